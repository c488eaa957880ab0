// sweep_tc_fp128.cu — instantiation of the tcgen05 half-sweep for padded size 128 (its own
// translation unit so the variants compile in parallel).
#include "sweep_tc_kernel.cuh"

namespace als {
namespace tcg {
cudaError_t configure_128(size_t smem) { return configure_fp<128, false>(smem); }
void launch_128(const Params &p, const Geometry &g, int grid, cudaStream_t st) {
    launch_fp<128, false>(p, g, grid, st);
}
}  // namespace tcg
}  // namespace als
