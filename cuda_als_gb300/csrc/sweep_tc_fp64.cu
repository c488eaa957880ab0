// sweep_tc_fp64.cu — instantiation of the tcgen05 half-sweep for padded size 64 (its own
// translation unit so the variants compile in parallel).
#include "sweep_tc_kernel.cuh"

namespace als {
namespace tcg {
cudaError_t configure_64(size_t smem) { return configure_fp<64, false>(smem); }
void launch_64(const Params &p, const Geometry &g, int grid, cudaStream_t st) {
    launch_fp<64, false>(p, g, grid, st);
}
}  // namespace tcg
}  // namespace als
