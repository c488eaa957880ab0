// sweep_tc_fp32_e4m3.cu — instantiation of the tcgen05 half-sweep with FP8 (e4m3) operands
// for padded size 32 (its own translation unit so the variants compile in parallel).
#include "sweep_tc_kernel.cuh"

namespace als {
namespace tcg {
cudaError_t configure_32_e4m3(size_t smem) { return configure_fp<32, true>(smem); }
void launch_32_e4m3(const Params &p, const Geometry &g, int grid, cudaStream_t st) {
    launch_fp<32, true>(p, g, grid, st);
}
}  // namespace tcg
}  // namespace als
