// Compensated FP32 instantiations of the fused directional passes (lines up
// to 32 cells) and the dispatch over the line length.
#include "pass_dispatch.cuh"
namespace gpss {
GPSS_DECLARE_COMP_N(64)
GPSS_DECLARE_COMP_N(128)
GPSS_DECLARE_COMP_N(256)

cudaError_t launch_comp_f32(bool xl, int n, const PassArgs<float> &a, int blocks, cudaStream_t s)
{
    switch (n) {
    case 2: return xl ? launch_comp_mode<2, true>(a, blocks, s) : launch_comp_mode<2, false>(a, blocks, s);
    case 4: return xl ? launch_comp_mode<4, true>(a, blocks, s) : launch_comp_mode<4, false>(a, blocks, s);
    case 8: return xl ? launch_comp_mode<8, true>(a, blocks, s) : launch_comp_mode<8, false>(a, blocks, s);
    case 16: return xl ? launch_comp_mode<16, true>(a, blocks, s) : launch_comp_mode<16, false>(a, blocks, s);
    case 32: return xl ? launch_comp_mode<32, true>(a, blocks, s) : launch_comp_mode<32, false>(a, blocks, s);
    case 64: return launch_comp_f32_64(xl, a, blocks, s);
    case 128: return launch_comp_f32_128(xl, a, blocks, s);
    case 256: return launch_comp_f32_256(xl, a, blocks, s);
    default: return cudaErrorInvalidValue;
    }
}
}  // namespace gpss
