// FP32 instantiations of the directional pass kernels for lines of 64 cells.
#include "pass_dispatch.cuh"
namespace gpss {
GPSS_DEFINE_PASS_N(float, f32, 64)
}
