// Compensated FP32 instantiations of the fused directional passes for lines of 256 cells.
#include "pass_dispatch.cuh"
namespace gpss {
GPSS_DEFINE_COMP_N(256)
}
