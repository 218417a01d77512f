// FP64 instantiations of the directional pass kernels for lines of 128 cells.
#include "pass_dispatch.cuh"
namespace gpss {
GPSS_DEFINE_PASS_N(double, f64, 128)
}
