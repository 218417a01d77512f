// FP64 instantiations of the directional pass kernels.
#include "pass_dispatch.cuh"
namespace gpss {
GPSS_DEFINE_PASS_DISPATCH(double, f64)
}
