// FP32 instantiations of the directional pass kernels (lines up to 32 cells,
// the pipelined kernel) and the dispatch over the line length.
#include "pass_dispatch.cuh"
namespace gpss {
GPSS_DEFINE_PASS_DISPATCH(float, f32)
}
