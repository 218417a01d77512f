// Instantiations and launch of the generic-length directional pass
// (pass_generic.cuh) for both precisions.
#include "gpss_internal.h"
#include "pass_generic.cuh"

namespace gpss {

namespace {

template <typename T, int MODE> cudaError_t gen_launch_mode(const PassArgs<T> &a, const GenPlan &p, cudaStream_t s)
{
    auto k = gen_pass_kernel<T, MODE>;
    const size_t smem = 2 * (size_t)p.W * (size_t)p.n * sizeof(vec2<T>);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, nb = 0, nsm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, GEN_THREADS, smem)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if (nb < 1) return cudaErrorInvalidConfiguration;
    const int tiles = (a.nlines + p.W - 1) / p.W;
    const int grid = tiles < nb * nsm ? tiles : nb * nsm;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(GEN_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, a, p);
}

template <typename T> cudaError_t gen_launch(int mode, const PassArgs<T> &a, const GenPlan &p, cudaStream_t s)
{
    // the generic pass has none of the merged imaginary-time, adjoint, stacked
    // plane or compensated features
    if (a.nl_pre || a.dot_with || a.pre_out || a.adj_pre || a.plane_nl || a.plane_scale || a.comp)
        return cudaErrorInvalidValue;
    switch (mode) {
    case MODE_FUSED:
        if (!a.phase && !a.mask_lim) return cudaErrorInvalidValue;
        return gen_launch_mode<T, MODE_FUSED>(a, p, s);
    case MODE_FWD: return gen_launch_mode<T, MODE_FWD>(a, p, s);
    case MODE_INV: return gen_launch_mode<T, MODE_INV>(a, p, s);
    case MODE_DIAG: return gen_launch_mode<T, MODE_DIAG>(a, p, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_gen_f32(int mode, const PassArgs<float> &a, const GenPlan &p, cudaStream_t s)
{
    return gen_launch<float>(mode, a, p, s);
}
cudaError_t launch_gen_f64(int mode, const PassArgs<double> &a, const GenPlan &p, cudaStream_t s)
{
    return gen_launch<double>(mode, a, p, s);
}

}  // namespace gpss
