// pass_dispatch.cuh -- host-side dispatch from run-time (mode, layout, n) to
// the pass_kernel instantiation.  Included once per precision.
#pragma once
#include "pass_kernel.cuh"
#include "pass_pipe.cuh"

namespace gpss {

// `tiles` = ceil(nlines / lines per CTA).  The grid is the smaller of that and
// GPSS_PASS_WAVES full waves of resident CTAs (0: no cap); the kernel loops
// over the remaining tiles.
#ifndef GPSS_PASS_WAVES
#define GPSS_PASS_WAVES 1
#endif

// SMs of the current device (cached per device)
static int sm_count()
{
    static int cache[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 1;
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) return 1;
        cache[dev] = n;
    }
    return cache[dev];
}

template <typename T, int N, bool XL, int MODE, int FEAT = FEAT_ALL>
static cudaError_t launch_pass_inst(const PassArgs<T> &a, int tiles, cudaStream_t s)
{
    using S = PassShape<T, N, XL, FEAT>;
    tiles = (a.nlines + S::W - 1) / S::W;  // this instantiation's tiles (the host counts default ones)
    auto k = pass_kernel<T, N, XL, MODE, FEAT>;
    static int wave[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    const bool cached = dev >= 0 && dev < 64 && wave[dev] > 0;
    int grid_cap = cached ? wave[dev] : 0;
    if (!cached) {
        // opt in to the dynamic shared memory this instantiation needs (the
        // default limit counts dynamic + static bytes against 48 KB) and size
        // one wave from the occupancy; once per device.  The shared/L1 split
        // stays the driver's choice: forcing the largest shared carveout
        // (smallest L1) made the 256^3 passes 13-16% slower.
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM_BYTES);
        if (e != cudaSuccess) return e;
        int nb = 0, nsm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, S::THREADS, S::SMEM_BYTES);
        if (e != cudaSuccess) return e;
        e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        if (nb < 1) return cudaErrorInvalidConfiguration;
        grid_cap = GPSS_PASS_WAVES > 0 ? nb * nsm * GPSS_PASS_WAVES : (1 << 30);
        if (dev >= 0 && dev < 64) wave[dev] = grid_cap;
    }
    const int grid = tiles < grid_cap ? tiles : grid_cap;
    // programmatic stream serialization: the kernel waits for the previous
    // grid itself (griddepcontrol.wait) after loading its constant tables
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(S::THREADS);
    cfg.dynamicSmemBytes = S::SMEM_BYTES;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, a);
}

// compensated FP32 fused passes (FEAT_COMP), instantiated in pass_f32c*.cu
cudaError_t launch_comp_f32(bool xl, int n, const PassArgs<float> &a, int blocks, cudaStream_t s);

template <int N, bool XL>
static cudaError_t launch_comp_mode(const PassArgs<float> &a, int blocks, cudaStream_t s)
{
    // the split-step kinetic passes only: phase, prescale, NL epilogue, sums,
    // and the discrete adjoint's epilogues (pre_out, adj_pre)
    if (a.mask_lim || a.acc || a.nl_pre || a.dot_with || a.plane_nl || a.plane_scale || !a.phase)
        return cudaErrorInvalidValue;
    const bool diag = (a.red & (RED_POINT | RED_KIN)) || a.prow != 0;
    const bool nl = a.nl_mode != NL_NONE || (a.red & RED_MASS);
    if (a.pre_out || a.adj_pre) {  // per-thread grids: the adjoint runs without the mass lock
        if (diag || a.grid_mass || a.red) return cudaErrorInvalidValue;
        if (nl) return launch_pass_inst<float, N, XL, MODE_FUSED, FEAT_COMP | FEAT_ADJ | FEAT_NL>(a, blocks, s);
        return launch_pass_inst<float, N, XL, MODE_FUSED, FEAT_COMP | FEAT_ADJ>(a, blocks, s);
    }
    if (diag) return launch_pass_inst<float, N, XL, MODE_FUSED, FEAT_COMP | FEAT_ALL>(a, blocks, s);
    if (a.grid_mass) {  // one grid per pass from the mass bound
        if (nl) return launch_pass_inst<float, N, XL, MODE_FUSED, FEAT_COMP | FEAT_GRIDM | FEAT_NL>(a, blocks, s);
        return launch_pass_inst<float, N, XL, MODE_FUSED, FEAT_COMP | FEAT_GRIDM>(a, blocks, s);
    }
    if (nl) return launch_pass_inst<float, N, XL, MODE_FUSED, FEAT_COMP | FEAT_NL>(a, blocks, s);
    return launch_pass_inst<float, N, XL, MODE_FUSED, FEAT_COMP>(a, blocks, s);
}

template <typename T, int N, bool XL>
static cudaError_t launch_pass_mode(int mode, const PassArgs<T> &a, int blocks, cudaStream_t s)
{
    if constexpr (sizeof(T) == 4) {
        if (mode == MODE_FUSED && a.comp) return launch_comp_f32(XL, N, a, blocks, s);
    }
    switch (mode) {
    case MODE_FUSED: {
        // the leanest instantiation that does everything the arguments ask for
        const bool adj = a.pre_out != nullptr || a.adj_pre != nullptr;
        const bool diag = (a.red & (RED_POINT | RED_KIN)) || a.prow != 0;
        const bool acc = a.acc != nullptr;
        const bool nl = a.nl_mode != NL_NONE || (a.red & RED_MASS);
        if (a.mask_lim) {
            if (diag || acc || adj || nl || a.nl_pre || a.dot_with) return cudaErrorInvalidValue;
            return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_MASK>(a, blocks, s);
        }
        if (!a.phase) return cudaErrorInvalidValue;  // every other fused pass reads a phase table
        if (a.nl_pre || a.dot_with) {
            if (diag || acc || adj || a.nl_mode != NL_NONE) return cudaErrorInvalidValue;
            return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_IMAGM>(a, blocks, s);
        }
        if constexpr (sizeof(T) == 4 && N >= 64) {
            if (a.plane_nl || a.plane_scale) {
                if (diag || acc || adj) return cudaErrorInvalidValue;  // planes: no energy sums, rotation, adjoint
                if (nl) return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_PLANE | FEAT_NL>(a, blocks, s);
                return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_PLANE>(a, blocks, s);
            }
        }
        if constexpr (sizeof(T) == 4 && !XL && N >= 64) {
            // y/z columns of a 3D field with a tensor map: tiles arrive by TMA
            if (a.tmap && !diag && !acc && !adj) {
                if (nl) return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_TMA | FEAT_NL>(a, blocks, s);
                return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_TMA>(a, blocks, s);
            }
        }
        if (diag || (acc && (adj || nl))) return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_ALL>(a, blocks, s);
        if (acc) return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_ACC>(a, blocks, s);
        if constexpr (sizeof(T) == 4 && !XL && N >= 64) {
            // fewer default tiles than SMs: the 128-thread y/z instantiation
            if (blocks < sm_count()) {
                constexpr int kSmallAdjNL = FEAT_ADJ | FEAT_NL | FEAT_SMALL;
                if (adj && nl) return launch_pass_inst<T, N, XL, MODE_FUSED, kSmallAdjNL>(a, blocks, s);
                if (adj) return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_ADJ | FEAT_SMALL>(a, blocks, s);
                if (nl) return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_NL | FEAT_SMALL>(a, blocks, s);
                return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_SMALL>(a, blocks, s);
            }
        }
        if (adj) {
            if (nl) return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_ADJ | FEAT_NL>(a, blocks, s);
            return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_ADJ>(a, blocks, s);
        }
        if (nl) return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_NL>(a, blocks, s);
        return launch_pass_inst<T, N, XL, MODE_FUSED, FEAT_NONE>(a, blocks, s);
    }
    case MODE_FWD: return launch_pass_inst<T, N, XL, MODE_FWD>(a, blocks, s);
    case MODE_INV: return launch_pass_inst<T, N, XL, MODE_INV>(a, blocks, s);
    case MODE_DIAG: return launch_pass_inst<T, N, XL, MODE_DIAG>(a, blocks, s);
    default: return cudaErrorInvalidValue;
    }
}

template <typename T, int N>
static cudaError_t launch_pass_n(int mode, bool xl, const PassArgs<T> &a, int blocks, cudaStream_t s)
{
    return xl ? launch_pass_mode<T, N, true>(mode, a, blocks, s)
              : launch_pass_mode<T, N, false>(mode, a, blocks, s);
}

template <typename T, int N, bool XL>
static cudaError_t launch_pipe_inst(const PassArgs<T> &a, int ntiles, cudaStream_t s)
{
    using S = PipeShape<T, N, XL>;
    auto k = pass_pipe_kernel<T, N, XL>;
    static int blocks_per_sm[64] = {0};
    static int sms[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    const int d = (dev >= 0 && dev < 64) ? dev : 0;
    if (!blocks_per_sm[d] || dev != d) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM_BYTES);
        if (e != cudaSuccess) return e;
        int nb = 0, nsm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, S::THREADS, S::SMEM_BYTES);
        if (e != cudaSuccess) return e;
        e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        if (nb < 1) return cudaErrorInvalidConfiguration;
        blocks_per_sm[d] = nb;
        sms[d] = nsm;
    }
    int grid = blocks_per_sm[d] * sms[d];
    if (grid > ntiles) grid = ntiles;
    k<<<grid, S::THREADS, S::SMEM_BYTES, s>>>(a, ntiles);
    return cudaGetLastError();
}

template <typename T, int N> static int lines_per_cta_n(bool xl)
{
    return xl ? PassShape<T, N, true>::W : PassShape<T, N, false>::W;
}

// The instantiations for n = 64, 128 and 256 (the large ones) live in their
// own translation units (pass_<prec>_<n>.cu), compiled in parallel.
#define GPSS_DECLARE_PASS_N(T, SUFFIX, N)                                                      \
    cudaError_t launch_pass_##SUFFIX##_##N(int mode, bool xl, const PassArgs<T> &a, int blocks, \
                                           cudaStream_t s);
#define GPSS_DEFINE_PASS_N(T, SUFFIX, N)                                                       \
    cudaError_t launch_pass_##SUFFIX##_##N(int mode, bool xl, const PassArgs<T> &a, int blocks, \
                                           cudaStream_t s)                                     \
    {                                                                                          \
        return launch_pass_n<T, N>(mode, xl, a, blocks, s);                                    \
    }

#define GPSS_DEFINE_PASS_DISPATCH(T, SUFFIX)                                                   \
    GPSS_DECLARE_PASS_N(T, SUFFIX, 64)                                                         \
    GPSS_DECLARE_PASS_N(T, SUFFIX, 128)                                                        \
    GPSS_DECLARE_PASS_N(T, SUFFIX, 256)                                                        \
    cudaError_t launch_pipe_##SUFFIX(bool xl, int n, const PassArgs<T> &a, int ntiles,         \
                                     cudaStream_t s)                                           \
    {                                                                                          \
        switch (n) {                                                                           \
        case 64: return xl ? launch_pipe_inst<T, 64, true>(a, ntiles, s)                       \
                           : launch_pipe_inst<T, 64, false>(a, ntiles, s);                     \
        case 128: return xl ? launch_pipe_inst<T, 128, true>(a, ntiles, s)                     \
                            : launch_pipe_inst<T, 128, false>(a, ntiles, s);                   \
        case 256: return xl ? launch_pipe_inst<T, 256, true>(a, ntiles, s)                     \
                            : launch_pipe_inst<T, 256, false>(a, ntiles, s);                   \
        default: return cudaErrorInvalidValue;                                                 \
        }                                                                                      \
    }                                                                                          \
    cudaError_t launch_pass_##SUFFIX(int mode, bool xl, int n, const PassArgs<T> &a,           \
                                     int blocks, cudaStream_t s)                               \
    {                                                                                          \
        switch (n) {                                                                           \
        case 2: return launch_pass_n<T, 2>(mode, xl, a, blocks, s);                            \
        case 4: return launch_pass_n<T, 4>(mode, xl, a, blocks, s);                            \
        case 8: return launch_pass_n<T, 8>(mode, xl, a, blocks, s);                            \
        case 16: return launch_pass_n<T, 16>(mode, xl, a, blocks, s);                          \
        case 32: return launch_pass_n<T, 32>(mode, xl, a, blocks, s);                          \
        case 64: return launch_pass_##SUFFIX##_64(mode, xl, a, blocks, s);                     \
        case 128: return launch_pass_##SUFFIX##_128(mode, xl, a, blocks, s);                   \
        case 256: return launch_pass_##SUFFIX##_256(mode, xl, a, blocks, s);                   \
        default: return cudaErrorInvalidValue;                                                 \
        }                                                                                      \
    }                                                                                          \
    int pass_lines_per_cta_##SUFFIX(int n, bool xl)                                            \
    {                                                                                          \
        switch (n) {                                                                           \
        case 2: return lines_per_cta_n<T, 2>(xl);                                              \
        case 4: return lines_per_cta_n<T, 4>(xl);                                              \
        case 8: return lines_per_cta_n<T, 8>(xl);                                              \
        case 16: return lines_per_cta_n<T, 16>(xl);                                            \
        case 32: return lines_per_cta_n<T, 32>(xl);                                            \
        case 64: return lines_per_cta_n<T, 64>(xl);                                            \
        case 128: return lines_per_cta_n<T, 128>(xl);                                          \
        case 256: return lines_per_cta_n<T, 256>(xl);                                          \
        default: return 0;                                                                     \
        }                                                                                      \
    }

#define GPSS_DEFINE_COMP_N(N)                                                                    \
    cudaError_t launch_comp_f32_##N(bool xl, const PassArgs<float> &a, int blocks, cudaStream_t s) \
    {                                                                                          \
        return xl ? launch_comp_mode<N, true>(a, blocks, s) : launch_comp_mode<N, false>(a, blocks, s); \
    }
#define GPSS_DECLARE_COMP_N(N)                                                                   \
    cudaError_t launch_comp_f32_##N(bool xl, const PassArgs<float> &a, int blocks, cudaStream_t s);

}  // namespace gpss
