// pass_pipe.cuh -- persistent, pipelined form of the fused directional pass.
//
// Same arithmetic as pass_kernel<MODE_FUSED> (stage A / B / C of a line
// FFT -> phase -> iFFT, nonlinear epilogue, reductions), but tiles move
// between HBM and shared memory by the asynchronous bulk-copy engine:
//
//   * a CTA owns tiles blockIdx.x, blockIdx.x + gridDim.x, ... (W lines each);
//   * S = 3 tile buffers: while tile i is computed, tile i+1 is being loaded
//     and tile i-1 is being stored, so HBM traffic overlaps the FFT work;
//   * a tile is transformed in place in its buffer: raw layout on arrival,
//     (k1, r) working layout between the stages, raw layout again for the
//     store, so no per-element global address arithmetic is left in the
//     compute;
//   * x lines (contiguous) arrive as one bulk copy per tile; y/z tiles (W
//     adjacent columns, one row of W values per position) as one bulk copy
//     per row, issued by the lanes of warp 0.
//
// Shared-memory layouts (slots of one complex value):
//   XL   raw(w, p) = w*N + p;  work(w, k1, r) = w*N + k1*N2 + (r ^ (k1 mod N2))
//        (the XOR spreads a stage-B gather over all banks without padding)
//   COL  raw(w, p) = p*W + w;  work(w, k1, r) = (k1*N2 + r)*W + w
//
// Every wait on a barrier is bounded; on timeout the CTA records status 2
// (reported as GPSS_ETIMEOUT), waits for its own copies and returns.
#pragma once
#include "bulk_async.cuh"
#include "pass_kernel.cuh"

namespace gpss {

template <typename T, int N, bool XL> struct PipeShape {
    static constexpr int N1 = Split<N>::N1;
    static constexpr int N2 = Split<N>::N2;
    static constexpr int P = N2;
    static constexpr int THREADS = 256;
    static constexpr int W = THREADS / P;
    static constexpr int S = 3;  // tile buffers
    static constexpr int TILE = W * N;  // complex slots per tile
    static constexpr size_t TILE_BYTES = sizeof(vec2<T>) * TILE;
    static constexpr size_t ROW_BYTES = sizeof(vec2<T>) * W;  // COL: one position of W lines
    // buffers, twiddles A/B (hi, lo), phase (hi, lo), barriers
    static constexpr size_t SMEM_BYTES = S * TILE_BYTES + sizeof(vec2<T>) * 6 * N + 8 * S;
};

constexpr uint32_t kPipeWaitPolls = 1u << 22;

template <typename T, int N, bool XL>
__global__ void __launch_bounds__(256)
pass_pipe_kernel(const PassArgs<T> a, int ntiles)
{
    using V = vec2<T>;
    using S = PipeShape<T, N, XL>;
    constexpr int N1 = S::N1, N2 = S::N2, P = S::P, W = S::W, THREADS = S::THREADS, NS = S::S;

    extern __shared__ __align__(128) unsigned char smem_raw[];
    V *bufs = reinterpret_cast<V *>(smem_raw);
    V *stw = bufs + NS * S::TILE;   // stage A: hi[N], lo[N]
    V *stwB = stw + 2 * N;          // stage B: hi[N], lo[N]
    V *sph = stw + 4 * N;           // phase: hi[N], lo[N]
    uint64_t *bar = reinterpret_cast<uint64_t *>(sph + 2 * N);

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < 4 * N; i += THREADS) stw[i] = a.tw[i];
    if (a.prow == 0)
        for (int i = tid; i < 2 * N; i += THREADS) sph[i] = a.phase[i];
    if (tid == 0) {
        for (int b = 0; b < NS; b++) mbar_init(&bar[b], 1);
        fence_mbar_init();
    }
    __syncthreads();

    const int w = XL ? tid / P : tid % W;
    const int r = XL ? tid % P : tid / W;
    auto raw = [&](int p) -> int {
        if constexpr (XL) return w * N + p;
        else return p * W + w;
    };
    auto work = [&](int k1, int rr) -> int {
        if constexpr (XL) return w * N + k1 * N2 + (rr ^ (k1 & (N2 - 1)));
        else return (k1 * N2 + rr) * W + w;
    };
    auto line_base = [&](int g) -> int64_t {
        return (int64_t)(g % a.m0) * a.s0 + (int64_t)(g / a.m0) * a.s1;
    };
    // issue the copies that bring tile `t` into buffer `b` (warp 0)
    auto load_tile = [&](int t, int b) {
        V *dst = bufs + b * S::TILE;
        const int g0 = t * W;
        if (lane == 0) mbar_arrive_expect_tx(&bar[b], (uint32_t)S::TILE_BYTES);
        __syncwarp();
        if constexpr (XL) {
            if (lane == 0) bulk_g2s(dst, a.in + line_base(g0), (uint32_t)S::TILE_BYTES, &bar[b]);
        } else {
            const int64_t b0 = line_base(g0);
            for (int p = lane; p < N; p += 32)
                bulk_g2s(dst + p * W, a.in + b0 + (int64_t)p * a.stride, (uint32_t)S::ROW_BYTES, &bar[b]);
        }
    };
    auto store_tile = [&](int t, int b) {
        const V *src = bufs + b * S::TILE;
        const int g0 = t * W;
        if constexpr (XL) {
            if (lane == 0) bulk_s2g(a.out + line_base(g0), src, (uint32_t)S::TILE_BYTES);
        } else {
            const int64_t b0 = line_base(g0);
            for (int p = lane; p < N; p += 32)
                bulk_s2g(a.out + b0 + (int64_t)p * a.stride, src + p * W, (uint32_t)S::ROW_BYTES);
        }
        bulk_commit();
    };

    const bool scaled = a.scale != nullptr;
    const T scale = scaled ? load_scale<T>(a.scale) : (T)1;
    const T kmult = a.kmult;
    T acc_mass = 0, acc_pot = 0, acc_int = 0, acc_kin = 0, acc_rot = 0;
    const NLConst<T> nlc = nl_const<T>(a.nl_split, a.nl_beta, a.nl_dt);
    const bool imag = a.nl_mode == NL_IMAG;
    bool timed_out = false;
    int wait_b = 0, pref_b = -1;       // barriers with loads possibly in flight at a timeout
    uint32_t wait_par = 0, pref_par = 0;

    if (warp == 0 && (int)blockIdx.x < ntiles) load_tile(blockIdx.x, 0);

    for (int it = 0;; it++) {
        const int tile = blockIdx.x + it * gridDim.x;
        if (tile >= ntiles) break;
        const int b = it % NS;
        // prefetch the next tile; its buffer last held tile it-2, whose store
        // (all but this lane's newest bulk group) must have finished reading
        const int nt = tile + gridDim.x;
        if (warp == 0 && nt < ntiles) {
            bulk_wait_read<1>();
            __syncwarp();
            load_tile(nt, (it + 1) % NS);
        }
        wait_b = b;
        wait_par = (uint32_t)((it / NS) & 1);
        pref_b = nt < ntiles ? (it + 1) % NS : -1;
        pref_par = (uint32_t)(((it + 1) / NS) & 1);
        const bool ok = mbar_wait_bounded(&bar[b], wait_par, a.wait_polls ? a.wait_polls - 1 : kPipeWaitPolls);
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        V *buf = bufs + b * S::TILE;
        const int g = tile * W + w;
        const int row = g % a.rowmod;

        // ---- stage A
        V v[N1];
#pragma unroll
        for (int j = 0; j < N1; j++) v[j] = buf[raw(r + N2 * j)];
        dft<N1, -1>(v);
        __syncthreads();  // the raw tile has been read by every thread
#pragma unroll
        for (int k1 = 0; k1 < N1; k1++) {
            const int m = k1 * N2 + r;
            buf[work(k1, r)] = (k1 == 0 || r == 0) ? v[k1] : cmul2(v[k1], stw[m], stw[N + m]);
        }
        __syncthreads();
        // ---- stage B (each (k1, rr) is read and rewritten by the same thread)
        constexpr int NI = N1 / N2;
#pragma unroll
        for (int i = 0; i < NI; i++) {
            const int k1 = r + P * i;
            V u[N2];
#pragma unroll
            for (int rr = 0; rr < N2; rr++) u[rr] = buf[work(k1, rr)];
            dft<N2, -1>(u);
            if (a.red & RED_KIN) {
                T s2 = 0, s1 = 0;
#pragma unroll
                for (int k2 = 0; k2 < N2; k2++) {
                    const int k = k1 + N1 * k2;
                    const int kk = k < N / 2 ? k : k - N;
                    const T xi = (T)kk * kmult;
                    const T m2 = u[k2].x * u[k2].x + u[k2].y * u[k2].y;
                    s2 += xi * xi * m2;
                    s1 += xi * m2;
                }
                acc_kin += s2 * (T)(1.0 / N);
                if (a.coord) acc_rot += s1 * (T)(1.0 / N) * (T)a.coord[row];
            }
#pragma unroll
            for (int k2 = 0; k2 < N2; k2++) {
                const int k = k1 + N1 * k2;
                const V ph = a.prow ? a.phase[row * a.prow + k] : sph[k];
                const V pl = a.prow ? a.phase[row * a.prow + N + k] : sph[N + k];
                u[k2] = cmul2(u[k2], ph, pl);
                if (scaled) u[k2] = cscale(u[k2], scale);
            }
            dft<N2, +1>(u);
#pragma unroll
            for (int rr = 0; rr < N2; rr++) {
                const int mb = rr * N1 + k1;
                buf[work(k1, rr)] = (k1 == 0 || rr == 0) ? u[rr] : cmulc2(u[rr], stwB[mb], stwB[N + mb]);
            }
        }
        __syncthreads();
        // ---- stage C
#pragma unroll
        for (int k1 = 0; k1 < N1; k1++) v[k1] = buf[work(k1, r)];
        dft<N1, +1>(v);
        const int64_t gb = (a.V || (a.red & RED_POINT)) ? line_base(g) : 0;
        if (a.nl_mode != NL_NONE) {
#pragma unroll
            for (int j = 0; j < N1; j++) {
                const T vv = a.V ? a.V[gb + (int64_t)(r + N2 * j) * a.stride] : (T)0;
                v[j] = nl_apply(v[j], vv, nlc, imag);
            }
        }
        if (a.red & RED_POINT) {
#pragma unroll
            for (int j = 0; j < N1; j++) {
                const T rho = v[j].x * v[j].x + v[j].y * v[j].y;
                acc_mass += rho;
                acc_int += rho * rho;
                if (a.V) acc_pot += a.V[gb + (int64_t)(r + N2 * j) * a.stride] * rho;
            }
        } else if (a.red & RED_MASS) {
#pragma unroll
            for (int j = 0; j < N1; j++) acc_mass += v[j].x * v[j].x + v[j].y * v[j].y;
        }
        __syncthreads();  // every (k1, r) has been read
#pragma unroll
        for (int j = 0; j < N1; j++) buf[raw(r + N2 * j)] = v[j];
        fence_proxy_async_smem();
        __syncthreads();
        if (warp == 0) store_tile(tile, b);
    }

    if (timed_out) {
        if (tid == 0 && a.fin_status) atomicOr(a.fin_status, 2);
        // let in-flight loads land (bounded) before the CTA releases its shared memory
        mbar_wait_bounded(&bar[wait_b], wait_par, kPipeWaitPolls);
        if (pref_b >= 0) mbar_wait_bounded(&bar[pref_b], pref_par, kPipeWaitPolls);
    }
    if (warp == 0) bulk_wait<0>();

    if (a.red) {
        __shared__ T red_smem[THREADS / 32];
        if (a.red & (RED_POINT | RED_MASS)) block_sum_store<T, THREADS>(acc_mass, a.partials, RQ_MASS, red_smem);
        if (a.red & RED_POINT) {
            block_sum_store<T, THREADS>(acc_pot, a.partials, RQ_POT, red_smem);
            block_sum_store<T, THREADS>(acc_int, a.partials, RQ_INT, red_smem);
        }
        if (a.red & RED_KIN) {
            block_sum_store<T, THREADS>(acc_kin, a.partials, RQ_KIN, red_smem);
            block_sum_store<T, THREADS>(acc_rot, a.partials, RQ_ROT, red_smem);
        }
        unsigned qmask = 0;
        if (a.red & (RED_POINT | RED_MASS)) qmask |= 1u << RQ_MASS;
        if (a.red & RED_POINT) qmask |= (1u << RQ_POT) | (1u << RQ_INT);
        if (a.red & RED_KIN) qmask |= (1u << RQ_KIN) | (1u << RQ_ROT);
        finish_reduction<T, THREADS>(a, qmask);
    }
}

}  // namespace gpss
