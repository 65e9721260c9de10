// fengine.cu -- the F-engine: int8 frames -> channel spectra, one fused kernel.
//
// Replaces the reference's per-chunk chain zero_invalid_frames_kernel ->
// int8_to_float_kernel -> cufftExecR2C (corr-cuda/src/kernels.cu:130-174 and
// :806-835) with one persistent kernel per launch:
//
//   * each CTA walks a strided list of (frame, station) items;
//   * the int8 frame of the next item is prefetched into shared memory with a
//     TMA bulk copy (cp.async.bulk + mbarrier) while the current item computes,
//     so HBM latency is hidden behind the FFT;
//   * a frame whose validity bit is clear is never read: its spectrum is written
//     as zeros, which is what zeroing the samples and transforming them gives;
//   * the real frame x[0..L) (L = 2M) is packed as M complex points
//     z[n] = x[2n] + i*x[2n+1] and transformed by a Stockham autosort FFT in
//     shared memory (radix-16 passes, one final radix-2/4/8 pass), FP32 in
//     registers, twiddles from host-computed double-precision tables;
//   * the split X[k] = Fe[k] + w^k Fo[k] turns Z into the L-point real spectrum;
//     bins 0..M-1 are written, the Nyquist bin M is dropped and nothing is
//     normalised (reference semantics, HANDOFF.md:583-602).
//
// Output layout: y[(frame*n_station + station)*M + k], complex64. One row per
// (frame, station), channel-contiguous, so the X-engines read a channel tile of
// every station of a frame as n_station coalesced segments.

#include <cmath>
#include <vector>

#include "engine.h"
#include "ptx.cuh"

namespace corrgb {
namespace {

// Shared-memory index padding: one float2 of padding per 16, which makes the
// stride-16 scatter of the first Stockham pass conflict-free.
__device__ __forceinline__ int padi(int i) { return i + (i >> 4); }

// ---------------------------------------------------------------------------
// Small DFTs in registers, forward sign (exp(-2*pi*i*n*k/R)), natural order.
// ---------------------------------------------------------------------------

template <int R>
struct Dft;

template <>
struct Dft<2> {
    static __device__ __forceinline__ void run(float2 *v) {
        const float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

template <>
struct Dft<4> {
    static __device__ __forceinline__ void run(float2 *v) {
        const float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
        const float2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
        v[0] = cadd(s02, s13);
        v[2] = csub(s02, s13);
        v[1] = make_float2(d02.x + d13.y, d02.y - d13.x); // d02 - i*d13
        v[3] = make_float2(d02.x - d13.y, d02.y + d13.x); // d02 + i*d13
    }
};

// cos(pi/4), cos(pi/8), sin(pi/8)
#define CORR_H 0.70710678118654752440f
#define CORR_C1 0.92387953251128675613f
#define CORR_S1 0.38268343236508977173f

template <>
struct Dft<8> {
    static __device__ __forceinline__ void run(float2 *v) {
        float2 e[4] = {v[0], v[2], v[4], v[6]};
        float2 o[4] = {v[1], v[3], v[5], v[7]};
        Dft<4>::run(e);
        Dft<4>::run(o);
        // o[k] *= exp(-i*pi*k/4)
        o[1] = make_float2(CORR_H * (o[1].x + o[1].y), CORR_H * (o[1].y - o[1].x));
        o[2] = make_float2(o[2].y, -o[2].x);
        o[3] = make_float2(CORR_H * (o[3].y - o[3].x), -CORR_H * (o[3].x + o[3].y));
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[k] = cadd(e[k], o[k]);
            v[k + 4] = csub(e[k], o[k]);
        }
    }
};

template <>
struct Dft<16> {
    // 16 = 4 x 4: n = 4*n1 + n2, k = k1 + 4*k2.
    static __device__ __forceinline__ void run(float2 *v) {
        float2 b[4][4];
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) {
            float2 t[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
            Dft<4>::run(t);
#pragma unroll
            for (int k1 = 0; k1 < 4; ++k1) b[n2][k1] = t[k1];
        }
        // b[n2][k1] *= exp(-2*pi*i*n2*k1/16)
        const float2 w1 = make_float2(CORR_C1, -CORR_S1);
        const float2 w3 = make_float2(CORR_S1, -CORR_C1);
        const float2 w9 = make_float2(-CORR_C1, CORR_S1);
        b[1][1] = cmul(b[1][1], w1);
        b[1][2] = make_float2(CORR_H * (b[1][2].x + b[1][2].y), CORR_H * (b[1][2].y - b[1][2].x));
        b[1][3] = cmul(b[1][3], w3);
        b[2][1] = make_float2(CORR_H * (b[2][1].x + b[2][1].y), CORR_H * (b[2][1].y - b[2][1].x));
        b[2][2] = make_float2(b[2][2].y, -b[2][2].x);
        b[2][3] = make_float2(CORR_H * (b[2][3].y - b[2][3].x), -CORR_H * (b[2][3].x + b[2][3].y));
        b[3][1] = cmul(b[3][1], w3);
        b[3][2] = make_float2(CORR_H * (b[3][2].y - b[3][2].x), -CORR_H * (b[3][2].x + b[3][2].y));
        b[3][3] = cmul(b[3][3], w9);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            float2 t[4] = {b[0][k1], b[1][k1], b[2][k1], b[3][k1]};
            Dft<4>::run(t);
#pragma unroll
            for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
        }
    }
};

// exp(-2*pi*i*u/M) for 0 <= u < M from the two-level table in shared memory.
__device__ __forceinline__ float2 tw_pass(const float2 *lo, const float2 *hi, int u) {
    return cmul(lo[u & 63], hi[u >> 6]);
}

// v[r] *= w^r with w = exp(-2*pi*i*u/M). w, w^4 and w^8 are read from the
// table; the other powers are at most two products away from those.
template <int R>
__device__ __forceinline__ void apply_twiddles(float2 *v, int u, const float2 *lo,
                                               const float2 *hi) {
    const float2 w1 = tw_pass(lo, hi, u);
    if constexpr (R == 2) {
        v[1] = cmul(v[1], w1);
    } else {
        const float2 w2 = cmul(w1, w1);
        const float2 w3 = cmul(w2, w1);
        v[1] = cmul(v[1], w1);
        v[2] = cmul(v[2], w2);
        v[3] = cmul(v[3], w3);
        if constexpr (R >= 8) {
            const float2 w4 = tw_pass(lo, hi, 4 * u);
            v[4] = cmul(v[4], w4);
            v[5] = cmul(v[5], cmul(w4, w1));
            v[6] = cmul(v[6], cmul(w4, w2));
            v[7] = cmul(v[7], cmul(w4, w3));
            if constexpr (R == 16) {
                const float2 w8 = tw_pass(lo, hi, 8 * u);
                const float2 w12 = cmul(w8, w4);
                v[8] = cmul(v[8], w8);
                v[9] = cmul(v[9], cmul(w8, w1));
                v[10] = cmul(v[10], cmul(w8, w2));
                v[11] = cmul(v[11], cmul(w8, w3));
                v[12] = cmul(v[12], w12);
                v[13] = cmul(v[13], cmul(w12, w1));
                v[14] = cmul(v[14], cmul(w12, w2));
                v[15] = cmul(v[15], cmul(w12, w3));
            }
        }
    }
}

// One Stockham pass of radix R over M points with sub-transform size NS:
//   out[(j/NS)*NS*R + j%NS + r*NS] = DFT_R( in[j + r*M/R] * w^(r*(j%NS)) )
// Each of the T threads owns P = M/T points, i.e. P/R butterflies. The pass
// is in place: every thread reads all of its inputs, the CTA synchronises,
// then every thread writes. The first pass reads int8 pairs instead.
template <int M, int T, int R, int NS, bool FIRST>
__device__ __forceinline__ void fft_pass(float2 *__restrict__ sd, const char2 *__restrict__ sx,
                                         const float2 *lo, const float2 *hi, int tid) {
    constexpr int P = M / T;
    constexpr int NB = P / R;
    constexpr int STRIDE = M / R;
    static_assert(NB >= 1 && NB * R == P, "bad radix plan");
    float2 v[NB][R];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int j = tid + q * T;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = j + r * STRIDE;
            if constexpr (FIRST) {
                const char2 c = sx[i];
                v[q][r] = make_float2(static_cast<float>(c.x), static_cast<float>(c.y));
            } else {
                v[q][r] = sd[padi(i)];
            }
        }
        if constexpr (NS > 1) {
            const int u = (j & (NS - 1)) * (M / (NS * R));
            apply_twiddles<R>(v[q], u, lo, hi);
        }
        Dft<R>::run(v[q]);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int j = tid + q * T;
        const int base = (j & ~(NS - 1)) * R + (j & (NS - 1));
#pragma unroll
        for (int r = 0; r < R; ++r) sd[padi(base + r * NS)] = v[q][r];
    }
    __syncthreads();
}

template <int M, int T, int NS>
__device__ __forceinline__ void fft_rest(float2 *sd, const float2 *lo, const float2 *hi,
                                         int tid) {
    if constexpr (NS < M) {
        constexpr int REM = M / NS;
        constexpr int R = REM >= 16 ? 16 : REM;
        fft_pass<M, T, R, NS, false>(sd, nullptr, lo, hi, tid);
        fft_rest<M, T, NS * R>(sd, lo, hi, tid);
    }
}

struct TwPtrs {
    const float2 *pass_lo, *pass_hi, *post_lo, *post_hi;
};

template <int LOGM>
struct FeCfg {
    static constexpr int M = 1 << LOGM;
    static constexpr int P = (LOGM >= 13) ? 32 : 16;   // points per thread
    static constexpr int T = M / P;                    // threads per CTA
    static constexpr int N_PASS_HI = M / 64;
    static constexpr int N_POST_HI = M / 128 + 1;
    // shared memory layout (bytes)
    static constexpr int OFF_X0 = 0;                   // int8 frame, buffer 0
    static constexpr int OFF_X1 = 2 * M;               // int8 frame, buffer 1
    static constexpr int OFF_D = 4 * M;                // padded complex data
    static constexpr int OFF_PLO = OFF_D + (M + M / 16) * 8;
    static constexpr int OFF_PHI = OFF_PLO + 64 * 8;
    static constexpr int OFF_QLO = OFF_PHI + N_PASS_HI * 8;
    static constexpr int OFF_QHI = OFF_QLO + 64 * 8;
    static constexpr int OFF_BAR = (OFF_QHI + N_POST_HI * 8 + 15) / 16 * 16;
    static constexpr int OFF_FLAG = OFF_BAR + 16;
    static constexpr int SMEM = OFF_FLAG + 16;
    static constexpr int MIN_BLOCKS = (LOGM >= 14) ? 1 : (LOGM == 13 ? 2 : 1);
};

__device__ __forceinline__ bool frame_present(const FengineArgs &a, int f, int s) {
    if (a.mask == nullptr) return true;
    const int bit = a.mask_bit0 + f;
    const uint8_t byte = a.mask[static_cast<size_t>(s) * a.mask_station_stride + (bit >> 3)];
    return (byte >> (bit & 7)) & 1u;
}

template <int LOGM>
__global__ void __launch_bounds__(FeCfg<LOGM>::T, FeCfg<LOGM>::MIN_BLOCKS)
    fengine_kernel(FengineArgs a, TwPtrs tw) {
    using C = FeCfg<LOGM>;
    constexpr int M = C::M;
    constexpr int T = C::T;
    extern __shared__ __align__(128) unsigned char smem[];
    char2 *const sx0 = reinterpret_cast<char2 *>(smem + C::OFF_X0);
    char2 *const sx1 = reinterpret_cast<char2 *>(smem + C::OFF_X1);
    float2 *sd = reinterpret_cast<float2 *>(smem + C::OFF_D);
    float2 *plo = reinterpret_cast<float2 *>(smem + C::OFF_PLO);
    float2 *phi = reinterpret_cast<float2 *>(smem + C::OFF_PHI);
    float2 *qlo = reinterpret_cast<float2 *>(smem + C::OFF_QLO);
    float2 *qhi = reinterpret_cast<float2 *>(smem + C::OFF_QHI);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + C::OFF_BAR);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + C::OFF_FLAG);

    const int tid = threadIdx.x;
    for (int i = tid; i < 64; i += T) {
        plo[i] = tw.pass_lo[i];
        qlo[i] = tw.post_lo[i];
    }
    for (int i = tid; i < C::N_PASS_HI; i += T) phi[i] = tw.pass_hi[i];
    for (int i = tid; i < C::N_POST_HI; i += T) qhi[i] = tw.post_hi[i];
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        *abort_flag = 0;
        fence_mbar_init();
    }
    __syncthreads();

    const int n_items = a.frames * a.n_station;
    const uint32_t frame_bytes = 2u * M;
    auto src_of = [&](int item) {
        const int f = item / a.n_station;
        const int s = item - f * a.n_station;
        return a.samples + static_cast<size_t>(s) * a.station_stride +
               static_cast<size_t>(f) * a.frame_stride;
    };
    auto present = [&](int item) {
        const int f = item / a.n_station;
        return frame_present(a, f, item - f * a.n_station);
    };

    int item = blockIdx.x;
    if (tid == 0 && item < n_items && present(item)) {
        mbar_arrive_expect_tx(&bar[0], frame_bytes);
        bulk_copy_g2s(sx0, src_of(item), frame_bytes, &bar[0]);
    }
    uint32_t parity_bits = 0u;   // bit b = phase parity of bar[b]

    for (int n = 0; item < n_items; ++n, item += gridDim.x) {
        const int buf = n & 1;
        const int next = item + gridDim.x;
        bool next_issued = false;
        if (tid == 0 && next < n_items && present(next)) {
            // The other buffer was last read by the previous item's first
            // pass, which every thread finished before its first barrier.
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[buf ^ 1], frame_bytes);
            bulk_copy_g2s(buf ? sx0 : sx1, src_of(next), frame_bytes, &bar[buf ^ 1]);
            next_issued = true;
        }
        float2 *yrow = a.y + static_cast<size_t>(item) * M;

        if (!present(item)) {
            // Missing frame: its samples count as zeros, so does its spectrum.
            for (int k = tid; k < M; k += T) yrow[k] = make_float2(0.f, 0.f);
            continue;
        }

        if (!mbar_wait_bounded(&bar[buf], (parity_bits >> buf) & 1u, a.err,
                               kErrFengineCopyTimeout))
            *abort_flag = 1;
        __syncthreads();
        if (*abort_flag) {
            // Let whatever copy is still in flight land before the CTA exits.
            if (tid == 0 && next_issued)
                mbar_wait_bounded(&bar[buf ^ 1], (parity_bits >> (buf ^ 1)) & 1u, nullptr, 0);
            return;
        }
        parity_bits ^= 1u << buf;

        fft_pass<M, T, 16, 1, true>(sd, buf ? sx1 : sx0, plo, phi, tid);
        fft_rest<M, T, 16>(sd, plo, phi, tid);

        // Real split: X[k] = Fe + w^k Fo, X[M-k] = conj(Fe - w^k Fo), with
        // Fe = (Z[k] + conj(Z[M-k]))/2, Fo = -i (Z[k] - conj(Z[M-k]))/2.
#pragma unroll 4
        for (int k = tid; k < M / 2; k += T) {
            const float2 zk = sd[padi(k)];
            float2 zm = sd[padi((M - k) & (M - 1))];
            zm.y = -zm.y;
            const float2 fe = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y + zm.y));
            const float2 fo = make_float2(0.5f * (zk.y - zm.y), -0.5f * (zk.x - zm.x));
            const float2 w = cmul(qlo[k & 63], qhi[k >> 6]);
            const float2 wf = cmul(w, fo);
            yrow[k] = cadd(fe, wf);
            if (k != 0) yrow[M - k] = make_float2(fe.x - wf.x, wf.y - fe.y);
        }
        if (tid == 0) {
            const float2 zh = sd[padi(M / 2)];
            yrow[M / 2] = make_float2(zh.x, -zh.y);
        }
        // The next item's first pass synchronises before it overwrites sd.
    }
}

template <int LOGM>
corr_status launch_one(const FengineArgs &a, const TwiddleTables &tw, int num_sms,
                       cudaStream_t stream) {
    using C = FeCfg<LOGM>;
    static bool configured = false;
    static int per_sm = 1;
    if (!configured) {
        corr_status st = cuda_check(
            cudaFuncSetAttribute(fengine_kernel<LOGM>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM),
            "cudaFuncSetAttribute(fengine)");
        if (st != CORR_OK) return st;
        int blocks = 0;
        st = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                            &blocks, fengine_kernel<LOGM>, C::T, C::SMEM),
                        "cudaOccupancyMaxActiveBlocksPerMultiprocessor(fengine)");
        if (st != CORR_OK) return st;
        if (blocks < 1)
            return fail(CORR_ERR_INTERNAL, "F-engine kernel cannot be resident on an SM");
        per_sm = blocks;
        configured = true;
    }
    const int items = a.frames * a.n_station;
    if (items <= 0) return CORR_OK;
    int grid = num_sms * per_sm;
    if (grid > items) grid = items;
    TwPtrs p{tw.pass_lo, tw.pass_hi, tw.post_lo, tw.post_hi};
    fengine_kernel<LOGM><<<grid, C::T, C::SMEM, stream>>>(a, p);
    return cuda_check(cudaGetLastError(), "fengine_kernel launch");
}

int ilog2(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

} // namespace

corr_status fengine_prepare(int n_freq, TwiddleTables *tw) {
    const int M = n_freq;
    const double pi = 3.14159265358979323846;
    std::vector<float2> h_plo(64), h_phi(static_cast<size_t>(M / 64)), h_qlo(64),
        h_qhi(static_cast<size_t>(M / 128 + 1));
    for (int u = 0; u < 64; ++u) {
        const double a = -2.0 * pi * u / M;
        h_plo[u] = make_float2(static_cast<float>(std::cos(a)), static_cast<float>(std::sin(a)));
        const double b = -pi * u / M;
        h_qlo[u] = make_float2(static_cast<float>(std::cos(b)), static_cast<float>(std::sin(b)));
    }
    for (int u = 0; u < M / 64; ++u) {
        const double a = -2.0 * pi * 64.0 * u / M;
        h_phi[u] = make_float2(static_cast<float>(std::cos(a)), static_cast<float>(std::sin(a)));
    }
    for (int u = 0; u < M / 128 + 1; ++u) {
        const double b = -pi * 64.0 * u / M;
        h_qhi[u] = make_float2(static_cast<float>(std::cos(b)), static_cast<float>(std::sin(b)));
    }
    tw->n_pass_hi = M / 64;
    tw->n_post_hi = M / 128 + 1;
    const size_t n_all = 64 + h_phi.size() + 64 + h_qhi.size();
    float2 *d = nullptr;
    corr_status st = cuda_check(cudaMalloc(&d, n_all * sizeof(float2)), "cudaMalloc(twiddles)");
    if (st != CORR_OK) return st;
    std::vector<float2> all;
    all.reserve(n_all);
    all.insert(all.end(), h_plo.begin(), h_plo.end());
    all.insert(all.end(), h_phi.begin(), h_phi.end());
    all.insert(all.end(), h_qlo.begin(), h_qlo.end());
    all.insert(all.end(), h_qhi.begin(), h_qhi.end());
    st = cuda_check(cudaMemcpy(d, all.data(), n_all * sizeof(float2), cudaMemcpyHostToDevice),
                    "cudaMemcpy(twiddles)");
    if (st != CORR_OK) {
        cudaFree(d);
        return st;
    }
    tw->pass_lo = d;
    tw->pass_hi = d + 64;
    tw->post_lo = tw->pass_hi + h_phi.size();
    tw->post_hi = tw->post_lo + 64;
    return CORR_OK;
}

void fengine_release(TwiddleTables *tw) {
    if (tw->pass_lo != nullptr) cudaFree(tw->pass_lo);
    *tw = TwiddleTables{};
}

corr_status fengine_launch(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                           int num_sms, cudaStream_t stream) {
    switch (ilog2(n_freq)) {
    case 9: return launch_one<9>(a, tw, num_sms, stream);
    case 10: return launch_one<10>(a, tw, num_sms, stream);
    case 11: return launch_one<11>(a, tw, num_sms, stream);
    case 12: return launch_one<12>(a, tw, num_sms, stream);
    case 13: return launch_one<13>(a, tw, num_sms, stream);
    case 14: return launch_one<14>(a, tw, num_sms, stream);
    default:
        return failf(CORR_ERR_ARG, "F-engine: n_freq=%d is not a power of two in [512, 16384]",
                     n_freq);
    }
}

} // namespace corrgb
