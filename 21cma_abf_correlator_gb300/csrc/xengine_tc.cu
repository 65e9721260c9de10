// xengine_tc.cu -- tensor-core X-engine: tcgen05 MMA, FP16 spectra, FP32 in TMEM.
//
// The same sum as the plain X-engine (reference corr_kernel,
// corr-cuda/src/kernels.cu:194-265), recast as one small real GEMM per channel.
// For channel c let D be the frames x 2N real matrix whose columns are
// (Re Y_0, Im Y_0, Re Y_1, Im Y_1, ...). Then S = D^T D holds everything:
//     Re V[j,k] = S[2j][2k] + S[2j+1][2k+1]
//     Im V[j,k] = S[2j+1][2k] - S[2j][2k+1]
// The tensor cores compute S with K = frames, FP16 operands and FP32 accumulation
// in tensor memory (TMEM), accumulated over the whole launch.
//
// Precision forms:
//   FP16       : D rounded once to FP16 (11-bit significand); one MMA per K step.
//   FP16 split : D = Dh + Dl, Dh = fp16(D), Dl = fp16(D - Dh) (about 22 bits).
//                S ~ Dh^T Dh + Dh^T Dl + Dl^T Dh, the Dl^T Dl term dropped: three
//                MMAs per K step into the same accumulator.
// Scale: spectra of int8 frames satisfy |Y| <= 128*L, so multiplying by the
// power of two 2^-(log2 L - 8) keeps every value below 2^15 (< FP16 max) in
// every channel for every input; being a power of two it is undone exactly.
// The int8 quantisation floor keeps |Y| >= ~sqrt(L/12) in every channel of real
// data, so the scaled values sit in FP16's normal range and no per-channel
// adaptive scale is needed.
//
// Persistent CTAs (one per SM: TMEM), 256 threads, CT channels per tile (CT/4
// spectra tiles, each a contiguous block per stage in the channel-tiled layout):
//   * thread 0 streams KT = 16 frames x N stations x CT channels of FP32 spectra
//     per stage into a 3-deep shared-memory ring with 1-D TMA bulk copies
//     (cp.async.bulk + mbarrier), running ahead across tile boundaries;
//   * all threads convert a landed stage (scale, round, split) into the K-major
//     no-swizzle UMMA operand layout (8-row x 16-byte core matrices), 2-deep;
//   * thread 0 issues the stage's tcgen05.mma (M=128, N=2N rounded to 16, K=16)
//     and commits them to the operand buffer's mbarrier;
//   * after a tile's last stage: commit, wait, tcgen05.ld the accumulators, form
//     V and add it into the row; the next tile's loads are already in flight.
// Every wait is clock-bounded.

#include <algorithm>

#include <cuda_fp16.h>

#include "engine.h"
#include "ptx.cuh"

namespace corrgb {
namespace {

constexpr int kThreads = 256;
constexpr int kKT = 16;                      // frames per stage = one MMA K step
constexpr int kLoadStages = 3;               // fp32 ring depth (TMA)
constexpr int kOpStages = 2;                 // operand ring depth
constexpr int kSBO = (kKT / 8) * 128;        // bytes per 8-row group (all K of a stage)
constexpr int kLBO = 128;                    // bytes between K-adjacent core matrices

struct TcGeom {
    int n_station;
    int lo_row;        // first Dl row (2N rounded up to 8); split form only
    int rows_valid;    // rows written per channel
    int n_mma;         // 2N rounded up to a multiple of 16 (MMA N, TMEM columns)
    int ct;            // channels per tile (multiple of kYTile)
    int tmem_cols;     // allocated columns (power of two >= 32)
    int chan_stride;   // operand bytes per channel (+16 B bank skew)
    int op_stage;      // operand bytes per stage (incl. slack read by the last A)
    int ld_stage;      // fp32 bytes per stage = KT * N * CT * 8
    int e_stride;      // floats per epilogue row
    int epi_bytes;
    int smem;
    bool split;
};

TcGeom make_geom(int n_station, bool split) {
    TcGeom g{};
    g.n_station = n_station;
    g.split = split;
    g.lo_row = (2 * n_station + 7) / 8 * 8;
    g.rows_valid = split ? g.lo_row + 2 * n_station : 2 * n_station;
    g.n_mma = std::max(16, (2 * n_station + 15) / 16 * 16);
    int ct = 8;
    while (ct > kYTile && ct * g.n_mma > 512) ct /= 2;
    g.ct = ct;
    int cols = 32;
    while (cols < ct * g.n_mma) cols *= 2;
    g.tmem_cols = cols;
    const int groups = (g.rows_valid + 7) / 8;
    g.chan_stride = groups * kSBO + 16;
    // rows read from a channel base: A reads 128 rows from Dh (and from Dl in
    // the split form), B reads n_mma rows from the same bases
    const int max_row = std::max((split ? g.lo_row : 0) + 128, g.rows_valid);
    const int slack = std::max(0, (max_row + 7) / 8 * kSBO - g.chan_stride) + 128;
    g.op_stage = (g.ct * g.chan_stride + slack + 127) / 128 * 128;
    g.ld_stage = kKT * n_station * g.ct * 8;
    g.e_stride = g.n_mma + 1;
    const int n_baseline = n_station * (n_station + 1) / 2;
    g.epi_bytes = (128 * g.e_stride * 4 + 15) / 16 * 16 + n_baseline * g.ct * 8;
    // the epilogue reuses the operand ring (free once a tile's MMAs are done)
    g.smem = kLoadStages * g.ld_stage + std::max(kOpStages * g.op_stage, g.epi_bytes) + 128;
    // Two CTAs on one SM would both need more than half of TMEM and the second
    // would stall in tcgen05.alloc for the first's whole (persistent) life:
    // claim more than half of shared memory so the scheduler never pairs them.
    if (g.tmem_cols > 256) g.smem = std::max(g.smem, 120 * 1024);
    return g;
}

// --- tcgen05 wrappers ------------------------------------------------------

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    // K-major, no swizzle: start>>4 | LBO>>4 << 16 | SBO>>4 << 32 | descriptor version 1 << 46
    return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) |
           (static_cast<uint64_t>((kLBO >> 4) & 0x3FFF) << 16) |
           (static_cast<uint64_t>((kSBO >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ uint32_t instr_desc_f16_f32(int m, int n) {
    // D = F32 (bit 4), A = B = F16 (0), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
    return (1u << 4) | (static_cast<uint32_t>(n >> 3) << 17) |
           (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Byte offset of (row r, frame group kq of 8) inside one channel's operand region.
__device__ __forceinline__ int core_off(int r, int kq) {
    return (r >> 3) * kSBO + kq * kLBO + (r & 7) * 16;
}

__device__ __forceinline__ uint32_t half2_bits(__half2 h) {
    return *reinterpret_cast<const uint32_t *>(&h);
}

struct TcParams {
    const float2 *y;
    int y_frames;
    int n_station;
    int n_freq;
    int frames;
    float2 *acc;
    int *err;
    float scale;       // power of two applied before rounding to fp16
    float inv_scale2;  // 1/scale^2
    TcGeom g;
};

__global__ void __launch_bounds__(kThreads, 1) xengine_tc_kernel(TcParams p) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
    __shared__ uint64_t load_bar[kLoadStages];
    __shared__ uint64_t mma_bar[kOpStages];
    __shared__ uint64_t fin_bar;
    __shared__ uint32_t s_tmem_base;
    __shared__ int s_abort;

    const TcGeom &g = p.g;
    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const int N = p.n_station;
    const int n_tiles = p.n_freq / g.ct;
    const int my_tiles = (n_tiles - static_cast<int>(blockIdx.x) + static_cast<int>(gridDim.x) - 1) /
                         static_cast<int>(gridDim.x);
    const int n_stages = (p.frames + kKT - 1) / kKT;
    const int total = my_tiles * n_stages;    // stages this CTA processes
    float *ld_ring = reinterpret_cast<float *>(smem);
    unsigned char *op_ring = smem + kLoadStages * g.ld_stage;
    const int tiles_per_ct = g.ct / kYTile;
    const size_t ytile_stride = static_cast<size_t>(p.y_frames) * N * kYTile;   // float2

    // Operand rows never written (padding to 128-row blocks) must be finite.
    for (int i = tid; i < kOpStages * g.op_stage / 16; i += kThreads)
        reinterpret_cast<uint4 *>(op_ring)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        for (int s = 0; s < kLoadStages; ++s) mbar_init(&load_bar[s], 1);
        for (int s = 0; s < kOpStages; ++s) mbar_init(&mma_bar[s], 1);
        mbar_init(&fin_bar, 1);
        s_abort = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(&s_tmem_base)),
                     "r"(g.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem_base;

    // Producer side (thread 0): load global stage gs into ring slot gs % kLoadStages.
    auto issue_load = [&](int gs) {
        const int tl = gs / n_stages;
        const int st = gs - tl * n_stages;
        const int tile = static_cast<int>(blockIdx.x) + tl * static_cast<int>(gridDim.x);
        const int f0 = st * kKT;
        const int nfr = min(kKT, p.y_frames - f0);
        const uint32_t piece = static_cast<uint32_t>(nfr) * N * kYTile * 8;
        const int slot = gs % kLoadStages;
        float2 *dst = reinterpret_cast<float2 *>(ld_ring + slot * (g.ld_stage / 4));
        mbar_arrive_expect_tx(&load_bar[slot], piece * tiles_per_ct);
        for (int t = 0; t < tiles_per_ct; ++t) {
            const int ytile = tile * tiles_per_ct + t;
            const float2 *src = p.y + ytile * ytile_stride + static_cast<size_t>(f0) * N * kYTile;
            bulk_copy_g2s(dst + t * (kKT * N * kYTile), src, piece, &load_bar[slot]);
        }
    };
    if (tid == 0)
        for (int gs = 0; gs < kLoadStages && gs < total; ++gs) issue_load(gs);

    const uint32_t idesc = instr_desc_f16_f32(128, g.n_mma);
    const int items = g.ct * N * (kKT / 8);
    uint32_t ld_phase = 0, mma_phase = 0, fin_phase = 0;   // bit s: parity of next completion
    const int n_baseline = N * (N + 1) / 2;

    for (int gs = 0; gs < total; ++gs) {
        const int tl = gs / n_stages;
        const int st = gs - tl * n_stages;
        const int c0 = (static_cast<int>(blockIdx.x) + tl * static_cast<int>(gridDim.x)) * g.ct;
        const int lb = gs % kLoadStages;
        const int ob = gs & 1;
        bool ok = mbar_wait_bounded(&load_bar[lb], (ld_phase >> lb) & 1u, p.err,
                                    kErrXengineMmaTimeout);
        ld_phase ^= 1u << lb;
        if (gs >= kOpStages) {
            ok = ok && mbar_wait_bounded(&mma_bar[ob], (mma_phase >> ob) & 1u, p.err,
                                         kErrXengineMmaTimeout);
            mma_phase ^= 1u << ob;
        }
        if (!ok) s_abort = 1;

        // ld layout: [tile-in-CT][frame][station][kYTile channels]
        const float2 *ld = reinterpret_cast<const float2 *>(ld_ring + lb * (g.ld_stage / 4));
        unsigned char *op = op_ring + ob * g.op_stage;
        const int f0 = st * kKT;
        for (int q = tid; q < items; q += kThreads) {
            const int c = q % g.ct;
            const int rest = q / g.ct;
            const int s = rest % N;
            const int kq = rest / N;
            const float2 *col = ld + (c / kYTile) * (kKT * N * kYTile) + s * kYTile + (c % kYTile);
            uint32_t hre[4], him[4], lre[4], lim[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int fa = kq * 8 + 2 * i;
                float2 va = col[fa * N * kYTile];
                float2 vb = col[(fa + 1) * N * kYTile];
                if (f0 + fa >= p.frames) va = make_float2(0.f, 0.f);
                if (f0 + fa + 1 >= p.frames) vb = make_float2(0.f, 0.f);
                const float a0 = va.x * p.scale, a1 = vb.x * p.scale;
                const float b0 = va.y * p.scale, b1 = vb.y * p.scale;
                const __half2 hr = __floats2half2_rn(a0, a1);
                const __half2 hi = __floats2half2_rn(b0, b1);
                hre[i] = half2_bits(hr);
                him[i] = half2_bits(hi);
                if (g.split) {
                    const float2 fr = __half22float2(hr);
                    const float2 fi = __half22float2(hi);
                    lre[i] = half2_bits(__floats2half2_rn(a0 - fr.x, a1 - fr.y));
                    lim[i] = half2_bits(__floats2half2_rn(b0 - fi.x, b1 - fi.y));
                }
            }
            unsigned char *ch = op + c * g.chan_stride;
            *reinterpret_cast<uint4 *>(ch + core_off(2 * s, kq)) =
                make_uint4(hre[0], hre[1], hre[2], hre[3]);
            *reinterpret_cast<uint4 *>(ch + core_off(2 * s + 1, kq)) =
                make_uint4(him[0], him[1], him[2], him[3]);
            if (g.split) {
                *reinterpret_cast<uint4 *>(ch + core_off(g.lo_row + 2 * s, kq)) =
                    make_uint4(lre[0], lre[1], lre[2], lre[3]);
                *reinterpret_cast<uint4 *>(ch + core_off(g.lo_row + 2 * s + 1, kq)) =
                    make_uint4(lim[0], lim[1], lim[2], lim[3]);
            }
        }
        fence_proxy_async_smem();   // operand stores -> visible to the tensor cores
        __syncthreads();
        if (s_abort) break;
        if (tid == 0) {
            // the fp32 slot is consumed: refill it kLoadStages stages ahead
            if (gs + kLoadStages < total) {
                fence_proxy_async_smem();
                issue_load(gs + kLoadStages);
            }
            tc_fence_after();
            const uint32_t base = smem_addr(op);
            const uint32_t acc_flag = st > 0 ? 1u : 0u;
            for (int c = 0; c < g.ct; ++c) {
                const uint32_t chb = base + c * g.chan_stride;
                const uint32_t d = tmem + static_cast<uint32_t>(c * g.n_mma);
                const uint64_t hdesc = smem_desc(chb);
                umma_f16(d, hdesc, hdesc, idesc, acc_flag);
                if (g.split) {
                    const uint64_t ldesc = smem_desc(chb + (g.lo_row / 8) * kSBO);
                    umma_f16(d, hdesc, ldesc, idesc, 1u);
                    umma_f16(d, ldesc, hdesc, idesc, 1u);
                }
            }
            umma_commit(&mma_bar[ob]);
        }

        if (st == n_stages - 1) {
            // Tile complete: wait for all of its MMAs, then read the accumulators.
            if (tid == 0) umma_commit(&fin_bar);
            if (!mbar_wait_bounded(&fin_bar, fin_phase, p.err, kErrXengineMmaTimeout))
                s_abort = 1;
            fin_phase ^= 1u;
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            if (s_abort) break;
            // Epilogue scratch aliases the operand ring: every MMA reading it is done.
            float *E = reinterpret_cast<float *>(op_ring);
            float2 *Vs = reinterpret_cast<float2 *>(op_ring + (128 * g.e_stride * 4 + 15) / 16 * 16);
            const int quad = warp & 3;
            const int half = warp >> 2;
            const int nchunks = g.n_mma / 16;
            for (int c = 0; c < g.ct; ++c) {
                if (quad * 32 < 2 * N) {   // warp-uniform
                    for (int cc = half; cc < nchunks; cc += 2) {
                        float v[16];
                        const uint32_t taddr = tmem + (static_cast<uint32_t>(quad * 32) << 16) +
                                               static_cast<uint32_t>(c * g.n_mma + cc * 16);
                        tmem_ld16(taddr, v);
                        float *row = E + (quad * 32 + lane) * g.e_stride + cc * 16;
#pragma unroll
                        for (int i = 0; i < 16; ++i) row[i] = v[i];
                    }
                }
                __syncthreads();
                for (int b = tid; b < n_baseline; b += kThreads) {
                    int j = 0, rem = b;
                    while (rem >= N - j) {
                        rem -= N - j;
                        ++j;
                    }
                    const int k = j + rem;
                    const float *e2j = E + (2 * j) * g.e_stride;
                    const float *e2j1 = e2j + g.e_stride;
                    const float re = e2j[2 * k] + e2j1[2 * k + 1];
                    const float im = e2j1[2 * k] - e2j[2 * k + 1];
                    Vs[b * g.ct + c] = make_float2(re * p.inv_scale2, im * p.inv_scale2);
                }
                __syncthreads();
            }
            for (int q = tid; q < n_baseline * g.ct; q += kThreads) {
                const int b = q / g.ct;
                const int c = q - b * g.ct;
                float2 *dst = p.acc + static_cast<size_t>(b) * p.n_freq + c0 + c;
                float2 a = *dst;
                const float2 v = Vs[q];
                a.x += v.x;
                a.y += v.y;
                *dst = a;
            }
            // The next tile's first conversion overwrites the operand ring (and the
            // next MMA the accumulators): everyone must be past the epilogue.
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
        }
    }

    if (s_abort) {
        // Let every MMA and bulk copy this CTA started land before TMEM and the
        // CTA go away.
        if (tid == 0) {
            umma_commit(&fin_bar);
            mbar_wait_bounded(&fin_bar, fin_phase, nullptr, 0);
            for (int s = 0; s < kLoadStages; ++s)
                mbar_wait_bounded(&load_bar[s], (ld_phase >> s) & 1u, nullptr, 0);
        }
        tc_fence_before();
        __syncthreads();
    }
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(g.tmem_cols)
                     : "memory");
    }
}

int ilog2(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

} // namespace

size_t xengine_tc_workspace_bytes(int, int) { return 0; }

corr_status xengine_tc_launch(const XengineArgs &a, bool split, int num_sms,
                              cudaStream_t stream) {
    if (a.frames <= 0) return CORR_OK;
    const TcGeom g = make_geom(a.n_station, split);
    if (g.smem > 227 * 1024)
        return failf(CORR_ERR_INTERNAL, "tensor X-engine needs %d bytes of shared memory", g.smem);
    if (a.n_freq % g.ct != 0)
        return failf(CORR_ERR_ARG, "n_freq=%d is not a multiple of %d channels", a.n_freq, g.ct);
    if (a.y_frames < a.frames)
        return fail(CORR_ERR_INTERNAL, "spectra buffer shallower than the launch");
    static int configured_smem = 0;
    if (configured_smem < g.smem) {
        corr_status st = cuda_check(
            cudaFuncSetAttribute(xengine_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 g.smem),
            "cudaFuncSetAttribute(xengine_tc)");
        if (st != CORR_OK) return st;
        configured_smem = g.smem;
    }
    TcParams p{};
    p.y = a.y;
    p.y_frames = a.y_frames;
    p.n_station = a.n_station;
    p.n_freq = a.n_freq;
    p.frames = a.frames;
    p.acc = a.acc;
    p.err = a.err;
    const int shift = ilog2(2 * a.n_freq) - 8;   // |Y| <= 128*L -> |Y*2^-shift| <= 2^15
    p.scale = ldexpf(1.0f, -shift);
    p.inv_scale2 = ldexpf(1.0f, 2 * shift);
    p.g = g;
    const int n_tiles = a.n_freq / g.ct;
    const int grid = std::min(n_tiles, std::max(1, num_sms));
    xengine_tc_kernel<<<grid, kThreads, g.smem, stream>>>(p);
    return cuda_check(cudaGetLastError(), "xengine_tc_kernel launch");
}

} // namespace corrgb
