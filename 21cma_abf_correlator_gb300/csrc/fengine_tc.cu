// fengine_tc.cu -- the F-engine on the tensor cores: n_freq 16384, FP16 spectra.
//
// FFT plan 2 at n_freq 16384 for the FP16 tensor X-engine. A frame's 32768
// int8 samples, packed as M = 16384 complex points z[n] = x[2n] + i x[2n+1],
// are transformed by three DFT stages, each a matrix product on tcgen05
// (kind::f16, FP32 accumulators in TMEM):
//
//   n = 512 a + b,  b = 16 c + d;   k = k1 + 32 k2a + 1024 k2b
//   stage 1: DFT-32 over a  for the 512 rows b          -> k1, then * W_M^(b k1)
//   stage 2: DFT-32 over c  for the 512 rows (k1, d)    -> k2a, then * W_512^(d k2a)
//   stage 3: DFT-16 over d  for the 1024 rows (k1, k2a) -> k2b
//
// A stage's operand A (rows x the DFT's inputs, re/im interleaved along K) is
// FP16 in shared memory in the K-major no-swizzle layout (8-row x 16-byte core
// matrices); the DFT matrices (real 2R x 2R forms) are the B operands, each the
// sum of an FP16 "hi" and "lo" part issued as two MMAs into one accumulator,
// so the matrices carry about 22 bits and the data one FP16 rounding per stage.
// The twiddles between the stages, the FP16 conversion and the real-FFT split
// after stage 3 run on the CUDA cores, which read the accumulators with
// tcgen05.ld. Rows are ordered so that every stage's scatter into the next
// operand is free of shared-memory bank conflicts where it matters, and so that
// after stage 3 the rows holding Z[k] and Z[M-k] sit in the same TMEM lane of
// two tiles (one thread does the split of both).
//
// Magnitudes: |z| <= 180, stage 1 outputs <= 5760 (FP16 holds them), stage 2
// outputs are scaled by 1/32 (folded into its twiddle table) before FP16, and
// stage 3 stays in FP32. The spectrum goes out as FP16 pairs scaled by
// y_scale (x32 to undo the 1/32), exactly as the CUDA-core F-engine writes them.
//
// One CTA per SM (229.5 KB of shared memory, 512 TMEM columns), persistent over
// (frame, station) items like fengine.cu, with two warp groups of 256 threads
// that each carry their own items: a group has its own int8 frame buffer (the
// next item's frame arrives by a TMA bulk copy once the current one has been
// read), its own 64 KB operand buffer, 256 TMEM columns, mbarriers and named
// barrier. Within an item a group's stages run in order: its threads convert,
// one of them issues the MMAs, all wait for them (clock-bounded mbarrier waits)
// and run the epilogue; meanwhile the other group's MMAs or epilogue run.
// Missing frames and lost packets are handled as in fengine.cu.

#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_fp16.h>

#include "engine.h"
#include "fft_common.cuh"
#include "ptx.cuh"

namespace corrgb {
namespace {

constexpr int kM = 16384;
constexpr int kThreads = 512;
constexpr int kLBO = 128;                 // bytes between K-adjacent core matrices
constexpr int kSboA12 = 1024;             // stages 1, 2: 512 rows x 64 FP16 per row
constexpr int kSboA3 = 512;               // stage 3: 1024 rows x 32 FP16 per row
constexpr int kSboB1 = 1024;              // DFT-32 (64 x 64)
constexpr int kSboB3 = 512;               // DFT-16 (32 x 32)
constexpr int kB1Bytes = 64 * 64 * 2;
constexpr int kB3Bytes = 32 * 32 * 2;
constexpr int kTw1 = 512;                 // W_M^b, b < 512
constexpr int kTw2 = 512;                 // W_512^(d k2a) / 32, [k2a][d]
constexpr int kTw3 = 520;                 // exp(-2 pi i k / L), k <= 512
constexpr int kImageBytes = 2 * kB1Bytes + 2 * kB3Bytes + (kTw1 + kTw2 + kTw3) * 8;
static_assert(kImageBytes % 16 == 0, "image copied in 16-byte pieces");
constexpr float kStage2Scale = 1.0f / 32.0f;
constexpr int kGroup = 256;               // threads per warp group
constexpr int kIssuers = 4;               // MMA-issuing threads per group (lane 0 of its first warps)
constexpr uint32_t kTmemPerGroup = 256;
constexpr uint32_t kTmemCols = 2 * kTmemPerGroup;

// shared memory (bytes)
constexpr int OFF_X0 = 0;                 // int8 frame of warp group 0 (32 KB)
constexpr int OFF_X1 = 2 * kM;            // warp group 1
constexpr int OFF_A = 4 * kM;             // stage operand of warp group 0 (64 KB)
constexpr int OFF_AY = OFF_A + 65536;     // warp group 1
constexpr int OFF_IMG = OFF_AY + 65536;   // B1 hi, B1 lo, B3 hi, B3 lo, tw1, tw2, tw3
constexpr int OFF_B1H = OFF_IMG;
constexpr int OFF_B1L = OFF_B1H + kB1Bytes;
constexpr int OFF_B3H = OFF_B1L + kB1Bytes;
constexpr int OFF_B3L = OFF_B3H + kB3Bytes;
constexpr int OFF_TW1 = OFF_B3L + kB3Bytes;
constexpr int OFF_TW2 = OFF_TW1 + kTw1 * 8;
constexpr int OFF_TW3 = OFF_TW2 + kTw2 * 8;
constexpr int OFF_BAR = OFF_IMG + kImageBytes;   // frame[2], MMA[2] (one each per group)
constexpr int OFF_MISC = OFF_BAR + 48;           // TMEM base, abort flag
constexpr int kSmem = OFF_MISC + 16;
static_assert(OFF_A % 1024 == 0 && OFF_AY % 1024 == 0 && OFF_IMG % 16 == 0 && OFF_BAR % 16 == 0,
              "alignment");
static_assert(kSmem <= 227 * 1024, "shared memory");

// --- row orders (a numpy model of these maps checks the whole transform) ---

// Stage-1 row r1 = 128 t + 32 q + l holds b = 16 c + d with
// d = (l & 7) + 8 ((4t+q) & 1), c = (l >> 3) + 4 ((4t+q) >> 1).
__host__ __device__ __forceinline__ int b_of_r1(int r1) {
    const int g = r1 >> 5, l = r1 & 31;
    return 16 * ((l >> 3) + 4 * (g >> 1)) + (l & 7) + 8 * (g & 1);
}
// Stage-2 row of (k1, d): 32 G + 4 (k1 & 7) + (d & 3) with G = 4 (k1 >> 3) + (d >> 2),
// so that a warp's 32 rows are eight k1 by four d: its scatter into the stage-3
// operand then hits 32 banks (the stage-1 scatter into this one hits 16).
__host__ __device__ __forceinline__ int r2_of(int k1, int d) {
    return 32 * (4 * (k1 >> 3) + (d >> 2)) + 4 * (k1 & 7) + (d & 3);
}
// Stage-3 row of (k1, k2a): k1 + 32 k2a for k2a < 16; the other half holds the
// rows of Z[M-k] in the same lane of the tile four further on.
__host__ __device__ __forceinline__ int r3_of(int k1, int k2a) {
    if (k2a < 16) return k1 + 32 * k2a;
    if (k1 == 0) return 512 + 32 * (k2a == 16 ? 0 : 32 - k2a);
    return 512 + (32 - k1) + 32 * (31 - k2a);
}
// Byte offset of complex element e of row r in an operand with `sbo`.
__host__ __device__ __forceinline__ uint32_t a_off(int r, int e, int sbo) {
    return static_cast<uint32_t>((r >> 3) * sbo + (e >> 2) * kLBO + (r & 7) * 16 + (e & 3) * 4);
}
// Byte offset of element (n, k) of a B operand (N rows, K-major) with `sbo`.
__host__ __device__ __forceinline__ uint32_t b_off(int n, int k, int sbo) {
    return static_cast<uint32_t>((n >> 3) * sbo + (k >> 3) * kLBO + (n & 7) * 16 + (k & 7) * 2);
}

// --- tcgen05 wrappers ---

__device__ __forceinline__ uint64_t sdesc(uint32_t addr, int sbo) {
    // K-major, no swizzle: start>>4 | LBO>>4 << 16 | SBO>>4 << 32 | version 1 << 46
    return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) |
           (static_cast<uint64_t>((kLBO >> 4) & 0x3FFF) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ uint32_t idesc_f16(int m, int n) {
    // D = F32, A = B = F16, both K-major, N >> 3 at bit 17, M >> 4 at bit 24
    return (1u << 4) | (static_cast<uint32_t>(n >> 3) << 17) |
           (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                    uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tc_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Two signed bytes -> FP16 pair, exactly: the biased bytes (b + 128) become the
// low mantissa bits of 1024 (0x6400), and 1152 is subtracted.
__device__ __forceinline__ uint32_t int8_pair_to_half2(uint32_t u16) {
    const uint32_t x = u16 ^ 0x8080u;
    const uint32_t h = __byte_perm(x, 0x64646464u, 0x4140);
    const __half2 v = __hsub2(*reinterpret_cast<const __half2 *>(&h),
                              __floats2half2_rn(1152.0f, 1152.0f));
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void put_half2(unsigned char *base, int off, float2 v) {
    *reinterpret_cast<__half2 *>(base + off) = __floats2half2_rn(v.x, v.y);
}

// Stage 1 or 2, tile t of four: D = A (128 x 64) . B^T (64 x 64) at columns 64 t,
// the hi and lo parts of B into one accumulator. Each of four threads issues one
// tile (issuing many small MMAs from one thread is slower than the tensor cores).
__device__ __forceinline__ void issue_dft32(uint32_t tmem, uint32_t a, uint32_t bh, uint32_t bl,
                                            int t) {
    const uint32_t id = idesc_f16(128, 64);
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        const uint64_t da = sdesc(a + t * 16 * kSboA12 + ks * 2 * kLBO, kSboA12);
        mma(tmem + 64 * t, da, sdesc(bh + ks * 2 * kLBO, kSboB1), id, ks > 0 ? 1u : 0u);
        mma(tmem + 64 * t, da, sdesc(bl + ks * 2 * kLBO, kSboB1), id, 1u);
    }
}

// Stage 3, tiles t and t + 4 of eight: D = A (128 x 32) . B^T (32 x 32) at columns 32 t.
__device__ __forceinline__ void issue_dft16(uint32_t tmem, uint32_t a, uint32_t bh, uint32_t bl,
                                            int t) {
    const uint32_t id = idesc_f16(128, 32);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int tt = t + 4 * h;
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            const uint64_t da = sdesc(a + tt * 16 * kSboA3 + ks * 2 * kLBO, kSboA3);
            mma(tmem + 32 * tt, da, sdesc(bh + ks * 2 * kLBO, kSboB3), id, ks > 0 ? 1u : 0u);
            mma(tmem + 32 * tt, da, sdesc(bl + ks * 2 * kLBO, kSboB3), id, 1u);
        }
    }
}

// Two warp groups of 256 threads share the SM, each carrying its own items
// through the three stages with its own frame buffer, operand buffer, 256 TMEM
// columns and barriers (named barrier 1 + group): while one group runs an
// epilogue on the CUDA cores, the other's MMAs run on the tensor cores.
template <bool CONTIG>
__global__ void __launch_bounds__(kThreads, 1)
    fengine_tc_kernel(FengineArgs a, const uint4 *__restrict__ image) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const float2 *tw1 = reinterpret_cast<const float2 *>(smem + OFF_TW1);
    const float2 *tw2 = reinterpret_cast<const float2 *>(smem + OFF_TW2);
    const float2 *tw3 = reinterpret_cast<const float2 *>(smem + OFF_TW3);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + OFF_BAR);   // frame[2], MMA[2]
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(smem + OFF_MISC);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + OFF_MISC + 4);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = warp >> 3, gtid = tid & (kGroup - 1);
    const int gw = warp & 7;                             // warp within the group
    const bool issuer = lane == 0 && gw < kIssuers;      // issues the MMAs of tile (pair) gw
    const int q = warp & 3, th = (warp >> 2) & 1;   // TMEM lane quarter; tiles th, th + 2
    {
        uint4 *dst = reinterpret_cast<uint4 *>(smem + OFF_IMG);
        for (int i = tid; i < kImageBytes / 16; i += kThreads) dst[i] = image[i];
    }
    if (tid == 0) {
        mbar_init(&bar[0], 1);                  // frames: one arrival + the copy's bytes
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], kIssuers);           // MMAs: one commit per issuing thread
        mbar_init(&bar[3], kIssuers);
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(s_tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = *s_tmem + kTmemPerGroup * grp;
    unsigned char *const sA = smem + (grp ? OFF_AY : OFF_A);
    unsigned char *const sx = smem + (grp ? OFF_X1 : OFF_X0);
    uint64_t *const fbar = &bar[grp];
    uint64_t *const mbar = &bar[2 + grp];
    const uint32_t a_addr = smem_addr(sA);
    const uint32_t lane_base = static_cast<uint32_t>(32 * q) << 16;
    auto group_sync = [&]() { asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "n"(kGroup) : "memory"); };

    const int n_items = a.frames * a.n_station;
    const int stride = 2 * static_cast<int>(gridDim.x);
    constexpr uint32_t frame_bytes = 2u * kM;
    const int ytile_shift = __ffs(a.ytile) - 1;
    const float out_scale = a.y_scale * 32.0f;   // undo stage 2's 1/32
    auto src_of = [&](int it) {
        const int f = it / a.n_station;
        const int s = it - f * a.n_station;
        return a.samples + static_cast<size_t>(s) * a.station_stride +
               static_cast<size_t>(f) * a.frame_stride;
    };
    auto present = [&](int it) {
        const int f = it / a.n_station;
        return frame_present<kM>(a, f, it - f * a.n_station);
    };
    bool copy_pending = false;   // (gtid 0) a frame copy into this group's buffer
    auto fetch = [&](int it) {   // gtid 0: request item it's frame if it has one
        if (it < n_items && present(it)) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(fbar, frame_bytes);
            bulk_copy_g2s(sx, src_of(it), frame_bytes, fbar);
            copy_pending = true;
        }
    };

    int item = 2 * static_cast<int>(blockIdx.x) + grp;
    if (gtid == 0) fetch(item);
    uint32_t fpar = 0u, mpar = 0u;
    bool mma_pending = false;     // (issuers) MMAs issued, completion not yet seen
    uint32_t pending_par = 0u;    // the phase their completion ends
    bool failed = false;

    auto issued = [&]() {
        mma_commit(mbar);
        mma_pending = true;
        pending_par = mpar;
    };
    auto wait_mma = [&]() {
        if (!mbar_wait_bounded(mbar, mpar, a.err, kErrFengineCopyTimeout, abort_flag))
            *abort_flag = 1;
        tc_after();
    };
    // End of a phase: operand writes visible to the tensor cores, TMEM reads
    // done, the group in step; the abort flag is read after the barrier.
    auto end_phase = [&]() -> bool {
        fence_proxy_async_smem();
        tc_before();
        group_sync();
        return *abort_flag == 0;
    };

    for (; item < n_items; item += stride) {
        using Row = YRow<kSpectraF16, CONTIG>;
        const Row yrow{reinterpret_cast<typename Row::T *>(a.y) + static_cast<size_t>(item) * a.ytile,
                       static_cast<uint32_t>(a.y_frames) * a.n_station * a.ytile, ytile_shift,
                       out_scale, 0.5f * out_scale};
        if (!present(item)) {
            for (int k = gtid; k < kM; k += kGroup) yrow.put(k, make_float2(0.f, 0.f));
            if (gtid == 0) fetch(item + stride);
            continue;
        }
        if (!mbar_wait_bounded(fbar, fpar, a.err, kErrFengineCopyTimeout, abort_flag))
            *abort_flag = 1;
        fpar ^= 1u;
        if (a.pmask != nullptr) {
            const int f = item / a.n_station;
            const uint32_t kept = packets_kept<kM>(a, f, item - f * a.n_station);
            if (kept != all_packets<kM>()) {
                uint4 *x16 = reinterpret_cast<uint4 *>(sx);
                for (int i = gtid; i < kM / 8; i += kGroup)
                    if (!((kept >> (i >> 6)) & 1u)) x16[i] = make_uint4(0u, 0u, 0u, 0u);
                group_sync();
            }
        }

        // Stage-1 operand: row r1 (b), complex elements a = 0..31, four per
        // 16-byte store; a quarter warp stores one whole core matrix.
        {
            const uint16_t *px = reinterpret_cast<const uint16_t *>(sx);
#pragma unroll 4
            for (int i = 0; i < 16; ++i) {
                const int idx = gtid + kGroup * i;
                const int j = idx >> 9, r1 = idx & 511;
                const int b = b_of_r1(r1);
                uint4 v;
                v.x = int8_pair_to_half2(px[512 * (4 * j + 0) + b]);
                v.y = int8_pair_to_half2(px[512 * (4 * j + 1) + b]);
                v.z = int8_pair_to_half2(px[512 * (4 * j + 2) + b]);
                v.w = int8_pair_to_half2(px[512 * (4 * j + 3) + b]);
                *reinterpret_cast<uint4 *>(sA + (r1 >> 3) * kSboA12 + j * kLBO + (r1 & 7) * 16) = v;
            }
        }
        if (!end_phase()) {
            failed = true;
            break;
        }
        if (gtid == 0) {
            copy_pending = false;    // landed and read
            fetch(item + stride);    // the group's next frame, into the buffer just read
        }
        if (issuer) {
            tc_after();
            issue_dft32(tmem, a_addr, smem_addr(smem + OFF_B1H), smem_addr(smem + OFF_B1L), gw);
            issued();
        }
        wait_mma();
        mpar ^= 1u;

        // Stage-1 epilogue: row b, outputs k1 -> * W_M^(b k1) -> stage-2 row (k1, d), element c.
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
            const int t = th + 2 * h;
            const int b = b_of_r1(128 * t + 32 * q + lane);
            const int c = b >> 4, d = b & 15;
            uint32_t v[64];
            const uint32_t ta = tmem + lane_base + 64 * t;
            tmem_ld16(ta, v);
            tmem_ld16(ta + 16, v + 16);
            tmem_wait_ld();
            tmem_ld16(ta + 32, v + 32);   // lands while the first half is worked
            tmem_ld16(ta + 48, v + 48);
            const float2 w = tw1[b];
            float2 wk = make_float2(1.f, 0.f);
            // row r2_of(k1, d) = r2_of(0, d) + 128 (k1 >> 3) + 4 (k1 & 7): 16 groups per
            // k1 >> 3, and (k1 & 7) adds 4 rows, i.e. half a group (k1 & 1) plus whole
            // groups (k1 >> 1 & 3); d & 3 < 4 keeps the low rows inside their group
            unsigned char *const dst = sA + a_off(r2_of(0, d), c, kSboA12);
#pragma unroll
            for (int k1 = 0; k1 < 32; ++k1) {
                if (k1 == 16) tmem_wait_ld();
                float2 y = make_float2(__uint_as_float(v[2 * k1]), __uint_as_float(v[2 * k1 + 1]));
                if (k1 > 0) {
                    wk = cmul(wk, w);
                    y = cmul(y, wk);
                }
                const int drows = 128 * (k1 >> 3) + 4 * (k1 & 7);
                put_half2(dst, (drows >> 3) * kSboA12 + (drows & 7) * 16, y);
            }
        }
        if (!end_phase()) {
            failed = true;
            break;
        }
        if (issuer) {
            mma_pending = false;
            tc_after();
            issue_dft32(tmem, a_addr, smem_addr(smem + OFF_B1H), smem_addr(smem + OFF_B1L), gw);
            issued();
        }
        wait_mma();
        mpar ^= 1u;

        // Stage-2 epilogue: row (k1, d), outputs k2a -> * W_512^(d k2a)/32 ->
        // stage-3 row (k1, k2a), element d.
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
            const int t = th + 2 * h;
            const int g = 4 * t + q;
            const int k1 = 8 * (g >> 2) + (lane >> 2), d = 4 * (g & 3) + (lane & 3);
            uint32_t v[64];
            const uint32_t ta = tmem + lane_base + 64 * t;
            tmem_ld16(ta, v);
            tmem_ld16(ta + 16, v + 16);
            tmem_wait_ld();
            tmem_ld16(ta + 32, v + 32);   // lands while the first half is worked
            tmem_ld16(ta + 48, v + 48);
            // k2a < 16: rows k1 + 32 k2a (4 row groups apart per k2a). k2a >= 16:
            // rows of the partner half, 4 groups back per k2a from k2a = 16, except
            // that k1 = 0 at k2a = 16 is row 512.
            unsigned char *const lo = sA + a_off(k1, d, kSboA3);
            const uint32_t hi16 = a_off(r3_of(k1, 16), d, kSboA3);
            const uint32_t hi17 = a_off(r3_of(k1, 17), d, kSboA3) + 4 * kSboA3;
            unsigned char *const hi = sA + hi17;
#pragma unroll
            for (int k2a = 0; k2a < 32; ++k2a) {
                if (k2a == 16) tmem_wait_ld();
                const float2 y = cmul(
                    make_float2(__uint_as_float(v[2 * k2a]), __uint_as_float(v[2 * k2a + 1])),
                    tw2[k2a * 16 + d]);
                if (k2a < 16)
                    put_half2(lo, k2a * 4 * kSboA3, y);
                else if (k2a == 16)
                    put_half2(sA, static_cast<int>(hi16), y);
                else
                    put_half2(hi, -(k2a - 16) * 4 * kSboA3, y);
            }
        }
        if (!end_phase()) {
            failed = true;
            break;
        }
        if (issuer) {
            mma_pending = false;
            tc_after();
            issue_dft16(tmem, a_addr, smem_addr(smem + OFF_B3H), smem_addr(smem + OFF_B3L), gw);
            issued();
        }
        wait_mma();
        mpar ^= 1u;

        // Stage-3 epilogue: thread p (row k1 + 32 k2a = p, k2a < 16) holds Z[p + 1024 i]
        // in za[i] and, in the partner row, Z[M - p - 1024 i] in zb[15 - i]; the real
        // split gives X at both. Row p = 0 ((0, 0)) and its partner (0, 16) pair
        // with themselves.
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
            const int t = th + 2 * h;
            const int p = 128 * t + 32 * q + lane;
            uint32_t u[32], w[32];
            tmem_ld16(tmem + lane_base + 32 * t, u);
            tmem_ld16(tmem + lane_base + 32 * t + 16, u + 16);
            tmem_ld16(tmem + lane_base + 32 * (t + 4), w);
            tmem_ld16(tmem + lane_base + 32 * (t + 4) + 16, w + 16);
            tmem_wait_ld();   // both rows feed every split below
            float2 za[16], zb[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                za[i] = make_float2(__uint_as_float(u[2 * i]), __uint_as_float(u[2 * i + 1]));
                zb[i] = make_float2(__uint_as_float(w[2 * i]), __uint_as_float(w[2 * i + 1]));
            }
            const bool t0 = (p == 0);
            const float2 wp = scale_tw(tw3[p], yrow.half);   // split_store takes h*w
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const float2 zmk = t0 ? za[(16 - i) & 15] : zb[15 - i];
                split_store(za[i], zmk, mul_w32(wp, i), p + 1024 * i, kM, !(t0 && i == 0), yrow);
            }
            const int kB = t0 ? 512 : p + 8192;
            const float2 wB = t0 ? scale_tw(tw3[512], yrow.half) : mul_w32(wp, 8);
#pragma unroll
            for (int i = 8; i < 16; ++i) {
                const float2 zk = t0 ? zb[i - 8] : za[i];
                const float2 zmk = t0 ? zb[23 - i] : zb[15 - i];
                split_store(zk, zmk, mul_w32(wB, i - 8), kB + 1024 * (i - 8), kM, true, yrow);
            }
            if (t0) yrow.put(kM / 2, make_float2(za[8].x * out_scale, -za[8].y * out_scale));
        }
        if (!end_phase()) {
            failed = true;
            break;
        }
        mma_pending = false;
    }
    if (failed) {
        // let this group's copy and MMAs in flight finish before the CTA and its
        // accumulators go (each wait bounded; the error is already recorded)
        if (gtid == 0 && copy_pending) mbar_wait_bounded(fbar, fpar, nullptr, 0);
        if (issuer && mma_pending) mbar_wait_bounded(mbar, pending_par, nullptr, 0);
    }
    __syncthreads();
    if (warp == 0) {
        tc_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(
                         *s_tmem),
                     "r"(kTmemCols)
                     : "memory");
    }
}

template <bool CONTIG>
corr_status launch(const FengineArgs &a, const void *image, int num_sms, cudaStream_t stream) {
    static PerDevice setup;   // the shared-memory limit is a per-device setting
    corr_status st = setup.run([](int) {
        return cuda_check(cudaFuncSetAttribute(fengine_tc_kernel<CONTIG>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem),
                          "cudaFuncSetAttribute(fengine_tc)");
    });
    if (st != CORR_OK) return st;
    const int items = a.frames * a.n_station;
    if (items <= 0) return CORR_OK;
    const int pairs = (items + 1) / 2;   // each CTA carries two items at a time
    const int grid = pairs < num_sms ? pairs : num_sms;
    fengine_tc_kernel<CONTIG><<<grid, kThreads, kSmem, stream>>>(
        a, static_cast<const uint4 *>(image));
    return cuda_check(cudaGetLastError(), "fengine_tc_kernel launch");
}

} // namespace

corr_status fengine_tc_prepare(void **d_image) {
    *d_image = nullptr;
    const double pi = 3.14159265358979323846;
    std::vector<unsigned char> img(kImageBytes, 0);
    auto put_half = [&](size_t off, double v) {
        const __half h = __float2half_rn(static_cast<float>(v));
        std::memcpy(&img[off], &h, 2);
    };
    // B = the real 2R x 2R form of the DFT-R matrix, rows n = 2k + (0 re, 1 im),
    // columns (K) 2a + (0 re, 1 im): [[cos, sin], [-sin, cos]] of 2 pi a k / R.
    auto build = [&](int R, size_t off_hi, size_t off_lo, int sbo) {
        for (int n = 0; n < 2 * R; ++n)
            for (int k = 0; k < 2 * R; ++k) {
                const double th = 2.0 * pi * static_cast<double>((k >> 1) * (n >> 1)) / R;
                const double c = std::cos(th), s = std::sin(th);
                const double v = (n & 1) == 0 ? ((k & 1) == 0 ? c : s) : ((k & 1) == 0 ? -s : c);
                const __half hi = __float2half_rn(static_cast<float>(v));
                const double lo = v - static_cast<double>(__half2float(hi));
                const size_t o = b_off(n, k, sbo);
                std::memcpy(&img[off_hi + o], &hi, 2);
                put_half(off_lo + o, lo);
            }
    };
    build(32, OFF_B1H - OFF_IMG, OFF_B1L - OFF_IMG, kSboB1);
    build(16, OFF_B3H - OFF_IMG, OFF_B3L - OFF_IMG, kSboB3);
    auto put_c = [&](size_t off, double re, double im) {
        const float2 v = make_float2(static_cast<float>(re), static_cast<float>(im));
        std::memcpy(&img[off], &v, 8);
    };
    for (int b = 0; b < kTw1; ++b) {
        const double th = -2.0 * pi * b / kM;
        put_c(OFF_TW1 - OFF_IMG + 8 * b, std::cos(th), std::sin(th));
    }
    for (int k2a = 0; k2a < 32; ++k2a)
        for (int d = 0; d < 16; ++d) {
            const double th = -2.0 * pi * d * k2a / 512.0;
            put_c(OFF_TW2 - OFF_IMG + 8 * (k2a * 16 + d), kStage2Scale * std::cos(th),
                  kStage2Scale * std::sin(th));
        }
    for (int k = 0; k < kTw3; ++k) {
        const double th = -2.0 * pi * k / (2.0 * kM);
        put_c(OFF_TW3 - OFF_IMG + 8 * k, std::cos(th), std::sin(th));
    }
    void *d = nullptr;
    corr_status st = cuda_check(cudaMalloc(&d, kImageBytes), "cudaMalloc(tensor FFT tables)");
    if (st != CORR_OK) return st;
    st = cuda_check(cudaMemcpy(d, img.data(), kImageBytes, cudaMemcpyHostToDevice),
                    "cudaMemcpy(tensor FFT tables)");
    if (st != CORR_OK) {
        cudaFree(d);
        return st;
    }
    *d_image = d;
    return CORR_OK;
}

} // namespace corrgb

extern "C" corr_status corrx_tc_fft_maps(int32_t *b_of_row, int32_t *row2, int32_t *row3,
                                         uint32_t *off12, uint32_t *off3) {
    using namespace corrgb;
    for (int r = 0; b_of_row != nullptr && r < 512; ++r) b_of_row[r] = b_of_r1(r);
    for (int k1 = 0; k1 < 32; ++k1) {
        for (int d = 0; row2 != nullptr && d < 16; ++d) row2[k1 * 16 + d] = r2_of(k1, d);
        for (int k2a = 0; row3 != nullptr && k2a < 32; ++k2a) row3[k1 * 32 + k2a] = r3_of(k1, k2a);
    }
    for (int r = 0; off12 != nullptr && r < 512; ++r)
        for (int e = 0; e < 32; ++e) off12[r * 32 + e] = a_off(r, e, kSboA12);
    for (int r = 0; off3 != nullptr && r < 1024; ++r)
        for (int e = 0; e < 16; ++e) off3[r * 16 + e] = a_off(r, e, kSboA3);
    return CORR_OK;
}

namespace corrgb {

corr_status fengine_tc_launch(const FengineArgs &a, const void *image, int num_sms,
                              cudaStream_t stream) {
    if (image == nullptr) return fail(CORR_ERR_INTERNAL, "tensor FFT tables not prepared");
    if (a.y_fmt != kSpectraF16)
        return fail(CORR_ERR_ARG, "FFT plan 2 writes FP16 spectra only (the FP16 tensor X-engine)");
    return a.ytile == kM ? launch<true>(a, image, num_sms, stream)
                         : launch<false>(a, image, num_sms, stream);
}

} // namespace corrgb
