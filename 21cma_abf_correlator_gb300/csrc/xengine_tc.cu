// xengine_tc.cu -- tensor-core X-engine: tcgen05 MMA, FP16 operands, FP32 in TMEM.
//
// The same sum as the plain X-engine (reference corr_kernel,
// corr-cuda/src/kernels.cu:194-265), recast as small real GEMMs per channel.
// For channel c let D be the frames x 2N real matrix whose columns are
// (Re Y_0, Im Y_0, Re Y_1, Im Y_1, ...). Then S = D^T D holds everything:
//     Re V[j,k] = S[2j][2k] + S[2j+1][2k+1]
//     Im V[j,k] = S[2j+1][2k] - S[2j][2k+1]
// The tensor cores compute S with K = frames, FP16 operands and FP32 accumulation
// in tensor memory (TMEM), accumulated over the whole launch.
//
// Precision forms (the F-engine stores the spectra already in the form's
// operand precision, scaled, so the converters here only transpose):
//   FP16       : D rounded once to FP16 (11-bit significand).
//   FP16 split : D = Dh + Dl, Dh = fp16(D), Dl = fp16(D - Dh) (about 22 bits);
//                S ~ H + P + P^T with H = Dh^T Dh and P = Dl^T Dh (Dl^T Dl dropped).
// Scale: spectra of int8 frames satisfy |Y| <= 128*L, so multiplying by the
// power of two 2^-(ceil(log2 L) - 8) keeps every value at or below 2^15
// (< FP16 max) in every channel for every input; being a power of two it is
// undone exactly.
// The int8 quantisation floor keeps |Y| >= ~sqrt(L/12) in every channel of real
// data, so the scaled values sit in FP16's normal range and no per-channel
// adaptive scale is needed.
//
// Operand regions. Per K step each region gets exactly one MMA: M = 128 rows of
// A read from the region's start, N = nb rows of B from the same start.
// R = 2N rounded up to 8 (the rows of one channel's D):
//   split, N <= 32 ("stacked"): rows [0,2N) Dh, [R,R+2N) Dl; nb = 2N (to 16):
//       TMEM lanes [0,2N) x cols [0,2N) = H, lanes [R,R+2N) x cols [0,2N) = P.
//   split, N > 32 ("wide"):  same rows; nb = R+2N (to 16), so B carries Dl and
//       lanes [0,2N) hold H in cols [0,2N) and T = Dh^T Dl = P^T in [R,R+2N).
//   fp16, N <= 32 ("paired"): two channels per region, rows [0,2N) and [R,R+2N);
//       nb = R+2N (to 16): the two diagonal blocks are the two channels' S.
//   fp16, N > 32: one channel per region, rows [0,2N), nb = 2N (to 16).
// The cross term: with Q[j][k] formed from rows 2j, 2j+1 of P exactly as V from
// S, P + P^T adds Q[j][k] + conj(Q[k][j]) to V[j][k] (the same holds with T in
// place of P), so the epilogue stages Q and folds it in as it adds V to the row.
// An MMA with M = 128 reads 4 KB of A whatever the form; stacking the split
// operands (pairing channels) makes that read serve three (two) products
// instead of one, which keeps the tensor cores' shared-memory reads below the
// stage's DRAM time.
//
// Warp-specialised persistent CTAs, one per SM (TMEM), CT channels per tile:
//   warp 0 (lane 0): stage loads into a ring as deep as shared memory allows.
//     Contiguous rows (ytile = n_freq): one 4-D TMA box {CT channels, N
//     stations, KT frames, 1 tile} per stage; the map ends at the launch's last
//     frame, so a partial stage arrives zero-padded. Tiles of CT channels
//     (ytile = CT): the stage is one contiguous block and one bulk copy brings
//     the launch's frames of it; the converters read the rest as zeros.
//   warps 1..kIssuers (lane 0): the MMAs of a stage once its operands are
//     written, the operand regions dealt round robin over the issuers.
//   converter warps: regroup a landed stage (FP16 bins, frame-major) into the
//     K-major no-swizzle operand layout (8-row x 16-byte core matrices, frames
//     along K) with byte permutes.
//   last four warps (epilogue, one per TMEM lane quarter): after a tile's last MMA,
//     read the accumulators (tcgen05.ld), pair rows 2j/2j+1 with one shuffle,
//     stage V (and Q), release TMEM, then add V into the row in global memory
//     with 16-byte read-modify-writes (one owner per channel tile and launch).
// The roles meet only at mbarriers, all waited on with clock-bounded waits, so
// a stuck party makes the others time out and report instead of hanging.

#include <algorithm>
#include <mutex>
#include <type_traits>

#include <cuda.h>
#include <cuda_fp16.h>

#include "engine.h"
#include "ptx.cuh"

namespace corrgb {
namespace {

// Warp layout (512 threads): warp 0 TMA; warps 1..kIssuers MMA issue (one
// thread each, operand regions dealt round robin: the issue of tcgen05.mma
// costs the issuing thread more than the tensor cores need per small MMA, so
// independent accumulators are issued from several threads); then converter
// warps; the last four warps are the epilogue (one per TMEM lane quarter).
constexpr int kIssuers = 4;
constexpr int kThreads = 512;
constexpr int kEpilogue = 128;
constexpr int kFirstConverterWarp = 1 + kIssuers;
constexpr int kConverters = kThreads - kEpilogue - 32 * kFirstConverterWarp;
constexpr int kFirstEpilogueWarp = kFirstConverterWarp + kConverters / 32;
static_assert(kConverters >= 192 && kFirstEpilogueWarp * 32 + kEpilogue == kThreads, "layout");
constexpr int kMaxLoadStages = 6;
constexpr int kMaxOpStages = 3;
constexpr int kMaxItems = 4;                     // conversion items per converter thread
constexpr int kLBO = 128;                        // bytes between K-adjacent core matrices
// Dynamic shared memory of any feasible shape: the 227 KB a CTA may opt into,
// less 1 KB left for the kernel's static shared variables.
constexpr int kMaxSmem = 227 * 1024 - 1024;

enum TcForm : int { kSplitStacked = 0, kSplitWide = 1, kFp16Paired = 2, kFp16Wide = 3 };

struct TcGeom {
    int n_station;
    int form;
    bool split;
    int ct;            // channels per tile
    int kt;            // frames per stage (16 or 32)
    int R;             // first row of a region's second block (>= 2N, a multiple of 8)
    int nb;            // MMA N
    int regions;       // operand regions per stage
    int sbo;           // bytes between 8-row groups = (kt/8) * 128
    int region_stride; // bytes between regions (multiple of 128, one 128-byte pad)
    int tmem_cols;
    int acc_cols;      // TMEM columns of one accumulator set (a tile)
    int n_acc;         // accumulator sets (2 = the next tile's MMAs overlap the epilogue)
    int op_stage;      // operand bytes per stage
    int elem;          // bytes per spectrum bin: 8 (FP32 pairs) or 4 (FP16 pairs)
    int ld_stage;      // spectra bytes per stage = kt * N * ct * elem
    int n_ld;
    int n_op;
    int vs_bytes;      // staged V: ct planes of n_baseline float2, k-major triangle
    int qs_bytes;      // staged Q: ct planes of N*N float2, [k][j] (split forms)
    int smem;
    int items;         // conversion items per stage = ct * N * kt/8
    bool ok;
};

int round_up(int v, int m) { return (v + m - 1) / m * m; }

// 16-byte bank skew of region r: the eight 16-byte stores of a quarter warp
// (eight channels, one station) land in eight distinct slots of a bank line.
__host__ __device__ inline int region_skew(int r) {
    return ((r & 1) | ((r & 2) << 1) | ((r & 4) >> 1)) * 16;
}

TcGeom make_geom(int n_station, bool split, int ct, int kt) {
    TcGeom g{};
    g.ok = false;
    g.n_station = n_station;
    g.split = split;
    g.ct = ct;
    g.kt = kt;
    const int N = n_station;
    if (N < 1 || N > 64 || (kt != 16 && kt != 32 && kt != 64) || ct < 2 || ct > 8 ||
        (ct & (ct - 1)))
        return g;
    // Both forms read FP16 spectra written so by the F-engine: pairs (4 bytes)
    // or hi/lo pairs (8 bytes); a TMA box row of CT of them must be a multiple
    // of 16 bytes.
    g.elem = split ? 8 : 4;
    if (ct * g.elem < 16) return g;
    g.R = round_up(2 * N, 8);
    // A region's second block (Dl, or the second channel) starts at row 64
    // when it fits: its accumulator rows then fall in TMEM lane quarters 2-3,
    // so the four epilogue warps share the read-out evenly.
    const bool stacks = g.R + 2 * N <= 128;
    if (stacks) g.R = std::max(g.R, 64);
    int rows_valid;
    if (split) {
        g.form = stacks ? kSplitStacked : kSplitWide;
        g.nb = g.form == kSplitStacked ? std::max(16, round_up(2 * N, 16))
                                       : round_up(g.R + 2 * N, 16);
        g.regions = ct;
        rows_valid = g.R + 2 * N;
    } else {
        g.form = stacks ? kFp16Paired : kFp16Wide;
        g.nb = g.form == kFp16Paired ? round_up(g.R + 2 * N, 16)
                                     : std::max(16, round_up(2 * N, 16));
        g.regions = g.form == kFp16Paired ? ct / 2 : ct;
        rows_valid = g.form == kFp16Paired ? g.R + 2 * N : 2 * N;
    }
    if (g.nb > 256) return g;
    // highest TMEM column any epilogue read touches (reads are 16 columns wide)
    int max_col = g.regions * g.nb;
    const int chunk = round_up(2 * N, 16);
    if (g.form == kSplitWide) max_col = std::max(max_col, (ct - 1) * g.nb + g.R + chunk);
    if (g.form == kFp16Paired)
        max_col = std::max(max_col, (g.regions - 1) * g.nb + g.R + chunk);
    if (max_col > 512) return g;
    g.acc_cols = round_up(max_col, 32);
    // Two accumulator sets when they fit: tile t+1 accumulates while the
    // epilogue still reads tile t.
    g.n_acc = 2 * g.acc_cols <= 512 ? 2 : 1;
    int cols = 32;
    while (cols < g.n_acc * g.acc_cols) cols *= 2;
    g.tmem_cols = cols;
    g.sbo = (kt / 8) * 128;
    const int groups = (rows_valid + 7) / 8;
    g.region_stride = groups * g.sbo + 128;
    // A reads 128 rows (16 groups), B nb rows, from the last region's start,
    // plus its skew.
    const int reach = std::max(16, g.nb / 8) * g.sbo;
    const int slack = std::max(0, reach - g.region_stride) + 7 * 16 + 128;
    g.op_stage = round_up(g.regions * g.region_stride + slack, 128);
    g.ld_stage = kt * N * ct * g.elem;
    // paired form: items enumerate stations in groups of four (see the converters)
    g.items = ct * (g.form == kFp16Paired ? round_up(N, 4) : N) * (kt / 8);
    if (g.items > kMaxItems * kConverters) return g;
    const int n_baseline = N * (N + 1) / 2;
    g.vs_bytes = round_up(n_baseline * ct * 8, 128);
    g.qs_bytes = split ? round_up(N * N * ct * 8, 128) : 0;
    const int jk_bytes = round_up(n_baseline * 2, 128);
    const int budget = kMaxSmem;
    const int fixed = g.vs_bytes + g.qs_bytes + jk_bytes + 128;
    g.n_op = 2;
    if (fixed + g.n_op * g.op_stage + 2 * g.ld_stage > budget) return g;
    // a third operand stage when it still leaves a four-deep load ring
    if (fixed + 3 * g.op_stage + 4 * g.ld_stage <= budget) g.n_op = 3;
    g.n_ld = std::min(kMaxLoadStages, (budget - fixed - g.n_op * g.op_stage) / g.ld_stage);
    g.smem = g.n_ld * g.ld_stage + g.n_op * g.op_stage + fixed;
    // Two CTAs on one SM would both need more than half of TMEM and the second
    // would stall in tcgen05.alloc for the first's whole (persistent) life:
    // claim more than half of shared memory so the scheduler never pairs them.
    if (g.tmem_cols > 256) g.smem = std::max(g.smem, 120 * 1024);
    g.ok = true;
    return g;
}

// --- tcgen05 / TMA wrappers -------------------------------------------------

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, int sbo) {
    // K-major, no swizzle: start>>4 | LBO>>4 << 16 | SBO>>4 << 32 | descriptor version 1 << 46
    return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) |
           (static_cast<uint64_t>((kLBO >> 4) & 0x3FFF) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
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

// Issue a 32-lane x 16-column TMEM load without waiting (tmem_ld_wait completes it).
__device__ __forceinline__ void tmem_ld16_issue(uint32_t taddr, uint32_t *r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ void tmem_ld_wait() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 4-D TMA tile load global -> shared, completing on `bar`.
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            int w, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w),
        "r"(smem_addr(bar))
        : "memory");
}

struct TcParams {
    int ytile;
    int bulk;          // ytile == CT: a stage is one contiguous block, loaded by one bulk copy
    const unsigned char *y;   // spectra (bulk loads)
    int y_frames;      // frames per spectra tile (bulk loads)
    int in_fmt;        // SpectraFormat: FP16 pairs, or FP16 hi/lo pairs (already scaled)
    int n_station;
    int n_freq;
    int frames;
    void *acc;         // float2 row, or double2 row when acc64
    int acc64;
    int *err;
    float inv_scale2;  // 1/scale^2: undoes the F-engine's spectra scale in S
    TcGeom g;
};

struct TcBars {
    uint64_t load_full[kMaxLoadStages];  // a stage's TMA load landed (tx-count)
    uint64_t load_empty[kMaxLoadStages]; // converters finished reading a slot (256 arrivals)
    uint64_t op_full[kMaxOpStages];      // converters wrote a stage's operands (256 arrivals)
    uint64_t op_empty[kMaxOpStages];     // MMAs reading an operand buffer finished (commit)
    uint64_t acc_full[2];                // a tile's MMAs finished (commit), per set
    uint64_t acc_empty[2];               // epilogue read a set (128 arrivals)
    uint64_t epi;                        // epilogue-only sync (128 arrivals, twice per tile)
    uint64_t fin;                        // abort path: every MMA this CTA issued finished
};

__global__ void __launch_bounds__(kThreads, 1)
    xengine_tc_kernel(const __grid_constant__ CUtensorMap ymap, TcParams p) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
    __shared__ TcBars bars;
    __shared__ uint32_t s_tmem_base;
    __shared__ int s_abort;
    __shared__ uint32_t s_ld_issued;   // TMA loads issued (abort drain)

    const TcGeom &g = p.g;
    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const int N = p.n_station;
    const int n_tiles = p.n_freq / g.ct;
    const int my_tiles = (n_tiles - static_cast<int>(blockIdx.x) + static_cast<int>(gridDim.x) - 1) /
                         static_cast<int>(gridDim.x);
    const int n_stages = (p.frames + g.kt - 1) / g.kt;
    const int total = my_tiles * n_stages;
    const int n_baseline = N * (N + 1) / 2;
    unsigned char *ld_ring = smem;
    unsigned char *op_ring = smem + g.n_ld * g.ld_stage;
    float2 *Vs = reinterpret_cast<float2 *>(op_ring + g.n_op * g.op_stage);
    float2 *Qs = reinterpret_cast<float2 *>(reinterpret_cast<unsigned char *>(Vs) + g.vs_bytes);
    uint16_t *jk = reinterpret_cast<uint16_t *>(reinterpret_cast<unsigned char *>(Qs) + g.qs_bytes);

    // Operand rows no conversion writes (a region's padding rows, the reach of
    // the last region's A) must hold finite values: zero them once, and make
    // the zeros visible to the tensor cores' (async-proxy) reads.
    for (int i = tid; i < g.n_op * g.op_stage / 16; i += kThreads)
        reinterpret_cast<uint4 *>(op_ring)[i] = make_uint4(0, 0, 0, 0);
    fence_proxy_async_smem();
    for (int b = tid; b < n_baseline; b += kThreads) {
        int j = 0, rem = b;
        while (rem >= N - j) {
            rem -= N - j;
            ++j;
        }
        jk[b] = static_cast<uint16_t>((j << 8) | (j + rem));
    }
    if (tid == 0) {
        for (int s = 0; s < g.n_ld; ++s) {
            mbar_init(&bars.load_full[s], 1);
            mbar_init(&bars.load_empty[s], kConverters);
        }
        for (int s = 0; s < g.n_op; ++s) {
            mbar_init(&bars.op_full[s], kConverters);
            mbar_init(&bars.op_empty[s], kIssuers);
        }
        for (int s = 0; s < 2; ++s) {
            mbar_init(&bars.acc_full[s], kIssuers);
            mbar_init(&bars.acc_empty[s], kEpilogue);
        }
        mbar_init(&bars.epi, kEpilogue);
        mbar_init(&bars.fin, kIssuers);
        s_abort = 0;
        s_ld_issued = 0;
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
    const volatile int *abort_flag = &s_abort;

    auto tile_c0 = [&](int tl) {
        return (static_cast<int>(blockIdx.x) + tl * static_cast<int>(gridDim.x)) * g.ct;
    };

    if (warp == 0) {
        // ---------------------------- TMA loads ----------------------------
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&ymap))
                         : "memory");
            for (int gs = 0; gs < total && *abort_flag == 0; ++gs) {
                const int tl = gs / n_stages;
                const int st = gs - tl * n_stages;
                const int slot = gs % g.n_ld;
                const int use = gs / g.n_ld;
                if (use > 0 &&
                    !mbar_wait_bounded(&bars.load_empty[slot], static_cast<uint32_t>(use - 1) & 1u,
                                       p.err, kErrXengineMmaTimeout, abort_flag)) {
                    s_abort = 1;
                    break;
                }
                const int c0 = tile_c0(tl);
                if (p.bulk) {
                    // channel tiles of CT bins: the stage's frames x stations x CT
                    // bins are contiguous. Only the launch's frames are copied; the
                    // converters treat the rest of a last, partial stage as zeros.
                    const int f0 = st * g.kt;
                    const int nf = min(g.kt, p.frames - f0);
                    const uint32_t row = static_cast<uint32_t>(N * g.ct * g.elem);
                    const unsigned char *src =
                        p.y + (static_cast<size_t>(c0 / g.ct) * p.y_frames + f0) * row;
                    mbar_arrive_expect_tx(&bars.load_full[slot], nf * row);
                    bulk_copy_g2s(ld_ring + slot * g.ld_stage, src, nf * row,
                                  &bars.load_full[slot]);
                } else {
                    mbar_arrive_expect_tx(&bars.load_full[slot],
                                          static_cast<uint32_t>(g.ld_stage));
                    // frames past `frames` (the map's last frame) arrive as zeros
                    tma_load_4d(ld_ring + slot * g.ld_stage, &ymap, c0 % p.ytile, 0,
                                st * g.kt, c0 / p.ytile, &bars.load_full[slot]);
                }
                ++s_ld_issued;
            }
        }
    } else if (warp < kFirstConverterWarp) {
        // ------------------------------ MMAs ------------------------------
        // issuer i: regions i, i + kIssuers, ... Every issuer commits every
        // stage (op_empty and acc_full count kIssuers arrivals), with or
        // without MMAs of its own.
        const int issuer = warp - 1;
        if (lane == 0) {
            const uint32_t idesc = instr_desc_f16_f32(128, g.nb);
            const int ksteps = g.kt / 16;
            // Descriptors differ only in their start-address field, which
            // cannot carry: (address >> 4) of shared memory fits its 14 bits.
            const uint64_t desc0 = smem_desc(smem_addr(op_ring), g.sbo);
            for (int gs = 0; gs < total && *abort_flag == 0; ++gs) {
                const int tl = gs / n_stages;
                const int st = gs - tl * n_stages;
                const int ob = gs % g.n_op;
                const int aset = tl % g.n_acc;
                const int use = tl / g.n_acc;   // earlier tiles that used this set
                if (st == 0 && use > 0) {
                    // this set's previous tile must be read before it is overwritten
                    if (!mbar_wait_bounded(&bars.acc_empty[aset], static_cast<uint32_t>(use - 1) & 1u,
                                           p.err, kErrXengineMmaTimeout, abort_flag)) {
                        s_abort = 1;
                        break;
                    }
                }
                if (!mbar_wait_bounded(&bars.op_full[ob], static_cast<uint32_t>(gs / g.n_op) & 1u,
                                       p.err, kErrXengineMmaTimeout, abort_flag)) {
                    s_abort = 1;
                    break;
                }
                tc_fence_after();
                const uint64_t dstage = desc0 + (static_cast<uint32_t>(ob * g.op_stage) >> 4);
                const uint32_t dset = tmem + static_cast<uint32_t>(aset * g.acc_cols);
                for (int r = issuer; r < g.regions; r += kIssuers) {
                    const uint32_t d = dset + static_cast<uint32_t>(r * g.nb);
                    const uint64_t dr =
                        dstage + (static_cast<uint32_t>(r * g.region_stride + region_skew(r)) >> 4);
                    for (int ks = 0; ks < ksteps; ++ks) {
                        const uint64_t desc = dr + static_cast<uint32_t>(ks * 2 * kLBO / 16);
                        umma_f16(d, desc, desc, idesc, (st > 0 || ks > 0) ? 1u : 0u);
                    }
                }
                umma_commit(&bars.op_empty[ob]);
                if (st == n_stages - 1) umma_commit(&bars.acc_full[aset]);
            }
        }
    } else if (warp < kFirstEpilogueWarp) {
        // --------------------------- converters ---------------------------
        const int wt = tid - 32 * kFirstConverterWarp;
        // This thread's items (channel c, station s, 8-frame group kq) are the
        // same every stage: keep their fp32 and operand offsets.
        int n_item = 0;
        uint32_t item_ok = 0;                   // bit i: item i exists (station groups may be short)
        uint32_t it_ld[kMaxItems], it_op[kMaxItems];
        int it_f0[kMaxItems];                   // first frame of the item's 8-frame group
        const int lo_off = (g.R / 8) * g.sbo;   // Dl rows start at row R
#pragma unroll
        for (int i = 0; i < kMaxItems; ++i) {
            it_ld[i] = 0;
            it_op[i] = 0;
            it_f0[i] = 0;
            const int q = wt + i * kConverters;
            int c, s, kq;
            if (g.form == kFp16Paired) {
                // A quarter warp (whose 16-byte stores share one bank line) takes
                // every region x four consecutive stations of one channel half.
                // Rows 2s of four stations fall in four distinct 16-byte slots and
                // the region skew separates the regions; the two halves of a
                // region are R = 64 rows = 8 row groups apart, the same slot, so
                // they go to different quarter warps.
                const int regions = g.ct / 2;
                int rest = q / regions;
                const int s_lo = rest % 4;
                rest /= 4;
                const int half = rest % 2;
                rest /= 2;
                const int groups = (N + 3) / 4;
                s = (rest % groups) * 4 + s_lo;
                kq = rest / groups;
                c = (q % regions) * 2 + half;
            } else {
                c = q % g.ct;
                const int rest = q / g.ct;
                s = rest % N;
                kq = rest / N;
            }
            if (q < g.items && s < N) {
                int region = c, row = 2 * s;
                if (g.form == kFp16Paired) {
                    region = c >> 1;
                    row += (c & 1) * g.R;
                }
                it_ld[i] = static_cast<uint32_t>((kq * 8 * N + s) * g.ct + c);
                it_op[i] = static_cast<uint32_t>(region * g.region_stride + region_skew(region) +
                                                 (row >> 3) * g.sbo + kq * kLBO + (row & 7) * 16);
                it_f0[i] = kq * 8;
                n_item = i + 1;
                item_ok |= 1u << i;
            }
        }
        const int row_step = N * g.ct;   // float2 between consecutive frames of a slot
        for (int gs = 0; gs < total; ++gs) {
            const int lb = gs % g.n_ld;
            const int ob = gs % g.n_op;
            bool ok = mbar_wait_bounded(&bars.load_full[lb], static_cast<uint32_t>(gs / g.n_ld) & 1u,
                                        p.err, kErrXengineMmaTimeout, abort_flag);
            if (ok && gs >= g.n_op)
                ok = mbar_wait_bounded(&bars.op_empty[ob],
                                       static_cast<uint32_t>(gs / g.n_op - 1) & 1u, p.err,
                                       kErrXengineMmaTimeout, abort_flag);
            if (!ok) {
                s_abort = 1;
                break;
            }
            // spectra slot: [frame][station][CT channels]
            const float2 *ld = reinterpret_cast<const float2 *>(ld_ring + lb * g.ld_stage);
            unsigned char *op = op_ring + ob * g.op_stage;
            // Frames of a bulk-loaded last stage past the launch's frames were not
            // copied (stale bytes): they convert as zeros. A tensor-map load
            // zero-fills them itself.
            const int st_here = gs % n_stages;
            const int n_valid = p.bulk ? min(g.kt, p.frames - st_here * g.kt) : g.kt;
            auto convert = [&](auto guard_tag) {
                constexpr bool kGuard = decltype(guard_tag)::value;
                if (p.in_fmt == kSpectraF16) {
                    // FP16 pairs (re, im) per frame: regroup into 8-frame rows of re
                    // and of im, two byte-permutes per frame pair
                    const uint32_t *ld16 = reinterpret_cast<const uint32_t *>(ld);
#pragma unroll
                    for (int it = 0; it < kMaxItems; ++it) {
                        if (it >= n_item) break;
                        if (!((item_ok >> it) & 1u)) continue;
                        const uint32_t *src = ld16 + it_ld[it];
                        uint32_t hre[4], him[4];
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            uint32_t w0 = 0, w1 = 0;
                            if (!kGuard || it_f0[it] + 2 * i < n_valid) w0 = src[(2 * i) * row_step];
                            if (!kGuard || it_f0[it] + 2 * i + 1 < n_valid)
                                w1 = src[(2 * i + 1) * row_step];
                            hre[i] = __byte_perm(w0, w1, 0x5410);
                            him[i] = __byte_perm(w0, w1, 0x7632);
                        }
                        unsigned char *dst = op + it_op[it];
                        *reinterpret_cast<uint4 *>(dst) = make_uint4(hre[0], hre[1], hre[2], hre[3]);
                        *reinterpret_cast<uint4 *>(dst + 16) =
                            make_uint4(him[0], him[1], him[2], him[3]);
                    }
                } else {
                    // FP16 hi/lo pairs per frame: the Dh rows from the h words, the
                    // Dl rows from the l words
                    const uint2 *ld2 = reinterpret_cast<const uint2 *>(ld);
#pragma unroll
                    for (int it = 0; it < kMaxItems; ++it) {
                        if (it >= n_item) break;
                        if (!((item_ok >> it) & 1u)) continue;
                        const uint2 *src = ld2 + it_ld[it];
                        uint32_t hre[4], him[4], lre[4], lim[4];
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            uint2 w0 = make_uint2(0u, 0u), w1 = make_uint2(0u, 0u);
                            if (!kGuard || it_f0[it] + 2 * i < n_valid) w0 = src[(2 * i) * row_step];
                            if (!kGuard || it_f0[it] + 2 * i + 1 < n_valid)
                                w1 = src[(2 * i + 1) * row_step];
                            hre[i] = __byte_perm(w0.x, w1.x, 0x5410);
                            him[i] = __byte_perm(w0.x, w1.x, 0x7632);
                            lre[i] = __byte_perm(w0.y, w1.y, 0x5410);
                            lim[i] = __byte_perm(w0.y, w1.y, 0x7632);
                        }
                        unsigned char *dst = op + it_op[it];
                        *reinterpret_cast<uint4 *>(dst) = make_uint4(hre[0], hre[1], hre[2], hre[3]);
                        *reinterpret_cast<uint4 *>(dst + 16) =
                            make_uint4(him[0], him[1], him[2], him[3]);
                        *reinterpret_cast<uint4 *>(dst + lo_off) =
                            make_uint4(lre[0], lre[1], lre[2], lre[3]);
                        *reinterpret_cast<uint4 *>(dst + lo_off + 16) =
                            make_uint4(lim[0], lim[1], lim[2], lim[3]);
                    }
                }
            };
            if (n_valid == g.kt)
                convert(std::false_type{});
            else
                convert(std::true_type{});
            mbar_arrive(&bars.load_empty[lb]);   // the spectra slot may be refilled
            fence_proxy_async_smem();   // operand stores -> visible to the tensor cores
            mbar_arrive(&bars.op_full[ob]);
        }
    } else {
        // ---------------------------- epilogue ----------------------------
        const int et = tid - 32 * kFirstEpilogueWarp;
        const int quad = warp & 3;             // TMEM lanes [32*quad, 32*quad+32)
        const int nchunks = (2 * N + 15) / 16;
        const int nq = g.ct / 2;                // float4 (two channels) per baseline
        const int nblk = g.split ? 2 : 1;
        // Staging, one plane per channel, j fastest so that the row lanes of a
        // warp (consecutive j) store to consecutive addresses:
        //   Vt[c][k(k+1)/2 + j] = V[j][k] (j <= k),  Qs[c][k][j] = Q[j][k].
        const int plane_v = n_baseline;
        for (int tl = 0; tl < my_tiles; ++tl) {
            const int aset = tl % g.n_acc;
            if (!mbar_wait_bounded(&bars.acc_full[aset], static_cast<uint32_t>(tl / g.n_acc) & 1u,
                                   p.err, kErrXengineMmaTimeout, abort_flag)) {
                s_abort = 1;
                break;
            }
            tc_fence_after();
            const uint32_t tbase = tmem + (static_cast<uint32_t>(quad * 32) << 16) +
                                   static_cast<uint32_t>(aset * g.acc_cols);
            for (int c = 0; c < g.ct; ++c) {
                for (int bk = 0; bk < nblk; ++bk) {
                    // block = rows [lb, lb+2N) x columns [cb, cb+2N) of the set
                    const bool isq = bk == 1;
                    int lb = 0, cb = c * g.nb;
                    if (g.form == kFp16Paired) {
                        lb = (c & 1) * g.R;
                        cb = (c >> 1) * g.nb + (c & 1) * g.R;
                    } else if (isq && g.form == kSplitStacked) {
                        lb = g.R;
                    } else if (isq) {
                        cb += g.R;   // wide split: T = P^T in columns [R, R+2N)
                    }
                    // warp-uniform: does this quarter hold any of the block's rows?
                    if (quad * 32 + 32 <= lb || quad * 32 >= lb + 2 * N) continue;
                    const int m = quad * 32 + lane - lb;
                    const bool row_lane = ((m & 1) == 0) && m >= 0 && m < 2 * N;
                    const int j = m >> 1;
                    // up to four 16-column chunks per TMEM wait
                    for (int c0 = 0; c0 < nchunks; c0 += 4) {
                        uint32_t r[4][16];
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            if (c0 + q < nchunks) tmem_ld16_issue(tbase + cb + (c0 + q) * 16, r[q]);
                        tmem_ld_wait();
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            if (c0 + q >= nchunks) break;
                            float v[16], w[16];
#pragma unroll
                            for (int i = 0; i < 16; ++i) {
                                v[i] = __uint_as_float(r[q][i]);
                                w[i] = __shfl_down_sync(0xffffffffu, v[i], 1);
                            }
                            if (row_lane) {
#pragma unroll
                                for (int t = 0; t < 8; ++t) {
                                    const int k = (c0 + q) * 8 + t;
                                    // v = row 2j, w = row 2j+1
                                    const float re = (v[2 * t] + w[2 * t + 1]) * p.inv_scale2;
                                    const float im = (w[2 * t] - v[2 * t + 1]) * p.inv_scale2;
                                    if (k < N) {
                                        if (isq)
                                            Qs[(c * N + k) * N + j] = make_float2(re, im);
                                        else if (k >= j)
                                            Vs[c * plane_v + k * (k + 1) / 2 + j] =
                                                make_float2(re, im);
                                    }
                                }
                            }
                        }
                    }
                }
            }
            // this set is read: the MMAs of tile tl + n_acc may start
            tc_fence_before();
            mbar_arrive(&bars.acc_empty[aset]);
            mbar_arrive(&bars.epi);
            if (!mbar_wait_bounded(&bars.epi, 0u, p.err, kErrXengineMmaTimeout, abort_flag)) {
                s_abort = 1;
                break;
            }
            // V (+ Q[j][k] + conj(Q[k][j])) into the row: this CTA is the only
            // writer of these channels in this launch.
            const int c0 = tile_c0(tl);
            // Four read-modify-writes per thread in flight: all loads first.
            constexpr int kBatch = 4;
            const int n_items = n_baseline * nq;
            // visibilities of channels c, c+1 of item q's baseline
            auto vis = [&](int q, float2 &v0, float2 &v1) {
                const int b = q / nq;
                const int c = (q - b * nq) * 2;
                const int j = jk[b] >> 8, k = jk[b] & 0xff;
                const int tri = k * (k + 1) / 2 + j;
                v0 = Vs[c * plane_v + tri];
                v1 = Vs[(c + 1) * plane_v + tri];
                if (g.split) {
                    const float2 qa0 = Qs[(c * N + k) * N + j], qb0 = Qs[(c * N + j) * N + k];
                    const float2 qa1 = Qs[((c + 1) * N + k) * N + j];
                    const float2 qb1 = Qs[((c + 1) * N + j) * N + k];
                    v0.x += qa0.x + qb0.x;
                    v0.y += qa0.y - qb0.y;
                    v1.x += qa1.x + qb1.x;
                    v1.y += qa1.y - qb1.y;
                }
            };
            auto row_offset = [&](int q) {
                const int b = q / nq;
                const int c = (q - b * nq) * 2;
                return static_cast<size_t>(b) * p.n_freq + c0 + c;
            };
            if (p.acc64) {
                // complex128 row: the launch's FP32 sums are added in double, as
                // reductions performed in L2 (red.global.add.f64): this CTA is the
                // only writer of these values in the launch, so the result is the
                // same as a read-modify-write, without waiting for the reads.
                double *acc = static_cast<double *>(p.acc);
                for (int q = et; q < n_items; q += kEpilogue) {
                    float2 v0, v1;
                    vis(q, v0, v1);
                    double *dst = acc + 2 * row_offset(q);
                    red_add_f64(dst + 0, v0.x);
                    red_add_f64(dst + 1, v0.y);
                    red_add_f64(dst + 2, v1.x);
                    red_add_f64(dst + 3, v1.y);
                }
            } else {
                float2 *acc = static_cast<float2 *>(p.acc);
                for (int q0 = et; q0 < n_items; q0 += kEpilogue * kBatch) {
                    float4 a[kBatch];
#pragma unroll
                    for (int u = 0; u < kBatch; ++u) {
                        const int q = q0 + u * kEpilogue;
                        if (q < n_items) a[u] = *reinterpret_cast<const float4 *>(acc + row_offset(q));
                    }
#pragma unroll
                    for (int u = 0; u < kBatch; ++u) {
                        const int q = q0 + u * kEpilogue;
                        if (q >= n_items) break;
                        float2 v0, v1;
                        vis(q, v0, v1);
                        a[u].x += v0.x;
                        a[u].y += v0.y;
                        a[u].z += v1.x;
                        a[u].w += v1.y;
                        *reinterpret_cast<float4 *>(acc + row_offset(q)) = a[u];
                    }
                }
            }
            // everyone done with Vs/Qs before the next tile overwrites them
            mbar_arrive(&bars.epi);
            if (!mbar_wait_bounded(&bars.epi, 1u, p.err, kErrXengineMmaTimeout, abort_flag)) {
                s_abort = 1;
                break;
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    if (s_abort && warp >= 1 && warp < kFirstConverterWarp && lane == 0) {
        // Let every MMA this CTA issued finish before TMEM goes away (bounded;
        // the watchdog code is already recorded). A commit covers the issuing
        // thread's earlier MMAs; fin completes once every issuer committed.
        umma_commit(&bars.fin);
        mbar_wait_bounded(&bars.fin, 0u, nullptr, 0);
    }
    if (s_abort && tid == 0) {
        // Let every TMA load land before the CTA's shared memory goes away. A
        // slot whose load was consumed completed its phase; one still in flight
        // completes the phase after the last one consumed.
        for (int s = 0; s < g.n_ld; ++s) {
            // loads issued into slot s (round robin from stage 0); the last
            // one's completion is phase n_s - 1 of that slot's barrier
            const uint32_t n_s = (s_ld_issued + g.n_ld - 1 - s) / g.n_ld;
            if (n_s > 0) mbar_wait_bounded(&bars.load_full[s], (n_s - 1) & 1u, nullptr, 0);
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(g.tmem_cols)
                     : "memory");
    }
}

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
// (no link-time dependency on libcuda).
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(f);
        else
            cudaGetLastError();
    });
    return fn;
}

} // namespace

bool xengine_tc_shape_ok(int n_station, bool split, int ct, int kt) {
    return make_geom(n_station, split, ct, kt).ok;
}

} // namespace corrgb

extern "C" corr_status corrx_tc_geometry(int32_t n_station, int32_t split, int32_t ct,
                                         int32_t kt, corrx_tc_geom *out) {
    using namespace corrgb;
    if (out == nullptr) return fail(CORR_ERR_ARG, "out must not be NULL");
    if (out->struct_size != sizeof(corrx_tc_geom))
        return failf(CORR_ERR_ABI, "corrx_tc_geom.struct_size=%u, expected %zu", out->struct_size,
                     sizeof(corrx_tc_geom));
    const TcGeom g = make_geom(n_station, split != 0, ct, kt);
    const uint32_t size = out->struct_size;
    *out = corrx_tc_geom{};
    out->struct_size = size;
    if (!g.ok) return CORR_OK;
    out->ok = 1;
    out->form = g.form;
    out->elem = g.elem;
    out->R = g.R;
    out->nb = g.nb;
    out->regions = g.regions;
    out->sbo = g.sbo;
    out->region_stride = g.region_stride;
    out->op_stage = g.op_stage;
    out->ld_stage = g.ld_stage;
    out->n_op = g.n_op;
    out->n_ld = g.n_ld;
    out->acc_cols = g.acc_cols;
    out->n_acc = g.n_acc;
    out->tmem_cols = g.tmem_cols;
    out->items = g.items;
    out->smem = g.smem;
    return CORR_OK;
}

namespace corrgb {

void xengine_tc_default_shape(int n_station, bool split, int *ct, int *kt) {
    // 32-frame stages halve the per-stage handoffs of 16-frame ones; then the
    // widest tile that fits.
    *ct = 0;
    *kt = 0;
    for (int k : {32, 16})
        for (int c = 8; c >= 2; c /= 2)
            if (make_geom(n_station, split, c, k).ok) {
                *ct = c;
                *kt = k;
                return;
            }
}

corr_status xengine_tc_launch(const XengineArgs &a, bool split, int ct, int kt, int num_sms,
                              cudaStream_t stream) {
    if (a.frames <= 0) return CORR_OK;
    const TcGeom g = make_geom(a.n_station, split, ct, kt);
    if (!g.ok)
        return failf(CORR_ERR_NOT_IMPL,
                     "tensor X-engine: no %s tile of %d channels x %d frames for %d inputs",
                     split ? "split" : "fp16", ct, kt, a.n_station);
    if (a.n_freq % g.ct != 0)
        return failf(CORR_ERR_ARG, "n_freq=%d is not a multiple of %d channels", a.n_freq, g.ct);
    if (a.y_frames < a.frames)
        return fail(CORR_ERR_INTERNAL, "spectra buffer shallower than the launch");
    if (a.ytile < g.ct || a.ytile % g.ct != 0 || a.n_freq % a.ytile != 0)
        return failf(CORR_ERR_INTERNAL, "spectra tiles of %d channels, tensor tiles of %d",
                     a.ytile, g.ct);
    if ((reinterpret_cast<uintptr_t>(a.acc) & 15) != 0)
        return fail(CORR_ERR_ARG, "the tensor X-engine needs a 16-byte aligned accumulator");
    if (a.y_fmt != (split ? kSpectraF16Split : kSpectraF16))
        return fail(CORR_ERR_INTERNAL, "spectra format does not match the X-engine form");
    if ((a.ytile * g.elem) % 16 != 0)
        return failf(CORR_ERR_ARG, "spectra tiles of %d bins are not a multiple of 16 bytes",
                     a.ytile);
    EncodeTiledFn enc = encode_tiled();
    if (enc == nullptr)
        return fail(CORR_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    // Spectra as a 4-D array of bins (4 or 8 bytes), innermost first:
    // (channel within its tile, station, frame, tile); a stage is KT*N rows of
    // CT bins. The frame extent is the launch's, so frames past it read as zeros.
    CUtensorMap map;
    const cuuint64_t row = static_cast<cuuint64_t>(a.ytile) * g.elem;
    const CUtensorMapDataType etype =
        g.elem == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32;
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const cuuint64_t dims[4] = {static_cast<cuuint64_t>(a.ytile),
                                static_cast<cuuint64_t>(a.n_station),
                                static_cast<cuuint64_t>(a.frames),
                                static_cast<cuuint64_t>(a.n_freq / a.ytile)};
    const cuuint64_t strides[3] = {row, row * a.n_station, row * a.n_station * a.y_frames};
    const cuuint32_t box[4] = {static_cast<cuuint32_t>(g.ct), static_cast<cuuint32_t>(a.n_station),
                               static_cast<cuuint32_t>(g.kt), 1};
    const CUresult cr =
        enc(&map, etype, 4, const_cast<float2 *>(a.y), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS)
        return failf(CORR_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", static_cast<int>(cr));
    // The shared-memory limit is a per-device setting: raise it once on each
    // device to the most any feasible shape uses (kMaxSmem), not per shape.
    static PerDevice setup;
    corr_status st = setup.run([](int) {
        return cuda_check(cudaFuncSetAttribute(xengine_tc_kernel,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               kMaxSmem),
                          "cudaFuncSetAttribute(xengine_tc)");
    });
    if (st != CORR_OK) return st;
    TcParams p{};
    p.ytile = a.ytile;
    p.bulk = a.ytile == g.ct;
    p.y = reinterpret_cast<const unsigned char *>(a.y);
    p.y_frames = a.y_frames;
    if (p.bulk && (reinterpret_cast<uintptr_t>(a.y) & 15) != 0)
        return fail(CORR_ERR_INTERNAL, "spectra buffer is not 16-byte aligned");
    p.in_fmt = a.y_fmt;
    p.n_station = a.n_station;
    p.n_freq = a.n_freq;
    p.frames = a.frames;
    p.acc = a.acc;
    p.acc64 = a.acc64;
    p.err = a.err;
    const float scale = spectra_scale(a.n_freq);   // applied by the F-engine
    p.inv_scale2 = 1.0f / (scale * scale);
    p.g = g;
    const int n_tiles = a.n_freq / g.ct;
    const int grid = std::min(n_tiles, std::max(1, num_sms));
    xengine_tc_kernel<<<grid, kThreads, g.smem, stream>>>(map, p);
    return cuda_check(cudaGetLastError(), "xengine_tc_kernel launch");
}

} // namespace corrgb
