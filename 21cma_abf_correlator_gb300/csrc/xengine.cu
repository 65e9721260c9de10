// xengine.cu -- plain FP32 X-engine and the row scaling kernel.
//
// Replaces corr_kernel (corr-cuda/src/kernels.cu:194-265): for every baseline
// b = (j,k), j <= k, and channel c,
//     acc[b][c] += sum_f Y_j[f][c] * conj(Y_k[f][c])
// with the reference's complex multiply-accumulate convention
//     re += xr*yr + xi*yi,  im += xi*yr - xr*yi          (kernels.cu:243-245)
// in FP32 and in that order (the product pair rounded, then added to the
// accumulator), issued as packed FP32x2 instructions.
//
// Shape: a CTA owns a tile of 32 channels (lane = channel) and a group of 4x4
// station blocks (warp = block pair). Spectra for 2 to 12 frames of every
// station in the tile are staged in shared memory by a 3-deep cp.async ring;
// each thread keeps 16 complex accumulators in registers for the whole launch
// and adds them into the row once at the end. Unlike the reference (one thread
// per baseline, <= 1024 threads per block) the station-block tiling gives each
// shared-memory load four multiply-accumulates.

#include <algorithm>
#include <type_traits>

#include "engine.h"
#include "ptx.cuh"

namespace corrgb {
namespace {

constexpr int kXch = 32;     // channels per CTA, one per lane
constexpr int kXstages = 3;  // cp.async ring depth
// frames per pipeline stage: as many of 12, 8, 4, 2 as three stages fit in
// shared memory (12 up to 24 padded stations, 8 up to 36, 4 up to 72, 2 up to
// 144); fewer stages mean fewer CTA barriers
constexpr int kXfsWidest = 12, kXfsWide = 8, kXfsNarrow = 4, kXfsTiny = 2;
constexpr int kBlk = 4;      // stations per block

__device__ __forceinline__ void decode_pair(int p, int nb, int *bj, int *bk) {
    int j = 0;
    while (p >= nb - j) {
        p -= nb - j;
        ++j;
    }
    *bj = j;
    *bk = j + p;
}

template <int kXfs>
__global__ void __launch_bounds__(1024, 1)
    xengine_plain_kernel(const float2 *__restrict__ y, int y_frames, int ytile, int n_station,
                         int npad, int n_freq, int frames, void *__restrict__ acc,
                         int acc64, int pairs_per_cta, int pair_first, int n_pairs,
                         const int32_t *__restrict__ pair_list) {
    extern __shared__ __align__(16) float2 xs[];   // [stage][frame][npad][32]
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nthreads = blockDim.x;
    const int c0 = blockIdx.y * kXch;
    const int nb = npad / kBlk;
    const int q = blockIdx.x * pairs_per_cta + warp;   // among the pairs computed
    const bool active = q < n_pairs && warp < pairs_per_cta;
    const int p = !active ? 0 : pair_list != nullptr ? pair_list[q] : pair_first + q;
    int bj = 0, bk = 0;
    if (active) decode_pair(p, nb, &bj, &bk);

    const int stage_elems = kXfs * npad * kXch;
    const int chunks = stage_elems / 2;   // 16-byte pieces per stage
    const int n_stages = (frames + kXfs - 1) / kXfs;

    // Every thread copies the same two channels (blockDim is a multiple of 16):
    // piece `part` of each (frame, station) row of the stage.
    const int part = threadIdx.x & 15;
    const int cq = c0 + part * 2;
    const float2 *ybase = y + y_index(cq, 0, 0, n_station, y_frames, ytile);
    auto load_stage = [&](int s) {
        float2 *dst = xs + (s % kXstages) * stage_elems;
        const int f0 = s * kXfs;
        for (int q = threadIdx.x; q < chunks; q += nthreads) {
            const int row = q >> 4;                  // frame*npad + station
            const int fi = row / npad;
            const int st = row - fi * npad;
            const int f = f0 + fi;
            const bool ok = (st < n_station) && (f < frames);
            // two channels per 16-byte piece, inside one channel tile
            const float2 *src =
                ok ? ybase + (static_cast<size_t>(f) * n_station + st) * ytile : y;
            cp_async16(dst + row * kXch + part * 2, src, ok ? 16u : 0u);
        }
    };

    float2 a[kBlk][kBlk];
#pragma unroll
    for (int i = 0; i < kBlk; ++i)
#pragma unroll
        for (int l = 0; l < kBlk; ++l) a[i][l] = make_float2(0.f, 0.f);

#pragma unroll
    for (int s = 0; s < kXstages - 1; ++s) {
        if (s < n_stages) load_stage(s);
        cp_async_commit();
    }
    for (int s = 0; s < n_stages; ++s) {
        cp_async_wait<kXstages - 2>();
        __syncthreads();
        if (s + kXstages - 1 < n_stages) load_stage(s + kXstages - 1);
        cp_async_commit();
        if (active) {
            const float2 *st = xs + (s % kXstages) * stage_elems;
            // A warp whose two blocks are the same keeps only j <= k: it loads
            // one block and skips the pairs below the diagonal (uniform per warp).
            auto stage = [&](auto diag) {
                constexpr bool DIAG = decltype(diag)::value;
#pragma unroll
                for (int fi = 0; fi < kXfs; ++fi) {
                    const float2 *fr = st + fi * npad * kXch + lane;
                    float2 xj[kBlk], xk[kBlk];
#pragma unroll
                    for (int i = 0; i < kBlk; ++i) {
                        xj[i] = fr[(bj * kBlk + i) * kXch];
                        xk[i] = DIAG ? xj[i] : fr[(bk * kBlk + i) * kXch];
                    }
                    // a += xj * conj(xk) in the reference's rounding order (the
                    // pair's product, then one add to the accumulator), packed:
                    //   t = (xj.x, xj.y) * (xk.x, xk.x)
                    //   t = (xj.y, -xj.x) * (xk.y, xk.y) + t
                    //   (re, im) += t
                    // the swapped and broadcast operands built once per station
                    float2 xjs[kBlk];
#pragma unroll
                    for (int i = 0; i < kBlk; ++i) xjs[i] = make_float2(xj[i].y, -xj[i].x);
#pragma unroll
                    for (int l = 0; l < kBlk; ++l) {
                        const float2 kx = make_float2(xk[l].x, xk[l].x);
                        const float2 ky = make_float2(xk[l].y, xk[l].y);
#pragma unroll
                        for (int i = 0; i < kBlk; ++i)
                            if (!DIAG || i <= l)
                                a[i][l] = cadd(a[i][l], fma2(xjs[i], ky, mul2(xj[i], kx)));
                    }
                }
            };
            if (bj == bk)
                stage(std::true_type{});
            else
                stage(std::false_type{});
        }
    }
    cp_async_wait<0>();

    if (!active) return;
    const int c = c0 + lane;
#pragma unroll
    for (int i = 0; i < kBlk; ++i) {
        const int j = bj * kBlk + i;
#pragma unroll
        for (int l = 0; l < kBlk; ++l) {
            const int k = bk * kBlk + l;
            if (j <= k && k < n_station) {
                const int b = j * n_station - j * (j - 1) / 2 + (k - j);
                const size_t at = static_cast<size_t>(b) * n_freq + c;
                if (acc64) {   // complex128 row: the launch's FP32 sum added in double
                    double2 *dst = static_cast<double2 *>(acc) + at;
                    double2 v = *dst;
                    v.x += a[i][l].x;
                    v.y += a[i][l].y;
                    *dst = v;
                } else {
                    float2 *dst = static_cast<float2 *>(acc) + at;
                    float2 v = *dst;
                    v.x += a[i][l].x;
                    v.y += a[i][l].y;
                    *dst = v;
                }
            }
        }
    }
}

__global__ void scale_kernel(float2 *__restrict__ acc, size_t n, float s) {
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        float2 v = acc[i];
        v.x *= s;
        v.y *= s;
        acc[i] = v;
    }
}

__global__ void scale64_kernel(double2 *__restrict__ acc, size_t n, double s) {
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        double2 v = acc[i];
        v.x *= s;
        v.y *= s;
        acc[i] = v;
    }
}

__global__ void add64_kernel(double2 *__restrict__ dst, const double2 *__restrict__ src,
                             size_t n) {
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        double2 v = dst[i];
        const double2 w = src[i];
        v.x += w.x;
        v.y += w.y;
        dst[i] = v;
    }
}

// Two channels per thread: 32 bytes of complex128 in, 16 bytes of complex64 out.
__global__ void dump64_kernel(float2 *__restrict__ out, size_t out_row,
                              const double2 *__restrict__ src, size_t src_row,
                              const int32_t *__restrict__ gmap, const int32_t *__restrict__ lmap,
                              int n_map, int half_freq, int rows, double s) {
    const size_t per_row = static_cast<size_t>(n_map) * half_freq;
    const size_t n = per_row * rows;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        const int r = static_cast<int>(i / per_row);
        const size_t q = i - static_cast<size_t>(r) * per_row;
        const int m = static_cast<int>(q / half_freq);
        const int c2 = static_cast<int>(q - static_cast<size_t>(m) * half_freq);
        const int gb = gmap ? gmap[m] : m;
        const int lb = lmap ? lmap[m] : m;
        const double2 *a = src + r * src_row + (static_cast<size_t>(lb) * half_freq + c2) * 2;
        const double2 a0 = a[0], a1 = a[1];
        float4 v;
        v.x = static_cast<float>(a0.x * s);
        v.y = static_cast<float>(a0.y * s);
        v.z = static_cast<float>(a1.x * s);
        v.w = static_cast<float>(a1.y * s);
        *reinterpret_cast<float4 *>(out + r * out_row +
                                    (static_cast<size_t>(gb) * half_freq + c2) * 2) = v;
    }
}

// One thread records the GPU's global nanosecond timer: the latency marks of a
// captured batch (a kernel node keeps its place in the graph's order, where an
// event recorded during capture would only express a dependency).
__global__ void stamp_kernel(unsigned long long *slot) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *slot = t;
}

// One thread waits on an mbarrier whose phase never completes (nothing arrives
// on it), with a caller-chosen budget; the bounded wait gives up and records
// kErrSelftestTimeout. The barrier is then retired by arriving on it so the CTA
// exits with nothing pending.
__global__ void watchdog_selftest_kernel(int *err, long long budget) {
    __shared__ uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    fence_mbar_init();
    const long long t0 = clock64();
    bool done = false;
    while (!(done = mbar_try_wait(&bar, 0u))) {
        if (clock64() - t0 > budget) break;
    }
    if (!done) atomicExch(err, kErrSelftestTimeout);
    mbar_arrive(&bar);
}

} // namespace

corr_status watchdog_selftest_launch(int *err, long long budget_cycles, cudaStream_t stream) {
    watchdog_selftest_kernel<<<1, 32, 0, stream>>>(err, budget_cycles);
    return cuda_check(cudaGetLastError(), "watchdog_selftest_kernel launch");
}

corr_status xengine_plain_launch(const XengineArgs &a, int num_sms, cudaStream_t stream) {
    (void)num_sms;
    if (a.frames <= 0) return CORR_OK;
    const int npad = (a.n_station + kBlk - 1) / kBlk * kBlk;
    const int nb = npad / kBlk;
    const int all_pairs = nb * (nb + 1) / 2;
    const bool list = a.pair_list != nullptr && a.pair_count > 0 && a.pair_count <= all_pairs;
    const bool part = list || (a.pair_count > 0 && a.pair_first >= 0 &&
                               a.pair_first + a.pair_count <= all_pairs);
    const int pair_first = part && !list ? a.pair_first : 0;
    const int n_pairs = part ? a.pair_count : all_pairs;
    const int groups = (n_pairs + 31) / 32;
    const int per_cta = (n_pairs + groups - 1) / groups;
    const size_t per_frame = static_cast<size_t>(kXstages) * npad * kXch * sizeof(float2);
    // Deeper stages mean fewer CTA barriers, but a CTA of few warps (as when only
    // some block pairs are computed) needs others beside it on its SM: take the
    // deepest stages among those that give an SM the most warps, up to 16.
    int fs = 0, best = -1;
    for (int f : {kXfsWidest, kXfsWide, kXfsNarrow, kXfsTiny}) {
        const size_t bytes = per_frame * f;
        if (bytes > 227 * 1024) continue;
        const int warps = std::min(16, static_cast<int>((227 * 1024) / bytes) * per_cta);
        if (warps > best) {
            best = warps;
            fs = f;
        }
    }
    if (fs == 0 || per_frame * fs > 227 * 1024)
        return failf(CORR_ERR_ARG, "plain X-engine: %d stations do not fit in shared memory",
                     a.n_station);
    const size_t smem = per_frame * fs;
    static PerDevice setup;   // the shared-memory limit is a per-device setting
    corr_status st = setup.run([](int) {
        for (auto k : {xengine_plain_kernel<kXfsWidest>, xengine_plain_kernel<kXfsWide>,
                       xengine_plain_kernel<kXfsNarrow>, xengine_plain_kernel<kXfsTiny>}) {
            corr_status s2 =
                cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                227 * 1024),
                           "cudaFuncSetAttribute(xengine_plain)");
            if (s2 != CORR_OK) return s2;
        }
        return CORR_OK;
    });
    if (st != CORR_OK) return st;
    dim3 grid(groups, a.n_freq / kXch);
    auto k = fs == kXfsWidest ? xengine_plain_kernel<kXfsWidest>
           : fs == kXfsWide   ? xengine_plain_kernel<kXfsWide>
           : fs == kXfsNarrow ? xengine_plain_kernel<kXfsNarrow>
                              : xengine_plain_kernel<kXfsTiny>;
    k<<<grid, per_cta * 32, smem, stream>>>(a.y, a.y_frames, a.ytile, a.n_station, npad,
                                            a.n_freq, a.frames, a.acc, a.acc64, per_cta,
                                            pair_first, n_pairs, list ? a.pair_list : nullptr);
    return cuda_check(cudaGetLastError(), "xengine_plain_kernel launch");
}

int xengine_plain_block_pair(int n_station, int j, int k) {
    const int nb = (n_station + kBlk - 1) / kBlk;
    const int bj = j / kBlk, bk = k / kBlk;
    // block pairs (bj, bk), bj <= bk, row-major
    return bj * nb - bj * (bj - 1) / 2 + (bk - bj);
}

corr_status scale_launch(float2 *acc, size_t n, float s, cudaStream_t stream) {
    if (n == 0) return CORR_OK;
    size_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    scale_kernel<<<static_cast<unsigned>(blocks), 256, 0, stream>>>(acc, n, s);
    return cuda_check(cudaGetLastError(), "scale_kernel launch");
}

namespace {
unsigned grid_for(size_t n, unsigned cap) {
    size_t blocks = (n + 255) / 256;
    if (blocks > cap) blocks = cap;
    return static_cast<unsigned>(blocks < 1 ? 1 : blocks);
}
} // namespace

corr_status scale64_launch(double2 *acc, size_t n, double s, cudaStream_t stream) {
    if (n == 0) return CORR_OK;
    scale64_kernel<<<grid_for(n, 4096), 256, 0, stream>>>(acc, n, s);
    return cuda_check(cudaGetLastError(), "scale64_kernel launch");
}

corr_status add64_launch(double2 *dst, const double2 *src, size_t n, cudaStream_t stream) {
    if (n == 0) return CORR_OK;
    add64_kernel<<<grid_for(n, 4096), 256, 0, stream>>>(dst, src, n);
    return cuda_check(cudaGetLastError(), "add64_kernel launch");
}

corr_status dump64_launch(float2 *out, size_t out_row, const double2 *src, size_t src_row,
                          const int32_t *gmap, const int32_t *lmap, int n_map, int n_freq,
                          int rows, double s, cudaStream_t stream) {
    if (n_freq % 2 != 0) return fail(CORR_ERR_INTERNAL, "dump64: n_freq must be even");
    const size_t n = static_cast<size_t>(n_map) * (n_freq / 2) * static_cast<size_t>(rows);
    if (n == 0) return CORR_OK;
    dump64_kernel<<<grid_for(n, 4096), 256, 0, stream>>>(out, out_row, src, src_row, gmap, lmap,
                                                          n_map, n_freq / 2, rows, s);
    return cuda_check(cudaGetLastError(), "dump64_kernel launch");
}

// MurmurHash3's 32-bit finaliser (a published integer mixing function).
__device__ __forceinline__ uint32_t mix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

// Sum of four uniform bytes, centred and scaled: close to N(0, 24^2), in int8.
__global__ void synth_fill_kernel(int8_t *x, size_t n, uint32_t seed) {
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        const uint32_t h = mix32(static_cast<uint32_t>(i) ^ mix32(static_cast<uint32_t>(i >> 32) + seed));
        const int sum = static_cast<int>((h & 0xff) + ((h >> 8) & 0xff) + ((h >> 16) & 0xff) +
                                         (h >> 24)) - 510;
        const int v = __float2int_rn(static_cast<float>(sum) * 0.1624f);
        x[i] = static_cast<int8_t>(max(-127, min(127, v)));
    }
}

corr_status synth_fill_launch(int8_t *x, size_t n, uint32_t seed, cudaStream_t stream) {
    if (n == 0) return CORR_OK;
    size_t blocks = (n + 255) / 256;
    if (blocks > 16384) blocks = 16384;
    synth_fill_kernel<<<static_cast<unsigned>(blocks), 256, 0, stream>>>(x, n, seed);
    return cuda_check(cudaGetLastError(), "synth_fill_kernel launch");
}

corr_status stamp_launch(unsigned long long *slot, cudaStream_t stream) {
    stamp_kernel<<<1, 1, 0, stream>>>(slot);
    return cuda_check(cudaGetLastError(), "stamp_kernel launch");
}

} // namespace corrgb
