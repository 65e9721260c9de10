// frontend.cu -- on-device synthetic front end (corrx_frontend_fill).
//
// Generates, on the GPU, the int8 frames and validity mask that the reference's
// receive path would assemble from its test transmitter's packets:
//   * packet contents: corr-rs/src/bin/replay.rs:212-266 (prng_sample,
//     build_packet: zero / counter / prng / sine);
//   * which packets exist: replay.rs:361-372 (per-station start counter and
//     sample delay), :417-426 (gap and uniform loss), :431-441 (delay ladder),
//     :314-320 (ladder origin);
//   * frame assembly: frame id = counter / P, the packet's samples at
//     (counter % P) * 4096 in the frame (corr-rs/src/frame.rs:74-89), and a frame
//     is valid only when all P of its packets arrived (corr-rs/src/assemble.rs:
//     1000-1070, the validity mask of corr_cuda.h).
//
// One launch writes both outputs. Work unit for the samples: one packet (4096
// bytes) per warp, grid-stride over (station, frame, packet). PRNG and SINE are
// functions of the sample index, so lane l computes 16 consecutive bytes at
// 16*l + 512*j and the warp's 16-byte stores are contiguous. COUNTER is a
// sequential xorshift64 chain over the packet's 4096 bytes; xorshift64 is
// linear over GF(2), so lane l jumps to step 128*l with a precomputed 64x64 bit
// matrix T^(128*l) (built per CTA in shared memory from the step itself) and
// then runs its 128 steps. Mask bytes (8 frames each) are done by the same
// threads after the samples.
//
// Integer results are bit-exact with the transmitter. SINE uses IEEE double
// with every multiply, add and divide rounded separately (no contraction), as
// the transmitter's Rust code evaluates it; its sin() is CUDA's, which can
// differ from the host libm's in the last bit, and that can move the rounded
// sample only when 4*sin(t) lies within a few ulp of a half-integer.

#include <cmath>

#include "engine.h"

namespace corrgb {
namespace {

constexpr int kSamplesPerPacket = 4096;          // corr-rs/src/config.rs:26
constexpr int kMaxSt = CORRX_FRONTEND_MAX_STATIONS;
constexpr int kThreads = 256;
constexpr int kJumpStride = 65;                  // padded row of the jump table (u64)

struct FrontArgs {
    int8_t *samples;
    size_t station_stride, frame_stride;
    int align;                                   // 16, 4 or 1: alignment of every frame
    uint8_t *mask;
    size_t mask_station_stride;
    int station0, n_station, frames, ppf;        // ppf = packets per frame
    int mask_bytes;                              // ceil(frames / 8)
    uint64_t frame0;
    int pattern;
    uint64_t seed;
    double tone;
    uint64_t start_counter, n_packets;
    int drop;                                    // drop_rate > 0
    uint64_t drop_threshold;                     // (uint64)(drop_rate * 1e6)
    uint64_t gap_at, gap_len;
    uint64_t ladder_frames, ladder_steps, ladder_origin;
    int64_t delay[kMaxSt];
    uint64_t offset[kMaxSt];
};

// x mod 9 for a 64-bit x without a 64-bit division: 2^24 = 1 (mod 9), so x is
// congruent to the sum of its three 24-bit digits (< 3 * 2^24).
__device__ __forceinline__ int mod9(uint64_t x) {
    const uint32_t r = static_cast<uint32_t>(x & 0xFFFFFFu) +
                       static_cast<uint32_t>((x >> 24) & 0xFFFFFFu) +
                       static_cast<uint32_t>(x >> 48);
    return static_cast<int>(r % 9u);
}

// replay.rs:212-226: the sample at absolute index i.
__device__ __forceinline__ int prng_sample(int64_t i, uint64_t seed) {
    uint64_t x = (static_cast<uint64_t>(i) + seed) * 0x9E3779B97F4A7C15ull;
    x ^= x >> 30;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27;
    x *= 0x94D049BB133111EBull;
    x ^= x >> 31;
    return mod9(x >> 8) - 4;
}

__device__ __forceinline__ uint64_t xorshift_step(uint64_t x) {
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return x;
}

// y = M x over GF(2), M given by its columns (images of the basis vectors).
__device__ __forceinline__ uint64_t gf2_apply(const uint64_t *col, uint64_t x) {
    uint64_t y = 0;
#pragma unroll 16
    for (int b = 0; b < 64; ++b)
        if ((x >> b) & 1ull) y ^= col[b];
    return y;
}

// replay.rs:421-426: is packet `counter` of station s lost to uniform loss?
__device__ __forceinline__ bool lost(const FrontArgs &a, uint64_t counter, int s) {
    if (!a.drop) return false;
    uint64_t x = counter * 0x2545F4914F6CDD1Dull + static_cast<uint64_t>(s);
    x ^= x >> 33;
    return (x % 1000000ull) < a.drop_threshold;
}

// replay.rs:361-426: did station s put packet `counter` on the wire?
__device__ __forceinline__ bool packet_arrives(const FrontArgs &a, uint64_t counter, int s) {
    const uint64_t first = a.start_counter + a.offset[s];
    if (counter < first) return false;
    const uint64_t n = counter - first;
    if (a.n_packets != 0 && n >= a.n_packets) return false;
    if (a.gap_len > 0 && n >= a.gap_at && n < a.gap_at + a.gap_len) return false;
    return !lost(a, counter, s);
}

// replay.rs:431-441: the sample delay of station s in frame `frame`.
__device__ __forceinline__ int64_t frame_delay(const FrontArgs &a, uint64_t frame, int s) {
    if (a.ladder_frames == 0) return a.delay[s];
    uint64_t k = frame >= a.ladder_origin ? 1 + (frame - a.ladder_origin) / a.ladder_frames : 1;
    if (a.ladder_steps > 0 && k > a.ladder_steps) k = a.ladder_steps;
    return a.delay[s] * static_cast<int64_t>(k);
}

// 16 bytes at dst, with the widest stores the destination's alignment allows
// (the staging ring's station stride is the reference's unpadded formula).
__device__ __forceinline__ void store16(int8_t *dst, uint32_t w0, uint32_t w1, uint32_t w2,
                                        uint32_t w3, int align) {
    if (align >= 16) {
        *reinterpret_cast<uint4 *>(dst) = make_uint4(w0, w1, w2, w3);
    } else if (align >= 4) {
        uint32_t *d = reinterpret_cast<uint32_t *>(dst);
        d[0] = w0;
        d[1] = w1;
        d[2] = w2;
        d[3] = w3;
    } else {
        const uint32_t w[4] = {w0, w1, w2, w3};
#pragma unroll
        for (int i = 0; i < 16; ++i) dst[i] = static_cast<int8_t>((w[i >> 2] >> (8 * (i & 3))) & 0xFFu);
    }
}

__device__ __forceinline__ uint32_t pack4(int b0, int b1, int b2, int b3) {
    return (static_cast<uint32_t>(b0) & 0xFFu) | ((static_cast<uint32_t>(b1) & 0xFFu) << 8) |
           ((static_cast<uint32_t>(b2) & 0xFFu) << 16) | ((static_cast<uint32_t>(b3) & 0xFFu) << 24);
}

// replay.rs:257-264: round(4 sin t) with t = phase + k*tone*2pi/4096, each
// operation rounded on its own as the host evaluates it.
__device__ __forceinline__ int sine_sample(double phase, double tone, int k) {
    constexpr double kTau = 6.283185307179586;   // f64 nearest to 2*pi
    const double step = __ddiv_rn(__dmul_rn(__dmul_rn(static_cast<double>(k), tone), kTau),
                                  static_cast<double>(kSamplesPerPacket));
    const double t = __dadd_rn(phase, step);
    return static_cast<int>(round(__dmul_rn(sin(t), 4.0)));
}

__global__ void __launch_bounds__(kThreads)
frontend_kernel(const FrontArgs a) {
    __shared__ uint64_t jump[32 * kJumpStride];   // T^(128*l), columns, l = 0..31
    __shared__ uint64_t scratch[2][64];

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int warps_per_cta = kThreads / 32;

    if (a.pattern == CORRX_PATTERN_COUNTER && a.samples != nullptr) {
        // P = T (one xorshift step), squared 7 times: T^128. Then
        // jump[l] = jump[l-1] * T^128, jump[0] = I.
        const int j = threadIdx.x;
        if (j < 64) {
            scratch[0][j] = xorshift_step(1ull << j);
            jump[j] = 1ull << j;
        }
        __syncthreads();
        int cur = 0;
        for (int sq = 0; sq < 7; ++sq) {
            if (j < 64) scratch[cur ^ 1][j] = gf2_apply(scratch[cur], scratch[cur][j]);
            cur ^= 1;
            __syncthreads();
        }
        for (int l = 1; l < 32; ++l) {
            if (j < 64)
                jump[l * kJumpStride + j] = gf2_apply(&jump[(l - 1) * kJumpStride], scratch[cur][j]);
            __syncthreads();
        }
    }

    if (a.samples != nullptr) {
        const uint64_t n_units = static_cast<uint64_t>(a.n_station) * a.frames * a.ppf;
        const uint64_t warp_id = static_cast<uint64_t>(blockIdx.x) * warps_per_cta + warp;
        const uint64_t n_warps = static_cast<uint64_t>(gridDim.x) * warps_per_cta;
        for (uint64_t u = warp_id; u < n_units; u += n_warps) {
            const int p = static_cast<int>(u % a.ppf);
            const uint64_t sf = u / a.ppf;
            const int f = static_cast<int>(sf % a.frames);
            const int si = static_cast<int>(sf / a.frames);   // output station
            const int s = a.station0 + si;                      // transmitter's index
            const uint64_t frame = a.frame0 + f;
            const uint64_t counter = frame * a.ppf + p;
            int8_t *dst = a.samples + si * a.station_stride + f * a.frame_stride +
                          static_cast<size_t>(p) * kSamplesPerPacket;
            if (a.pattern == CORRX_PATTERN_COUNTER) {
                // replay.rs:235-249; lane l owns bytes [128 l, 128 l + 128).
                const uint64_t x0 = counter * 0x9E3779B97F4A7C15ull +
                                    static_cast<uint64_t>(s) * 0x12345678ull;
                uint64_t x = gf2_apply(&jump[lane * kJumpStride], x0);
                int8_t *out = dst + lane * 128;
#pragma unroll 1
                for (int q = 0; q < 8; ++q) {
                    uint32_t w[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        int b[4];
#pragma unroll
                        for (int t = 0; t < 4; ++t) {
                            x = xorshift_step(x);
                            b[t] = mod9(x >> 3) - 4;
                        }
                        w[e] = pack4(b[0], b[1], b[2], b[3]);
                    }
                    store16(out + 16 * q, w[0], w[1], w[2], w[3], a.align);
                }
            } else if (a.pattern == CORRX_PATTERN_PRNG) {
                // replay.rs:251-256: sample k of the packet is prng_sample(
                // counter*4096 - delay + k).
                const int64_t first = static_cast<int64_t>(counter * kSamplesPerPacket) -
                                      frame_delay(a, frame, s);
#pragma unroll 1
                for (int q = 0; q < kSamplesPerPacket / 512; ++q) {
                    const int k0 = q * 512 + lane * 16;
                    uint32_t w[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        w[e] = pack4(prng_sample(first + k0 + 4 * e, a.seed),
                                     prng_sample(first + k0 + 4 * e + 1, a.seed),
                                     prng_sample(first + k0 + 4 * e + 2, a.seed),
                                     prng_sample(first + k0 + 4 * e + 3, a.seed));
                    store16(dst + k0, w[0], w[1], w[2], w[3], a.align);
                }
            } else if (a.pattern == CORRX_PATTERN_SINE) {
                constexpr double kTau = 6.283185307179586;
                const double phase = __dmul_rn(
                    __dmul_rn(__dadd_rn(static_cast<double>(counter),
                                        __dmul_rn(static_cast<double>(a.seed),
                                                  static_cast<double>(s))),
                              a.tone),
                    kTau);
#pragma unroll 1
                for (int q = 0; q < kSamplesPerPacket / 512; ++q) {
                    const int k0 = q * 512 + lane * 16;
                    uint32_t w[4];
#pragma unroll 1
                    for (int e = 0; e < 4; ++e)
                        w[e] = pack4(sine_sample(phase, a.tone, k0 + 4 * e),
                                     sine_sample(phase, a.tone, k0 + 4 * e + 1),
                                     sine_sample(phase, a.tone, k0 + 4 * e + 2),
                                     sine_sample(phase, a.tone, k0 + 4 * e + 3));
                    store16(dst + k0, w[0], w[1], w[2], w[3], a.align);
                }
            } else {
                for (int q = 0; q < kSamplesPerPacket / 512; ++q)
                    store16(dst + q * 512 + lane * 16, 0u, 0u, 0u, 0u, a.align);
            }
        }
    }

    if (a.mask != nullptr) {
        const uint64_t n_bytes = static_cast<uint64_t>(a.n_station) * a.mask_bytes;
        const uint64_t tid = static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x;
        const uint64_t n_threads = static_cast<uint64_t>(gridDim.x) * kThreads;
        for (uint64_t i = tid; i < n_bytes; i += n_threads) {
            const int si = static_cast<int>(i / a.mask_bytes);
            const int s = a.station0 + si;
            const int byte = static_cast<int>(i % a.mask_bytes);
            uint32_t bits = 0;
            for (int t = 0; t < 8; ++t) {
                const int f = byte * 8 + t;
                if (f >= a.frames) break;
                const uint64_t c0 = (a.frame0 + f) * a.ppf;
                bool ok = true;
                for (int p = 0; p < a.ppf && ok; ++p) ok = packet_arrives(a, c0 + p, s);
                if (ok) bits |= 1u << t;
            }
            a.mask[si * a.mask_station_stride + byte] = static_cast<uint8_t>(bits);
        }
    }
}

}  // namespace
}  // namespace corrgb

using namespace corrgb;

extern "C" corr_status corrx_frontend_fill(const corrx_frontend *fe, int32_t station0,
                                           int32_t n_station, int32_t n_freq, int64_t frame0,
                                           int32_t frames,
                                           int8_t *samples, size_t station_stride,
                                           size_t frame_stride, uint8_t *mask,
                                           size_t mask_station_stride, void *stream) {
    if (fe == nullptr) return fail(CORR_ERR_ARG, "fe must not be NULL");
    if (fe->struct_size != sizeof(corrx_frontend))
        return failf(CORR_ERR_ABI, "corrx_frontend.struct_size=%u, expected %zu", fe->struct_size,
                     sizeof(corrx_frontend));
    if (station0 < 0 || n_station < 1 || station0 + n_station > kMaxSt)
        return failf(CORR_ERR_ARG, "stations [%d, %d) outside [0, %d)", station0,
                     station0 + n_station, kMaxSt);
    if (n_freq < 2048 || (2 * n_freq) % kSamplesPerPacket != 0)
        return failf(CORR_ERR_ARG,
                     "n_freq=%d: a frame of 2*n_freq samples must hold whole 4096-sample packets",
                     n_freq);
    if (frames < 1 || frame0 < 0) return fail(CORR_ERR_ARG, "frames must be >= 1, frame0 >= 0");
    if (fe->pattern < CORRX_PATTERN_ZERO || fe->pattern > CORRX_PATTERN_SINE)
        return failf(CORR_ERR_ARG, "unknown pattern %d", fe->pattern);
    if (!(fe->drop_rate >= 0.0 && fe->drop_rate < 1.0))
        return fail(CORR_ERR_ARG, "drop_rate must be in [0, 1)");
    if (fe->pattern == CORRX_PATTERN_SINE && !std::isfinite(fe->tone))
        return fail(CORR_ERR_ARG, "tone must be finite");
    const size_t L = 2 * static_cast<size_t>(n_freq);
    if (samples != nullptr) {
        if (frame_stride < L) return fail(CORR_ERR_ARG, "frame_stride is shorter than a frame");
    }
    const int mask_bytes = (frames + 7) / 8;
    if (mask != nullptr && n_station > 1 && mask_station_stride < static_cast<size_t>(mask_bytes))
        return fail(CORR_ERR_ARG, "mask_station_stride is shorter than one station's mask");
    if (samples == nullptr && mask == nullptr) return CORR_OK;

    FrontArgs a{};
    a.samples = samples;
    a.station_stride = station_stride;
    a.frame_stride = frame_stride;
    const uintptr_t bits = reinterpret_cast<uintptr_t>(samples) | frame_stride |
                           (n_station > 1 ? station_stride : 0);
    a.align = bits % 16 == 0 ? 16 : bits % 4 == 0 ? 4 : 1;
    a.mask = mask;
    a.mask_station_stride = mask_station_stride;
    a.station0 = station0;
    a.n_station = n_station;
    a.frames = frames;
    a.ppf = static_cast<int>(L / kSamplesPerPacket);
    a.mask_bytes = mask_bytes;
    a.frame0 = static_cast<uint64_t>(frame0);
    a.pattern = fe->pattern;
    a.seed = fe->seed;
    a.tone = fe->tone;
    a.start_counter = fe->start_counter;
    a.n_packets = fe->n_packets;
    a.drop = fe->drop_rate > 0.0;
    a.drop_threshold = static_cast<uint64_t>(fe->drop_rate * 1000000.0);
    a.gap_at = fe->gap_at;
    a.gap_len = fe->gap_len;
    a.ladder_frames = fe->ladder_frames;
    a.ladder_steps = fe->ladder_steps;
    if (fe->ladder_frames > 0) {
        // replay.rs:315-320 (unsigned, wrapping like the transmitter's u64)
        const uint64_t first_frame = (fe->start_counter * kSamplesPerPacket) / L;
        a.ladder_origin = (first_frame + fe->ladder_frames - 1) / fe->ladder_frames * fe->ladder_frames;
    }
    for (int s = 0; s < kMaxSt; ++s) {
        a.delay[s] = fe->sample_delay[s];
        a.offset[s] = fe->counter_offset[s];
    }

    int dev = 0, sms = 0;
    corr_status st = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (st != CORR_OK) return st;
    st = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                    "cudaDeviceGetAttribute(SM count)");
    if (st != CORR_OK) return st;
    // CTAs: one warp per packet, one thread per mask byte, at most 8 CTAs of 256
    // threads per SM (grid-stride beyond that).
    const uint64_t packets = samples != nullptr ? static_cast<uint64_t>(n_station) * frames * a.ppf : 0;
    const uint64_t bytes = mask != nullptr ? static_cast<uint64_t>(n_station) * mask_bytes : 0;
    const uint64_t want = std::max((packets + kThreads / 32 - 1) / (kThreads / 32),
                                   (bytes + kThreads - 1) / kThreads);
    const uint64_t cap = static_cast<uint64_t>(sms) * 8;
    const unsigned grid = static_cast<unsigned>(std::max<uint64_t>(1, std::min(want, cap)));
    frontend_kernel<<<grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(a);
    return cuda_check(cudaGetLastError(), "frontend_kernel launch");
}
