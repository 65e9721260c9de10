// fft_common.cuh -- pieces shared by the F-engines (fengine.cu, fengine_tc.cu):
// constant twiddles (32nd roots of unity), the spectra row writer (YRow), the
// real-FFT split and the frame / packet presence tests.

#ifndef CORR_GB300_FFT_COMMON_CUH
#define CORR_GB300_FFT_COMMON_CUH

#include <cstdint>
#include <type_traits>

#include <cuda_fp16.h>

#include "engine.h"
#include "ptx.cuh"

namespace corrgb {
namespace {

// cos(2*pi*m/32) and sin(2*pi*m/32) for m in [0, 32), built from the first octant.
__host__ __device__ constexpr float cos32_q(int r) {
    return r == 0 ? 1.0f
         : r == 1 ? 0.98078528040323044913f
         : r == 2 ? 0.92387953251128675613f
         : r == 3 ? 0.83146961230254523708f
         : r == 4 ? 0.70710678118654752440f
         : r == 5 ? 0.55557023301960222474f
         : r == 6 ? 0.38268343236508977173f
         : r == 7 ? 0.19509032201612826785f
                  : 0.0f;
}
__host__ __device__ constexpr float cos32(int m) {
    return (m & 31) < 8    ? cos32_q(m & 31)
         : (m & 31) < 16 ? -cos32_q(16 - (m & 31))
         : (m & 31) < 24 ? -cos32_q((m & 31) - 16)
                         : cos32_q(32 - (m & 31));
}
__host__ __device__ constexpr float sin32(int m) { return cos32(m - 8); }

// a * exp(-2*pi*i*m/32); m is a compile-time constant after unrolling.
__device__ __forceinline__ float2 mul_w32(float2 a, int m) {
    m &= 31;
    if (m == 0) return a;
    if (m == 8) return make_float2(a.y, -a.x);
    if (m == 16) return make_float2(-a.x, -a.y);
    if (m == 24) return make_float2(-a.y, a.x);
    const float c = cos32(m), s = sin32(m);
    return make_float2(fmaf(a.x, c, a.y * s), fmaf(a.y, c, -a.x * s));
}

// Where bin k of the current (frame, station) goes in the channel-tiled layout.
// (Element indices fit 32 bits: the spectra buffer holds < 2^32 values.)
// Bin formats: FP32 pairs; FP16 pairs scaled by `scale` (a power of two, so the
// scaling is exact), the FP16 tensor X-engine's operands; or the split form's
// operands, the FP16 pair h = fp16(v*scale) followed by l = fp16(v*scale - h).
// put() takes v already multiplied by `scale`: the real-FFT split folds it
// into its factor 1/2 (half = scale/2), which is exact for the same reason.
// CONTIG: ytile = n_freq, one contiguous row, bin k at base[k].
// STEP 2: the row takes every other bin, put(k) writing bin 2k + odd (the even
// or the odd bins of a frame transformed as two half-length sequences).
template <int FMT, bool CONTIG, int STEP = 1>
struct YRow {
    using T = typename std::conditional<
        FMT == kSpectraF32, float2,
        typename std::conditional<FMT == kSpectraF16, __half2, uint2>::type>::type;
    T *base;               // y + (f*n_station + s)*ytile
    uint32_t tile_stride;  // y_frames*n_station*ytile
    int shift;             // log2(ytile)
    float scale;
    float half;            // scale / 2
    int odd = 0;           // STEP 2: 0 = even bins, 1 = odd bins
    __device__ __forceinline__ void put(int k, float2 v) const {
        if constexpr (STEP == 2) k = 2 * k + odd;
        T *dst = CONTIG ? base + k
                        : base + (static_cast<uint32_t>(k >> shift) * tile_stride +
                                  static_cast<uint32_t>(k & ((1 << shift) - 1)));
        if constexpr (FMT == kSpectraF16) {
            *dst = __floats2half2_rn(v.x, v.y);
        } else if constexpr (FMT == kSpectraF16Split) {
            const float x = v.x, y = v.y;
            const __half2 h = __floats2half2_rn(x, y);
            const float2 hf = __half22float2(h);
            const __half2 l = __floats2half2_rn(x - hf.x, y - hf.y);
            *dst = make_uint2(*reinterpret_cast<const uint32_t *>(&h),
                              *reinterpret_cast<const uint32_t *>(&l));
        } else {
            *dst = v;
        }
    }
};

// X[k] = Fe + w_k Fo and X[M-k] = conj(Fe - w_k Fo), with Z = FFT of the packed
// pairs, Fe = (Z[k] + conj(Z[M-k]))/2, Fo = -i (Z[k] - conj(Z[M-k]))/2 and
// w_k = exp(-2*pi*i*k/L). `both` = false skips X[M-k] (k = 0: Nyquist).
// Both outputs come out multiplied by the row's scale, folded into the 1/2:
// h = yrow.half = scale/2 is a power of two, and the caller passes hw = h*w_k.
// With s = Z[k] + conj(Z[M-k]) and d = -i (Z[k] - conj(Z[M-k])), the outputs
// are h*s + hw*d and conj(h*s - hw*d), an FMA per component. Scaling by a power
// of two is exact, so these are the same numbers as scaling Fe and Fo first
// (one multiply per component fewer).
template <class Row>
__device__ __forceinline__ void split_store(float2 zk, float2 zmk, float2 hw, int k, int M,
                                            bool both, const Row &yrow) {
    const float h = yrow.half;
    const float2 s = make_float2(zk.x + zmk.x, zk.y - zmk.y);
    const float2 d = make_float2(zk.y + zmk.y, zmk.x - zk.x);
    const float2 wf = cmul(hw, d);
    yrow.put(k, fma2(make_float2(h, h), s, wf));
    if (both) yrow.put(M - k, make_float2(fmaf(h, s.x, -wf.x), fmaf(-h, s.y, wf.y)));
}

// h*w for the power of two h = yrow.half (exact).
__device__ __forceinline__ float2 scale_tw(float2 w, float h) {
    return make_float2(w.x * h, w.y * h);
}

// Packets of 1024 samples (512 int8 pairs) kept for frame f of station s: all
// of them without a packet mask, else the frame's word cut to its M/512 packets.
template <int M>
__host__ __device__ constexpr uint32_t all_packets() {
    return (M >> 9) >= 32 ? 0xffffffffu : (1u << (M >> 9)) - 1u;
}

template <int M>
__device__ __forceinline__ uint32_t packets_kept(const FengineArgs &a, int f, int s) {
    if (a.pmask == nullptr) return all_packets<M>();
    return a.pmask[static_cast<size_t>(s) * a.pmask_station_stride + a.pmask_frame0 + f] &
           all_packets<M>();
}

template <int M>
__device__ __forceinline__ bool frame_present(const FengineArgs &a, int f, int s) {
    if (a.mask != nullptr) {
        const int bit = a.mask_bit0 + f;
        const uint8_t byte = a.mask[static_cast<size_t>(s) * a.mask_station_stride + (bit >> 3)];
        if (!((byte >> (bit & 7)) & 1u)) return false;
    }
    // a frame whose packets were all lost is all zeros: the same as a missing one
    return packets_kept<M>(a, f, s) != 0u;
}

} // namespace
} // namespace corrgb

#endif // CORR_GB300_FFT_COMMON_CUH
