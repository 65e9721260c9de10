// fengine_impl.cuh -- the F-engine's kernel and launch templates, shared by
// the translation units that instantiate them (fengine.cu and
// fengine_large.cu / fengine_split_*.cu, one group of transform lengths each,
// so that they compile in parallel). What the kernel does is described in
// fengine.cu.

#ifndef CORR_GB300_FENGINE_IMPL_CUH
#define CORR_GB300_FENGINE_IMPL_CUH

#include <cmath>
#include <type_traits>
#include <vector>

#include <cuda_fp16.h>

#include "engine.h"
#include "fft_common.cuh"
#include "ptx.cuh"

namespace corrgb {

// Launchers of the groups of lengths compiled apart from fengine.cu.
corr_status fengine_launch_large(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                                 int num_sms, cudaStream_t stream);   // 10240 .. 16384
corr_status fengine_launch_split_a(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                                   int num_sms, cudaStream_t stream); // 18432, 20480
corr_status fengine_launch_split_b(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                                   int num_sms, cudaStream_t stream); // 22528, 24576
corr_status fengine_launch_split_c(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                                   int num_sms, cudaStream_t stream); // 26624, 28672
corr_status fengine_launch_split_d(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                                   int num_sms, cudaStream_t stream); // 30720, 32768

namespace {

// ---------------------------------------------------------------------------
// Small DFTs in registers, forward sign (exp(-2*pi*i*n*k/R)), natural order.
// The power-of-two radices' constant twiddles are 32nd roots of unity; the odd
// radices 3 .. 15 (first pass of lengths R x 2^k) use their own.
// ---------------------------------------------------------------------------

template <int R>
struct Dft;

// Scaled elements. Inside the radix-8/16/32 DFTs an element is kept as
// (s.x * v.x, s.y * v.y), where the lanes' scales s are compile-time constants
// once the loops are unrolled. A constant twiddle c - i*s in tangent form,
// c*(x + t*y, y - t*x) with t = s/c (or the cotangent form when |s| > |c|),
// costs two FMAs instead of a complex product's four and leaves its cosine (or
// sine) in the scales; the butterflies that follow take the scales in as FMAs
// in place of their additions, choosing the side whose scale is +-1, so the
// DFT's outputs come out with unit scales. Two FP32 operations fewer per
// constant twiddle; the rounding is that of the FMA forms.
struct Sv {
    float2 v, s;
};

// One lane of as*av + bs*bv in one operation: the new (v, s).
__device__ __forceinline__ void sv_lane(float av, float as, float bv, float bs, float &v,
                                        float &s) {
    if (as == bs) {
        v = av + bv;
        s = as;
    } else if (as == -bs) {
        v = av - bv;
        s = as;
    } else if (fabsf(as) == 1.0f || fabsf(bs) != 1.0f) {
        v = fmaf(bs / as, bv, av);
        s = as;
    } else {
        v = fmaf(as / bs, av, bv);
        s = bs;
    }
}
// Whether sv_lane keeps a's scale (a is the addend).
__host__ __device__ constexpr bool sv_keeps_a(float as, float bs) {
    return as == bs || as == -bs || as == 1.0f || as == -1.0f || (bs != 1.0f && bs != -1.0f);
}

// a + b (minus: a - b); one packed instruction where both lanes keep a's scale.
__device__ __forceinline__ Sv sv_comb(const Sv &a, const Sv &b, bool minus) {
    const float bsx = minus ? -b.s.x : b.s.x, bsy = minus ? -b.s.y : b.s.y;
    if (sv_keeps_a(a.s.x, bsx) && sv_keeps_a(a.s.y, bsy)) {
        const float qx = bsx / a.s.x, qy = bsy / a.s.y;
        float2 v;
        if (qx == 1.0f && qy == 1.0f)
            v = cadd(a.v, b.v);
        else if (qx == -1.0f && qy == -1.0f)
            v = csub(a.v, b.v);
        else
            v = fma2(make_float2(qx, qy), b.v, a.v);
        return {v, a.s};
    }
    Sv r;
    sv_lane(a.v.x, a.s.x, b.v.x, bsx, r.v.x, r.s.x);
    sv_lane(a.v.y, a.s.y, b.v.y, bsy, r.v.y, r.s.y);
    return r;
}
// a - i*b (minus: a + i*b), lane by lane (the swap keeps it out of the packed form).
__device__ __forceinline__ Sv sv_comb_mi(const Sv &a, const Sv &b, bool minus) {
    // -i*b = (b.y, -b.x)
    const float bsx = minus ? -b.s.y : b.s.y, bsy = minus ? b.s.x : -b.s.x;
    Sv r;
    sv_lane(a.v.x, a.s.x, b.v.y, bsx, r.v.x, r.s.x);
    sv_lane(a.v.y, a.s.y, b.v.x, bsy, r.v.y, r.s.y);
    return r;
}
// a * exp(-2*pi*i*m/32), m a compile-time constant.
__device__ __forceinline__ Sv sv_twiddle(const Sv &a, int m) {
    m &= 31;
    if (m == 0) return a;
    if (m == 8) return {make_float2(a.v.y, a.v.x), make_float2(a.s.y, -a.s.x)};    // * -i
    if (m == 16) return {a.v, make_float2(-a.s.x, -a.s.y)};
    if (m == 24) return {make_float2(a.v.y, a.v.x), make_float2(-a.s.y, a.s.x)};   // * i
    const float c = cos32(m), s = sin32(m);
    if (fabsf(c) >= fabsf(s)) {
        // re = c*sx*(vx + t*(sy/sx)*vy), im = c*sy*(vy - t*(sx/sy)*vx)
        const float t = s / c;
        return {make_float2(fmaf(t * a.s.y / a.s.x, a.v.y, a.v.x),
                            fmaf(-t * a.s.x / a.s.y, a.v.x, a.v.y)),
                make_float2(c * a.s.x, c * a.s.y)};
    }
    // re = s*sy*(vy + u*(sx/sy)*vx), im = -s*sx*(vx - u*(sy/sx)*vy), u = c/s
    const float u = c / s;
    return {make_float2(fmaf(u * a.s.x / a.s.y, a.v.x, a.v.y),
                        fmaf(-u * a.s.y / a.s.x, a.v.y, a.v.x)),
            make_float2(s * a.s.y, -s * a.s.x)};
}
// The plain value (the scales are 1 at a DFT's outputs; this folds away then).
__device__ __forceinline__ float2 sv_value(const Sv &a) {
    return make_float2(a.s.x == 1.0f ? a.v.x : a.s.x * a.v.x,
                       a.s.y == 1.0f ? a.v.y : a.s.y * a.v.y);
}

template <>
struct Dft<2> {
    static __device__ __forceinline__ void run(float2 *v) {
        const float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
    static __device__ __forceinline__ void run_sv(Sv *v) {
        const Sv a = v[0], b = v[1];
        v[0] = sv_comb(a, b, false);
        v[1] = sv_comb(a, b, true);
    }
};

template <>
struct Dft<4> {
    static __device__ __forceinline__ void finish(float2 s02, float2 d02, float2 s13, float2 d13,
                                                  float2 *v) {
        v[0] = cadd(s02, s13);
        v[2] = csub(s02, s13);
        v[1] = make_float2(d02.x + d13.y, d02.y - d13.x); // d02 - i*d13
        v[3] = make_float2(d02.x - d13.y, d02.y + d13.x); // d02 + i*d13
    }
    static __device__ __forceinline__ void run(float2 *v) {
        finish(cadd(v[0], v[2]), csub(v[0], v[2]), cadd(v[1], v[3]), csub(v[1], v[3]), v);
    }
    // Inputs still carrying the int8 unpacking's offset B (x[n] = b[n] + B, every
    // value an integer below 2^24): x0 - x2 = b0 - b2 and x0 + (x2 - 2B) = b0 + b2
    // exactly, so the offset goes in one subtraction per pair instead of one per
    // input, with the same results as run() on b.
    static __device__ __forceinline__ void run_biased(float2 *v, float2 two_b) {
        finish(cadd(v[0], csub(v[2], two_b)), csub(v[0], v[2]), cadd(v[1], csub(v[3], two_b)),
               csub(v[1], v[3]), v);
    }
    static __device__ __forceinline__ void run_sv(Sv *v) {
        const Sv s02 = sv_comb(v[0], v[2], false), d02 = sv_comb(v[0], v[2], true);
        const Sv s13 = sv_comb(v[1], v[3], false), d13 = sv_comb(v[1], v[3], true);
        v[0] = sv_comb(s02, s13, false);
        v[2] = sv_comb(s02, s13, true);
        v[1] = sv_comb_mi(d02, d13, false);   // d02 - i*d13
        v[3] = sv_comb_mi(d02, d13, true);    // d02 + i*d13
    }
};

// cos(2*pi*m/R) and sin(2*pi*m/R) for the odd radices R = 3, 5, ..., 15 and
// m = 1..(R-1)/2 (the values of the circle functions at those angles, to 21
// digits). Radices 3, 5 and 7 lead the plans of lengths 3, 5, 7 x 2^k; 9, 11,
// 13 and 15 those of the half-length sequences of n_freq 18432 .. 30720.
__host__ __device__ constexpr float pick7(int m, float a1, float a2 = 0.f, float a3 = 0.f,
                                          float a4 = 0.f, float a5 = 0.f, float a6 = 0.f,
                                          float a7 = 0.f) {
    return m == 1 ? a1 : m == 2 ? a2 : m == 3 ? a3 : m == 4 ? a4 : m == 5 ? a5 : m == 6 ? a6 : a7;
}
__host__ __device__ constexpr float cos_odd(int R, int m) {
    return R == 3 ? -0.5f
         : R == 5 ? pick7(m, 0.309016994374947424102f, -0.809016994374947424102f)
         : R == 7 ? pick7(m, 0.623489801858733530525f, -0.222520933956314404289f,
                          -0.900968867902419126236f)
         : R == 9 ? pick7(m, 0.766044443118978035202f, 0.173648177666930348852f, -0.5f,
                          -0.939692620785908384054f)
         : R == 11 ? pick7(m, 0.841253532831181168862f, 0.415415013001886425529f,
                           -0.142314838273285140444f, -0.654860733945285064057f,
                           -0.95949297361449738989f)
         : R == 13 ? pick7(m, 0.8854560256532098959f, 0.568064746731155802512f,
                           0.120536680255323053349f, -0.35460488704253562597f,
                           -0.748510748171101098635f, -0.970941817426052027157f)
                   : pick7(m, 0.913545457642600895502f, 0.669130606358858213826f,
                           0.309016994374947424102f, -0.1045284632676534714f, -0.5f,
                           -0.809016994374947424102f, -0.978147600733805637929f);
}
__host__ __device__ constexpr float sin_odd(int R, int m) {
    return R == 3 ? 0.866025403784438646764f
         : R == 5 ? pick7(m, 0.951056516295153572116f, 0.587785252292473129169f)
         : R == 7 ? pick7(m, 0.781831482468029808708f, 0.974927912181823607018f,
                          0.433883739117558120476f)
         : R == 9 ? pick7(m, 0.642787609686539326323f, 0.984807753012208059367f,
                          0.866025403784438646764f, 0.342020143325668733044f)
         : R == 11 ? pick7(m, 0.540640817455597582108f, 0.909631995354518371412f,
                           0.989821441880932732376f, 0.755749574354258283774f,
                           0.281732556841429697711f)
         : R == 13 ? pick7(m, 0.464723172043768545656f, 0.82298386589365639458f,
                           0.992708874098053992801f, 0.93501624268541482344f,
                           0.663122658240795202377f, 0.239315664287557767149f)
                   : pick7(m, 0.406736643075800207754f, 0.743144825477394235015f,
                           0.951056516295153572116f, 0.994521895368273336923f,
                           0.866025403784438646764f, 0.587785252292473129169f,
                           0.207911690817759337102f);
}

// Odd R: the inputs n and R-n meet the same cosine and opposite sines, so with
// s_n = x[n] + x[R-n] and d_n = x[n] - x[R-n] (n = 1..H, H = (R-1)/2)
//   X[k]   = x[0] + sum_n s_n cos(2*pi*n*k/R) - i sum_n d_n sin(2*pi*n*k/R)
//   X[R-k] = the same with +i,                     k = 1..H.
// BIASED: the inputs still carry the int8 unpacking's offset B (every value an
// integer below 2^24): s_n = x[n] + (x[R-n] - 2B), d_n = x[n] - x[R-n] and
// x[0] - B are then exact, the same numbers as from the unbiased inputs.
template <int R>
struct DftOdd {
    static constexpr int H = (R - 1) / 2;
    template <bool BIASED = false>
    static __device__ __forceinline__ void run(float2 *v, float2 two_b = float2{}) {
        float2 s[H], d[H];
        const float2 x0 = BIASED ? csub(v[0], make_float2(0.5f * two_b.x, 0.5f * two_b.y)) : v[0];
        float2 sum = x0;
#pragma unroll
        for (int n = 1; n <= H; ++n) {
            s[n - 1] = cadd(v[n], BIASED ? csub(v[R - n], two_b) : v[R - n]);
            d[n - 1] = csub(v[n], v[R - n]);
            sum = cadd(sum, s[n - 1]);
        }
#pragma unroll
        for (int k = 1; k <= H; ++k) {
            float2 a = x0, b = make_float2(0.f, 0.f);
#pragma unroll
            for (int n = 1; n <= H; ++n) {
                // angle 2*pi*m/R; beyond H the sine changes sign; for a composite
                // R (9, 15) n*k can be a multiple of R: angle 0
                const int m = (n * k) % R;
                const int mm = m <= H ? m : R - m;
                const float c = mm == 0 ? 1.0f : cos_odd(R, mm);
                const float sn = mm == 0 ? 0.0f : m <= H ? sin_odd(R, mm) : -sin_odd(R, mm);
                a = make_float2(fmaf(s[n - 1].x, c, a.x), fmaf(s[n - 1].y, c, a.y));
                b = make_float2(fmaf(d[n - 1].x, sn, b.x), fmaf(d[n - 1].y, sn, b.y));
            }
            v[k] = make_float2(a.x + b.y, a.y - b.x);       // a - i*b
            v[R - k] = make_float2(a.x - b.y, a.y + b.x);   // a + i*b
        }
        v[0] = sum;
    }
};
template <> struct Dft<3> : DftOdd<3> {};
template <> struct Dft<5> : DftOdd<5> {};
template <> struct Dft<7> : DftOdd<7> {};
template <> struct Dft<9> : DftOdd<9> {};
template <> struct Dft<11> : DftOdd<11> {};
template <> struct Dft<13> : DftOdd<13> {};

// 15 = 3 x 5, coprime: the prime-factor (Good-Thomas) form has no twiddles.
// Input n = (5*n1 + 3*n2) mod 15 and output k = (10*k1 + 6*k2) mod 15 (10 = 5 *
// (5^-1 mod 3), 6 = 3 * (3^-1 mod 5)): five-point DFTs over n2 for each n1, then
// three-point DFTs over n1 for each k2. About 60 % of the direct form's
// operations, and fewer values live at once.
template <>
struct Dft<15> {
    static __device__ __forceinline__ void run(float2 *v) {
        float2 y[3][5];
#pragma unroll
        for (int n1 = 0; n1 < 3; ++n1) {
#pragma unroll
            for (int n2 = 0; n2 < 5; ++n2) y[n1][n2] = v[(5 * n1 + 3 * n2) % 15];
            Dft<5>::run(y[n1]);
        }
#pragma unroll
        for (int k2 = 0; k2 < 5; ++k2) {
            float2 t[3] = {y[0][k2], y[1][k2], y[2][k2]};
            Dft<3>::run(t);
#pragma unroll
            for (int k1 = 0; k1 < 3; ++k1) v[(10 * k1 + 6 * k2) % 15] = t[k1];
        }
    }
};

// R = 4 x (R/4): n = (R/4)*n1 + n2, k = k1 + 4*k2, on scaled elements (Sv) with
// the constant twiddles between the two stages in tangent form. BIASED: the
// inputs still carry the int8 unpacking's offset (Dft<4>::run_biased).
template <int R>
struct Dft {
    static_assert(R == 8 || R == 16 || R == 32, "radix");
    static constexpr int R2 = R / 4;
    template <bool BIASED = false>
    static __device__ __forceinline__ void run(float2 *v, float2 two_b = float2{}) {
        Sv e[R];
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) {
            Sv t[4];
            if constexpr (BIASED) {
                float2 f[4] = {v[n2], v[R2 + n2], v[2 * R2 + n2], v[3 * R2 + n2]};
                Dft<4>::run_biased(f, two_b);
#pragma unroll
                for (int k1 = 0; k1 < 4; ++k1) t[k1] = {f[k1], make_float2(1.0f, 1.0f)};
            } else {
#pragma unroll
                for (int n1 = 0; n1 < 4; ++n1) t[n1] = {v[n1 * R2 + n2], make_float2(1.0f, 1.0f)};
                Dft<4>::run_sv(t);
            }
#pragma unroll
            for (int k1 = 0; k1 < 4; ++k1) e[n2 * 4 + k1] = sv_twiddle(t[k1], n2 * k1 * (32 / R));
        }
        second_stage(e, v);
    }
    // Inputs already scaled (the inner DFT of a larger one).
    static __device__ __forceinline__ void run_sv(Sv *x) {
        Sv e[R];
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) {
            Sv t[4] = {x[n2], x[R2 + n2], x[2 * R2 + n2], x[3 * R2 + n2]};
            Dft<4>::run_sv(t);
#pragma unroll
            for (int k1 = 0; k1 < 4; ++k1) e[n2 * 4 + k1] = sv_twiddle(t[k1], n2 * k1 * (32 / R));
        }
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            Sv t[R2];
#pragma unroll
            for (int n2 = 0; n2 < R2; ++n2) t[n2] = e[n2 * 4 + k1];
            Dft<R2>::run_sv(t);
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) x[k1 + 4 * k2] = t[k2];
        }
    }

  private:
    // e[n2*4 + k1] (twiddled first-stage outputs) -> v[k1 + 4*k2], unit scales.
    static __device__ __forceinline__ void second_stage(Sv *e, float2 *v) {
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            Sv t[R2];
#pragma unroll
            for (int n2 = 0; n2 < R2; ++n2) t[n2] = e[n2 * 4 + k1];
            Dft<R2>::run_sv(t);
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) v[k1 + 4 * k2] = sv_value(t[k2]);
        }
    }
};

// exp(-2*pi*i*u/M) for 0 <= u < M from the two-level table in shared memory.
__device__ __forceinline__ float2 tw_pass(const float2 *lo, const float2 *hi, int u) {
    return cmul(lo[u & 63], hi[u >> 6]);
}

// v[r] *= w^r with w = exp(-2*pi*i*u/M), u*R < M. w, w^4, w^8 and w^16 come
// from the table; every other power is at most three products from those.
template <int R>
__device__ __forceinline__ void apply_twiddles(float2 *v, int u, const float2 *lo,
                                               const float2 *hi) {
    float2 w[R];
    w[1] = tw_pass(lo, hi, u);
    // w^4, w^8, w^16: lo[(k*u) & 63] = lo[k*(u & (64/k - 1))], read from the
    // compact copies lo[64 + ...] (k = 4), lo[80 + ...] (8), lo[88 + ...] (16)
    // so that a warp's lanes hit distinct banks
    if constexpr (R >= 4) {
        w[2] = cmul(w[1], w[1]);
        w[3] = cmul(w[2], w[1]);
    }
    if constexpr (R >= 8) {
        w[4] = cmul(lo[64 + (u & 15)], hi[(4 * u) >> 6]);
#pragma unroll
        for (int r = 5; r < 8; ++r) w[r] = cmul(w[4], w[r - 4]);
    }
    if constexpr (R >= 16) {
        w[8] = cmul(lo[80 + (u & 7)], hi[(8 * u) >> 6]);
#pragma unroll
        for (int r = 9; r < 16; ++r) w[r] = cmul(w[8], w[r - 8]);
    }
    if constexpr (R >= 32) {
        w[16] = cmul(lo[88 + (u & 3)], hi[(16 * u) >> 6]);
#pragma unroll
        for (int r = 17; r < 32; ++r) w[r] = cmul(w[16], w[r - 16]);
    }
#pragma unroll
    for (int r = 1; r < R; ++r) v[r] = cmul(v[r], w[r]);
}

// Radix plan per transform length M: three passes R0 x R1 x R2 = M, P = 2*R2
// points per thread, T = M/P threads. The last pass (radix R2) is fused with
// the real-FFT split: thread t owns butterflies t and J - t (J = M/R2), so Z[k]
// and Z[M-k] meet in its registers. Plan 0 of a power of two has three passes
// (R0 x R1 x R2, R1b = 1); plan 1, where a size has one, has four
// (R0 x R1 x R1b x R2) with half the points per thread and twice the threads:
// one more shared-memory pass against twice the warps to hide latency. The
// autotuner times both. A length of 3, 5 or 7 x 2^k (the multiples of 2048 up
// to 16384 that are not powers of two: a frame of whole 4096-sample packets)
// starts with that odd radix, whose pass has no twiddles, then three
// power-of-two passes.
template <int M, int PLAN>
struct FePlan;
template <> struct FePlan<16384, 0> { static constexpr int R0 = 32, R1 = 32, R1b = 1, R2 = 16; };
template <> struct FePlan<16384, 1> { static constexpr int R0 = 16, R1 = 16, R1b = 8, R2 = 8; };
template <> struct FePlan<14336, 0> { static constexpr int R0 = 7, R1 = 16, R1b = 8, R2 = 16; };
template <> struct FePlan<12288, 0> { static constexpr int R0 = 3, R1 = 32, R1b = 8, R2 = 16; };
template <> struct FePlan<10240, 0> { static constexpr int R0 = 5, R1 = 16, R1b = 8, R2 = 16; };
template <> struct FePlan<8192, 0> { static constexpr int R0 = 32, R1 = 16, R1b = 1, R2 = 16; };
template <> struct FePlan<6144, 0> { static constexpr int R0 = 3, R1 = 16, R1b = 8, R2 = 16; };
template <> struct FePlan<4096, 0> { static constexpr int R0 = 16, R1 = 16, R1b = 1, R2 = 16; };
template <> struct FePlan<2048, 0> { static constexpr int R0 = 16, R1 = 8, R1b = 1, R2 = 16; };
template <> struct FePlan<1024, 0> { static constexpr int R0 = 16, R1 = 8, R1b = 1, R2 = 8; };
template <> struct FePlan<512, 0> { static constexpr int R0 = 16, R1 = 4, R1b = 1, R2 = 8; };
// Half lengths of n_freq 18432, 22528, 26624 and 30720 (the other half lengths
// above, 10240 .. 16384, use their own plans).
template <> struct FePlan<15360, 0> { static constexpr int R0 = 15, R1 = 16, R1b = 4, R2 = 16; };
template <> struct FePlan<13312, 0> { static constexpr int R0 = 13, R1 = 16, R1b = 4, R2 = 16; };
template <> struct FePlan<11264, 0> { static constexpr int R0 = 11, R1 = 16, R1b = 4, R2 = 16; };
template <> struct FePlan<9216, 0> { static constexpr int R0 = 9, R1 = 16, R1b = 4, R2 = 16; };

// HALF: MM is half of n_freq; a CTA holds the whole frame of 4*MM int8 samples
// (one buffer: two would not fit beside the data) and transforms its two
// half-length sequences one after the other.
template <int MM, int PLAN, bool HALF = false>
struct FeCfg {
    using Plan = FePlan<MM, PLAN>;
    static constexpr int M = MM;
    static constexpr int R0 = Plan::R0, R1 = Plan::R1, R1b = Plan::R1b, R2 = Plan::R2;
    static_assert(R0 * R1 * R1b * R2 == M, "radix plan must cover M");
    static_assert(M % 64 == 0, "the two-level twiddle tables step by 64");
    static constexpr int P = 2 * R2;                // points per thread
    static constexpr int T = M / P;                 // threads per CTA
    static constexpr int J = M / R2;                // butterflies of the last pass
    static constexpr int PADSHIFT = (R0 == 32) ? 5 : 4;
    static constexpr int N_PASS_HI = M / 64;
    static constexpr int N_POST_HI = M / 64;
    static constexpr int FRAME = HALF ? 4 * M : 2 * M;   // int8 bytes of one frame
    // shared memory layout (bytes)
    static constexpr int OFF_X0 = 0;                      // int8 frame, buffer 0
    static constexpr int OFF_X1 = HALF ? 0 : FRAME;       // int8 frame, buffer 1
    static constexpr int OFF_D = HALF ? FRAME : 2 * FRAME;   // padded complex data
    static constexpr int OFF_PLO = OFF_D + (M + (M >> PADSHIFT)) * 8;
    static constexpr int OFF_PHI = OFF_PLO + 92 * 8;   // lo[64] + lo4[16] + lo8[8] + lo16[4]
    static constexpr int OFF_QLO = OFF_PHI + N_PASS_HI * 8;
    static constexpr int OFF_QHI = OFF_QLO + 64 * 8;
    static constexpr int OFF_T2 = OFF_QHI + N_POST_HI * 8;   // second-pass twiddles
    static constexpr int OFF_BAR = (OFF_T2 + R0 * R1 * 8 + 15) / 16 * 16;
    static constexpr int OFF_FLAG = OFF_BAR + 16;
    static constexpr int OFF_SHIFT = OFF_FLAG + 8;        // HALF: odd_shift
    static constexpr int SMEM = OFF_FLAG + 16;
    static_assert(SMEM <= 227 * 1024, "shared memory");
    // CTAs per SM the launch bounds plan for: as many as shared memory allows,
    // with at most 128 registers per thread (64 at 1024 threads).
    static constexpr int BY_SMEM = (220 * 1024) / SMEM;
    static constexpr int BY_REGS = T >= 1024 ? 1 : 65536 / (T * 128);
    static constexpr int MIN_BLOCKS =
        (BY_SMEM < BY_REGS ? BY_SMEM : BY_REGS) < 1 ? 1 : (BY_SMEM < BY_REGS ? BY_SMEM : BY_REGS);
};

// Two signed bytes (little-endian pair) -> two floats, exactly, without the
// conversion unit: flipping the sign bit gives b + 128 in [0, 255]; placed in the
// low byte of 0x4B000000 that is the float 2^23 + b + 128 (int8_pair_to_biased),
// and subtracting B = 2^23 + 128 leaves b (int8_pair_to_float2). The first
// passes keep the biased values and take B out in their first butterflies.
constexpr float kInt8Bias = 8388736.0f;   // 2^23 + 128
__device__ __forceinline__ float2 int8_pair_to_biased(uint16_t u) {
    const uint32_t x = static_cast<uint32_t>(u) ^ 0x8080u;
    return make_float2(__uint_as_float(__byte_perm(x, 0x4B000000u, 0x7440)),
                       __uint_as_float(__byte_perm(x, 0x4B000000u, 0x7441)));
}
__device__ __forceinline__ float2 int8_pair_to_float2(uint16_t u) {
    const float2 x = int8_pair_to_biased(u);
    return make_float2(x.x - kInt8Bias, x.y - kInt8Bias);
}

// Shared-memory index padding: one float2 per R0 elements, which makes the
// stride-R0 scatter of the first pass conflict-free and keeps every other
// access a contiguous run.
template <int SHIFT>
__device__ __forceinline__ int padi(int i) { return i + (i >> SHIFT); }

// j / D and j % D for a compile-time D and j >= 0: a shift and a mask for a
// power of two, a multiply-high otherwise.
template <int D>
__device__ __forceinline__ int div_c(int j) {
    return static_cast<int>(static_cast<unsigned>(j) / static_cast<unsigned>(D));
}
template <int D>
__device__ __forceinline__ int mod_c(int j) {
    return static_cast<int>(static_cast<unsigned>(j) % static_cast<unsigned>(D));
}

// Where a pass reads its input: the data in shared memory, or (first pass)
// the int8 frame: its M sample pairs as M complex points; or, for a frame of
// 2M pairs split into two half-length sequences (one radix-2 step of
// decimation in frequency, z = the 2M points), z[e] + z[e+M] (the sequence
// whose transform is the even bins) or (z[e] - z[e+M]) * exp(-pi*i*e/M) (the
// odd bins).
enum PassSource : int { kFromShared = 0, kFromInt8 = 1, kFromInt8Sum = 2, kFromInt8Diff = 3 };

// Stockham pass of radix R over M points with sub-transform size NS:
//   out[(j/NS)*NS*R + j%NS + r*NS] = DFT_R( in[j + r*M/R] * w^(r*(j%NS)) )
// for the M/R butterflies j. Each thread owns ceil(P/R) of them (j = tid + q*T);
// where R does not divide P (an odd first radix) the last round of butterflies
// is partial and the threads past M/R sit it out. In place: read all, barrier,
// write all, barrier. The odd-radix first pass of a split frame (which also
// combines two points and, for the odd bins, multiplies each by a twiddle)
// reads the int8 frame, not the data it writes, so it instead waits once at
// the start (for the previous transform's last reads of the data) and then
// writes each butterfly as soon as it is computed, holding R values at a time
// instead of ceil(P/R)*R. (The plain odd-radix first pass keeps the first
// order: streaming it made n_freq 6144 5 % slower and 10240, 14336 no faster.)
// TAB: the pass's twiddles w^(r*(j%NS)) (NS*R of them) come from table `t2`
// laid out [r][j%NS] instead of from the two-level tables. qlo/qhi: the
// exp(-pi*i*e/M) tables that kFromInt8Diff multiplies by.
template <int M, int T, int P, int R, int NS, int SHIFT, int SRC, bool TAB = false>
__device__ __forceinline__ void fft_pass(float2 *__restrict__ sd, const char2 *__restrict__ sx,
                                         const float2 *lo, const float2 *hi, int tid,
                                         const float2 *t2 = nullptr, const float2 *qlo = nullptr,
                                         const float2 *qhi = nullptr) {
    constexpr int NB = (P + R - 1) / R;
    constexpr int STRIDE = M / R;
    constexpr bool EXACT = NB * R == P;   // NB*T == M/R: every thread has NB butterflies
    constexpr bool STREAM = (SRC == kFromInt8Sum || SRC == kFromInt8Diff) && (R % 2 == 1);
    static_assert(M % (NS * R) == 0, "bad radix plan");
    // Reads: a padded per-thread base plus a compile-time offset, since the read
    // stride is a multiple of the padding period. Writes likewise when the write
    // stride NS is (or, in a first pass of radix 2^SHIFT, stays inside one
    // period); otherwise (odd radices, and the pass after an odd first one) each
    // element's padded index is computed on its own.
    static_assert(STRIDE % (1 << SHIFT) == 0, "read stride");
    constexpr bool RUNS = NS % (1 << SHIFT) == 0 || (NS == 1 && R == (1 << SHIFT));
    constexpr int PSTRIDE = STRIDE + (STRIDE >> SHIFT);
    constexpr int PNS = (NS == 1) ? 1 : NS + (NS >> SHIFT);
    // The int8 first pass leaves the unpacking's offset in its inputs; the DFT's
    // first butterflies take it out (Dft<4>::run_biased, DftOdd).
    constexpr bool BIASED = SRC == kFromInt8 && (R == 3 || R == 5 || R == 7 || R == 8 ||
                                                 R == 16 || R == 32);
    static_assert(!BIASED || (NS == 1 && !TAB), "the biased inputs take no twiddles");
    const uint16_t *x16 = reinterpret_cast<const uint16_t *>(sx);
    auto gather = [&](int j, float2 *v) {
        if constexpr (BIASED) {
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = int8_pair_to_biased(x16[j + r * STRIDE]);
        } else if constexpr (SRC == kFromInt8) {
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = int8_pair_to_float2(x16[j + r * STRIDE]);
        } else if constexpr (SRC == kFromInt8Sum) {
            // with the offset B still in: x[e] + (x[e+M] - 2B) and x[e] - x[e+M]
            // are the integer sum and difference, exactly (Dft<4>::run_biased)
            const float2 two_b = make_float2(2.0f * kInt8Bias, 2.0f * kInt8Bias);
#pragma unroll
            for (int r = 0; r < R; ++r)
                v[r] = cadd(int8_pair_to_biased(x16[j + r * STRIDE]),
                            csub(int8_pair_to_biased(x16[j + r * STRIDE + M]), two_b));
        } else if constexpr (SRC == kFromInt8Diff) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int e = j + r * STRIDE;
                v[r] = cmul(csub(int8_pair_to_biased(x16[e]), int8_pair_to_biased(x16[e + M])),
                            cmul(qlo[e & 63], qhi[e >> 6]));
            }
        } else {
            const int pj = padi<SHIFT>(j);
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = sd[pj + r * PSTRIDE];
        }
        if constexpr (TAB) {
            const float2 *tj = t2 + mod_c<NS>(j);
#pragma unroll
            for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tj[r * NS]);
        } else if constexpr (NS > 1) {
            apply_twiddles<R>(v, mod_c<NS>(j) * (M / (NS * R)), lo, hi);
        }
    };
    auto transform = [&](float2 *v) {
        if constexpr (BIASED)
            Dft<R>::template run<true>(v, make_float2(2.0f * kInt8Bias, 2.0f * kInt8Bias));
        else
            Dft<R>::run(v);
    };
    auto store = [&](int j, const float2 *v) {
        const int base = div_c<NS>(j) * (NS * R) + mod_c<NS>(j);
        if constexpr (RUNS) {
            const int pb = padi<SHIFT>(base);
#pragma unroll
            for (int r = 0; r < R; ++r) sd[pb + r * PNS] = v[r];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) sd[padi<SHIFT>(base + r * NS)] = v[r];
        }
    };
    if constexpr (STREAM) {
        __syncthreads();
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int j = tid + q * T;
            if (!EXACT && j >= STRIDE) continue;
            float2 v[R];
            gather(j, v);
            transform(v);
            store(j, v);
        }
    } else {
        float2 v[NB][R];
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int j = tid + q * T;
            if (!EXACT && j >= STRIDE) continue;
            gather(j, v[q]);
            transform(v[q]);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int j = tid + q * T;
            if (!EXACT && j >= STRIDE) continue;
            store(j, v[q]);
        }
    }
    __syncthreads();
}

// Last pass (radix R2, NS = J) fused with the split and the global store.
// Thread t >= 1 owns butterflies t and J - t: Z[M - (t + r*J)] = Z[(J - t) + (R-1-r)*J],
// so its R pairs are (a[r], b[R-1-r]). Thread 0 owns the two self-paired
// butterflies 0 and J/2: pairs (a[r], a[R-r]) and (b[r], b[R-1-r]). All threads
// run the same R iterations (thread 0's operands are register selects), so no
// warp diverges; only X[M/2] = conj(Z[M/2]) is one extra store for thread 0.
// Split twiddles: k = j + i*J gives w_k = w_j * exp(-pi*i*i/R2), one table
// lookup per butterfly times compile-time constants.
template <int MM, int PLAN, class Row>
__device__ __forceinline__ void last_pass_store(const float2 *__restrict__ sd,
                                                const float2 *plo, const float2 *phi,
                                                const float2 *qlo, const float2 *qhi,
                                                const Row &yrow, int tid) {
    using C = FeCfg<MM, PLAN>;
    constexpr int M = C::M, J = C::J, R = C::R2, H = R / 2;
    static_assert(J % (1 << C::PADSHIFT) == 0, "last-pass stride");
    constexpr int PJ = J + (J >> C::PADSHIFT);
    const bool t0 = (tid == 0);
    const int j1 = tid;
    const int j2 = t0 ? J / 2 : J - tid;
    float2 a[R], b[R];
    const int p1 = padi<C::PADSHIFT>(j1), p2 = padi<C::PADSHIFT>(j2);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        a[r] = sd[p1 + r * PJ];
        b[r] = sd[p2 + r * PJ];
    }
    apply_twiddles<R>(a, j1, plo, phi);
    apply_twiddles<R>(b, j2, plo, phi);
    Dft<R>::run(a);   // a[r] = Z[j1 + r*J]
    Dft<R>::run(b);   // b[r] = Z[j2 + r*J]
    // h*w_{j1} and h*w_{j2} (thread 0: h*w_{J/2}), h = yrow.half (split_store)
    const float2 w1 = scale_tw(cmul(qlo[j1 & 63], qhi[j1 >> 6]), yrow.half);
    const float2 w2 = scale_tw(cmul(qlo[j2 & 63], qhi[j2 >> 6]), yrow.half);
    // Second half (i >= H): thread 0 pairs b with itself from k = J/2; the
    // others continue k = j1 + i*J. Both as a base index and a base twiddle
    // chosen once, stepped by compile-time constants.
    const int kB = t0 ? J / 2 : j1 + H * J;
    const float2 wB = t0 ? w2 : mul_w32(w1, H * (16 / R));
#pragma unroll
    for (int i = 0; i < R; ++i) {
        // exp(-pi*i*n/R) = exp(-2*pi*i*n*(16/R)/32)
        if (i < H) {
            // thread 0 (j1 = 0): Z[M - i*J] = Z[(R - i)*J] = a[(R - i) % R]
            const float2 zmk = t0 ? a[(R - i) % R] : b[R - 1 - i];
            split_store(a[i], zmk, mul_w32(w1, i * (16 / R)), j1 + i * J, M, !(t0 && i == 0),
                        yrow);
        } else {
            const float2 zk = t0 ? b[i - H] : a[i];
            const float2 zmk = t0 ? b[R - 1 - (i - H)] : b[R - 1 - i];
            split_store(zk, zmk, mul_w32(wB, (i - H) * (16 / R)), kB + (i - H) * J, M, true,
                        yrow);
        }
    }
    if (t0) yrow.put(M / 2, make_float2(a[H].x * yrow.scale, -a[H].y * yrow.scale));
}

// Last pass for the odd bins of a frame split into two half-length sequences:
// B[k'] = Z[2k'+1], k' < M (M = n_freq/2, this transform's length). Bin
// k = 2k'+1 of the real spectrum pairs with n_freq - k = 2(M-1-k')+1, that is
// B[k'] with B[M-1-k']; for k' = j + i*J the partner is butterfly J-1-j, output
// R-1-i. Thread t owns butterflies t and J-1-t (t < J/2 = T), so its R pairs
// are (a[i], b[R-1-i]) and no element pairs with itself. The split twiddle is
// exp(-2*pi*i*k/(2*n_freq)) = exp(-pi*i*k'/M) * exp(-pi*i/n_freq) (odd_shift).
// Row: a STEP 2 row of the odd bins, so index k' lands on bin 2k'+1.
template <int MM, int PLAN, class Row>
__device__ __forceinline__ void last_pass_store_odd(const float2 *__restrict__ sd,
                                                    const float2 *plo, const float2 *phi,
                                                    const float2 *qlo, const float2 *qhi,
                                                    float2 odd_shift, const Row &yrow, int tid) {
    using C = FeCfg<MM, PLAN>;
    constexpr int M = C::M, J = C::J, R = C::R2;
    static_assert(J % (1 << C::PADSHIFT) == 0 && J % 2 == 0, "last-pass stride");
    constexpr int PJ = J + (J >> C::PADSHIFT);
    const int j1 = tid, j2 = J - 1 - tid;
    float2 a[R], b[R];
    const int p1 = padi<C::PADSHIFT>(j1), p2 = padi<C::PADSHIFT>(j2);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        a[r] = sd[p1 + r * PJ];
        b[r] = sd[p2 + r * PJ];
    }
    apply_twiddles<R>(a, j1, plo, phi);
    apply_twiddles<R>(b, j2, plo, phi);
    Dft<R>::run(a);   // a[r] = B[j1 + r*J]
    Dft<R>::run(b);   // b[r] = B[j2 + r*J]
    const float2 w1 = scale_tw(cmul(cmul(qlo[j1 & 63], qhi[j1 >> 6]), odd_shift), yrow.half);
#pragma unroll
    for (int i = 0; i < R; ++i)   // exp(-pi*i*i/R) = exp(-2*pi*i*i*(16/R)/32)
        split_store(a[i], b[R - 1 - i], mul_w32(w1, i * (16 / R)), j1 + i * J, M - 1, true, yrow);
}

struct TwPtrs {
    const float2 *pass_lo, *pass_hi, *post_lo, *post_hi;
    const float2 *odd_shift;   // HALF only
};

// HALF (n_freq = 2*MM above 16384): each item's frame of 2*MM sample pairs is
// transformed as two MM-point sequences, even bins then odd bins, from one
// int8 buffer; the next item's copy is issued once the second sequence's first
// pass has read the frame, and lands during the rest of that transform.
template <int MM, int PLAN, int FMT, bool CONTIG, bool HALF>
__global__ void __launch_bounds__(FeCfg<MM, PLAN, HALF>::T, FeCfg<MM, PLAN, HALF>::MIN_BLOCKS)
    fengine_kernel(FengineArgs a, TwPtrs tw) {
    using C = FeCfg<MM, PLAN, HALF>;
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
    float2 *t2 = reinterpret_cast<float2 *>(smem + C::OFF_T2);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + C::OFF_BAR);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + C::OFF_FLAG);
    float2 *odd_shift = reinterpret_cast<float2 *>(smem + C::OFF_SHIFT);

    const int tid = threadIdx.x;
    if (HALF && tid == 0) *odd_shift = *tw.odd_shift;
    for (int i = tid; i < 64; i += T) {
        plo[i] = tw.pass_lo[i];
        qlo[i] = tw.post_lo[i];
    }
    for (int i = tid; i < 28; i += T)   // compact copies for w^4, w^8, w^16
        plo[64 + i] = i < 16 ? tw.pass_lo[4 * i] : i < 24 ? tw.pass_lo[8 * (i - 16)]
                                                           : tw.pass_lo[16 * (i - 24)];
    for (int i = tid; i < C::N_PASS_HI; i += T) phi[i] = tw.pass_hi[i];
    for (int i = tid; i < C::N_POST_HI; i += T) qhi[i] = tw.post_hi[i];
    // second pass: t2[r][jj] = exp(-2*pi*i*r*jj/(R0*R1)) = w^u, u = r*jj*M/(R0*R1)
    // (< M, as r < R1 and jj < R0)
    for (int i = tid; i < C::R0 * C::R1; i += T) {
        const int r = i / C::R0, jj = i - r * C::R0;
        const int u = r * jj * (M / (C::R0 * C::R1));
        t2[i] = cmul(tw.pass_lo[u & 63], tw.pass_hi[u >> 6]);
    }
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        if (!HALF) mbar_init(&bar[1], 1);
        *abort_flag = 0;
        fence_mbar_init();
    }
    __syncthreads();

    const int n_items = a.frames * a.n_station;
    const uint32_t frame_bytes = C::FRAME;
    const int ytile_shift = __ffs(a.ytile) - 1;
    const float out_scale = (FMT == kSpectraF32) ? 1.0f : a.y_scale;   // FP32 bins unscaled
    auto src_of = [&](int item) {
        const int f = item / a.n_station;
        const int s = item - f * a.n_station;
        return a.samples + static_cast<size_t>(s) * a.station_stride +
               static_cast<size_t>(f) * a.frame_stride;
    };
    auto present = [&](int item) {
        const int f = item / a.n_station;
        return frame_present<M>(a, f, item - f * a.n_station);
    };

    int item = blockIdx.x;
    if (tid == 0 && item < n_items && present(item)) {
        mbar_arrive_expect_tx(&bar[0], frame_bytes);
        bulk_copy_g2s(sx0, src_of(item), frame_bytes, &bar[0]);
    }
    uint32_t parity_bits = 0u;   // bit b = phase parity of bar[b]

    for (int n = 0; item < n_items; ++n, item += gridDim.x) {
        const int buf = HALF ? 0 : (n & 1);
        const int next = item + gridDim.x;
        bool next_issued = false;
        if (!HALF && tid == 0 && next < n_items && present(next)) {
            // The other buffer was last read by the previous item's first pass,
            // which every thread finished before that pass's first barrier.
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[buf ^ 1], frame_bytes);
            bulk_copy_g2s(buf ? sx0 : sx1, src_of(next), frame_bytes, &bar[buf ^ 1]);
            next_issued = true;
        }
        // HALF: the single buffer is free once this item's frame has been read
        // (or at once, for a missing frame, which was never copied).
        auto issue_next_into_buffer = [&] {
            if (tid == 0 && next < n_items && present(next)) {
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&bar[0], frame_bytes);
                bulk_copy_g2s(sx0, src_of(next), frame_bytes, &bar[0]);
            }
        };
        using Row = YRow<FMT, CONTIG>;
        const Row yrow{
            reinterpret_cast<typename Row::T *>(a.y) + static_cast<size_t>(item) * a.ytile,
            static_cast<uint32_t>(a.y_frames) * a.n_station * a.ytile, ytile_shift, out_scale,
            0.5f * out_scale};

        if (!present(item)) {
            if constexpr (HALF) issue_next_into_buffer();
            // Missing frame: its samples count as zeros, so does its spectrum.
            for (int k = tid; k < (HALF ? 2 * M : M); k += T) yrow.put(k, make_float2(0.f, 0.f));
            continue;
        }

        // Every thread waits for the frame itself: no CTA barrier here, so a
        // warp that has stored its part of the previous spectrum starts this
        // item's first pass (which reads only the int8 frame and writes sd after
        // its own barrier) while other warps are still storing.
        if (!mbar_wait_bounded(&bar[buf], (parity_bits >> buf) & 1u, a.err,
                               kErrFengineCopyTimeout))
            *abort_flag = 1;
        parity_bits ^= 1u << buf;

        if constexpr (HALF) {
            using RowH = YRow<FMT, CONTIG, 2>;
            const RowH even{yrow.base, yrow.tile_stride, yrow.shift, yrow.scale, yrow.half, 0};
            const RowH odd{yrow.base, yrow.tile_stride, yrow.shift, yrow.scale, yrow.half, 1};
            fft_pass<M, T, C::P, C::R0, 1, C::PADSHIFT, kFromInt8Sum>(sd, sx0, plo, phi, tid,
                                                                     nullptr, qlo, qhi);
            if (*abort_flag) return;   // nothing in flight: the next copy is not issued yet
            fft_pass<M, T, C::P, C::R1, C::R0, C::PADSHIFT, kFromShared, true>(sd, nullptr, plo,
                                                                              phi, tid, t2);
            if constexpr (C::R1b > 1)
                fft_pass<M, T, C::P, C::R1b, C::R0 * C::R1, C::PADSHIFT, kFromShared>(
                    sd, nullptr, plo, phi, tid);
            last_pass_store<MM, PLAN>(sd, plo, phi, qlo, qhi, even, tid);
            fft_pass<M, T, C::P, C::R0, 1, C::PADSHIFT, kFromInt8Diff>(sd, sx0, plo, phi, tid,
                                                                      nullptr, qlo, qhi);
            // that pass ended with a barrier: every thread has read the frame
            issue_next_into_buffer();
            fft_pass<M, T, C::P, C::R1, C::R0, C::PADSHIFT, kFromShared, true>(sd, nullptr, plo,
                                                                              phi, tid, t2);
            if constexpr (C::R1b > 1)
                fft_pass<M, T, C::P, C::R1b, C::R0 * C::R1, C::PADSHIFT, kFromShared>(
                    sd, nullptr, plo, phi, tid);
            last_pass_store_odd<MM, PLAN>(sd, plo, phi, qlo, qhi, *odd_shift, odd, tid);
            continue;
        }

        if (a.pmask != nullptr) {
            // Lost packets count as zeros: clear them in the landed copy before
            // the first pass reads it. The word is the same for every thread,
            // so the branch and its barrier are taken by the whole CTA.
            const int f = item / a.n_station;
            const uint32_t kept = packets_kept<M>(a, f, item - f * a.n_station);
            if (kept != all_packets<M>()) {
                uint4 *x16 = reinterpret_cast<uint4 *>(buf ? sx1 : sx0);
                for (int i = tid; i < M / 8; i += T)     // 64 uint4 per packet
                    if (!((kept >> (i >> 6)) & 1u)) x16[i] = make_uint4(0u, 0u, 0u, 0u);
                __syncthreads();
            }
        }

        fft_pass<M, T, C::P, C::R0, 1, C::PADSHIFT, kFromInt8>(sd, buf ? sx1 : sx0, plo, phi, tid);
        // the pass ends with a barrier: every thread sees the same flag
        if (*abort_flag) {
            // Let whatever copy is still in flight land before the CTA exits.
            if (tid == 0 && next_issued)
                mbar_wait_bounded(&bar[buf ^ 1], (parity_bits >> (buf ^ 1)) & 1u, nullptr, 0);
            return;
        }
        fft_pass<M, T, C::P, C::R1, C::R0, C::PADSHIFT, kFromShared, true>(sd, nullptr, plo, phi,
                                                                          tid, t2);
        if constexpr (C::R1b > 1)
            fft_pass<M, T, C::P, C::R1b, C::R0 * C::R1, C::PADSHIFT, kFromShared>(sd, nullptr, plo,
                                                                                phi, tid);
        last_pass_store<MM, PLAN>(sd, plo, phi, qlo, qhi, yrow, tid);
        // The next item's first pass synchronises before it overwrites sd.
    }
}

template <int MM, int PLAN, int FMT, bool CONTIG, bool HALF>
corr_status launch_one(const FengineArgs &a, const TwiddleTables &tw, int num_sms,
                       cudaStream_t stream) {
    using C = FeCfg<MM, PLAN, HALF>;
    // Shared-memory limit and residency are per device: set up once on each.
    static PerDevice setup;
    static int per_sm[kMaxDeviceOrdinals];
    corr_status st = setup.run([](int dev) {
        corr_status s2 = cuda_check(
            cudaFuncSetAttribute(fengine_kernel<MM, PLAN, FMT, CONTIG, HALF>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM),
            "cudaFuncSetAttribute(fengine)");
        if (s2 != CORR_OK) return s2;
        int blocks = 0;
        s2 = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                            &blocks, fengine_kernel<MM, PLAN, FMT, CONTIG, HALF>, C::T, C::SMEM),
                        "cudaOccupancyMaxActiveBlocksPerMultiprocessor(fengine)");
        if (s2 != CORR_OK) return s2;
        if (blocks < 1)
            return fail(CORR_ERR_INTERNAL, "F-engine kernel cannot be resident on an SM");
        per_sm[dev] = blocks;
        return CORR_OK;
    });
    if (st != CORR_OK) return st;
    int dev = 0;
    cudaGetDevice(&dev);
    const int items = a.frames * a.n_station;
    if (items <= 0) return CORR_OK;
    int grid = num_sms * per_sm[dev];
    if (grid > items) grid = items;
    TwPtrs p{tw.pass_lo, tw.pass_hi, tw.post_lo, tw.post_hi, tw.odd_shift};
    fengine_kernel<MM, PLAN, FMT, CONTIG, HALF><<<grid, C::T, C::SMEM, stream>>>(a, p);
    return cuda_check(cudaGetLastError(), "fengine_kernel launch");
}

template <int MM, int PLAN, bool HALF = false>
corr_status launch_plan(const FengineArgs &a, const TwiddleTables &tw, int num_sms,
                        cudaStream_t stream) {
    const bool contig = a.ytile == (HALF ? 2 * MM : MM);
    if (a.y_fmt == kSpectraF16)
        return contig ? launch_one<MM, PLAN, kSpectraF16, true, HALF>(a, tw, num_sms, stream)
                      : launch_one<MM, PLAN, kSpectraF16, false, HALF>(a, tw, num_sms, stream);
    if (a.y_fmt == kSpectraF16Split)
        return contig ? launch_one<MM, PLAN, kSpectraF16Split, true, HALF>(a, tw, num_sms, stream)
                      : launch_one<MM, PLAN, kSpectraF16Split, false, HALF>(a, tw, num_sms,
                                                                            stream);
    if (contig) return launch_one<MM, PLAN, kSpectraF32, true, HALF>(a, tw, num_sms, stream);
    return launch_one<MM, PLAN, kSpectraF32, false, HALF>(a, tw, num_sms, stream);
}

template <int MM>
corr_status launch_size(const FengineArgs &a, const TwiddleTables &tw, int num_sms,
                        cudaStream_t stream) {
    if constexpr (MM == 16384) {
        if (a.fplan == 1) return launch_plan<MM, 1>(a, tw, num_sms, stream);
        if (a.fplan == 2) return fengine_tc_launch(a, tw.tc_image, num_sms, stream);
    }
    if (a.fplan != 0)
        return failf(CORR_ERR_ARG, "FFT plan %d is not available at n_freq=%d", a.fplan, MM);
    return launch_plan<MM, 0>(a, tw, num_sms, stream);
}

// n_freq = 2*MH above 16384: two MH-point transforms per frame.
template <int MH>
corr_status launch_half(const FengineArgs &a, const TwiddleTables &tw, int num_sms,
                        cudaStream_t stream) {
    if (a.fplan != 0)
        return failf(CORR_ERR_ARG, "FFT plan %d is not available at n_freq=%d", a.fplan, 2 * MH);
    if (a.pmask != nullptr)
        return failf(CORR_ERR_ARG,
                     "n_freq=%d: packet masks cover frames of at most 32 packets (n_freq <= 16384)",
                     2 * MH);
    if (tw.odd_shift == nullptr)
        return failf(CORR_ERR_INTERNAL, "n_freq=%d: twiddle tables lack the odd-bin shift", 2 * MH);
    return launch_plan<MH, 0, true>(a, tw, num_sms, stream);
}

} // namespace
} // namespace corrgb

#endif // CORR_GB300_FENGINE_IMPL_CUH
