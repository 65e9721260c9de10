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
//     shared memory (three or four passes of radix 4..32, led by an odd radix
//     3..15 when M is not a power of two; FePlan in fengine_impl.cuh), FP32 in
//     registers, twiddles from host-computed double-precision tables; above
//     n_freq 16384 the M points are first split into two M/2-point sequences
//     (even and odd bins) that the CTA transforms in turn (HALF);
//   * the split X[k] = Fe[k] + w^k Fo[k] turns Z into the L-point real spectrum;
//     bins 0..M-1 are written, the Nyquist bin M is dropped and nothing is
//     normalised (reference semantics, HANDOFF.md:583-602).
//
// Output layout (engine.h, y_index): bins in channel tiles of `ytile`; bin k of
// (frame f, station s) lands at ((k/ytile)*y_frames + f)*n_station + s)*ytile +
// k%ytile, as FP32 pairs, FP16 pairs or FP16 hi/lo pairs (YRow). The fused last
// pass writes 32 consecutive bins per warp store.

#include <cmath>
#include <vector>

#include "fengine_impl.cuh"

// This file: the host side (twiddle tables, plans, dispatch by length) and the
// kernels of n_freq 512 .. 8192; fengine_impl.cuh holds the kernel templates.

namespace corrgb {

int fengine_plans(int n_freq) { return n_freq == 16384 ? 3 : 1; }

bool fengine_plan_ok(int n_freq, int fplan, int y_fmt) {
    if (fplan < 0 || fplan >= fengine_plans(n_freq)) return false;
    return fplan != 2 || y_fmt == kSpectraF16;   // the tensor-core plan writes FP16 only
}

void fengine_twiddles_host(int n_freq, std::vector<float2> *all) {
    const int M = fft_length(n_freq);
    const double pi = 3.14159265358979323846;
    auto cis = [](double a) {
        return make_float2(static_cast<float>(std::cos(a)), static_cast<float>(std::sin(a)));
    };
    all->clear();
    all->reserve(static_cast<size_t>(twiddle_entries(n_freq)));
    for (int u = 0; u < 64; ++u) all->push_back(cis(-2.0 * pi * u / M));            // pass_lo
    for (int u = 0; u < M / 64; ++u) all->push_back(cis(-2.0 * pi * 64.0 * u / M)); // pass_hi
    for (int u = 0; u < 64; ++u) all->push_back(cis(-pi * u / M));                  // post_lo
    for (int u = 0; u < M / 64; ++u) all->push_back(cis(-pi * 64.0 * u / M));       // post_hi
    if (M != n_freq) all->push_back(cis(-pi / n_freq));                           // odd_shift
    all->resize(static_cast<size_t>(twiddle_entries(n_freq)), make_float2(0.f, 0.f));
}

void twiddle_views(float2 *base, int n_freq, TwiddleTables *tw) {
    const int M = fft_length(n_freq);
    tw->n_pass_hi = M / 64;
    tw->n_post_hi = M / 64;
    tw->pass_lo = base;
    tw->pass_hi = base + 64;
    tw->post_lo = tw->pass_hi + tw->n_pass_hi;
    tw->post_hi = tw->post_lo + 64;
    tw->odd_shift = M != n_freq ? tw->post_hi + tw->n_post_hi : nullptr;
}

corr_status fengine_prepare(int n_freq, TwiddleTables *tw) {
    std::vector<float2> all;
    fengine_twiddles_host(n_freq, &all);
    const size_t n_all = all.size();
    float2 *d = nullptr;
    corr_status st = cuda_check(cudaMalloc(&d, n_all * sizeof(float2)), "cudaMalloc(twiddles)");
    if (st != CORR_OK) return st;
    st = cuda_check(cudaMemcpy(d, all.data(), n_all * sizeof(float2), cudaMemcpyHostToDevice),
                    "cudaMemcpy(twiddles)");
    if (st != CORR_OK) {
        cudaFree(d);
        return st;
    }
    twiddle_views(d, n_freq, tw);
    if (n_freq == 16384 && (st = fengine_tc_prepare(&tw->tc_image)) != CORR_OK) {
        fengine_release(tw);
        return st;
    }
    return CORR_OK;
}

void fengine_release(TwiddleTables *tw) {
    if (tw->pass_lo != nullptr) cudaFree(tw->pass_lo);
    if (tw->tc_image != nullptr) cudaFree(tw->tc_image);
    *tw = TwiddleTables{};
}

corr_status fengine_launch(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                           int num_sms, cudaStream_t stream) {
    switch (n_freq) {
    case 512: return launch_size<512>(a, tw, num_sms, stream);
    case 1024: return launch_size<1024>(a, tw, num_sms, stream);
    case 2048: return launch_size<2048>(a, tw, num_sms, stream);
    case 4096: return launch_size<4096>(a, tw, num_sms, stream);
    case 6144: return launch_size<6144>(a, tw, num_sms, stream);
    case 8192: return launch_size<8192>(a, tw, num_sms, stream);
    case 10240: case 12288: case 14336: case 16384:
        return fengine_launch_large(n_freq, tw, a, num_sms, stream);
    case 18432: case 20480: return fengine_launch_split_a(n_freq, tw, a, num_sms, stream);
    case 22528: case 24576: return fengine_launch_split_b(n_freq, tw, a, num_sms, stream);
    case 26624: case 28672: return fengine_launch_split_c(n_freq, tw, a, num_sms, stream);
    case 30720: case 32768: return fengine_launch_split_d(n_freq, tw, a, num_sms, stream);
    default:
        return failf(CORR_ERR_ARG,
                     "F-engine: n_freq=%d is neither a power of two in [512, 32768] nor a "
                     "multiple of 2048 up to 32768",
                     n_freq);
    }
}

} // namespace corrgb
