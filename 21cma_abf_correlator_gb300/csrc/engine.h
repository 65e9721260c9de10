// engine.h -- internal interface between the C ABI layer (abi.cpp), the
// device-resident extension API and the CUDA translation units.
//
// The reference splits its library the same way (corr-cuda/src/gpu_internal.h
// between corr_cuda.cpp and kernels.cu); the contents here are this engine's own:
// an FX plan (F-engine FFT + X-engine) that works on device pointers, and the
// staged pipeline (streams, events, row stack) the ABI drives.

#ifndef CORR_GB300_ENGINE_H
#define CORR_GB300_ENGINE_H

#include <cstddef>
#include <cstdint>
#include <algorithm>
#include <atomic>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "corr_cuda.h"
#include "corr_gb300.h"

namespace corrgb {

/// Thread-local failure message returned by corr_last_error().
std::string &last_error();
corr_status fail(corr_status st, const std::string &msg);
corr_status failf(corr_status st, const char *fmt, ...);
corr_status cuda_check(cudaError_t e, const char *what);

/// Device ordinals a process-wide per-device record can hold.
constexpr int kMaxDeviceOrdinals = 64;

/// A one-time set-up that must happen once on every device a kernel runs on
/// (cudaFuncSetAttribute and occupancy queries are per-device), safe against
/// concurrent first calls from several threads. run() executes `fn` with the
/// current device unless it already succeeded there; a failure is not recorded,
/// so the next call tries again.
class PerDevice {
public:
    template <class F> corr_status run(F &&fn) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) {
            cudaGetLastError();
            return fail_current();
        }
        if (dev < 0 || dev >= kMaxDeviceOrdinals) return fail_ordinal(dev);
        if (done_[dev].load(std::memory_order_acquire)) return CORR_OK;
        std::lock_guard<std::mutex> lock(mu_);
        if (done_[dev].load(std::memory_order_relaxed)) return CORR_OK;
        const corr_status st = fn(dev);
        if (st == CORR_OK) done_[dev].store(true, std::memory_order_release);
        return st;
    }

private:
    static corr_status fail_current();
    static corr_status fail_ordinal(int dev);
    std::mutex mu_;
    std::atomic<bool> done_[kMaxDeviceOrdinals] = {};
};

/// Watchdog codes a kernel writes into FxPlan::d_err when a bounded wait ran out.
enum : int {
    kErrNone = 0,
    kErrFengineCopyTimeout = 1,
    kErrXengineTmemTimeout = 2,
    kErrXengineMmaTimeout = 3,
    kErrSelftestTimeout = 4,
};

/// Twiddle tables, all computed on the host in double precision (libm) and
/// rounded once to float.
///   pass_lo[u]  = exp(-2*pi*i*u/M)        u in [0, 64)
///   pass_hi[u]  = exp(-2*pi*i*64*u/M)     u in [0, M/64)
///   post_lo[k]  = exp(-pi*i*k/M)          k in [0, 64)
///   post_hi[k]  = exp(-pi*i*64*k/M)       k in [0, M/64)
/// so exp(-2*pi*i*u/M) = pass_lo[u%64]*pass_hi[u/64] (u < M) and the real-FFT
/// split twiddle exp(-2*pi*i*k/L) = post_lo[k%64]*post_hi[k/64] (k < M).
struct TwiddleTables {
    float2 *pass_lo = nullptr;
    float2 *pass_hi = nullptr;
    float2 *post_lo = nullptr;
    float2 *post_hi = nullptr;
    int n_pass_hi = 0;
    int n_post_hi = 0;
    // n_freq above 16384 (two half-length transforms, M = n_freq/2 above):
    // exp(-pi*i/n_freq), the odd bins' offset in the real-FFT split twiddle
    float2 *odd_shift = nullptr;
    void *tc_image = nullptr;   // tensor-core FFT tables (plan 2, n_freq 16384)
};

/// Spectra layout shared by the F- and X-engines: channel tiles of `ytile`
/// channels (n_freq itself, or a power of two >= 2 that divides n_freq), each
/// tile holding every frame and station,
///   y[((c / ytile) * y_frames + f) * n_station + s) * ytile + c % ytile]
/// ytile = n_freq is one contiguous row of n_freq bins per (frame, station)
/// (the F-engine's cheapest store pattern); ytile equal to the tensor
/// X-engine's channels per tile makes each of its stages one contiguous block.
__host__ __device__ inline size_t y_index(int c, int f, int s, int n_station, int y_frames,
                                          int ytile) {
    return ((static_cast<size_t>(c / ytile) * y_frames + f) * n_station + s) * ytile +
           (c % ytile);
}

/// How the F-engine stores a bin for each X-engine: FP32 pairs (plain); FP16
/// pairs scaled by spectra_scale (FP16 tensor form); or the split form's operands,
/// the scaled FP16 pair h then l = fp16(scaled - h), 8 bytes like FP32.
enum SpectraFormat : int { kSpectraF32 = 0, kSpectraF16 = 1, kSpectraF16Split = 2 };

inline int spectra_format(int xmode) {
    return xmode == CORR_X_TC_FP16         ? kSpectraF16
           : xmode == CORR_X_TC_FP16_SPLIT ? kSpectraF16Split
                                           : kSpectraF32;
}

/// The power of two that FP16 spectra are scaled by: spectra of int8 frames
/// satisfy |Y| <= 128*L, so 2^-(ceil(log2 L) - 8) keeps every bin at or below
/// 2^15, inside FP16's range, for every input; products are unscaled by its
/// inverse square.
inline float spectra_scale(int n_freq) {
    int l = 0;
    while ((1 << l) < 2 * n_freq) ++l;
    return std::ldexp(1.0f, -(l - 8));
}

/// Arguments of one F-engine launch: `frames` x `n_station` real FFTs.
struct FengineArgs {
    const int8_t *samples;      // frame f of station s: samples + s*station_stride + f*frame_stride
    size_t station_stride;
    size_t frame_stride;
    const uint8_t *mask;        // nullable; bit (mask_bit0+f) of mask + s*mask_station_stride
    size_t mask_station_stride;
    int mask_bit0;
    // nullable; word pmask[s*pmask_station_stride + pmask_frame0 + f]: bit p set = the
    // p-th 1024-sample packet of frame f of station s arrived (the others are zeros)
    const uint32_t *pmask;
    size_t pmask_station_stride;
    int pmask_frame0;
    int n_station;
    int frames;
    float2 *y;                  // spectra (y_index)
    int y_frames;               // frames the spectra buffer holds
    int ytile;                  // channels per spectra tile
    int y_fmt;                  // SpectraFormat of the stored bins (scaled by y_scale if FP16)
    int fplan;                  // FFT radix plan (0 .. fengine_plans(n_freq) - 1)
    float y_scale;
    int *err;
};

/// Arguments of one X-engine launch over `frames` frames of spectra.
///
/// The launch sums its frames in FP32 (registers or tensor memory) and adds that
/// partial sum into the row once, in its epilogue: into complex64 values
/// (acc64 = 0) or into complex128 values (acc64 = 1), the cross-launch
/// integration accumulator that keeps long rows at the precision of one launch.
struct XengineArgs {
    const float2 *y;            // as FengineArgs::y
    int y_frames;               // frames the spectra buffer holds (>= frames)
    int ytile;                  // channels per spectra tile
    int y_fmt;                  // SpectraFormat of the bins
    int n_station;
    int n_freq;
    int frames;
    void *acc;                  // acc[b*n_freq + c] += (float2, or double2 if acc64)
    int acc64;
    int *err;
    // plain X-engine: compute only the station-block pairs [pair_first,
    // pair_first + pair_count) of its row-major enumeration (pair_count 0: all),
    // or, with pair_list, the pair_count pairs it names
    int pair_first;
    int pair_count;
    const int32_t *pair_list;
};

// fengine.cu
/// Length of the F-engine's complex FFT for n_freq: n_freq itself up to 16384
/// (one CTA's shared memory holds the frame); above that a frame is split by
/// one radix-2 step into two sequences of n_freq/2 points, transformed one
/// after the other by the same CTA (even bins, then odd bins).
constexpr int fft_length(int n_freq) { return n_freq > 16384 ? n_freq / 2 : n_freq; }
/// Entries reserved for n_freq's twiddle tables: the four tables of
/// M = fft_length(n_freq) (pass_lo, pass_hi, post_lo, post_hi), then, for the
/// split lengths, odd_shift; zero-padded up to this count.
constexpr int twiddle_entries(int n_freq) { return 128 + 2 * (n_freq / 64); }
/// The tables for n_freq, concatenated in that order (host, double precision
/// rounded once to float), twiddle_entries(n_freq) of them.
void fengine_twiddles_host(int n_freq, std::vector<float2> *all);
/// Point `tw` at the four tables stored concatenated from `base` (device memory).
void twiddle_views(float2 *base, int n_freq, TwiddleTables *tw);
corr_status fengine_prepare(int n_freq, TwiddleTables *tw);
/// How many FFT radix plans the F-engine has for n_freq (plan 0 always exists).
int fengine_plans(int n_freq);
void fengine_release(TwiddleTables *tw);
/// FFT plan 2 (n_freq 16384, FP16 spectra): the tensor-core F-engine (fengine_tc.cu).
corr_status fengine_tc_prepare(void **d_image);
corr_status fengine_tc_launch(const FengineArgs &a, const void *image, int num_sms,
                              cudaStream_t stream);
/// Whether FFT plan `fplan` can write spectra of format `y_fmt` at n_freq.
bool fengine_plan_ok(int n_freq, int fplan, int y_fmt);
corr_status fengine_launch(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                           int num_sms, cudaStream_t stream);

// xengine.cu
corr_status xengine_plain_launch(const XengineArgs &a, int num_sms, cudaStream_t stream);
/// The plain X-engine's station-block pair holding baseline (j, k), j <= k: its
/// index in the row-major enumeration of block pairs.
int xengine_plain_block_pair(int n_station, int j, int k);
corr_status scale_launch(float2 *acc, size_t n, float s, cudaStream_t stream);
/// acc[i] *= s in double precision over n complex128 values.
corr_status scale64_launch(double2 *acc, size_t n, double s, cudaStream_t stream);
/// dst[i] += src[i] over n complex128 values.
corr_status add64_launch(double2 *dst, const double2 *src, size_t n, cudaStream_t stream);
/// Complex128 rows to complex64: for r < rows, i < n_map, c < n_freq,
///   out[r*out_row + gmap[i]*n_freq + c] = (float2)(src[r*src_row + lmap[i]*n_freq + c] * s)
/// (gmap/lmap NULL: the identity over n_map baselines). n_freq is even.
corr_status dump64_launch(float2 *out, size_t out_row, const double2 *src, size_t src_row,
                          const int32_t *gmap, const int32_t *lmap, int n_map, int n_freq,
                          int rows, double s, cudaStream_t stream);
corr_status watchdog_selftest_launch(int *err, long long budget_cycles, cudaStream_t stream);
corr_status stamp_launch(unsigned long long *slot, cudaStream_t stream);
/// Deterministic pseudo-random int8 samples (roughly Gaussian, sigma ~ 24) for
/// the autotuner's timing passes.
corr_status synth_fill_launch(int8_t *x, size_t n, uint32_t seed, cudaStream_t stream);

// xengine_tc.cu
/// Is (ct channels per tile, kt frames per stage) a feasible tensor X-engine
/// tile for n_station inputs (TMEM columns, shared memory)?
bool xengine_tc_shape_ok(int n_station, bool split, int ct, int kt);
/// The widest feasible tile with 16-frame stages (*ct = 0: none).
void xengine_tc_default_shape(int n_station, bool split, int *ct, int *kt);
corr_status xengine_tc_launch(const XengineArgs &a, bool split, int ct, int kt, int num_sms,
                              cudaStream_t stream);

/// An FX plan: everything one device needs to turn int8 frames into added
/// visibilities, independent of where the frames came from.
struct FxPlan {
    int device = 0;
    int n_station = 0;
    int n_freq = 0;
    int n_baseline = 0;
    int max_frames = 0;   // frames per F/X pass (spectra buffer depth)
    int ytile = 0;        // channels per spectra tile (n_freq: contiguous rows)
    int xct = 0;          // tensor X-engine: channels per tile
    int xkt = 0;          // tensor X-engine: frames per stage
    int fplan = 0;        // F-engine FFT radix plan
    int xmode = CORR_X_PLAIN_FP32;
    int acc64 = 0;        // rows are complex128 (CORRX_ACC_FP64) instead of complex64
    int xpair_first = 0;  // plain X-engine: block pairs to compute (xpair_count 0: all)
    int xpair_count = 0;
    int32_t *d_xpair_list = nullptr;   // ... or the list of them (device memory)
    int num_sms = 0;
    float2 *d_y = nullptr;
    int *d_err = nullptr;
    TwiddleTables tw;
};

corr_status fxplan_create(int device, int n_station, int n_freq, int max_frames, int xmode,
                          FxPlan **out);
void fxplan_destroy(FxPlan *p);
corr_status fxplan_set_tiles(FxPlan *p, int ytile, int xct, int xkt, int fplan);
/// The plain X-engine computes only the station-block pairs that hold the given
/// baselines (indices of the row-major numbering over the plan's stations); the
/// other baselines of the row are left as they are. A device of a baseline-range
/// split owns a contiguous range of them, one of pair covering a scattered set.
/// The tensor forms compute every pair regardless.
corr_status fxplan_limit_baselines(FxPlan *p, const std::vector<int32_t> &baselines);
corr_status fxplan_autotune(FxPlan *p, cudaStream_t stream, corrx_tiles *out);

/// F then X over `frames` frames, in passes of at most max_frames.
corr_status fxplan_accumulate(FxPlan *p, const int8_t *samples, size_t station_stride,
                              size_t frame_stride, const uint8_t *mask,
                              size_t mask_station_stride, int mask_bit0, int frames,
                              void *acc, cudaStream_t stream,
                              const uint32_t *pmask = nullptr, size_t pmask_station_stride = 0,
                              int pmask_frame0 = 0);

/// Read and clear the device watchdog flag (synchronises the device).
corr_status fxplan_check(FxPlan *p);

/// Host-side validation shared by corr_create and corrx_create.
/// Stations one engine can correlate: the plain X-engine stages every station's
/// spectra for a tile of channels in shared memory (two frames a stage at 128);
/// the tensor forms take up to 64 (xengine_tc_default_shape).
constexpr int kMaxStations = 128;
/// Baselines the ABI lets one device own, the reference's per-device limit
/// (corr-cuda/src/kernels.cu:474-483): 44 stations on one device; more only
/// with the baselines split over several devices.
constexpr int kMaxBaselinesPerDevice = 1024;
/// n_station in [1, kMaxStations] and an n_freq the F-engine transforms.
corr_status check_geometry(int n_station, int n_freq);

} // namespace corrgb

#endif // CORR_GB300_ENGINE_H
