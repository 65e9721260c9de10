// noalloc.cu -- corrx_accumulate for callers that cannot allocate device memory.
//
// Some hosts of this library may not call cudaMalloc at all: an application
// that owns all device memory through its own pool and does not let plugins
// allocate, a real-time loop in which an allocation (and the device-wide
// synchronisation it can imply) would break the loop's deadline, or a process
// whose device-memory budget is fixed up front. corrx_accumulate_noalloc serves
// them: it runs the same F-engine and X-engine kernels as corrx_accumulate, but
// the spectra between the two live in a file-scope device array of fixed size
// instead of a buffer allocated by corrx_create, and the twiddle tables of every
// transform length live in a second fixed array.
//
// Properties a caller must know:
//   * scratch: kNoAllocScratchBytes (64 MiB) of spectra plus 86 KB of twiddle
//     tables, held by every GPU that loads the library until the process exits;
//   * one call may cover at most 64 MiB / (n_station * n_freq * e) frames, e the
//     bytes a spectrum bin takes between the engines (4 for the FP16 tensor
//     X-engine, 8 for the plain and split forms): 42 or 21 frames at 24 inputs
//     and n_freq 16384. Larger requests are rejected with CORR_ERR_ARG, nothing
//     is launched, and the caller splits them;
//   * the first call on a device does that device's set-up with it current: it
//     looks up the arrays' device addresses (cudaGetSymbolAddress) and copies
//     the twiddle tables into theirs (synchronous copies). Make that first call
//     before any stream capture;
//   * every call shares the spectra array: two calls whose kernels overlap on
//     the GPU (different streams, no ordering between them) race on it and give
//     wrong results. Calls on one stream are ordered and safe. Nothing in it has
//     to start at zero: each call writes every scratch value it reads;
//   * a bounded wait that runs out inside a kernel ends that kernel early
//     without a report (there is no engine to hold a watchdog flag); use
//     corrx_accumulate where that report matters.

#include <mutex>
#include <vector>

#include "engine.h"

namespace corrgb {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
// The transform lengths the F-engine takes, each with its tables in the array.
constexpr int kSizes[] = {512,   1024,  2048,  4096,  6144,  8192,  10240, 12288, 14336,
                          16384, 18432, 20480, 22528, 24576, 26624, 28672, 30720, 32768};
constexpr int kNumSizes = static_cast<int>(sizeof(kSizes) / sizeof(kSizes[0]));

// Offset of the twiddle tables of kSizes[i] channels in the twiddle array.
constexpr int twiddle_offset(int i) {
    return i == 0 ? 0 : twiddle_offset(i - 1) + twiddle_entries(kSizes[i - 1]);
}
constexpr int kTwEntries = twiddle_offset(kNumSizes);

static __device__ __align__(256) float2 g_noalloc_spectra[kNoAllocScratchBytes / sizeof(float2)];
static __device__ __align__(256) float2 g_noalloc_twiddles[kTwEntries];

struct DeviceScratch {
    float2 *spectra = nullptr;
    float2 *twiddles = nullptr;
    int num_sms = 0;
    bool ready = false;
};

std::mutex g_mu;
DeviceScratch g_dev[kMaxDeviceOrdinals];

// Set-up of `dev` (the current device), once: the arrays' device addresses, the
// SM count, and the twiddle tables of every supported length.
corr_status scratch_for(int dev, DeviceScratch *out) {
    if (dev < 0 || dev >= kMaxDeviceOrdinals)
        return failf(CORR_ERR_ARG, "device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_mu);
    DeviceScratch &d = g_dev[dev];
    if (!d.ready) {
        void *p = nullptr;
        corr_status st = cuda_check(cudaGetSymbolAddress(&p, g_noalloc_spectra),
                                    "cudaGetSymbolAddress(spectra scratch)");
        if (st != CORR_OK) return st;
        d.spectra = static_cast<float2 *>(p);
        st = cuda_check(cudaGetSymbolAddress(&p, g_noalloc_twiddles),
                        "cudaGetSymbolAddress(twiddle scratch)");
        if (st != CORR_OK) return st;
        d.twiddles = static_cast<float2 *>(p);
        std::vector<float2> all, tab;
        for (int i = 0; i < kNumSizes; ++i) {
            fengine_twiddles_host(kSizes[i], &tab);
            all.insert(all.end(), tab.begin(), tab.end());
        }
        st = cuda_check(cudaMemcpy(d.twiddles, all.data(), all.size() * sizeof(float2),
                                   cudaMemcpyHostToDevice),
                        "cudaMemcpy(twiddle scratch)");
        if (st != CORR_OK) return st;
        st = cuda_check(cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev),
                        "cudaDeviceGetAttribute(SM count)");
        if (st != CORR_OK) return st;
        d.ready = true;
    }
    *out = d;
    return CORR_OK;
}

} // namespace
} // namespace corrgb

using namespace corrgb;

extern "C" corr_status corrx_accumulate_noalloc(int32_t n_station, int32_t n_freq, int32_t xmode,
                                                const int8_t *d_samples, size_t station_stride,
                                                size_t frame_stride, const uint8_t *d_mask,
                                                size_t mask_station_stride, int32_t mask_bit0,
                                                int32_t frames, void *d_acc, void *stream) {
    corr_status st = check_geometry(n_station, n_freq);
    if (st != CORR_OK) return st;
    if (xmode != CORR_X_PLAIN_FP32 && xmode != CORR_X_TC_FP16 && xmode != CORR_X_TC_FP16_SPLIT)
        return failf(CORR_ERR_ARG, "unknown X-engine mode %d", xmode);
    if (d_samples == nullptr || d_acc == nullptr)
        return fail(CORR_ERR_ARG, "d_samples and d_acc must not be NULL");
    if (frames < 0 || mask_bit0 < 0) return fail(CORR_ERR_ARG, "frames and mask_bit0 must be >= 0");
    if (frame_stride < 2u * static_cast<size_t>(n_freq))
        return fail(CORR_ERR_ARG, "frame_stride is shorter than a frame");
    if ((reinterpret_cast<uintptr_t>(d_samples) | station_stride | frame_stride) % 16 != 0)
        return fail(CORR_ERR_ARG, "samples, station_stride and frame_stride must be 16-byte aligned");
    // bytes a bin takes between the engines: FP16 pairs, or 8-byte FP32 / hi-lo pairs
    const size_t bin_bytes = spectra_format(xmode) == kSpectraF16 ? 4 : 8;
    const size_t per_frame = static_cast<size_t>(n_station) * n_freq * bin_bytes;
    const int max_frames = static_cast<int>(kNoAllocScratchBytes / per_frame);
    if (frames > max_frames)
        return failf(CORR_ERR_ARG,
                     "frames=%d exceeds the %d frames the fixed %zu-byte scratch holds at "
                     "n_station=%d, n_freq=%d, X-engine mode %d; split the call",
                     frames, max_frames, kNoAllocScratchBytes, n_station, n_freq, xmode);
    if (frames == 0) return CORR_OK;

    int dev = 0;
    if ((st = cuda_check(cudaGetDevice(&dev), "cudaGetDevice")) != CORR_OK) return st;
    DeviceScratch d;
    if ((st = scratch_for(dev, &d)) != CORR_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    int size_index = 0;
    while (size_index < kNumSizes && kSizes[size_index] != n_freq) ++size_index;
    if (size_index == kNumSizes)
        return failf(CORR_ERR_INTERNAL, "no twiddle tables for n_freq=%d", n_freq);
    TwiddleTables tw;
    twiddle_views(d.twiddles + twiddle_offset(size_index), n_freq, &tw);

    FengineArgs fa{};
    fa.samples = d_samples;
    fa.station_stride = station_stride;
    fa.frame_stride = frame_stride;
    fa.mask = d_mask;
    fa.mask_station_stride = mask_station_stride;
    fa.mask_bit0 = mask_bit0;
    fa.n_station = n_station;
    fa.frames = frames;
    fa.y = d.spectra;
    fa.y_frames = frames;
    fa.ytile = n_freq;
    fa.y_fmt = spectra_format(xmode);
    fa.fplan = 0;
    fa.y_scale = spectra_scale(n_freq);
    fa.err = nullptr;
    if ((st = fengine_launch(n_freq, tw, fa, d.num_sms, s)) != CORR_OK) return st;

    XengineArgs xa{};
    xa.y = d.spectra;
    xa.y_frames = frames;
    xa.ytile = n_freq;
    xa.y_fmt = spectra_format(xmode);
    xa.n_station = n_station;
    xa.n_freq = n_freq;
    xa.frames = frames;
    xa.acc = d_acc;
    xa.acc64 = 0;
    xa.err = nullptr;
    if (xmode == CORR_X_PLAIN_FP32) return xengine_plain_launch(xa, d.num_sms, s);
    int ct = 0, kt = 0;
    xengine_tc_default_shape(n_station, xmode == CORR_X_TC_FP16_SPLIT, &ct, &kt);
    return xengine_tc_launch(xa, xmode == CORR_X_TC_FP16_SPLIT, ct, kt, d.num_sms, s);
}
