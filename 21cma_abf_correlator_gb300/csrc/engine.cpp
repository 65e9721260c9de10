// engine.cpp -- FX plan: device buffers + the F/X launch sequence, and the
// device-resident extension entry points declared in corr_gb300.h.
//
// One pass of the plan over `ft` frames is two launches on the caller's stream:
//   F-engine: ft*n_station int8 frames -> spectra y   (fengine.cu)
//   X-engine: spectra y -> acc += visibilities        (xengine.cu / xengine_tc.cu)
// The spectra buffer is sized for max_frames frames; longer requests are split
// into passes. This is the work the reference does per chunk in gpu_accumulate
// (corr-cuda/src/kernels.cu:806-845), minus the host copies, which belong to the
// caller (abi.cpp for the staging ring).

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "engine.h"

namespace corrgb {

std::string &last_error() {
    static thread_local std::string s;
    return s;
}

corr_status fail(corr_status st, const std::string &msg) {
    last_error() = msg;
    return st;
}

corr_status failf(corr_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    last_error() = buf;
    return st;
}

corr_status cuda_check(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return CORR_OK;
    cudaGetLastError();   // a failed call must not surface again at the next launch check
    return fail(CORR_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorName(e) + ": " + cudaGetErrorString(e));
}

corr_status PerDevice::fail_current() {
    return fail(CORR_ERR_CUDA, "cudaGetDevice failed: no current device");
}

corr_status PerDevice::fail_ordinal(int dev) {
    return failf(CORR_ERR_ARG, "device ordinal %d: at most %d devices are supported", dev,
                 kMaxDeviceOrdinals);
}

static bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

corr_status check_geometry(int n_station, int n_freq) {
    if (n_station < 1) return fail(CORR_ERR_ARG, "n_station must be >= 1");
    if (n_station > kMaxStations)
        return failf(CORR_ERR_ARG, "n_station=%d: an engine correlates at most %d stations",
                     n_station, kMaxStations);
    if (n_freq < 1) return fail(CORR_ERR_ARG, "n_freq must be >= 1");
    // Powers of two from 512, and the reference's multiples of 2048 (frames of
    // whole 4096-sample packets), up to 32768: the F-engine's transform lengths.
    const bool pow2 = is_pow2(n_freq) && n_freq >= 512;
    if ((!pow2 && n_freq % 2048 != 0) || n_freq > 32768) {
        if (n_freq % 2048 == 0)
            return failf(CORR_ERR_NOT_IMPL,
                         "n_freq=%d: frames longer than 65536 samples (n_freq above 32768) "
                         "are not supported",
                         n_freq);
        return failf(CORR_ERR_ARG,
                     "n_freq=%d is neither a multiple of 2048 nor a power of two in [512, 32768]",
                     n_freq);
    }
    return CORR_OK;
}

corr_status fxplan_create(int device, int n_station, int n_freq, int max_frames, int xmode,
                          FxPlan **out) {
    if (out == nullptr) return fail(CORR_ERR_ARG, "fxplan_create: out is NULL");
    *out = nullptr;
    corr_status st = check_geometry(n_station, n_freq);
    if (st != CORR_OK) return st;
    if (max_frames < 1) return fail(CORR_ERR_ARG, "max_frames must be >= 1");
    if (static_cast<uint64_t>(max_frames) * n_station * n_freq >= (uint64_t(1) << 32))
        return failf(CORR_ERR_ARG,
                     "max_frames=%d: the spectra buffer would hold 2^32 or more values",
                     max_frames);
    if (xmode != CORR_X_PLAIN_FP32 && xmode != CORR_X_TC_FP16 && xmode != CORR_X_TC_FP16_SPLIT)
        return failf(CORR_ERR_ARG, "unknown X-engine mode %d", xmode);
    if ((st = cuda_check(cudaSetDevice(device), "cudaSetDevice")) != CORR_OK) return st;

    FxPlan *p = new (std::nothrow) FxPlan();
    if (p == nullptr) return fail(CORR_ERR_NOMEM, "fxplan_create: out of host memory");
    p->device = device;
    p->n_station = n_station;
    p->n_freq = n_freq;
    p->n_baseline = n_station * (n_station + 1) / 2;
    p->max_frames = max_frames;
    p->ytile = n_freq;
    p->xmode = xmode;
    if (xmode != CORR_X_PLAIN_FP32) {
        xengine_tc_default_shape(n_station, xmode == CORR_X_TC_FP16_SPLIT, &p->xct, &p->xkt);
        if (p->xct == 0) {
            delete p;
            return failf(CORR_ERR_NOT_IMPL, "the tensor X-engine takes 1..64 inputs (n_station=%d)",
                         n_station);
        }
    }
    if ((st = cuda_check(cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount,
                                                device),
                         "cudaDeviceGetAttribute(SM count)")) != CORR_OK) {
        delete p;
        return st;
    }
    const size_t y_bytes = static_cast<size_t>(max_frames) * n_station * n_freq * sizeof(float2);
    if (cudaMalloc(&p->d_y, y_bytes) != cudaSuccess) {
        cudaGetLastError();
        delete p;
        return failf(CORR_ERR_NOMEM, "cudaMalloc(spectra, %zu bytes) failed", y_bytes);
    }
    if ((st = cuda_check(cudaMalloc(&p->d_err, sizeof(int)), "cudaMalloc(watchdog)")) !=
            CORR_OK ||
        (st = cuda_check(cudaMemset(p->d_err, 0, sizeof(int)), "cudaMemset(watchdog)")) !=
            CORR_OK ||
        (st = fengine_prepare(n_freq, &p->tw)) != CORR_OK) {
        fxplan_destroy(p);
        return st;
    }
    *out = p;
    return CORR_OK;
}

void fxplan_destroy(FxPlan *p) {
    if (p == nullptr) return;
    cudaSetDevice(p->device);
    fengine_release(&p->tw);
    if (p->d_y) cudaFree(p->d_y);
    if (p->d_err) cudaFree(p->d_err);
    if (p->d_xpair_list) cudaFree(p->d_xpair_list);
    delete p;
}

corr_status fxplan_accumulate(FxPlan *p, const int8_t *samples, size_t station_stride,
                              size_t frame_stride, const uint8_t *mask,
                              size_t mask_station_stride, int mask_bit0, int frames,
                              void *acc, cudaStream_t stream, const uint32_t *pmask,
                              size_t pmask_station_stride, int pmask_frame0) {
    if (frames < 0) return fail(CORR_ERR_ARG, "frames must be >= 0");
    const size_t frame_bytes = 2u * static_cast<size_t>(p->n_freq);
    if (frame_stride < frame_bytes)
        return fail(CORR_ERR_ARG, "frame_stride is shorter than a frame");
    if ((reinterpret_cast<uintptr_t>(samples) | station_stride | frame_stride) % 16 != 0)
        return fail(CORR_ERR_ARG,
                    "samples, station_stride and frame_stride must be 16-byte aligned "
                    "(the F-engine loads frames with TMA bulk copies)");
    for (int f0 = 0; f0 < frames; f0 += p->max_frames) {
        const int ft = frames - f0 < p->max_frames ? frames - f0 : p->max_frames;
        FengineArgs fa{};
        fa.samples = samples + static_cast<size_t>(f0) * frame_stride;
        fa.station_stride = station_stride;
        fa.frame_stride = frame_stride;
        fa.mask = mask;
        fa.mask_station_stride = mask_station_stride;
        fa.mask_bit0 = mask_bit0 + f0;
        fa.pmask = pmask;
        fa.pmask_station_stride = pmask_station_stride;
        fa.pmask_frame0 = pmask_frame0 + f0;
        fa.n_station = p->n_station;
        fa.frames = ft;
        fa.y = p->d_y;
        fa.y_frames = p->max_frames;
        fa.ytile = p->ytile;
        fa.y_fmt = spectra_format(p->xmode);
        fa.fplan = p->fplan;
        fa.y_scale = spectra_scale(p->n_freq);
        fa.err = p->d_err;
        corr_status st = fengine_launch(p->n_freq, p->tw, fa, p->num_sms, stream);
        if (st != CORR_OK) return st;
        XengineArgs xa{};
        xa.y = p->d_y;
        xa.y_frames = p->max_frames;
        xa.ytile = p->ytile;
        xa.y_fmt = spectra_format(p->xmode);
        xa.n_station = p->n_station;
        xa.n_freq = p->n_freq;
        xa.frames = ft;
        xa.acc = acc;
        xa.acc64 = p->acc64;
        xa.err = p->d_err;
        xa.pair_first = p->xpair_first;
        xa.pair_count = p->xpair_count;
        xa.pair_list = p->d_xpair_list;
        if (p->xmode == CORR_X_PLAIN_FP32)
            st = xengine_plain_launch(xa, p->num_sms, stream);
        else
            st = xengine_tc_launch(xa, p->xmode == CORR_X_TC_FP16_SPLIT, p->xct, p->xkt,
                                   p->num_sms, stream);
        if (st != CORR_OK) return st;
    }
    return CORR_OK;
}

corr_status fxplan_check(FxPlan *p) {
    corr_status st = cuda_check(cudaSetDevice(p->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    if ((st = cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize")) != CORR_OK) return st;
    int code = 0;
    if ((st = cuda_check(cudaMemcpy(&code, p->d_err, sizeof(int), cudaMemcpyDeviceToHost),
                         "cudaMemcpy(watchdog)")) != CORR_OK)
        return st;
    if (code != kErrNone) {
        cudaMemset(p->d_err, 0, sizeof(int));
        return failf(CORR_ERR_INTERNAL,
                     "device watchdog tripped (code %d): a bounded wait inside a kernel ran "
                     "out and the kernel returned early; results of that launch are invalid",
                     code);
    }
    return CORR_OK;
}

} // namespace corrgb

using namespace corrgb;

extern "C" corr_status corrx_create(const corrx_params *prm, void **out_eng) {
    if (out_eng == nullptr) return fail(CORR_ERR_ARG, "out_eng is NULL");
    *out_eng = nullptr;
    if (prm == nullptr) return fail(CORR_ERR_ARG, "params is NULL");
    if (prm->struct_size != sizeof(corrx_params))
        return failf(CORR_ERR_ABI, "corrx_params.struct_size=%u, expected %zu", prm->struct_size,
                     sizeof(corrx_params));
    int ndev = 0;
    corr_status st = cuda_check(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
    if (st != CORR_OK) return st;
    if (prm->device_id < 0 || prm->device_id >= ndev)
        return failf(CORR_ERR_ARG, "device_id=%d but %d device(s) are visible", prm->device_id,
                     ndev);
    FxPlan *p = nullptr;
    st = fxplan_create(prm->device_id, prm->n_station, prm->n_freq, prm->max_frames, prm->xmode,
                       &p);
    if (st != CORR_OK) return st;
    *out_eng = p;
    return CORR_OK;
}

extern "C" corr_status corrx_destroy(void *eng) {
    fxplan_destroy(static_cast<FxPlan *>(eng));
    return CORR_OK;
}

extern "C" corr_status corrx_accumulate(void *eng, const int8_t *d_samples,
                                        size_t station_stride, size_t frame_stride,
                                        const uint8_t *d_mask, size_t mask_station_stride,
                                        int32_t mask_bit0, int32_t frames, void *d_acc,
                                        void *stream) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr) return fail(CORR_ERR_ARG, "eng is NULL");
    if (d_samples == nullptr || d_acc == nullptr)
        return fail(CORR_ERR_ARG, "d_samples and d_acc must not be NULL");
    if (mask_bit0 < 0) return fail(CORR_ERR_ARG, "mask_bit0 must be >= 0");
    corr_status st = cuda_check(cudaSetDevice(p->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    return fxplan_accumulate(p, d_samples, station_stride, frame_stride, d_mask,
                             mask_station_stride, mask_bit0, frames, d_acc,
                             static_cast<cudaStream_t>(stream));
}

extern "C" corr_status corrx_accumulate_packets(void *eng, const int8_t *d_samples,
                                                size_t station_stride, size_t frame_stride,
                                                const uint8_t *d_mask, size_t mask_station_stride,
                                                int32_t mask_bit0, const uint32_t *d_pmask,
                                                size_t pmask_station_stride,
                                                int32_t pmask_frame0, int32_t frames,
                                                void *d_acc, void *stream) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr) return fail(CORR_ERR_ARG, "eng is NULL");
    if (d_samples == nullptr || d_acc == nullptr || d_pmask == nullptr)
        return fail(CORR_ERR_ARG, "d_samples, d_pmask and d_acc must not be NULL");
    if (mask_bit0 < 0 || pmask_frame0 < 0)
        return fail(CORR_ERR_ARG, "mask_bit0 and pmask_frame0 must be >= 0");
    if (reinterpret_cast<uintptr_t>(d_pmask) % alignof(uint32_t) != 0)
        return fail(CORR_ERR_ARG, "d_pmask must be 4-byte aligned");
    if (2 * p->n_freq > 32 * 1024)
        return fail(CORR_ERR_ARG, "packet masks hold 32 packets of 1024 samples per frame");
    corr_status st = cuda_check(cudaSetDevice(p->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    return fxplan_accumulate(p, d_samples, station_stride, frame_stride, d_mask,
                             mask_station_stride, mask_bit0, frames, d_acc,
                             static_cast<cudaStream_t>(stream), d_pmask, pmask_station_stride,
                             pmask_frame0);
}

extern "C" corr_status corrx_scale(void *eng, void *d_acc, uint64_t frames, void *stream) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr) return fail(CORR_ERR_ARG, "eng is NULL");
    if (frames == 0) return fail(CORR_ERR_ARG, "frames must be > 0");
    corr_status st = cuda_check(cudaSetDevice(p->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    const size_t n = static_cast<size_t>(p->n_baseline) * p->n_freq;
    if (p->acc64)
        return scale64_launch(static_cast<double2 *>(d_acc), n,
                              1.0 / static_cast<double>(frames), static_cast<cudaStream_t>(stream));
    return scale_launch(static_cast<float2 *>(d_acc), n, 1.0f / static_cast<float>(frames),
                        static_cast<cudaStream_t>(stream));
}

extern "C" corr_status corrx_set_accumulator(void *eng, int32_t precision) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr) return fail(CORR_ERR_ARG, "eng is NULL");
    if (precision != CORRX_ACC_FP32 && precision != CORRX_ACC_FP64)
        return failf(CORR_ERR_ARG, "unknown accumulator precision %d", precision);
    p->acc64 = precision == CORRX_ACC_FP64 ? 1 : 0;
    return CORR_OK;
}

extern "C" corr_status corrx_dump(void *eng, const void *d_acc, uint64_t frames, void *d_out,
                                  void *stream) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr) return fail(CORR_ERR_ARG, "eng is NULL");
    if (d_acc == nullptr || d_out == nullptr) return fail(CORR_ERR_ARG, "d_acc and d_out must be non-NULL");
    if (frames == 0) return fail(CORR_ERR_ARG, "frames must be > 0");
    if ((reinterpret_cast<uintptr_t>(d_acc) | reinterpret_cast<uintptr_t>(d_out)) % 16 != 0)
        return fail(CORR_ERR_ARG, "d_acc and d_out must be 16-byte aligned");
    corr_status st = cuda_check(cudaSetDevice(p->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    const size_t n = static_cast<size_t>(p->n_baseline) * p->n_freq;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (p->acc64)
        return dump64_launch(static_cast<float2 *>(d_out), n, static_cast<const double2 *>(d_acc),
                             n, nullptr, nullptr, p->n_baseline, p->n_freq, 1,
                             1.0 / static_cast<double>(frames), s);
    if (d_out != d_acc &&
        (st = cuda_check(cudaMemcpyAsync(d_out, d_acc, n * sizeof(float2),
                                         cudaMemcpyDeviceToDevice, s),
                         "cudaMemcpyAsync(dump)")) != CORR_OK)
        return st;
    return scale_launch(static_cast<float2 *>(d_out), n, 1.0f / static_cast<float>(frames), s);
}

extern "C" corr_status corrx_run_fengine(void *eng, const int8_t *d_samples,
                                         size_t station_stride, size_t frame_stride,
                                         const uint8_t *d_mask, size_t mask_station_stride,
                                         int32_t mask_bit0, int32_t frames, void *stream) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr) return fail(CORR_ERR_ARG, "eng is NULL");
    if (d_samples == nullptr) return fail(CORR_ERR_ARG, "d_samples is NULL");
    if (frames < 0 || frames > p->max_frames)
        return failf(CORR_ERR_ARG, "frames=%d outside [0, max_frames=%d]", frames, p->max_frames);
    if ((reinterpret_cast<uintptr_t>(d_samples) | station_stride | frame_stride) % 16 != 0)
        return fail(CORR_ERR_ARG, "samples and strides must be 16-byte aligned");
    corr_status st = cuda_check(cudaSetDevice(p->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    FengineArgs fa{};
    fa.samples = d_samples;
    fa.station_stride = station_stride;
    fa.frame_stride = frame_stride;
    fa.mask = d_mask;
    fa.mask_station_stride = mask_station_stride;
    fa.mask_bit0 = mask_bit0;
    fa.n_station = p->n_station;
    fa.frames = frames;
    fa.y = p->d_y;
    fa.y_frames = p->max_frames;
    fa.ytile = p->ytile;
    fa.y_fmt = spectra_format(p->xmode);
    fa.fplan = p->fplan;
    fa.y_scale = spectra_scale(p->n_freq);
    fa.err = p->d_err;
    return fengine_launch(p->n_freq, p->tw, fa, p->num_sms, static_cast<cudaStream_t>(stream));
}

extern "C" corr_status corrx_run_xengine(void *eng, int32_t frames, void *d_acc, void *stream) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr) return fail(CORR_ERR_ARG, "eng is NULL");
    if (d_acc == nullptr) return fail(CORR_ERR_ARG, "d_acc is NULL");
    if (frames < 0 || frames > p->max_frames)
        return failf(CORR_ERR_ARG, "frames=%d outside [0, max_frames=%d]", frames, p->max_frames);
    corr_status st = cuda_check(cudaSetDevice(p->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    XengineArgs xa{};
    xa.y = p->d_y;
    xa.y_frames = p->max_frames;
    xa.ytile = p->ytile;
    xa.y_fmt = spectra_format(p->xmode);
    xa.n_station = p->n_station;
    xa.n_freq = p->n_freq;
    xa.frames = frames;
    xa.acc = d_acc;
    xa.acc64 = p->acc64;
    xa.err = p->d_err;
    xa.pair_first = p->xpair_first;
    xa.pair_count = p->xpair_count;
    xa.pair_list = p->d_xpair_list;
    if (p->xmode == CORR_X_PLAIN_FP32)
        return xengine_plain_launch(xa, p->num_sms, static_cast<cudaStream_t>(stream));
    return xengine_tc_launch(xa, p->xmode == CORR_X_TC_FP16_SPLIT, p->xct, p->xkt, p->num_sms,
                             static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------------------
// Tile shapes and the autotuner.
// ---------------------------------------------------------------------------

namespace corrgb {

corr_status fxplan_limit_baselines(FxPlan *p, const std::vector<int32_t> &baselines) {
    p->xpair_first = p->xpair_count = 0;
    if (p->d_xpair_list != nullptr) {
        cudaSetDevice(p->device);
        cudaFree(p->d_xpair_list);
        p->d_xpair_list = nullptr;
    }
    const int n = p->n_station, nb = n * (n + 1) / 2;
    if (baselines.empty() || static_cast<int>(baselines.size()) == nb) return CORR_OK;
    // the block pair of each baseline (row-major over j <= k), in order, once
    std::vector<int> row_start(static_cast<size_t>(n) + 1, 0);
    for (int j = 0; j < n; ++j) row_start[static_cast<size_t>(j) + 1] = row_start[j] + (n - j);
    std::vector<int32_t> pairs;
    for (int32_t g : baselines) {
        if (g < 0 || g >= nb) return failf(CORR_ERR_INTERNAL, "baseline %d outside the row", g);
        const int j = static_cast<int>(std::upper_bound(row_start.begin(), row_start.end(), g) -
                                       row_start.begin()) - 1;
        const int k = j + (g - row_start[static_cast<size_t>(j)]);
        pairs.push_back(xengine_plain_block_pair(n, j, k));
    }
    std::sort(pairs.begin(), pairs.end());
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
    const int count = static_cast<int>(pairs.size());
    if (pairs.back() - pairs.front() + 1 == count) {   // a contiguous run: first and count
        p->xpair_first = pairs.front();
        p->xpair_count = count;
        return CORR_OK;
    }
    corr_status st = cuda_check(cudaSetDevice(p->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    const size_t bytes = pairs.size() * sizeof(int32_t);
    if ((st = cuda_check(cudaMalloc(&p->d_xpair_list, bytes), "cudaMalloc(block pairs)")) !=
            CORR_OK ||
        (st = cuda_check(cudaMemcpy(p->d_xpair_list, pairs.data(), bytes, cudaMemcpyHostToDevice),
                         "cudaMemcpy(block pairs)")) != CORR_OK)
        return st;
    p->xpair_count = count;
    return CORR_OK;
}

corr_status fxplan_set_tiles(FxPlan *p, int ytile, int xct, int xkt, int fplan) {
    if (fplan < 0 || fplan >= fengine_plans(p->n_freq))
        return failf(CORR_ERR_ARG, "FFT plan %d: n_freq=%d has plans 0..%d", fplan, p->n_freq,
                     fengine_plans(p->n_freq) - 1);
    if (!fengine_plan_ok(p->n_freq, fplan, spectra_format(p->xmode)))
        return failf(CORR_ERR_ARG, "FFT plan %d does not write the spectra of X-engine mode %d",
                     fplan, p->xmode);
    if (ytile != p->n_freq &&
        (ytile < 2 || (ytile & (ytile - 1)) != 0 || p->n_freq % ytile != 0))
        return failf(CORR_ERR_ARG,
                     "ytile=%d is neither n_freq=%d nor a power of two >= 2 dividing it", ytile,
                     p->n_freq);
    if (p->xmode != CORR_X_PLAIN_FP32) {
        if (!xengine_tc_shape_ok(p->n_station, p->xmode == CORR_X_TC_FP16_SPLIT, xct, xkt))
            return failf(CORR_ERR_ARG,
                         "no tensor X-engine tile of %d channels x %d frames for %d inputs", xct,
                         xkt, p->n_station);
        // The tensor forms read either contiguous rows (a TMA tile per stage)
        // or tiles of exactly their own width, where a stage is one contiguous
        // block (a single bulk copy per stage).
        if (ytile != p->n_freq && ytile != xct)
            return failf(CORR_ERR_ARG,
                         "the tensor X-engines read contiguous rows (ytile = n_freq = %d) or "
                         "tiles of their own width (ytile = xct = %d), not ytile = %d",
                         p->n_freq, xct, ytile);
        p->xct = xct;
        p->xkt = xkt;
    }
    p->ytile = ytile;
    p->fplan = fplan;
    return CORR_OK;
}

corr_status fxplan_autotune(FxPlan *p, cudaStream_t stream, corrx_tiles *out) {
    corr_status st = cuda_check(cudaSetDevice(p->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    struct Cand {
        int ytile, ct, kt;
    };
    std::vector<Cand> cands;
    if (p->xmode == CORR_X_PLAIN_FP32) {
        cands.push_back({p->n_freq, p->xct, p->xkt});
    } else {
        const bool split = p->xmode == CORR_X_TC_FP16_SPLIT;
        for (int ct = 8; ct >= 2; ct /= 2)
            for (int kt = 16; kt <= 64; kt *= 2)
                if (xengine_tc_shape_ok(p->n_station, split, ct, kt)) {
                    cands.push_back({p->n_freq, ct, kt});
                    if (ct < p->n_freq) cands.push_back({ct, ct, kt});
                }
    }
    if (cands.empty()) return fail(CORR_ERR_INTERNAL, "autotune: no candidate tile");
    const int frames = std::min(p->max_frames, 1024);
    const int L = 2 * p->n_freq;
    const size_t x_bytes = static_cast<size_t>(p->n_station) * frames * L;
    // room for a complex128 row, whichever accumulator the engine uses
    const size_t acc_bytes = static_cast<size_t>(p->n_baseline) * p->n_freq * sizeof(double2);
    int8_t *d_x = nullptr;
    void *d_acc = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const int ytile0 = p->ytile, ct0 = p->xct, kt0 = p->xkt;
    auto cleanup = [&] {
        if (d_x) cudaFree(d_x);
        if (d_acc) cudaFree(d_acc);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    if ((st = cuda_check(cudaMalloc(&d_x, x_bytes), "cudaMalloc(autotune frames)")) != CORR_OK ||
        (st = cuda_check(cudaMalloc(&d_acc, acc_bytes), "cudaMalloc(autotune row)")) != CORR_OK ||
        (st = cuda_check(cudaEventCreate(&e0), "cudaEventCreate")) != CORR_OK ||
        (st = cuda_check(cudaEventCreate(&e1), "cudaEventCreate")) != CORR_OK ||
        (st = synth_fill_launch(d_x, x_bytes, 0x2c1bu, stream)) != CORR_OK ||
        (st = cuda_check(cudaMemsetAsync(d_acc, 0, acc_bytes, stream), "cudaMemsetAsync")) !=
            CORR_OK) {
        cleanup();
        return st;
    }
    // time one launch of `run` (after one untimed launch): best of two
    auto timed = [&](auto &&run, float *ms) -> corr_status {
        corr_status s2 = run();
        float best = 1e30f;
        for (int r = 0; r < 2 && s2 == CORR_OK; ++r) {
            if ((s2 = cuda_check(cudaEventRecord(e0, stream), "cudaEventRecord")) != CORR_OK) break;
            if ((s2 = run()) != CORR_OK) break;
            if ((s2 = cuda_check(cudaEventRecord(e1, stream), "cudaEventRecord")) != CORR_OK) break;
            if ((s2 = cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize")) != CORR_OK) break;
            float t = 0.f;
            if ((s2 = cuda_check(cudaEventElapsedTime(&t, e0, e1), "cudaEventElapsedTime")) !=
                CORR_OK)
                break;
            best = std::min(best, t);
        }
        *ms = best;
        return s2;
    };
    auto run_f = [&] {
        return corrx_run_fengine(p, d_x, static_cast<size_t>(frames) * L, L, nullptr, 0, 0, frames,
                                 stream);
    };
    auto run_x = [&] { return corrx_run_xengine(p, frames, d_acc, stream); };
    // The F-engine's time depends on the FFT plan and the spectra layout, the
    // X-engine's on the layout and the tile. The plan is chosen on contiguous
    // rows; then every (layout, tile) is timed, the F-engine once per layout,
    // and the pair with the smallest F + X time wins.
    const int fplan0 = p->fplan;
    const int n_fplans = fengine_plans(p->n_freq);
    float best_f = 1e30f, best_x = 1e30f, best_sum = 1e30f;
    int best_fplan = fplan0;
    Cand best{ytile0, ct0, kt0};
    for (int fp = 0; fp < n_fplans && st == CORR_OK; ++fp) {
        if (!fengine_plan_ok(p->n_freq, fp, spectra_format(p->xmode))) continue;
        // Plan 2 rounds the data to FP16 between its DFT stages, which raises the
        // FP16 path's error by about half; it is chosen explicitly (corrx_set_tiles),
        // never by the autotuner, so an autotuned engine keeps plan 0/1 numerics.
        if (fp == 2) continue;
        if ((st = fxplan_set_tiles(p, p->n_freq, cands[0].ct, cands[0].kt, fp)) != CORR_OK) break;
        float f_ms = 0.f;
        if ((st = timed(run_f, &f_ms)) != CORR_OK) break;
        if (f_ms < best_f) {
            best_f = f_ms;
            best_fplan = fp;
        }
    }
    std::vector<std::pair<int, float>> f_by_layout;   // ytile -> F-engine ms
    for (const Cand &c : cands) {
        if (st != CORR_OK) break;
        if (fxplan_set_tiles(p, c.ytile, c.ct, c.kt, best_fplan) != CORR_OK)
            continue;   // not for this form
        float f_ms = -1.f;
        for (const auto &e : f_by_layout)
            if (e.first == c.ytile) f_ms = e.second;
        if (f_ms < 0.f) {
            if ((st = timed(run_f, &f_ms)) != CORR_OK) break;
            f_by_layout.emplace_back(c.ytile, f_ms);
        } else if ((st = run_f()) != CORR_OK) {   // the spectra this layout holds
            break;
        }
        float x_ms = 0.f;
        if ((st = timed(run_x, &x_ms)) != CORR_OK) break;
        if (f_ms + x_ms < best_sum) {
            best_sum = f_ms + x_ms;
            best_f = f_ms;
            best_x = x_ms;
            best = c;
        }
    }
    corr_status st_check = st == CORR_OK ? fxplan_check(p) : st;
    cleanup();
    if (st_check != CORR_OK) {
        fxplan_set_tiles(p, ytile0, ct0, kt0, fplan0);
        return st_check;
    }
    if ((st = fxplan_set_tiles(p, best.ytile, best.ct, best.kt, best_fplan)) != CORR_OK) return st;
    if (out != nullptr) {
        out->ytile = p->ytile;
        out->xct = p->xct;
        out->xkt = p->xkt;
        out->fplan = p->fplan;
        out->ms_fengine = best_f;
        out->ms_xengine = best_x;
    }
    return CORR_OK;
}

} // namespace corrgb

extern "C" corr_status corrx_get_tiles(void *eng, corrx_tiles *out) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr || out == nullptr) return fail(CORR_ERR_ARG, "eng and out must be non-NULL");
    if (out->struct_size != sizeof(corrx_tiles))
        return failf(CORR_ERR_ABI, "corrx_tiles.struct_size=%u, expected %zu", out->struct_size,
                     sizeof(corrx_tiles));
    out->ytile = p->ytile;
    out->xct = p->xct;
    out->xkt = p->xkt;
    out->fplan = p->fplan;
    out->ms_fengine = 0.f;
    out->ms_xengine = 0.f;
    return CORR_OK;
}

extern "C" corr_status corrx_set_tiles(void *eng, const corrx_tiles *t) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr || t == nullptr) return fail(CORR_ERR_ARG, "eng and t must be non-NULL");
    if (t->struct_size != sizeof(corrx_tiles))
        return failf(CORR_ERR_ABI, "corrx_tiles.struct_size=%u, expected %zu", t->struct_size,
                     sizeof(corrx_tiles));
    return fxplan_set_tiles(p, t->ytile, t->xct, t->xkt, t->fplan);
}

extern "C" corr_status corrx_autotune(void *eng, void *stream, corrx_tiles *out) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr) return fail(CORR_ERR_ARG, "eng is NULL");
    if (out != nullptr && out->struct_size != sizeof(corrx_tiles))
        return failf(CORR_ERR_ABI, "corrx_tiles.struct_size=%u, expected %zu", out->struct_size,
                     sizeof(corrx_tiles));
    return fxplan_autotune(p, static_cast<cudaStream_t>(stream), out);
}

extern "C" corr_status corrx_selftest_watchdog(void *eng, int64_t budget_cycles, void *stream) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr) return fail(CORR_ERR_ARG, "eng is NULL");
    if (budget_cycles < 1 || budget_cycles > 4000000000LL)
        return fail(CORR_ERR_ARG, "budget_cycles must be in [1, 4e9]");
    corr_status st = cuda_check(cudaSetDevice(p->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    return watchdog_selftest_launch(p->d_err, budget_cycles, static_cast<cudaStream_t>(stream));
}

extern "C" corr_status corrx_check(void *eng) {
    FxPlan *p = static_cast<FxPlan *>(eng);
    if (p == nullptr) return fail(CORR_ERR_ARG, "eng is NULL");
    return fxplan_check(p);
}

// ---------------------------------------------------------------------------
// Batched integration blocks captured in one CUDA graph.
// ---------------------------------------------------------------------------

namespace corrgb {
namespace {

struct FxBatch {
    FxPlan *plan = nullptr;
    int n_blocks = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaEvent_t> ev_fork;
    unsigned long long *d_stamps = nullptr;   // [block][start, row in host memory], ns
    double2 *d_acc64 = nullptr;   // complex128 accumulator of the block in flight (FP64 engines)
    cudaStream_t cap = nullptr, side = nullptr;
    cudaStream_t last_launch = nullptr;
};

void batch_free(FxBatch *b) {
    if (b == nullptr) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (cudaEvent_t e : b->ev_fork)
        if (e) cudaEventDestroy(e);
    if (b->d_stamps) cudaFree(b->d_stamps);
    if (b->d_acc64) cudaFree(b->d_acc64);
    if (b->cap) cudaStreamDestroy(b->cap);
    if (b->side) cudaStreamDestroy(b->side);
    delete b;
}

} // namespace
} // namespace corrgb

namespace corrgb {
namespace {

// Capture every block into one graph; block i runs on plans[block_engine[i]]
// (block_engine NULL: all on plans[0]).
// d_pmask (nullable): packet words, frame f of station s at
// d_pmask[s*pmask_station_stride + f], f counted like block_first.
corr_status batch_create(const std::vector<FxPlan *> &plans, const int32_t *block_engine,
                         const int8_t *d_samples, size_t station_stride, size_t frame_stride,
                         const uint8_t *d_mask, size_t mask_station_stride,
                         const uint32_t *d_pmask, size_t pmask_station_stride,
                         const int64_t *block_first, const int32_t *block_frames,
                         int32_t n_blocks, void *d_rows, void *h_rows, void **out_batch) {
    if (out_batch == nullptr) return fail(CORR_ERR_ARG, "out_batch is NULL");
    *out_batch = nullptr;
    if (plans.empty()) return fail(CORR_ERR_ARG, "no engine");
    for (FxPlan *q : plans)
        if (q == nullptr) return fail(CORR_ERR_ARG, "an engine is NULL");
    FxPlan *p = plans[0];
    for (FxPlan *q : plans)
        if (q->device != p->device || q->n_station != p->n_station || q->n_freq != p->n_freq ||
            q->acc64 != p->acc64)
            return fail(CORR_ERR_ARG,
                        "the engines of one batch must share device, n_station, n_freq and "
                        "accumulator precision");
    if (d_samples == nullptr || d_rows == nullptr || block_first == nullptr ||
        block_frames == nullptr)
        return fail(CORR_ERR_ARG, "d_samples, d_rows and the block arrays must be non-NULL");
    if (n_blocks < 1) return fail(CORR_ERR_ARG, "n_blocks must be >= 1");
    if (d_pmask != nullptr && reinterpret_cast<uintptr_t>(d_pmask) % alignof(uint32_t) != 0)
        return fail(CORR_ERR_ARG, "d_pmask must be 4-byte aligned");
    if (d_pmask != nullptr && 2 * p->n_freq > 32 * 1024)
        return fail(CORR_ERR_ARG, "packet masks hold 32 packets of 1024 samples per frame");
    const int n_plans = static_cast<int>(plans.size());
    for (int i = 0; i < n_blocks; ++i) {
        if (block_frames[i] < 1 || block_first[i] < 0)
            return failf(CORR_ERR_ARG, "block %d: first=%lld frames=%d", i,
                         (long long)block_first[i], block_frames[i]);
        if (block_engine != nullptr && (block_engine[i] < 0 || block_engine[i] >= n_plans))
            return failf(CORR_ERR_ARG, "block %d: engine %d of %d", i, block_engine[i], n_plans);
    }
    auto plan_of = [&](int i) { return plans[block_engine ? block_engine[i] : 0]; };
    corr_status st = cuda_check(cudaSetDevice(p->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    FxBatch *b = new (std::nothrow) FxBatch();
    if (b == nullptr) return fail(CORR_ERR_NOMEM, "cannot allocate the batch");
    b->plan = p;
    b->n_blocks = n_blocks;
    const size_t row_elems = static_cast<size_t>(p->n_baseline) * p->n_freq;
    float2 *rows = static_cast<float2 *>(d_rows);
    if ((st = cuda_check(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking),
                         "cudaStreamCreate(capture)")) != CORR_OK ||
        (st = cuda_check(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking),
                         "cudaStreamCreate(side)")) != CORR_OK) {
        batch_free(b);
        return st;
    }
    b->ev_fork.assign(n_blocks + 1, nullptr);
    st = cuda_check(cudaMalloc(&b->d_stamps, 2 * sizeof(unsigned long long) * n_blocks),
                    "cudaMalloc(stamps)");
    if (st == CORR_OK)
        st = cuda_check(cudaMemset(b->d_stamps, 0, 2 * sizeof(unsigned long long) * n_blocks),
                        "cudaMemset(stamps)");
    for (int i = 0; i <= n_blocks && st == CORR_OK; ++i)
        st = cuda_check(cudaEventCreateWithFlags(&b->ev_fork[i], cudaEventDisableTiming),
                        "cudaEventCreate");
    // FP64 engines accumulate each block in one complex128 row, reused block
    // after block (the blocks run in order on the capture stream), and dump it
    // scaled into the block's complex64 row.
    if (st == CORR_OK && p->acc64)
        st = cuda_check(cudaMalloc(&b->d_acc64, row_elems * sizeof(double2)),
                        "cudaMalloc(FP64 row)");
    void *acc_of_block = p->acc64 ? static_cast<void *>(b->d_acc64) : static_cast<void *>(rows);
    if (st != CORR_OK) {
        batch_free(b);
        return st;
    }
    // Kernels configure themselves on first use; do that outside the capture,
    // once for every engine a block uses.
    for (int e = 0; e < n_plans && st == CORR_OK; ++e) {
        bool used = false;
        for (int i = 0; i < n_blocks && !used; ++i) used = plan_of(i) == plans[e];
        if (used)
            st = fxplan_accumulate(plans[e], d_samples, station_stride, frame_stride, d_mask,
                                   mask_station_stride, static_cast<int>(block_first[0]), 1,
                                   acc_of_block, b->cap, d_pmask, pmask_station_stride,
                                   static_cast<int>(block_first[0]));
    }
    if (st == CORR_OK) st = cuda_check(cudaStreamSynchronize(b->cap), "warm-up");
    if (st != CORR_OK) {
        batch_free(b);
        return st;
    }

    st = cuda_check(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal),
                    "cudaStreamBeginCapture");
    for (int i = 0; i < n_blocks && st == CORR_OK; ++i) {
        float2 *row = rows + static_cast<size_t>(i) * row_elems;
        const int first = static_cast<int>(block_first[i]);
        const size_t acc_bytes = row_elems * (p->acc64 ? sizeof(double2) : sizeof(float2));
        void *acc = p->acc64 ? static_cast<void *>(b->d_acc64) : static_cast<void *>(row);
        if ((st = stamp_launch(b->d_stamps + 2 * i, b->cap)) != CORR_OK) break;
        if ((st = cuda_check(cudaMemsetAsync(acc, 0, acc_bytes, b->cap),
                             "cudaMemsetAsync(row)")) != CORR_OK)
            break;
        if ((st = fxplan_accumulate(plan_of(i),
                                    d_samples + static_cast<size_t>(first) * frame_stride,
                                    station_stride, frame_stride, d_mask, mask_station_stride,
                                    first, block_frames[i], acc, b->cap, d_pmask,
                                    pmask_station_stride, first)) != CORR_OK)
            break;
        if (p->acc64)
            st = dump64_launch(row, row_elems, b->d_acc64, row_elems, nullptr, nullptr,
                               p->n_baseline, p->n_freq, 1,
                               1.0 / static_cast<double>(block_frames[i]), b->cap);
        else
            st = scale_launch(row, row_elems, 1.0f / static_cast<float>(block_frames[i]), b->cap);
        if (st != CORR_OK) break;
        // dump on the side stream; the next block's kernels do not wait for it
        if ((st = cuda_check(cudaEventRecord(b->ev_fork[i], b->cap), "cudaEventRecord")) != CORR_OK ||
            (st = cuda_check(cudaStreamWaitEvent(b->side, b->ev_fork[i], 0), "cudaStreamWaitEvent")) !=
                CORR_OK)
            break;
        if (h_rows != nullptr &&
            (st = cuda_check(cudaMemcpyAsync(static_cast<float2 *>(h_rows) + i * row_elems, row,
                                             row_elems * sizeof(float2), cudaMemcpyDeviceToHost,
                                             b->side),
                             "cudaMemcpyAsync(row dump)")) != CORR_OK)
            break;
        if ((st = stamp_launch(b->d_stamps + 2 * i + 1, b->side)) != CORR_OK) break;
    }
    // join the side stream back into the capture
    if (st == CORR_OK)
        st = cuda_check(cudaEventRecord(b->ev_fork[n_blocks], b->side), "cudaEventRecord");
    if (st == CORR_OK)
        st = cuda_check(cudaStreamWaitEvent(b->cap, b->ev_fork[n_blocks], 0), "cudaStreamWaitEvent");
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->cap, &g);
    if (st == CORR_OK) st = cuda_check(e, "cudaStreamEndCapture");
    b->graph = g;
    if (st == CORR_OK)
        st = cuda_check(cudaGraphInstantiate(&b->exec, b->graph, 0), "cudaGraphInstantiate");
    if (st != CORR_OK) {
        batch_free(b);
        return st;
    }
    *out_batch = b;
    return CORR_OK;
}

} // namespace
} // namespace corrgb

extern "C" corr_status corrx_batch_create(void *eng, const int8_t *d_samples,
                                          size_t station_stride, size_t frame_stride,
                                          const uint8_t *d_mask, size_t mask_station_stride,
                                          const int64_t *block_first, const int32_t *block_frames,
                                          int32_t n_blocks, void *d_rows, void *h_rows,
                                          void **out_batch) {
    return corrgb::batch_create({static_cast<corrgb::FxPlan *>(eng)}, nullptr, d_samples,
                                station_stride, frame_stride, d_mask, mask_station_stride, nullptr,
                                0, block_first, block_frames, n_blocks, d_rows, h_rows, out_batch);
}

extern "C" corr_status corrx_batch_create_mixed(void *const *engines, int32_t n_engines,
                                                const int32_t *block_engine,
                                                const int8_t *d_samples, size_t station_stride,
                                                size_t frame_stride, const uint8_t *d_mask,
                                                size_t mask_station_stride,
                                                const int64_t *block_first,
                                                const int32_t *block_frames, int32_t n_blocks,
                                                void *d_rows, void *h_rows, void **out_batch) {
    using namespace corrgb;
    if (engines == nullptr || n_engines < 1 || block_engine == nullptr)
        return fail(CORR_ERR_ARG, "engines, n_engines >= 1 and block_engine are required");
    std::vector<FxPlan *> plans;
    for (int i = 0; i < n_engines; ++i) plans.push_back(static_cast<FxPlan *>(engines[i]));
    return batch_create(plans, block_engine, d_samples, station_stride, frame_stride, d_mask,
                        mask_station_stride, nullptr, 0, block_first, block_frames, n_blocks,
                        d_rows, h_rows, out_batch);
}

extern "C" corr_status corrx_batch_create_packets(
    void *const *engines, int32_t n_engines, const int32_t *block_engine,
    const int8_t *d_samples, size_t station_stride, size_t frame_stride, const uint8_t *d_mask,
    size_t mask_station_stride, const uint32_t *d_pmask, size_t pmask_station_stride,
    const int64_t *block_first, const int32_t *block_frames, int32_t n_blocks, void *d_rows,
    void *h_rows, void **out_batch) {
    using namespace corrgb;
    if (engines == nullptr || n_engines < 1 || (n_engines > 1 && block_engine == nullptr))
        return fail(CORR_ERR_ARG, "engines and n_engines >= 1 are required, and block_engine "
                                  "with more than one engine");
    if (d_pmask == nullptr) return fail(CORR_ERR_ARG, "d_pmask is NULL");
    std::vector<FxPlan *> plans;
    for (int i = 0; i < n_engines; ++i) plans.push_back(static_cast<FxPlan *>(engines[i]));
    return batch_create(plans, block_engine, d_samples, station_stride, frame_stride, d_mask,
                        mask_station_stride, d_pmask, pmask_station_stride, block_first,
                        block_frames, n_blocks, d_rows, h_rows, out_batch);
}

extern "C" corr_status corrx_batch_launch(void *batch, void *stream) {
    using namespace corrgb;
    FxBatch *b = static_cast<FxBatch *>(batch);
    if (b == nullptr) return fail(CORR_ERR_ARG, "batch is NULL");
    corr_status st = cuda_check(cudaSetDevice(b->plan->device), "cudaSetDevice");
    if (st != CORR_OK) return st;
    b->last_launch = static_cast<cudaStream_t>(stream);
    return cuda_check(cudaGraphLaunch(b->exec, b->last_launch), "cudaGraphLaunch");
}

extern "C" corr_status corrx_batch_block_ms(void *batch, float *out_ms, int32_t n) {
    using namespace corrgb;
    FxBatch *b = static_cast<FxBatch *>(batch);
    if (b == nullptr || out_ms == nullptr) return fail(CORR_ERR_ARG, "batch and out_ms must be non-NULL");
    if (n < b->n_blocks) return failf(CORR_ERR_ARG, "n=%d < %d blocks", n, b->n_blocks);
    corr_status st = cuda_check(cudaSetDevice(b->plan->device), "cudaSetDevice");
    if (st == CORR_OK) st = cuda_check(cudaStreamSynchronize(b->last_launch), "cudaStreamSynchronize");
    std::vector<unsigned long long> t(2 * static_cast<size_t>(b->n_blocks));
    if (st == CORR_OK)
        st = cuda_check(cudaMemcpy(t.data(), b->d_stamps, t.size() * sizeof(t[0]),
                                   cudaMemcpyDeviceToHost),
                        "cudaMemcpy(stamps)");
    if (st != CORR_OK) return st;
    for (int i = 0; i < b->n_blocks; ++i) {
        if (t[2 * i] == 0 || t[2 * i + 1] < t[2 * i])
            return failf(CORR_ERR_STATE, "block %d has no latency record (launch the batch first)", i);
        out_ms[i] = static_cast<float>(static_cast<double>(t[2 * i + 1] - t[2 * i]) * 1e-6);
    }
    return CORR_OK;
}

extern "C" corr_status corrx_batch_destroy(void *batch) {
    corrgb::batch_free(static_cast<corrgb::FxBatch *>(batch));
    return CORR_OK;
}
