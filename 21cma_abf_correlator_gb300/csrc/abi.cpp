// abi.cpp -- the extern "C" surface of corr_cuda.h (ABI v7) on one GB300.
//
// Same contract as the reference's C ABI layer (corr-cuda/src/corr_cuda.cpp):
// validation and error strings, the pinned staging ring and its layout, the
// slot state machine (free -> copying -> free), the row stack and its
// BUSY/STATE rules, the callback forms, the statistics. The device work behind
// it is the FX plan of engine.cpp.
//
// Streams and ordering, per context:
//   copy    : staging -> device chunk ring (2-D copies: samples, then mask)
//   compute : F-engine + X-engine per chunk, row scaling, accumulator clear
//   fetch   : row stack -> host
//   notify  : event waits + host callbacks for the *_submit entry points
// A three-deep device chunk ring lets the copy of chunk n+1 run under the
// kernels of chunk n. Events: h2d_done per staging slot, copy_done /
// compute_done per ring buffer, row_done, fetch_done.

#include <chrono>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "engine.h"

namespace corrgb {
namespace {

constexpr int kRing = 3;

uint64_t now_ns() {
    return static_cast<uint64_t>(std::chrono::duration_cast<std::chrono::nanoseconds>(
                                     std::chrono::steady_clock::now().time_since_epoch())
                                     .count());
}

enum class Slot { kFree, kCopying };

struct Layout {
    int8_t *base = nullptr;
    size_t frame_stride = 0, slot_stride = 0, validity_offset = 0, validity_bytes = 0;
    size_t station_stride = 0, total_bytes = 0;
};

// Staging layout, identical to the reference's compute_layout
// (corr-cuda/src/corr_cuda.cpp:535-553): per station, block_slots slots of
// frames_per_slot frames of 2*n_freq bytes, then block_slots masks of
// ceil(frames_per_slot/8) bytes; stations back to back.
Layout make_layout(const corr_config &c) {
    Layout s;
    s.frame_stride = 2u * static_cast<size_t>(c.n_freq);
    s.slot_stride = s.frame_stride * static_cast<size_t>(c.frames_per_slot);
    s.validity_bytes = (static_cast<size_t>(c.frames_per_slot) + 7u) / 8u;
    s.validity_offset = s.slot_stride * static_cast<size_t>(c.block_slots);
    s.station_stride = s.validity_offset + s.validity_bytes * static_cast<size_t>(c.block_slots);
    s.total_bytes = s.station_stride * static_cast<size_t>(c.n_station);
    return s;
}

struct Timing {
    uint64_t accumulate = 0, slot_free = 0, row_end = 0, rows_wait = 0, fetch = 0;
};

struct Context {
    corr_config cfg{};
    int device = 0;
    int n_baseline = 0;
    Layout lay;
    void *staging = nullptr;
    std::vector<Slot> slots;
    std::mutex mu;   // guards `slots`

    FxPlan *plan = nullptr;
    int8_t *d_samples[kRing] = {};   // [station][chunk_frames][2*n_freq]
    uint8_t *d_mask[kRing] = {};     // [station][validity_bytes]
    size_t ring_station_stride = 0;
    float2 *d_acc = nullptr;         // [rows_per_fetch][n_baseline][n_freq]
    size_t row_elems = 0;
    int cur_row = 0;
    int pending = 0;
    bool dirty = false;              // something accumulated since create/fetch
    uint64_t chunk_seq = 0;

    cudaStream_t s_copy = nullptr, s_compute = nullptr, s_fetch = nullptr, s_notify = nullptr;
    std::vector<cudaEvent_t> h2d_done;
    cudaEvent_t copy_done[kRing] = {}, compute_done[kRing] = {};
    cudaEvent_t row_done = nullptr, fetch_done = nullptr;

    uint64_t bytes_h2d = 0, bytes_d2h = 0, transfers = 0;
    uint64_t chunks_skipped = 0;   // chunks with no valid frame in any station
    Timing timing;

    size_t out_bytes() const {
        return row_elems * sizeof(float2) * static_cast<size_t>(cfg.rows_per_fetch);
    }
};

Context *as_ctx(void *h) { return static_cast<Context *>(h); }

corr_status use_device(Context *c) { return cuda_check(cudaSetDevice(c->device), "cudaSetDevice"); }

void free_context(Context *c) {
    if (c == nullptr) return;
    cudaSetDevice(c->device);
    for (cudaEvent_t e : c->h2d_done)
        if (e) cudaEventDestroy(e);
    for (int i = 0; i < kRing; ++i) {
        if (c->copy_done[i]) cudaEventDestroy(c->copy_done[i]);
        if (c->compute_done[i]) cudaEventDestroy(c->compute_done[i]);
        if (c->d_samples[i]) cudaFree(c->d_samples[i]);
        if (c->d_mask[i]) cudaFree(c->d_mask[i]);
    }
    if (c->row_done) cudaEventDestroy(c->row_done);
    if (c->fetch_done) cudaEventDestroy(c->fetch_done);
    for (cudaStream_t s : {c->s_copy, c->s_compute, c->s_fetch, c->s_notify})
        if (s) cudaStreamDestroy(s);
    if (c->d_acc) cudaFree(c->d_acc);
    fxplan_destroy(c->plan);
    if (c->staging) cudaFreeHost(c->staging);
    delete c;
}

// Checks that need no device (reference validate_config, corr_cuda.cpp:473-531).
corr_status validate(const corr_config *cfg) {
    if (cfg == nullptr) return fail(CORR_ERR_ARG, "cfg is NULL");
    if (cfg->abi_version != CORR_ABI_VERSION)
        return failf(CORR_ERR_ABI, "abi_version mismatch: library %u, caller %u", CORR_ABI_VERSION,
                     cfg->abi_version);
    if (cfg->struct_size != sizeof(corr_config))
        return failf(CORR_ERR_ABI, "struct_size mismatch: library %zu, caller %u",
                     sizeof(corr_config), cfg->struct_size);
    if (cfg->device_id < 0) return fail(CORR_ERR_ARG, "device_id is negative");
    if (cfg->n_devices < 0) return fail(CORR_ERR_ARG, "n_devices is negative");
    if (cfg->n_devices > static_cast<int32_t>(CORR_MAX_DEVICES))
        return failf(CORR_ERR_ARG, "n_devices=%d exceeds CORR_MAX_DEVICES=%u", cfg->n_devices,
                     CORR_MAX_DEVICES);
    if (cfg->split_mode != CORR_SPLIT_BASELINE_RANGE &&
        cfg->split_mode != CORR_SPLIT_PAIR_COVERING && cfg->split_mode != CORR_SPLIT_TIME_SLICE)
        return failf(CORR_ERR_ARG, "split_mode=%d is not a known split", cfg->split_mode);
    corr_status st = check_geometry(cfg->n_station, cfg->n_freq);
    if (st != CORR_OK) return st;
    if (cfg->frames_per_slot < 1) return fail(CORR_ERR_ARG, "frames_per_slot must be >= 1");
    if (cfg->chunk_frames < 1) return fail(CORR_ERR_ARG, "chunk_frames must be >= 1");
    if (cfg->chunk_frames > cfg->frames_per_slot)
        return failf(CORR_ERR_ARG, "chunk_frames=%d exceeds frames_per_slot=%d",
                     cfg->chunk_frames, cfg->frames_per_slot);
    if (cfg->block_slots < 2)
        return failf(CORR_ERR_ARG, "block_slots=%d must be >= 2", cfg->block_slots);
    if (cfg->rows_per_fetch < 1)
        return failf(CORR_ERR_ARG, "rows_per_fetch=%d must be >= 1", cfg->rows_per_fetch);
    return CORR_OK;
}

corr_status watchdog(Context *c) {
    int code = 0;
    corr_status st = cuda_check(
        cudaMemcpy(&code, c->plan->d_err, sizeof(int), cudaMemcpyDeviceToHost),
        "cudaMemcpy(watchdog)");
    if (st != CORR_OK) return st;
    if (code != kErrNone) {
        cudaMemset(c->plan->d_err, 0, sizeof(int));
        return failf(CORR_ERR_INTERNAL,
                     "device watchdog tripped (code %d); the rows in flight are invalid", code);
    }
    return CORR_OK;
}

corr_status notify_on(Context *c, cudaEvent_t ev, corr_notify_fn fn, void *user) {
    corr_status st = cuda_check(cudaStreamWaitEvent(c->s_notify, ev, 0), "cudaStreamWaitEvent(notify)");
    if (st != CORR_OK) return st;
    return cuda_check(cudaLaunchHostFunc(c->s_notify, reinterpret_cast<cudaHostFn_t>(fn), user),
                      "cudaLaunchHostFunc");
}

corr_status slot_of(Context *c, int64_t seq, int32_t *slot) {
    if (seq < 0) return failf(CORR_ERR_ARG, "slot_seq=%lld is negative", (long long)seq);
    *slot = static_cast<int32_t>(seq % c->cfg.block_slots);
    return CORR_OK;
}

void release_slot(Context *c, int32_t slot) {
    for (int s = 0; s < c->cfg.n_station; ++s)
        std::memset(c->lay.base + static_cast<size_t>(s) * c->lay.station_stride +
                        c->lay.validity_offset + static_cast<size_t>(slot) * c->lay.validity_bytes,
                    0, c->lay.validity_bytes);
    std::lock_guard<std::mutex> lock(c->mu);
    c->slots[static_cast<size_t>(slot)] = Slot::kFree;
}

corr_status expect_copying(Context *c, int32_t slot, int64_t seq) {
    std::lock_guard<std::mutex> lock(c->mu);
    if (c->slots[static_cast<size_t>(slot)] != Slot::kCopying)
        return failf(CORR_ERR_STATE, "slot %d (sequence %lld) was not submitted", slot,
                     (long long)seq);
    return CORR_OK;
}

// Does any station mark a frame of [f0, f0 + ft) of this slot valid? The mask
// bytes sit in host staging memory, written by the receive side before
// row_accumulate, so they are read here directly.
bool chunk_has_frames(const Context *c, const uint8_t *mask_base, int f0, int ft) {
    const Layout &L = c->lay;
    const int b0 = f0 >> 3, b1 = (f0 + ft - 1) >> 3;
    const uint8_t lo = static_cast<uint8_t>(0xFFu << (f0 & 7));
    const uint8_t hi = static_cast<uint8_t>(0xFFu >> (7 - ((f0 + ft - 1) & 7)));
    for (int s = 0; s < c->cfg.n_station; ++s) {
        const uint8_t *m = mask_base + static_cast<size_t>(s) * L.station_stride;
        for (int b = b0; b <= b1; ++b) {
            uint8_t keep = 0xFF;
            if (b == b0) keep &= lo;
            if (b == b1) keep &= hi;
            if (m[b] & keep) return true;
        }
    }
    return false;
}

// The chunked copy + F/X sequence of one slot. A chunk in which no station has
// a valid frame contributes exactly zero to the row (every frame of it would be
// zero-filled): it is skipped -- no copy, no F-engine, no X-engine.
corr_status accumulate_slot(Context *c, int32_t slot, int32_t frames) {
    const corr_config &cfg = c->cfg;
    const Layout &L = c->lay;
    const int n = cfg.n_station;
    float2 *row = c->d_acc + static_cast<size_t>(c->cur_row) * c->row_elems;
    const int8_t *slot_base = L.base + static_cast<size_t>(slot) * L.slot_stride;
    const uint8_t *mask_base = reinterpret_cast<const uint8_t *>(L.base) + L.validity_offset +
                               static_cast<size_t>(slot) * L.validity_bytes;
    corr_status st = CORR_OK;
    for (int f0 = 0; f0 < frames; f0 += cfg.chunk_frames) {
        const int ft = frames - f0 < cfg.chunk_frames ? frames - f0 : cfg.chunk_frames;
        if (!chunk_has_frames(c, mask_base, f0, ft)) {
            ++c->chunks_skipped;
            continue;
        }
        const int d = static_cast<int>(c->chunk_seq++ % kRing);
        const size_t width = static_cast<size_t>(ft) * L.frame_stride;
        if ((st = cuda_check(cudaStreamWaitEvent(c->s_copy, c->compute_done[d], 0),
                             "cudaStreamWaitEvent(compute_done)")) != CORR_OK)
            return st;
        if ((st = cuda_check(cudaMemcpy2DAsync(c->d_samples[d], c->ring_station_stride,
                                               slot_base + static_cast<size_t>(f0) * L.frame_stride,
                                               L.station_stride, width, static_cast<size_t>(n),
                                               cudaMemcpyHostToDevice, c->s_copy),
                             "cudaMemcpy2DAsync(samples)")) != CORR_OK)
            return st;
        if ((st = cuda_check(cudaMemcpy2DAsync(c->d_mask[d], L.validity_bytes, mask_base,
                                               L.station_stride, L.validity_bytes,
                                               static_cast<size_t>(n), cudaMemcpyHostToDevice,
                                               c->s_copy),
                             "cudaMemcpy2DAsync(mask)")) != CORR_OK)
            return st;
        c->bytes_h2d += static_cast<uint64_t>(width * n + L.validity_bytes * n);
        ++c->transfers;
        if ((st = cuda_check(cudaEventRecord(c->copy_done[d], c->s_copy),
                             "cudaEventRecord(copy_done)")) != CORR_OK ||
            (st = cuda_check(cudaStreamWaitEvent(c->s_compute, c->copy_done[d], 0),
                             "cudaStreamWaitEvent(copy_done)")) != CORR_OK)
            return st;
        if ((st = fxplan_accumulate(c->plan, c->d_samples[d], c->ring_station_stride,
                                    L.frame_stride, c->d_mask[d], L.validity_bytes, f0, ft, row,
                                    c->s_compute)) != CORR_OK)
            return st;
        if ((st = cuda_check(cudaEventRecord(c->compute_done[d], c->s_compute),
                             "cudaEventRecord(compute_done)")) != CORR_OK)
            return st;
    }
    c->dirty = true;
    return cuda_check(cudaEventRecord(c->h2d_done[static_cast<size_t>(slot)], c->s_copy),
                      "cudaEventRecord(h2d_done)");
}

corr_status fetch_submit(Context *c, void *out, size_t out_bytes, int32_t *out_rows,
                         corr_notify_fn cb, void *user) {
    if (out_bytes < c->out_bytes())
        return failf(CORR_ERR_ARG, "out_bytes=%zu but %zu are required for rows_per_fetch=%d",
                     out_bytes, c->out_bytes(), c->cfg.rows_per_fetch);
    const int32_t rows = c->pending;
    *out_rows = rows;
    if (rows == 0) return CORR_OK;
    const size_t bytes = c->row_elems * sizeof(float2) * static_cast<size_t>(rows);
    corr_status st;
    if ((st = cuda_check(cudaStreamWaitEvent(c->s_fetch, c->row_done, 0),
                         "cudaStreamWaitEvent(row_done)")) != CORR_OK ||
        (st = cuda_check(cudaMemcpyAsync(out, c->d_acc, bytes, cudaMemcpyDeviceToHost, c->s_fetch),
                         "cudaMemcpyAsync(rows)")) != CORR_OK ||
        (st = cuda_check(cudaEventRecord(c->fetch_done, c->s_fetch),
                         "cudaEventRecord(fetch_done)")) != CORR_OK ||
        (st = cuda_check(cudaStreamWaitEvent(c->s_compute, c->fetch_done, 0),
                         "cudaStreamWaitEvent(fetch_done)")) != CORR_OK ||
        (st = cuda_check(cudaMemsetAsync(c->d_acc, 0, bytes, c->s_compute),
                         "cudaMemsetAsync(acc)")) != CORR_OK)
        return st;
    c->bytes_d2h += bytes;
    if (cb != nullptr && (st = notify_on(c, c->fetch_done, cb, user)) != CORR_OK) return st;
    c->pending = 0;
    c->cur_row = 0;
    c->dirty = false;
    return CORR_OK;
}

corr_status query(cudaEvent_t e, const char *what) {
    cudaError_t r = cudaEventQuery(e);
    if (r == cudaSuccess) return CORR_OK;
    if (r == cudaErrorNotReady) return CORR_ERR_BUSY;
    return cuda_check(r, what);
}

} // namespace
} // namespace corrgb

using namespace corrgb;

extern "C" const char *corr_abi_banner(void) {
    static std::string banner;
    static std::once_flag once;
    std::call_once(once, [] {
        int rt = 0, drv = 0;
        cudaRuntimeGetVersion(&rt);
        cudaDriverGetVersion(&drv);
        banner = "corr_gb300 0.1.0 abi=" + std::to_string(CORR_ABI_VERSION) +
                 " cudart=" + std::to_string(rt) + " driver=" + std::to_string(drv) +
                 " fft=own-stockham arch=sm_103a target=GB300";
    });
    return banner.c_str();
}

extern "C" const char *corr_last_error(void) { return last_error().c_str(); }

extern "C" corr_status corr_create(const corr_config *cfg, void **out_ctx) {
    if (out_ctx == nullptr) return fail(CORR_ERR_ARG, "out_ctx is NULL");
    *out_ctx = nullptr;
    corr_status st = validate(cfg);
    if (st != CORR_OK) return st;

    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(CORR_ERR_CUDA, std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
    }
    if (ndev == 0) return fail(CORR_ERR_ARG, "no CUDA device is visible");
    std::vector<int> devices;
    if (cfg->n_devices > 0)
        devices.assign(cfg->devices, cfg->devices + cfg->n_devices);
    else
        devices.push_back(cfg->device_id);
    for (size_t i = 0; i < devices.size(); ++i) {
        if (devices[i] < 0 || devices[i] >= ndev)
            return failf(CORR_ERR_ARG, "devices[%zu]=%d but only %d device(s) are visible", i,
                         devices[i], ndev);
        for (size_t j = 0; j < i; ++j)
            if (devices[j] == devices[i])
                return failf(CORR_ERR_ARG, "devices[%zu]=%d repeats an earlier entry", i,
                             devices[i]);
    }
    if (devices.size() > 1)
        return failf(CORR_ERR_NOT_IMPL,
                     "n_devices=%zu: this library drives one GPU per context; run one context "
                     "per device and add the rows on the host",
                     devices.size());

    Context *c = new (std::nothrow) Context();
    if (c == nullptr) return fail(CORR_ERR_NOMEM, "cannot allocate the context");
    c->cfg = *cfg;
    c->device = devices[0];
    c->n_baseline = cfg->n_station * (cfg->n_station + 1) / 2;
    c->lay = make_layout(*cfg);
    c->row_elems = static_cast<size_t>(c->n_baseline) * static_cast<size_t>(cfg->n_freq);
    c->ring_station_stride = static_cast<size_t>(cfg->chunk_frames) * c->lay.frame_stride;

    if ((st = use_device(c)) != CORR_OK) {
        delete c;
        return st;
    }
    e = cudaHostAlloc(&c->staging, c->lay.total_bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        cudaGetLastError();
        c->staging = nullptr;
        const size_t want = c->lay.total_bytes;
        free_context(c);
        return failf(CORR_ERR_NOMEM, "cudaHostAlloc(%zu bytes) failed: %s; check RLIMIT_MEMLOCK",
                     want, cudaGetErrorString(e));
    }
    std::memset(c->staging, 0, c->lay.total_bytes);
    c->lay.base = static_cast<int8_t *>(c->staging);
    c->slots.assign(static_cast<size_t>(cfg->block_slots), Slot::kFree);

    if ((st = fxplan_create(c->device, cfg->n_station, cfg->n_freq, cfg->chunk_frames,
                            CORR_X_PLAIN_FP32, &c->plan)) != CORR_OK) {
        free_context(c);
        return st;
    }
    const size_t ring_bytes = c->ring_station_stride * static_cast<size_t>(cfg->n_station);
    const size_t mask_bytes = c->lay.validity_bytes * static_cast<size_t>(cfg->n_station);
    for (int i = 0; i < kRing && st == CORR_OK; ++i) {
        if (cudaMalloc(&c->d_samples[i], ring_bytes) != cudaSuccess ||
            cudaMalloc(&c->d_mask[i], mask_bytes) != cudaSuccess) {
            cudaGetLastError();
            st = failf(CORR_ERR_NOMEM, "cudaMalloc(chunk ring, %zu bytes) failed", ring_bytes);
        }
    }
    const size_t acc_bytes = c->out_bytes();
    if (st == CORR_OK && cudaMalloc(&c->d_acc, acc_bytes) != cudaSuccess) {
        cudaGetLastError();
        st = failf(CORR_ERR_NOMEM, "cudaMalloc(row stack, %zu bytes) failed", acc_bytes);
    }
    if (st == CORR_OK) st = cuda_check(cudaMemset(c->d_acc, 0, acc_bytes), "cudaMemset(acc)");
    for (cudaStream_t *s : {&c->s_copy, &c->s_compute, &c->s_fetch, &c->s_notify})
        if (st == CORR_OK)
            st = cuda_check(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking), "cudaStreamCreate");
    c->h2d_done.assign(static_cast<size_t>(cfg->block_slots), nullptr);
    for (auto &ev : c->h2d_done)
        if (st == CORR_OK)
            st = cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
    for (int i = 0; i < kRing; ++i)
        for (cudaEvent_t *ev : {&c->copy_done[i], &c->compute_done[i]})
            if (st == CORR_OK)
                st = cuda_check(cudaEventCreateWithFlags(ev, cudaEventDisableTiming),
                                "cudaEventCreate");
    for (cudaEvent_t *ev : {&c->row_done, &c->fetch_done})
        if (st == CORR_OK)
            st = cuda_check(cudaEventCreateWithFlags(ev, cudaEventDisableTiming), "cudaEventCreate");
    // Prime every "previous use finished" event so the first wait returns.
    for (int i = 0; i < kRing && st == CORR_OK; ++i)
        st = cuda_check(cudaEventRecord(c->compute_done[i], c->s_compute), "cudaEventRecord");
    for (auto &ev : c->h2d_done)
        if (st == CORR_OK) st = cuda_check(cudaEventRecord(ev, c->s_copy), "cudaEventRecord");
    if (st == CORR_OK) st = cuda_check(cudaEventRecord(c->row_done, c->s_compute), "cudaEventRecord");
    if (st == CORR_OK) st = cuda_check(cudaEventRecord(c->fetch_done, c->s_fetch), "cudaEventRecord");
    if (st == CORR_OK) st = cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize(create)");
    if (st != CORR_OK) {
        const std::string msg = last_error();
        free_context(c);
        return fail(st, msg);
    }
    *out_ctx = c;
    return CORR_OK;
}

extern "C" corr_status corr_destroy(void *h) {
    Context *c = as_ctx(h);
    if (c == nullptr) return CORR_OK;
    corr_status st = use_device(c);
    if (st == CORR_OK) st = cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize(destroy)");
    const std::string msg = last_error();
    free_context(c);
    if (st != CORR_OK) return fail(st, msg);
    return CORR_OK;
}

extern "C" corr_status corr_staging_info(void *h, int32_t station, corr_staging *out) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (out == nullptr) return fail(CORR_ERR_ARG, "out is NULL");
    if (station < 0 || station >= c->cfg.n_station)
        return failf(CORR_ERR_ARG, "station %d out of range [0,%d)", station, c->cfg.n_station);
    out->base = c->lay.base + static_cast<size_t>(station) * c->lay.station_stride;
    out->frame_stride = c->lay.frame_stride;
    out->slot_stride = c->lay.slot_stride;
    out->total_bytes = c->lay.station_stride;
    out->validity_offset = c->lay.validity_offset;
    out->validity_bytes_per_slot = c->lay.validity_bytes;
    return CORR_OK;
}

extern "C" corr_status corr_row_accumulate(void *h, int64_t slot_seq, int32_t frames) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    int32_t slot = 0;
    corr_status st = slot_of(c, slot_seq, &slot);
    if (st != CORR_OK) return st;
    if (frames < 1 || frames > c->cfg.frames_per_slot)
        return failf(CORR_ERR_ARG,
                     "frames=%d out of range [1,%d]; bytes past the caller's count are stale",
                     frames, c->cfg.frames_per_slot);
    {
        std::lock_guard<std::mutex> lock(c->mu);
        if (c->slots[static_cast<size_t>(slot)] != Slot::kFree)
            return failf(CORR_ERR_BUSY,
                         "slot %d (sequence %lld) is not free; it was submitted and not "
                         "released with corr_row_slot_free",
                         slot, (long long)slot_seq);
        c->slots[static_cast<size_t>(slot)] = Slot::kCopying;
    }
    const uint64_t t0 = now_ns();
    if ((st = use_device(c)) == CORR_OK) st = accumulate_slot(c, slot, frames);
    c->timing.accumulate += now_ns() - t0;
    if (st != CORR_OK) {
        std::lock_guard<std::mutex> lock(c->mu);
        c->slots[static_cast<size_t>(slot)] = Slot::kFree;
    }
    return st;
}

extern "C" corr_status corr_row_slot_free(void *h, int64_t slot_seq) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    int32_t slot = 0;
    corr_status st = slot_of(c, slot_seq, &slot);
    if (st != CORR_OK || (st = expect_copying(c, slot, slot_seq)) != CORR_OK) return st;
    const uint64_t t0 = now_ns();
    if ((st = use_device(c)) == CORR_OK)
        st = cuda_check(cudaEventSynchronize(c->h2d_done[static_cast<size_t>(slot)]),
                        "cudaEventSynchronize(h2d_done)");
    c->timing.slot_free += now_ns() - t0;
    if (st != CORR_OK) return st;
    release_slot(c, slot);
    return CORR_OK;
}

extern "C" corr_status corr_row_slot_free_submit(void *h, int64_t slot_seq, corr_notify_fn cb,
                                                 void *user) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (cb == nullptr) return fail(CORR_ERR_ARG, "cb is NULL");
    int32_t slot = 0;
    corr_status st = slot_of(c, slot_seq, &slot);
    if (st != CORR_OK || (st = expect_copying(c, slot, slot_seq)) != CORR_OK) return st;
    const uint64_t t0 = now_ns();
    if ((st = use_device(c)) == CORR_OK)
        st = notify_on(c, c->h2d_done[static_cast<size_t>(slot)], cb, user);
    c->timing.slot_free += now_ns() - t0;
    return st;
}

extern "C" corr_status corr_row_slot_free_finish(void *h, int64_t slot_seq) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    int32_t slot = 0;
    corr_status st = slot_of(c, slot_seq, &slot);
    if (st != CORR_OK) return st;
    {
        std::lock_guard<std::mutex> lock(c->mu);
        if (c->slots[static_cast<size_t>(slot)] != Slot::kCopying)
            return failf(CORR_ERR_STATE,
                         "slot %d (sequence %lld) was not submitted, or its release has already "
                         "been finished",
                         slot, (long long)slot_seq);
    }
    // The copy is known complete (the callback fired); surface a failed copy.
    if ((st = use_device(c)) == CORR_OK)
        st = query(c->h2d_done[static_cast<size_t>(slot)], "cudaEventQuery(h2d_done)");
    if (st == CORR_ERR_BUSY)
        return fail(CORR_ERR_STATE, "the slot's copy has not completed; finish only after the "
                                    "callback has fired");
    if (st != CORR_OK) return st;
    release_slot(c, slot);
    return CORR_OK;
}

extern "C" corr_status corr_row_end(void *h, uint64_t frames) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (frames == 0) return fail(CORR_ERR_ARG, "row_end: frames must be > 0");
    if (c->pending >= c->cfg.rows_per_fetch)
        return fail(CORR_ERR_BUSY,
                    "row_end: all rows are closed and unfetched; continuing would overwrite data");
    const uint64_t t0 = now_ns();
    corr_status st = use_device(c);
    if (st == CORR_OK)
        st = scale_launch(c->d_acc + static_cast<size_t>(c->cur_row) * c->row_elems, c->row_elems,
                          1.0f / static_cast<float>(frames), c->s_compute);
    if (st == CORR_OK)
        st = cuda_check(cudaEventRecord(c->row_done, c->s_compute), "cudaEventRecord(row_done)");
    c->timing.row_end += now_ns() - t0;
    if (st != CORR_OK) return st;
    ++c->pending;
    if (++c->cur_row >= c->cfg.rows_per_fetch) c->cur_row = 0;
    return CORR_OK;
}

extern "C" corr_status corr_rows_wait(void *h) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    const uint64_t t0 = now_ns();
    corr_status st = use_device(c);
    if (st == CORR_OK)
        st = cuda_check(cudaEventSynchronize(c->row_done), "cudaEventSynchronize(row_done)");
    if (st == CORR_OK) st = watchdog(c);
    c->timing.rows_wait += now_ns() - t0;
    return st;
}

extern "C" corr_status corr_rows_wait_submit(void *h, corr_notify_fn cb, void *user) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (cb == nullptr) return fail(CORR_ERR_ARG, "cb is NULL");
    const uint64_t t0 = now_ns();
    corr_status st = use_device(c);
    if (st == CORR_OK) st = notify_on(c, c->row_done, cb, user);
    c->timing.rows_wait += now_ns() - t0;
    return st;
}

extern "C" corr_status corr_rows_ready(void *h) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    corr_status st = use_device(c);
    if (st == CORR_OK) st = query(c->row_done, "cudaEventQuery(row_done)");
    if (st == CORR_OK) st = watchdog(c);
    return st;
}

extern "C" corr_status corr_rows_pending(void *h, int32_t *out_pending) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (out_pending == nullptr) return fail(CORR_ERR_ARG, "out_pending is NULL");
    *out_pending = c->pending;
    return CORR_OK;
}

extern "C" corr_status corr_rows_fetch_submit(void *h, void *out, size_t out_bytes,
                                              int32_t *out_rows, corr_notify_fn cb, void *user) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (out == nullptr) return fail(CORR_ERR_ARG, "out is NULL");
    if (out_rows == nullptr) return fail(CORR_ERR_ARG, "out_rows is NULL");
    if (cb == nullptr) return fail(CORR_ERR_ARG, "cb is NULL");
    const uint64_t t0 = now_ns();
    corr_status st = use_device(c);
    if (st == CORR_OK) st = fetch_submit(c, out, out_bytes, out_rows, cb, user);
    c->timing.fetch += now_ns() - t0;
    return st;
}

extern "C" corr_status corr_rows_fetch_ready(void *h) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    corr_status st = use_device(c);
    if (st == CORR_OK) st = query(c->fetch_done, "cudaEventQuery(fetch_done)");
    return st;
}

extern "C" corr_status corr_rows_fetch(void *h, void *out, size_t out_bytes, int32_t *out_rows) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (out == nullptr) return fail(CORR_ERR_ARG, "out is NULL");
    if (out_rows == nullptr) return fail(CORR_ERR_ARG, "out_rows is NULL");
    const uint64_t t0 = now_ns();
    corr_status st = use_device(c);
    if (st == CORR_OK) st = fetch_submit(c, out, out_bytes, out_rows, nullptr, nullptr);
    if (st == CORR_OK && *out_rows > 0) {
        st = cuda_check(cudaEventSynchronize(c->fetch_done), "cudaEventSynchronize(fetch_done)");
        if (st == CORR_OK) st = watchdog(c);
    }
    c->timing.fetch += now_ns() - t0;
    return st;
}

extern "C" int32_t corr_n_baseline(int32_t n_station) {
    if (n_station < 1) return -1;
    return n_station * (n_station + 1) / 2;
}

extern "C" corr_status corr_baseline_pairs(int32_t n_station, int32_t *out_jk, int32_t out_len) {
    if (n_station < 1) return fail(CORR_ERR_ARG, "n_station must be >= 1");
    const int32_t nbl = corr_n_baseline(n_station);
    if (out_len != 2 * nbl)
        return failf(CORR_ERR_ARG, "out_len=%d but %d are required for n_station=%d", out_len,
                     2 * nbl, n_station);
    if (out_jk == nullptr) return fail(CORR_ERR_ARG, "out_jk is NULL");
    int32_t i = 0;
    for (int32_t j = 0; j < n_station; ++j)
        for (int32_t k = j; k < n_station; ++k) {
            out_jk[2 * i] = j;
            out_jk[2 * i + 1] = k;
            ++i;
        }
    return CORR_OK;
}

extern "C" int32_t corr_n_devices(void *h) { return h == nullptr ? -1 : 1; }

static corr_status check_index(Context *c, int32_t device_index) {
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (device_index != 0)
        return failf(CORR_ERR_ARG, "device_index %d out of range [0,1)", device_index);
    return CORR_OK;
}

extern "C" corr_status corr_device_plan_get(void *h, int32_t device_index, corr_device_plan *out) {
    Context *c = as_ctx(h);
    corr_status st = check_index(c, device_index);
    if (st != CORR_OK) return st;
    if (out == nullptr) return fail(CORR_ERR_ARG, "out is NULL");
    out->device_id = c->device;
    out->n_station_resident = c->cfg.n_station;
    out->first_baseline = 0;
    out->n_baseline = c->n_baseline;
    out->contiguous = 1;
    return CORR_OK;
}

extern "C" corr_status corr_device_stations(void *h, int32_t device_index, int32_t *out_stations,
                                            int32_t out_len) {
    Context *c = as_ctx(h);
    corr_status st = check_index(c, device_index);
    if (st != CORR_OK) return st;
    if (out_stations == nullptr) return fail(CORR_ERR_ARG, "out_stations is NULL");
    if (out_len < c->cfg.n_station)
        return failf(CORR_ERR_ARG, "out_len=%d but device 0 holds %d stations", out_len,
                     c->cfg.n_station);
    for (int32_t i = 0; i < c->cfg.n_station; ++i) out_stations[i] = i;
    return CORR_OK;
}

extern "C" corr_status corr_device_baselines(void *h, int32_t device_index, int32_t *out_baselines,
                                             int32_t out_len) {
    Context *c = as_ctx(h);
    corr_status st = check_index(c, device_index);
    if (st != CORR_OK) return st;
    if (out_baselines == nullptr) return fail(CORR_ERR_ARG, "out_baselines is NULL");
    if (out_len < c->n_baseline)
        return failf(CORR_ERR_ARG, "out_len=%d but device 0 owns %d baselines", out_len,
                     c->n_baseline);
    for (int32_t i = 0; i < c->n_baseline; ++i) out_baselines[i] = i;
    return CORR_OK;
}

extern "C" corr_status corr_device_stats_get(void *h, int32_t device_index, corr_device_stats *out) {
    Context *c = as_ctx(h);
    corr_status st = check_index(c, device_index);
    if (st != CORR_OK) return st;
    if (out == nullptr) return fail(CORR_ERR_ARG, "out is NULL");
    out->device_id = c->device;
    out->bytes_h2d = c->bytes_h2d;
    out->bytes_d2h = c->bytes_d2h;
    out->transfers = c->transfers;
    out->ns_accumulate = c->timing.accumulate;
    out->ns_slot_free = c->timing.slot_free;
    out->ns_row_end = c->timing.row_end;
    out->ns_rows_wait = c->timing.rows_wait;
    out->ns_fetch = c->timing.fetch;
    return CORR_OK;
}

extern "C" corr_status corr_host_alloc(size_t bytes, void **out) {
    if (out == nullptr) return fail(CORR_ERR_ARG, "out is NULL");
    if (bytes == 0) return fail(CORR_ERR_ARG, "bytes must be > 0");
    void *p = nullptr;
    cudaError_t e = cudaHostAlloc(&p, bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return failf(CORR_ERR_NOMEM, "cudaHostAlloc(%zu bytes) failed: %s", bytes,
                     cudaGetErrorString(e));
    }
    *out = p;
    return CORR_OK;
}

extern "C" void corr_host_free(void *p) {
    if (p != nullptr) cudaFreeHost(p);
}

extern "C" corr_status corr_set_xengine(void *h, int32_t mode) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (mode != CORR_X_PLAIN_FP32 && mode != CORR_X_TC_FP16 && mode != CORR_X_TC_FP16_SPLIT)
        return failf(CORR_ERR_ARG, "unknown X-engine mode %d", mode);
    if (c->dirty || c->pending != 0)
        return fail(CORR_ERR_STATE,
                    "the X-engine can only change while no row holds data (after create or a "
                    "fetch)");
    if (mode != CORR_X_PLAIN_FP32) {
        int ct = 0, kt = 0;
        corrgb::xengine_tc_default_shape(c->plan->n_station, mode == CORR_X_TC_FP16_SPLIT, &ct, &kt);
        if (ct == 0)
            return failf(CORR_ERR_NOT_IMPL, "the tensor X-engine takes 1..64 inputs (n_station=%d)",
                         c->plan->n_station);
        c->plan->xct = ct;
        c->plan->xkt = kt;
        if (c->plan->ytile < ct) c->plan->ytile = c->plan->n_freq;
    }
    c->plan->xmode = mode;
    // an FFT plan that cannot write this mode's spectra falls back to plan 0
    if (!corrgb::fengine_plan_ok(c->plan->n_freq, c->plan->fplan, corrgb::spectra_format(mode)))
        c->plan->fplan = 0;
    return CORR_OK;
}

extern "C" corr_status corr_get_tiles(void *h, corrx_tiles *out) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    return corrx_get_tiles(c->plan, out);
}

extern "C" corr_status corr_set_tiles(void *h, const corrx_tiles *t) {
    Context *c = as_ctx(h);
    if (c == nullptr || t == nullptr) return fail(CORR_ERR_ARG, "ctx and t must be non-NULL");
    if (c->dirty || c->pending != 0)
        return fail(CORR_ERR_STATE,
                    "tiles can only change while no row holds data (after create or a fetch)");
    return corrx_set_tiles(c->plan, t);
}

extern "C" corr_status corr_autotune(void *h, corrx_tiles *out) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (out != nullptr && out->struct_size != sizeof(corrx_tiles))
        return failf(CORR_ERR_ABI, "corrx_tiles.struct_size=%u, expected %zu", out->struct_size,
                     sizeof(corrx_tiles));
    if (c->dirty || c->pending != 0)
        return fail(CORR_ERR_STATE,
                    "tiles can only be tuned while no row holds data (after create or a fetch)");
    return corrgb::fxplan_autotune(c->plan, c->s_compute, out);
}
