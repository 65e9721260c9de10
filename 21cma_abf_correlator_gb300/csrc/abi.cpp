// abi.cpp -- the extern "C" surface of corr_cuda.h (ABI v7) on one or more GB300s.
//
// Same contract as the reference's C ABI layer (corr-cuda/src/corr_cuda.cpp):
// validation and error strings, the pinned staging ring and its layout, the
// slot state machine (free -> copying -> free), the row stack and its
// BUSY/STATE rules, the callback forms, the statistics, and the three ways of
// spreading a run over several devices. The device work behind it is the FX
// plan of engine.cpp.
//
// A context is a list of shares, one per configured device (placement.cpp
// decides what each holds). Share 0 is the home: it owns the fetch stream, the
// complex64 output rows and the notify stream through which every callback is
// delivered. Per share:
//   copy    : staging -> device chunk ring (2-D copies of its resident stations)
//   compute : F-engine + X-engine per chunk into a complex128 row stack,
//             row scaling, row clearing
// A three-deep chunk ring lets the copy of chunk n+1 run under the kernels of
// chunk n. Rows integrate in complex128: each X-engine launch adds its FP32
// partial sums once, so a row of thousands of chunks keeps one launch's
// precision. At fetch the home brings every other share's rows into its own
// memory (cudaMemcpyPeerAsync; the library's kernels never dereference a peer
// pointer) and either adds them (time slice: partial rows over disjoint frames)
// or takes the baselines each share owns (baseline range, pair covering), then
// rounds the result to complex64 and copies it to the caller in one transfer.

#include <chrono>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "engine.h"
#include "placement.h"

namespace corrgb {
namespace {

constexpr int kRing = 3;

uint64_t now_ns() {
    return static_cast<uint64_t>(std::chrono::duration_cast<std::chrono::nanoseconds>(
                                     std::chrono::steady_clock::now().time_since_epoch())
                                     .count());
}

// Configured device ordinal -> CUDA ordinal (corrx_set_device_map); empty = identity.
std::mutex g_map_mu;
std::vector<int> g_device_map;

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

// A run of consecutive global stations held by a share: one 2-D copy each.
struct StationRun {
    int global0 = 0, local0 = 0, count = 0;
};

// One configured device's part of a context.
struct Share {
    DevicePlacement pl;                // what it holds and owns (placement.h)
    int physical = 0;                  // CUDA ordinal
    std::vector<StationRun> runs;
    FxPlan *plan = nullptr;
    int8_t *d_samples[kRing] = {};     // [local station][chunk_frames][2*n_freq]
    uint8_t *d_mask[kRing] = {};       // [local station][validity_bytes]
    size_t ring_station_stride = 0;
    double2 *d_acc = nullptr;          // [rows_per_fetch][local baselines][n_freq] complex128
    size_t row_elems = 0;              // local baselines * n_freq
    int32_t *d_gmap = nullptr;         // on the home device: owned baselines, global index
    int32_t *d_lmap = nullptr;         //   ... and local index (baseline range, pair covering)
    uint64_t chunk_seq = 0;

    cudaStream_t s_copy = nullptr, s_compute = nullptr;
    std::vector<cudaEvent_t> h2d_done;
    cudaEvent_t copy_done[kRing] = {}, compute_done[kRing] = {};
    cudaEvent_t row_done = nullptr;
    cudaEvent_t taken = nullptr;       // home device: the fetch has read this share's rows

    uint64_t bytes_h2d = 0, bytes_d2h = 0, transfers = 0, chunks_skipped = 0;
    Timing timing;

    int n_local() const { return static_cast<int>(pl.stations.size()); }
};

struct Context {
    corr_config cfg{};
    int n_baseline = 0;
    bool time_slice = false;
    Layout lay;
    void *staging = nullptr;
    std::vector<Slot> slots;
    std::mutex mu;   // guards `slots`

    std::vector<std::unique_ptr<Share>> shares;   // [0] = home
    float2 *d_out = nullptr;       // home: [rows_per_fetch][n_baseline][n_freq] complex64
    double2 *d_peer = nullptr;     // home: one other share's rows, brought over at fetch
    size_t peer_elems = 0;
    cudaStream_t s_fetch = nullptr, s_notify = nullptr;   // home
    cudaEvent_t fetch_done = nullptr;                     // home

    int cur_row = 0;
    int pending = 0;
    bool dirty = false;   // something accumulated since create/fetch
    // The caller's frame count of each closed row. The division by it happens
    // when the row is rounded to complex64 at the fetch, after a time slice's
    // partial rows are added: the sum of complex128 partials is then the same
    // number one device would have, and so is the row.
    std::vector<uint64_t> row_frames;

    int n_devices() const { return static_cast<int>(shares.size()); }
    Share &home() { return *shares[0]; }
    size_t row_elems() const {
        return static_cast<size_t>(n_baseline) * static_cast<size_t>(cfg.n_freq);
    }
    size_t out_bytes() const {
        return row_elems() * sizeof(float2) * static_cast<size_t>(cfg.rows_per_fetch);
    }
};

Context *as_ctx(void *h) { return static_cast<Context *>(h); }

corr_status on_device(int physical) {
    return cuda_check(cudaSetDevice(physical), "cudaSetDevice");
}

void free_share(Share *s, int home_physical) {
    if (s == nullptr) return;
    cudaSetDevice(s->physical);
    for (cudaStream_t st : {s->s_copy, s->s_compute})
        if (st) cudaStreamSynchronize(st);
    for (cudaEvent_t e : s->h2d_done)
        if (e) cudaEventDestroy(e);
    for (int i = 0; i < kRing; ++i) {
        if (s->copy_done[i]) cudaEventDestroy(s->copy_done[i]);
        if (s->compute_done[i]) cudaEventDestroy(s->compute_done[i]);
        if (s->d_samples[i]) cudaFree(s->d_samples[i]);
        if (s->d_mask[i]) cudaFree(s->d_mask[i]);
    }
    if (s->row_done) cudaEventDestroy(s->row_done);
    for (cudaStream_t st : {s->s_copy, s->s_compute})
        if (st) cudaStreamDestroy(st);
    if (s->d_acc) cudaFree(s->d_acc);
    fxplan_destroy(s->plan);
    cudaSetDevice(home_physical);   // the maps and `taken` live on the home device
    if (s->taken) cudaEventDestroy(s->taken);
    if (s->d_gmap) cudaFree(s->d_gmap);
    if (s->d_lmap) cudaFree(s->d_lmap);
}

void free_context(Context *c) {
    if (c == nullptr) return;
    const int home_phys = c->shares.empty() ? 0 : c->shares[0]->physical;
    if (!c->shares.empty()) {
        cudaSetDevice(home_phys);
        for (cudaStream_t s : {c->s_fetch, c->s_notify})
            if (s) cudaStreamSynchronize(s);
    }
    for (auto &s : c->shares) free_share(s.get(), home_phys);
    if (!c->shares.empty()) {
        cudaSetDevice(home_phys);
        if (c->fetch_done) cudaEventDestroy(c->fetch_done);
        for (cudaStream_t s : {c->s_fetch, c->s_notify})
            if (s) cudaStreamDestroy(s);
        if (c->d_out) cudaFree(c->d_out);
        if (c->d_peer) cudaFree(c->d_peer);
    }
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
    // The reference's per-device baseline limit, on the placement the split
    // gives the configured devices (host-only: the ordinals are labels here).
    std::vector<int> ordinals;
    if (cfg->n_devices > 0)
        ordinals.assign(cfg->devices, cfg->devices + cfg->n_devices);
    else
        ordinals.push_back(cfg->device_id);
    std::vector<DevicePlacement> plan;
    if ((st = plan_devices(cfg->n_station, cfg->split_mode, ordinals, &plan)) != CORR_OK)
        return st;
    return check_device_baselines(plan);
}

// The configured device list, checked against what is visible and mapped to
// CUDA ordinals.
corr_status resolve_devices(const corr_config &cfg, std::vector<int> *ordinals,
                            std::vector<int> *physical) {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(CORR_ERR_CUDA, std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
    }
    if (ndev == 0) return fail(CORR_ERR_ARG, "no CUDA device is visible");
    std::vector<int> map;
    {
        std::lock_guard<std::mutex> lock(g_map_mu);
        map = g_device_map;
    }
    // Without a map set through the API, CORRX_DEVICE_MAP ("0,0,0,0") gives one:
    // it lets an unmodified caller of this ABI (the reference's C test drivers)
    // run its multi-device cases on a machine with fewer GPUs.
    if (map.empty()) {
        if (const char *env = std::getenv("CORRX_DEVICE_MAP")) {
            for (const char *p = env; *p != '\0';) {
                char *end = nullptr;
                const long v = std::strtol(p, &end, 10);
                if (end == p || v < 0 || v >= kMaxDeviceOrdinals)
                    return failf(CORR_ERR_ARG, "CORRX_DEVICE_MAP=\"%s\" is not a list of device "
                                               "ordinals", env);
                map.push_back(static_cast<int>(v));
                p = *end == ',' ? end + 1 : end;
                if (*end != ',' && *end != '\0')
                    return failf(CORR_ERR_ARG, "CORRX_DEVICE_MAP=\"%s\" is not a list of device "
                                               "ordinals", env);
            }
        }
    }
    const int n_ordinals = map.empty() ? ndev : static_cast<int>(map.size());
    if (cfg.n_devices > 0)
        ordinals->assign(cfg.devices, cfg.devices + cfg.n_devices);
    else
        ordinals->assign(1, cfg.device_id);
    physical->clear();
    for (size_t i = 0; i < ordinals->size(); ++i) {
        const int d = (*ordinals)[i];
        if (d < 0 || d >= n_ordinals)
            return failf(CORR_ERR_ARG, "devices[%zu]=%d but only %d device(s) are visible", i, d,
                         n_ordinals);
        for (size_t j = 0; j < i; ++j)
            if ((*ordinals)[j] == d)
                return failf(CORR_ERR_ARG, "devices[%zu]=%d repeats an earlier entry", i, d);
        const int p = map.empty() ? d : map[static_cast<size_t>(d)];
        if (p < 0 || p >= ndev)
            return failf(CORR_ERR_ARG, "device %d maps to CUDA device %d; %d are visible", d, p,
                         ndev);
        physical->push_back(p);
    }
    return CORR_OK;
}

corr_status watchdog(Share &s) {
    int code = 0;
    corr_status st = on_device(s.physical);
    if (st == CORR_OK)
        st = cuda_check(cudaMemcpy(&code, s.plan->d_err, sizeof(int), cudaMemcpyDeviceToHost),
                        "cudaMemcpy(watchdog)");
    if (st != CORR_OK) return st;
    if (code != kErrNone) {
        cudaMemset(s.plan->d_err, 0, sizeof(int));
        return failf(CORR_ERR_INTERNAL,
                     "device watchdog tripped (code %d) on device %d; the rows in flight are "
                     "invalid",
                     code, s.pl.ordinal);
    }
    return CORR_OK;
}

corr_status watchdog_all(Context *c) {
    for (auto &s : c->shares) {
        corr_status st = watchdog(*s);
        if (st != CORR_OK) return st;
    }
    return CORR_OK;
}

// Deliver `fn(user)` on the home notify stream once every event in `evs`
// (recorded on any of the context's devices) has completed.
corr_status notify_after(Context *c, const std::vector<cudaEvent_t> &evs, corr_notify_fn fn,
                         void *user) {
    corr_status st = on_device(c->home().physical);
    for (cudaEvent_t ev : evs)
        if (st == CORR_OK)
            st = cuda_check(cudaStreamWaitEvent(c->s_notify, ev, 0), "cudaStreamWaitEvent(notify)");
    if (st != CORR_OK) return st;
    return cuda_check(cudaLaunchHostFunc(c->s_notify, reinterpret_cast<cudaHostFn_t>(fn), user),
                      "cudaLaunchHostFunc");
}

corr_status slot_of(Context *c, int64_t seq, int32_t *slot) {
    if (seq < 0) return failf(CORR_ERR_ARG, "slot_seq=%lld is negative", (long long)seq);
    *slot = static_cast<int32_t>(seq % c->cfg.block_slots);
    return CORR_OK;
}

// The shares that read slot sequence `seq`: under the time slice only the one
// it was routed to (seq % n_devices, reference corr_cuda.cpp:841-851), otherwise
// every share.
void readers_of(const Context *c, int64_t seq, int *first, int *last) {
    if (c->time_slice) {
        *first = static_cast<int>(seq % c->n_devices());
        *last = *first + 1;
    } else {
        *first = 0;
        *last = c->n_devices();
    }
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

// Does any station the share holds mark a frame of [f0, f0 + ft) of this slot
// valid? The mask bytes sit in host staging memory, written by the receive side
// before row_accumulate, so they are read here directly.
bool chunk_has_frames(const Context *c, const Share &sh, const uint8_t *mask_base, int f0,
                      int ft) {
    const Layout &L = c->lay;
    const int b0 = f0 >> 3, b1 = (f0 + ft - 1) >> 3;
    const uint8_t lo = static_cast<uint8_t>(0xFFu << (f0 & 7));
    const uint8_t hi = static_cast<uint8_t>(0xFFu >> (7 - ((f0 + ft - 1) & 7)));
    for (int32_t s : sh.pl.stations) {
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

// The chunked copy + F/X sequence of one slot on one share. A chunk in which no
// station of the share has a valid frame contributes exactly zero (every frame
// of it would be zero-filled): it is skipped -- no copy, no F-engine, no X-engine.
corr_status accumulate_slot(Context *c, Share &sh, int32_t slot, int32_t frames) {
    const corr_config &cfg = c->cfg;
    const Layout &L = c->lay;
    double2 *row = sh.d_acc + static_cast<size_t>(c->cur_row) * sh.row_elems;
    const int8_t *slot_base = L.base + static_cast<size_t>(slot) * L.slot_stride;
    const uint8_t *mask_base = reinterpret_cast<const uint8_t *>(L.base) + L.validity_offset +
                               static_cast<size_t>(slot) * L.validity_bytes;
    corr_status st = CORR_OK;
    for (int f0 = 0; f0 < frames; f0 += cfg.chunk_frames) {
        const int ft = frames - f0 < cfg.chunk_frames ? frames - f0 : cfg.chunk_frames;
        if (!chunk_has_frames(c, sh, mask_base, f0, ft)) {
            ++sh.chunks_skipped;
            continue;
        }
        const int d = static_cast<int>(sh.chunk_seq++ % kRing);
        const size_t width = static_cast<size_t>(ft) * L.frame_stride;
        if ((st = cuda_check(cudaStreamWaitEvent(sh.s_copy, sh.compute_done[d], 0),
                             "cudaStreamWaitEvent(compute_done)")) != CORR_OK)
            return st;
        for (const StationRun &r : sh.runs) {
            const size_t g0 = static_cast<size_t>(r.global0) * L.station_stride;
            if ((st = cuda_check(
                     cudaMemcpy2DAsync(sh.d_samples[d] + r.local0 * sh.ring_station_stride,
                                       sh.ring_station_stride,
                                       slot_base + g0 + static_cast<size_t>(f0) * L.frame_stride,
                                       L.station_stride, width, static_cast<size_t>(r.count),
                                       cudaMemcpyHostToDevice, sh.s_copy),
                     "cudaMemcpy2DAsync(samples)")) != CORR_OK)
                return st;
            if ((st = cuda_check(
                     cudaMemcpy2DAsync(sh.d_mask[d] + r.local0 * L.validity_bytes,
                                       L.validity_bytes, mask_base + g0, L.station_stride,
                                       L.validity_bytes, static_cast<size_t>(r.count),
                                       cudaMemcpyHostToDevice, sh.s_copy),
                     "cudaMemcpy2DAsync(mask)")) != CORR_OK)
                return st;
        }
        sh.bytes_h2d += static_cast<uint64_t>((width + L.validity_bytes) * sh.n_local());
        ++sh.transfers;
        if ((st = cuda_check(cudaEventRecord(sh.copy_done[d], sh.s_copy),
                             "cudaEventRecord(copy_done)")) != CORR_OK ||
            (st = cuda_check(cudaStreamWaitEvent(sh.s_compute, sh.copy_done[d], 0),
                             "cudaStreamWaitEvent(copy_done)")) != CORR_OK)
            return st;
        if ((st = fxplan_accumulate(sh.plan, sh.d_samples[d], sh.ring_station_stride,
                                    L.frame_stride, sh.d_mask[d], L.validity_bytes, f0, ft, row,
                                    sh.s_compute)) != CORR_OK)
            return st;
        if ((st = cuda_check(cudaEventRecord(sh.compute_done[d], sh.s_compute),
                             "cudaEventRecord(compute_done)")) != CORR_OK)
            return st;
    }
    return cuda_check(cudaEventRecord(sh.h2d_done[static_cast<size_t>(slot)], sh.s_copy),
                      "cudaEventRecord(h2d_done)");
}

// Queue the fetch of the closed rows on the home device: bring each other
// share's rows over, combine, round to complex64, copy to `out`, then clear
// every share's rows once they have been read.
corr_status fetch_submit(Context *c, void *out, size_t out_bytes, int32_t *out_rows,
                         corr_notify_fn cb, void *user) {
    if (out_bytes < c->out_bytes())
        return failf(CORR_ERR_ARG, "out_bytes=%zu but %zu are required for rows_per_fetch=%d",
                     out_bytes, c->out_bytes(), c->cfg.rows_per_fetch);
    const int32_t rows = c->pending;
    *out_rows = rows;
    if (rows == 0) return CORR_OK;
    Share &home = c->home();
    const int nf = c->cfg.n_freq;
    const size_t out_row = c->row_elems();
    corr_status st = on_device(home.physical);
    for (auto &s : c->shares)
        if (st == CORR_OK)
            st = cuda_check(cudaStreamWaitEvent(c->s_fetch, s->row_done, 0),
                            "cudaStreamWaitEvent(row_done)");
    if (st != CORR_OK) return st;
    // rows of share `s`, readable on the home device
    auto bring = [&](Share &s, const double2 **src) -> corr_status {
        if (&s == &home) {
            *src = home.d_acc;
            return CORR_OK;
        }
        const size_t bytes = s.row_elems * sizeof(double2) * static_cast<size_t>(rows);
        corr_status s2 = cuda_check(cudaMemcpyPeerAsync(c->d_peer, home.physical, s.d_acc,
                                                        s.physical, bytes, c->s_fetch),
                                    "cudaMemcpyPeerAsync(partial rows)");
        if (s2 != CORR_OK) return s2;
        s.bytes_d2h += bytes;
        *src = c->d_peer;
        return cuda_check(cudaEventRecord(s.taken, c->s_fetch), "cudaEventRecord(taken)");
    };
    if (c->time_slice) {
        // Every share holds a partial row of every baseline over its own slots:
        // sum them (complex128) into the home's rows, then round once.
        for (int d = 1; d < c->n_devices() && st == CORR_OK; ++d) {
            const double2 *src = nullptr;
            if ((st = bring(*c->shares[static_cast<size_t>(d)], &src)) == CORR_OK)
                st = add64_launch(home.d_acc, src, home.row_elems * static_cast<size_t>(rows),
                                  c->s_fetch);
        }
        for (int r = 0; r < rows && st == CORR_OK; ++r)
            st = dump64_launch(c->d_out + static_cast<size_t>(r) * out_row, out_row,
                               home.d_acc + static_cast<size_t>(r) * home.row_elems,
                               home.row_elems, nullptr, nullptr, c->n_baseline, nf, 1,
                               1.0 / static_cast<double>(c->row_frames[static_cast<size_t>(r)]),
                               c->s_fetch);
        if (st == CORR_OK)
            st = cuda_check(cudaEventRecord(home.taken, c->s_fetch), "cudaEventRecord(taken)");
    } else {
        // Each share owns some baselines of its local matrix: place them.
        for (auto &sp : c->shares) {
            if (st != CORR_OK) break;
            Share &s = *sp;
            const double2 *src = nullptr;
            if ((st = bring(s, &src)) != CORR_OK) break;
            for (int r = 0; r < rows && st == CORR_OK; ++r)
                st = dump64_launch(
                    c->d_out + static_cast<size_t>(r) * out_row, out_row,
                    src + static_cast<size_t>(r) * s.row_elems, s.row_elems, s.d_gmap, s.d_lmap,
                    static_cast<int>(s.pl.baselines.size()), nf, 1,
                    1.0 / static_cast<double>(c->row_frames[static_cast<size_t>(r)]), c->s_fetch);
            if (st == CORR_OK && &s == &home)
                st = cuda_check(cudaEventRecord(home.taken, c->s_fetch), "cudaEventRecord(taken)");
        }
    }
    if (st != CORR_OK) return st;
    const size_t bytes = out_row * sizeof(float2) * static_cast<size_t>(rows);
    if ((st = cuda_check(cudaMemcpyAsync(out, c->d_out, bytes, cudaMemcpyDeviceToHost, c->s_fetch),
                         "cudaMemcpyAsync(rows)")) != CORR_OK ||
        (st = cuda_check(cudaEventRecord(c->fetch_done, c->s_fetch),
                         "cudaEventRecord(fetch_done)")) != CORR_OK)
        return st;
    home.bytes_d2h += bytes;
    // Clear each share's rows on its compute stream, behind the fetch's read of them.
    for (auto &sp : c->shares) {
        Share &s = *sp;
        if ((st = on_device(s.physical)) != CORR_OK ||
            (st = cuda_check(cudaStreamWaitEvent(s.s_compute, s.taken, 0),
                             "cudaStreamWaitEvent(taken)")) != CORR_OK ||
            (st = cuda_check(cudaMemsetAsync(s.d_acc, 0,
                                             s.row_elems * sizeof(double2) *
                                                 static_cast<size_t>(rows),
                                             s.s_compute),
                             "cudaMemsetAsync(rows)")) != CORR_OK)
            return st;
    }
    if (cb != nullptr && (st = notify_after(c, {c->fetch_done}, cb, user)) != CORR_OK) return st;
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

// Everything one share needs on its device; maps and `taken` on the home device.
corr_status build_share(Context *c, Share &s, int home_physical) {
    const corr_config &cfg = c->cfg;
    const int n = s.n_local();
    corr_status st = on_device(s.physical);
    if (st != CORR_OK) return st;
    for (int i = 0; i < n;) {
        StationRun r;
        r.local0 = i;
        r.global0 = s.pl.stations[static_cast<size_t>(i)];
        while (i < n && s.pl.stations[static_cast<size_t>(i)] == r.global0 + (i - r.local0)) ++i;
        r.count = i - r.local0;
        s.runs.push_back(r);
    }
    if ((st = fxplan_create(s.physical, n, cfg.n_freq, cfg.chunk_frames, CORR_X_PLAIN_FP32,
                            &s.plan)) != CORR_OK)
        return st;
    s.plan->acc64 = 1;
    // A device of the baseline-range or pair-covering split owns only some
    // baselines of its stations' matrix: the plain X-engine computes only the
    // station-block pairs that hold them, so the devices divide its work.
    if (!c->time_slice && (st = fxplan_limit_baselines(s.plan, s.pl.local)) != CORR_OK)
        return st;
    s.ring_station_stride = static_cast<size_t>(cfg.chunk_frames) * c->lay.frame_stride;
    s.row_elems = static_cast<size_t>(n * (n + 1) / 2) * static_cast<size_t>(cfg.n_freq);
    const size_t ring_bytes = s.ring_station_stride * static_cast<size_t>(n);
    const size_t mask_bytes = c->lay.validity_bytes * static_cast<size_t>(n);
    for (int i = 0; i < kRing; ++i) {
        if (cudaMalloc(&s.d_samples[i], ring_bytes) != cudaSuccess ||
            cudaMalloc(&s.d_mask[i], mask_bytes) != cudaSuccess) {
            cudaGetLastError();
            return failf(CORR_ERR_NOMEM, "cudaMalloc(chunk ring, %zu bytes) failed", ring_bytes);
        }
    }
    const size_t acc_bytes =
        s.row_elems * sizeof(double2) * static_cast<size_t>(cfg.rows_per_fetch);
    if (cudaMalloc(&s.d_acc, acc_bytes) != cudaSuccess) {
        cudaGetLastError();
        return failf(CORR_ERR_NOMEM, "cudaMalloc(row stack, %zu bytes) failed", acc_bytes);
    }
    if ((st = cuda_check(cudaMemset(s.d_acc, 0, acc_bytes), "cudaMemset(rows)")) != CORR_OK)
        return st;
    for (cudaStream_t *p : {&s.s_copy, &s.s_compute})
        if (st == CORR_OK)
            st = cuda_check(cudaStreamCreateWithFlags(p, cudaStreamNonBlocking), "cudaStreamCreate");
    // Events that other devices wait on are created without timing, which a
    // cross-device wait requires.
    s.h2d_done.assign(static_cast<size_t>(cfg.block_slots), nullptr);
    for (auto &ev : s.h2d_done)
        if (st == CORR_OK)
            st = cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
    for (int i = 0; i < kRing; ++i)
        for (cudaEvent_t *ev : {&s.copy_done[i], &s.compute_done[i]})
            if (st == CORR_OK)
                st = cuda_check(cudaEventCreateWithFlags(ev, cudaEventDisableTiming),
                                "cudaEventCreate");
    if (st == CORR_OK)
        st = cuda_check(cudaEventCreateWithFlags(&s.row_done, cudaEventDisableTiming),
                        "cudaEventCreate");
    // Prime every "previous use finished" event so the first wait returns.
    for (int i = 0; i < kRing && st == CORR_OK; ++i)
        st = cuda_check(cudaEventRecord(s.compute_done[i], s.s_compute), "cudaEventRecord");
    for (auto &ev : s.h2d_done)
        if (st == CORR_OK) st = cuda_check(cudaEventRecord(ev, s.s_copy), "cudaEventRecord");
    if (st == CORR_OK) st = cuda_check(cudaEventRecord(s.row_done, s.s_compute), "cudaEventRecord");
    if (st != CORR_OK) return st;

    if ((st = on_device(home_physical)) != CORR_OK) return st;
    if ((st = cuda_check(cudaEventCreateWithFlags(&s.taken, cudaEventDisableTiming),
                         "cudaEventCreate")) != CORR_OK)
        return st;
    if (!c->time_slice && !placement_is_identity(s.pl, c->cfg.n_station)) {
        const size_t nb = s.pl.baselines.size();
        if ((st = cuda_check(cudaMalloc(&s.d_gmap, nb * sizeof(int32_t)), "cudaMalloc(map)")) !=
                CORR_OK ||
            (st = cuda_check(cudaMalloc(&s.d_lmap, nb * sizeof(int32_t)), "cudaMalloc(map)")) !=
                CORR_OK ||
            (st = cuda_check(cudaMemcpy(s.d_gmap, s.pl.baselines.data(), nb * sizeof(int32_t),
                                        cudaMemcpyHostToDevice),
                             "cudaMemcpy(map)")) != CORR_OK ||
            (st = cuda_check(cudaMemcpy(s.d_lmap, s.pl.local.data(), nb * sizeof(int32_t),
                                        cudaMemcpyHostToDevice),
                             "cudaMemcpy(map)")) != CORR_OK)
            return st;
    }
    return CORR_OK;
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
        banner = "corr_gb300 0.2.0 abi=" + std::to_string(CORR_ABI_VERSION) +
                 " cudart=" + std::to_string(rt) + " driver=" + std::to_string(drv) +
                 " fft=own-stockham arch=sm_103a target=GB300";
    });
    return banner.c_str();
}

extern "C" const char *corr_last_error(void) { return last_error().c_str(); }

extern "C" corr_status corrx_set_device_map(const int32_t *physical, int32_t n) {
    if (n < 0 || n > kMaxDeviceOrdinals)
        return failf(CORR_ERR_ARG, "n=%d outside [0, %d]", n, kMaxDeviceOrdinals);
    if (n > 0 && physical == nullptr) return fail(CORR_ERR_ARG, "physical is NULL");
    for (int i = 0; i < n; ++i)
        if (physical[i] < 0 || physical[i] >= kMaxDeviceOrdinals)
            return failf(CORR_ERR_ARG, "physical[%d]=%d is not a device ordinal", i, physical[i]);
    std::lock_guard<std::mutex> lock(g_map_mu);
    g_device_map.assign(physical, physical + n);
    return CORR_OK;
}

extern "C" corr_status corr_create(const corr_config *cfg, void **out_ctx) {
    if (out_ctx == nullptr) return fail(CORR_ERR_ARG, "out_ctx is NULL");
    *out_ctx = nullptr;
    corr_status st = validate(cfg);
    if (st != CORR_OK) return st;
    std::vector<int> ordinals, physical;
    if ((st = resolve_devices(*cfg, &ordinals, &physical)) != CORR_OK) return st;
    std::vector<DevicePlacement> plan;
    if ((st = plan_devices(cfg->n_station, cfg->split_mode, ordinals, &plan)) != CORR_OK)
        return st;

    Context *c = new (std::nothrow) Context();
    if (c == nullptr) return fail(CORR_ERR_NOMEM, "cannot allocate the context");
    c->cfg = *cfg;
    c->n_baseline = cfg->n_station * (cfg->n_station + 1) / 2;
    c->time_slice = cfg->split_mode == CORR_SPLIT_TIME_SLICE;
    c->lay = make_layout(*cfg);
    for (size_t d = 0; d < plan.size(); ++d) {
        std::unique_ptr<Share> s(new (std::nothrow) Share());
        if (!s) {
            free_context(c);
            return fail(CORR_ERR_NOMEM, "cannot allocate the context");
        }
        s->pl = plan[d];
        s->physical = physical[d];
        c->shares.push_back(std::move(s));
    }
    const int home_phys = physical[0];
    if ((st = on_device(home_phys)) != CORR_OK) {
        free_context(c);
        return st;
    }
    // Portable: every device of the context copies out of this one allocation.
    cudaError_t e = cudaHostAlloc(&c->staging, c->lay.total_bytes, cudaHostAllocPortable);
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
    c->row_frames.assign(static_cast<size_t>(cfg->rows_per_fetch), 1);

    // home-device resources: output rows, peer staging, fetch/notify streams
    for (cudaStream_t *s : {&c->s_fetch, &c->s_notify})
        if (st == CORR_OK)
            st = cuda_check(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking), "cudaStreamCreate");
    if (st == CORR_OK)
        st = cuda_check(cudaEventCreateWithFlags(&c->fetch_done, cudaEventDisableTiming),
                        "cudaEventCreate");
    if (st == CORR_OK && cudaMalloc(&c->d_out, c->out_bytes()) != cudaSuccess) {
        cudaGetLastError();
        st = failf(CORR_ERR_NOMEM, "cudaMalloc(output rows, %zu bytes) failed", c->out_bytes());
    }
    for (size_t d = 1; d < c->shares.size(); ++d) {
        const int n = static_cast<int>(c->shares[d]->pl.stations.size());
        c->peer_elems = std::max(c->peer_elems, static_cast<size_t>(n * (n + 1) / 2) *
                                                    static_cast<size_t>(cfg->n_freq) *
                                                    static_cast<size_t>(cfg->rows_per_fetch));
    }
    if (st == CORR_OK && c->peer_elems > 0 &&
        cudaMalloc(&c->d_peer, c->peer_elems * sizeof(double2)) != cudaSuccess) {
        cudaGetLastError();
        st = failf(CORR_ERR_NOMEM, "cudaMalloc(peer rows, %zu bytes) failed",
                   c->peer_elems * sizeof(double2));
    }
    if (st == CORR_OK) st = cuda_check(cudaEventRecord(c->fetch_done, c->s_fetch), "cudaEventRecord");
    for (auto &s : c->shares)
        if (st == CORR_OK) st = build_share(c, *s, home_phys);
    // The first host function a process queues starts CUDA's callback thread;
    // do that here, so the first *_submit call costs what every later one does.
    if (st == CORR_OK && (st = on_device(home_phys)) == CORR_OK)
        st = cuda_check(cudaLaunchHostFunc(c->s_notify, [](void *) {}, nullptr),
                        "cudaLaunchHostFunc(warm-up)");
    for (auto &s : c->shares)
        if (st == CORR_OK && (st = on_device(s->physical)) == CORR_OK)
            st = cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize(create)");
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
    corr_status st = CORR_OK;
    for (auto &s : c->shares) {
        corr_status s2 = on_device(s->physical);
        if (s2 == CORR_OK)
            s2 = cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize(destroy)");
        if (s2 != CORR_OK && st == CORR_OK) st = s2;
    }
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
    int first = 0, last = 0;
    readers_of(c, slot_seq, &first, &last);
    for (int d = first; d < last && st == CORR_OK; ++d) {
        Share &s = *c->shares[static_cast<size_t>(d)];
        const uint64_t t0 = now_ns();
        if ((st = on_device(s.physical)) == CORR_OK) st = accumulate_slot(c, s, slot, frames);
        s.timing.accumulate += now_ns() - t0;
    }
    if (st != CORR_OK) {
        std::lock_guard<std::mutex> lock(c->mu);
        c->slots[static_cast<size_t>(slot)] = Slot::kFree;
        return st;
    }
    c->dirty = true;
    return CORR_OK;
}

extern "C" corr_status corr_row_slot_free(void *h, int64_t slot_seq) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    int32_t slot = 0;
    corr_status st = slot_of(c, slot_seq, &slot);
    if (st != CORR_OK || (st = expect_copying(c, slot, slot_seq)) != CORR_OK) return st;
    int first = 0, last = 0;
    readers_of(c, slot_seq, &first, &last);
    for (int d = first; d < last && st == CORR_OK; ++d) {
        Share &s = *c->shares[static_cast<size_t>(d)];
        const uint64_t t0 = now_ns();
        if ((st = on_device(s.physical)) == CORR_OK)
            st = cuda_check(cudaEventSynchronize(s.h2d_done[static_cast<size_t>(slot)]),
                            "cudaEventSynchronize(h2d_done)");
        s.timing.slot_free += now_ns() - t0;
    }
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
    int first = 0, last = 0;
    readers_of(c, slot_seq, &first, &last);
    std::vector<cudaEvent_t> evs;
    for (int d = first; d < last; ++d)
        evs.push_back(c->shares[static_cast<size_t>(d)]->h2d_done[static_cast<size_t>(slot)]);
    const uint64_t t0 = now_ns();
    st = notify_after(c, evs, cb, user);
    c->shares[static_cast<size_t>(first)]->timing.slot_free += now_ns() - t0;
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
    // The copies are known complete (the callback fired); surface a failed copy.
    int first = 0, last = 0;
    readers_of(c, slot_seq, &first, &last);
    for (int d = first; d < last && st == CORR_OK; ++d) {
        Share &s = *c->shares[static_cast<size_t>(d)];
        if ((st = on_device(s.physical)) == CORR_OK)
            st = query(s.h2d_done[static_cast<size_t>(slot)], "cudaEventQuery(h2d_done)");
    }
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
    // Every share closes the row at once. The division by `frames` (the
    // reference's scale_row_kernel, kernels.cu:178-185) is applied when the row
    // is rounded to complex64 at the fetch, in double precision.
    corr_status st = CORR_OK;
    for (auto &sp : c->shares) {
        Share &s = *sp;
        const uint64_t t0 = now_ns();
        if ((st = on_device(s.physical)) == CORR_OK)
            st = cuda_check(cudaEventRecord(s.row_done, s.s_compute), "cudaEventRecord(row_done)");
        s.timing.row_end += now_ns() - t0;
        if (st != CORR_OK) return st;
    }
    c->row_frames[static_cast<size_t>(c->cur_row)] = frames;
    ++c->pending;
    if (++c->cur_row >= c->cfg.rows_per_fetch) c->cur_row = 0;
    return CORR_OK;
}

extern "C" corr_status corr_rows_wait(void *h) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    for (auto &sp : c->shares) {
        Share &s = *sp;
        const uint64_t t0 = now_ns();
        corr_status st = on_device(s.physical);
        if (st == CORR_OK)
            st = cuda_check(cudaEventSynchronize(s.row_done), "cudaEventSynchronize(row_done)");
        if (st == CORR_OK) st = watchdog(s);
        s.timing.rows_wait += now_ns() - t0;
        if (st != CORR_OK) return st;
    }
    return CORR_OK;
}

extern "C" corr_status corr_rows_wait_submit(void *h, corr_notify_fn cb, void *user) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (cb == nullptr) return fail(CORR_ERR_ARG, "cb is NULL");
    std::vector<cudaEvent_t> evs;
    for (auto &s : c->shares) evs.push_back(s->row_done);
    const uint64_t t0 = now_ns();
    corr_status st = notify_after(c, evs, cb, user);
    c->home().timing.rows_wait += now_ns() - t0;
    return st;
}

extern "C" corr_status corr_rows_ready(void *h) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    for (auto &s : c->shares) {
        corr_status st = on_device(s->physical);
        if (st == CORR_OK) st = query(s->row_done, "cudaEventQuery(row_done)");
        if (st != CORR_OK) return st;
    }
    return watchdog_all(c);
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
    // As the reference (corr_cuda.cpp:1236-1240): pair covering over several
    // devices, whose devices report scattered baselines, has only the blocking
    // fetch.
    bool scattered = c->cfg.split_mode == CORR_SPLIT_PAIR_COVERING && c->n_devices() > 1;
    if (!c->time_slice)
        for (auto &s : c->shares) scattered = scattered || !s->pl.contiguous;
    if (scattered)
        return fail(CORR_ERR_NOT_IMPL,
                    "this split places scattered baselines into the row; corr_rows_fetch() "
                    "is the way to fetch under it");
    const uint64_t t0 = now_ns();
    corr_status st = fetch_submit(c, out, out_bytes, out_rows, cb, user);
    c->home().timing.fetch += now_ns() - t0;
    return st;
}

extern "C" corr_status corr_rows_fetch_ready(void *h) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    corr_status st = on_device(c->home().physical);
    if (st == CORR_OK) st = query(c->fetch_done, "cudaEventQuery(fetch_done)");
    return st;
}

extern "C" corr_status corr_rows_fetch(void *h, void *out, size_t out_bytes, int32_t *out_rows) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (out == nullptr) return fail(CORR_ERR_ARG, "out is NULL");
    if (out_rows == nullptr) return fail(CORR_ERR_ARG, "out_rows is NULL");
    const uint64_t t0 = now_ns();
    corr_status st = fetch_submit(c, out, out_bytes, out_rows, nullptr, nullptr);
    if (st == CORR_OK && *out_rows > 0) {
        if ((st = on_device(c->home().physical)) == CORR_OK)
            st = cuda_check(cudaEventSynchronize(c->fetch_done), "cudaEventSynchronize(fetch_done)");
        if (st == CORR_OK) st = watchdog_all(c);
    }
    c->home().timing.fetch += now_ns() - t0;
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

extern "C" int32_t corr_n_devices(void *h) {
    Context *c = as_ctx(h);
    return c == nullptr ? -1 : c->n_devices();
}

static corr_status share_at(Context *c, int32_t device_index, Share **out) {
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (device_index < 0 || device_index >= c->n_devices())
        return failf(CORR_ERR_ARG, "device_index %d out of range [0,%d)", device_index,
                     c->n_devices());
    *out = c->shares[static_cast<size_t>(device_index)].get();
    return CORR_OK;
}

extern "C" corr_status corr_device_plan_get(void *h, int32_t device_index, corr_device_plan *out) {
    Share *s = nullptr;
    corr_status st = share_at(as_ctx(h), device_index, &s);
    if (st != CORR_OK) return st;
    if (out == nullptr) return fail(CORR_ERR_ARG, "out is NULL");
    fill_device_plan(s->pl, out);
    return CORR_OK;
}

extern "C" corr_status corr_device_stations(void *h, int32_t device_index, int32_t *out_stations,
                                            int32_t out_len) {
    Share *s = nullptr;
    corr_status st = share_at(as_ctx(h), device_index, &s);
    if (st != CORR_OK) return st;
    if (out_stations == nullptr) return fail(CORR_ERR_ARG, "out_stations is NULL");
    if (out_len < s->n_local())
        return failf(CORR_ERR_ARG, "out_len=%d but device %d holds %d stations", out_len,
                     device_index, s->n_local());
    std::copy(s->pl.stations.begin(), s->pl.stations.end(), out_stations);
    return CORR_OK;
}

extern "C" corr_status corr_device_baselines(void *h, int32_t device_index, int32_t *out_baselines,
                                             int32_t out_len) {
    Share *s = nullptr;
    corr_status st = share_at(as_ctx(h), device_index, &s);
    if (st != CORR_OK) return st;
    if (out_baselines == nullptr) return fail(CORR_ERR_ARG, "out_baselines is NULL");
    const int nb = static_cast<int>(s->pl.baselines.size());
    if (out_len < nb)
        return failf(CORR_ERR_ARG, "out_len=%d but device %d owns %d baselines", out_len,
                     device_index, nb);
    std::copy(s->pl.baselines.begin(), s->pl.baselines.end(), out_baselines);
    return CORR_OK;
}

extern "C" corr_status corr_device_stats_get(void *h, int32_t device_index, corr_device_stats *out) {
    Share *s = nullptr;
    corr_status st = share_at(as_ctx(h), device_index, &s);
    if (st != CORR_OK) return st;
    if (out == nullptr) return fail(CORR_ERR_ARG, "out is NULL");
    out->device_id = s->pl.ordinal;
    out->bytes_h2d = s->bytes_h2d;
    out->bytes_d2h = s->bytes_d2h;
    out->transfers = s->transfers;
    out->ns_accumulate = s->timing.accumulate;
    out->ns_slot_free = s->timing.slot_free;
    out->ns_row_end = s->timing.row_end;
    out->ns_rows_wait = s->timing.rows_wait;
    out->ns_fetch = s->timing.fetch;
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

// --- extensions on ABI contexts (corr_gb300.h) --------------------------------

static corr_status idle(Context *c, const char *what) {
    if (c->dirty || c->pending != 0)
        return failf(CORR_ERR_STATE,
                     "%s can only change while no row holds data (after create or a fetch)", what);
    return CORR_OK;
}

extern "C" corr_status corr_set_xengine(void *h, int32_t mode) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (mode != CORR_X_PLAIN_FP32 && mode != CORR_X_TC_FP16 && mode != CORR_X_TC_FP16_SPLIT)
        return failf(CORR_ERR_ARG, "unknown X-engine mode %d", mode);
    corr_status st = idle(c, "the X-engine");
    if (st != CORR_OK) return st;
    for (auto &s : c->shares) {
        FxPlan *p = s->plan;
        if (mode != CORR_X_PLAIN_FP32) {
            int ct = 0, kt = 0;
            xengine_tc_default_shape(p->n_station, mode == CORR_X_TC_FP16_SPLIT, &ct, &kt);
            if (ct == 0)
                return failf(CORR_ERR_NOT_IMPL,
                             "the tensor X-engine takes 1..64 inputs (n_station=%d)", p->n_station);
        }
    }
    for (auto &s : c->shares) {
        FxPlan *p = s->plan;
        if (mode != CORR_X_PLAIN_FP32) {
            int ct = 0, kt = 0;
            xengine_tc_default_shape(p->n_station, mode == CORR_X_TC_FP16_SPLIT, &ct, &kt);
            p->xct = ct;
            p->xkt = kt;
            if (p->ytile < ct) p->ytile = p->n_freq;
        }
        p->xmode = mode;
        // an FFT plan that cannot write this mode's spectra falls back to plan 0
        if (!fengine_plan_ok(p->n_freq, p->fplan, spectra_format(mode))) p->fplan = 0;
    }
    return CORR_OK;
}

extern "C" corr_status corr_get_tiles(void *h, corrx_tiles *out) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    return corrx_get_tiles(c->home().plan, out);
}

extern "C" corr_status corr_set_tiles(void *h, const corrx_tiles *t) {
    Context *c = as_ctx(h);
    if (c == nullptr || t == nullptr) return fail(CORR_ERR_ARG, "ctx and t must be non-NULL");
    corr_status st = idle(c, "tiles");
    for (auto &s : c->shares)
        if (st == CORR_OK) st = corrx_set_tiles(s->plan, t);
    return st;
}

extern "C" corr_status corr_autotune(void *h, corrx_tiles *out) {
    Context *c = as_ctx(h);
    if (c == nullptr) return fail(CORR_ERR_ARG, "ctx is NULL");
    if (out != nullptr && out->struct_size != sizeof(corrx_tiles))
        return failf(CORR_ERR_ABI, "corrx_tiles.struct_size=%u, expected %zu", out->struct_size,
                     sizeof(corrx_tiles));
    corr_status st = idle(c, "tiles");
    // each device tunes for its own share (its resident station count)
    for (size_t d = 0; d < c->shares.size() && st == CORR_OK; ++d) {
        Share &s = *c->shares[d];
        if ((st = on_device(s.physical)) == CORR_OK)
            st = fxplan_autotune(s.plan, s.s_compute, d == 0 ? out : nullptr);
    }
    return st;
}
