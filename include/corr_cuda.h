/*
 * corr_cuda.h -- C ABI of the GB300 FX correlator engine.
 *
 * This is the drop-in contract for the GPU half of the 21CMA correlator: the
 * names, values, structure layouts and call semantics are those of ABI v7 of
 * the reference library (corr-cuda/include/corr_cuda.h), so a host built
 * against that header (the Rust corr-rs crate, or the C tests) links against
 * this library's libcorr_cuda.so unchanged. Each entry point below names the
 * reference declaration it replaces.
 *
 * What happens behind it is new: int8 frames are unpacked, zero-filled where the
 * validity mask says a frame is missing, and transformed by a hand-written
 * real-to-complex FFT (no cuFFT), then correlated over every baseline j <= k by
 * an X-engine (FP32 SIMT by default; tcgen05 tensor cores on request, see
 * corr_gb300.h).
 *
 * Accumulation model (unchanged from the reference):
 *
 *   create                  -> row stack zeroed, row 0 active
 *   accumulate(slot) * K    -> acc[row] += correlation of that slot's frames
 *   end(frames)             -> acc[row] /= frames; the next row becomes active
 *   rows_wait()             -> every closed row has been scaled
 *   rows_fetch(out)         -> one device-to-host copy of the closed rows, then clear
 *
 * Staging: the library owns a page-locked ring of `block_slots` slots per
 * station. Receive threads write int8 frames and validity bits into it; the
 * scheduler hands a slot to the GPU with corr_row_accumulate() and gets it back
 * with corr_row_slot_free(). A context is driven by one thread; the receive
 * threads only ever touch staging bytes.
 */

#ifndef CORR_CUDA_H
#define CORR_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ABI version. v7 is the version in which the validity mask is read by the
   device and cleared by corr_row_slot_free() (corr_cuda.h:94 in the reference). */
#define CORR_ABI_VERSION 7u

/* Split modes (reference corr_cuda.h:113-137): how a context with several
   devices shares the work. TIME_SLICE routes slot sequence s to device
   s % n_devices, each device holds every station and a partial row of every
   baseline, and the fetch adds the partial rows. BASELINE_RANGE and
   PAIR_COVERING copy every slot to every device; each device reports a set of
   baselines (a contiguous range of them, over every station; or the baselines
   among a subset of stations, each baseline on exactly one device) and the
   fetch assembles the row. corrx_plan_query (corr_gb300.h) states the
   placements exactly. */
#define CORR_SPLIT_BASELINE_RANGE 0
#define CORR_SPLIT_PAIR_COVERING 1
#define CORR_SPLIT_TIME_SLICE 2

/* Size of the fixed device list in corr_config (reference corr_cuda.h:141). */
#define CORR_MAX_DEVICES 8u

/* Status codes (reference corr_cuda.h:143-154). CORR_ERR_CUFFT keeps its value
   for layout compatibility; this library has no cuFFT and never returns it. */
typedef enum corr_status {
    CORR_OK           = 0,
    CORR_ERR_ARG      = 1, /* bad or inconsistent argument               */
    CORR_ERR_ABI      = 2, /* abi_version / struct_size mismatch         */
    CORR_ERR_CUDA     = 3, /* CUDA runtime or driver error               */
    CORR_ERR_CUFFT    = 4, /* reserved (reference: cuFFT error)          */
    CORR_ERR_STATE    = 5, /* call out of order for this context or slot */
    CORR_ERR_BUSY     = 6, /* slot or row stack still owned by the GPU   */
    CORR_ERR_NOMEM    = 7, /* host or device allocation failed           */
    CORR_ERR_NOT_IMPL = 8, /* not supported by this library              */
    CORR_ERR_INTERNAL = 9  /* device-side watchdog or invariant failure  */
} corr_status;

/*
 * Instance description, 76 bytes (reference corr_cuda.h:171-196).
 *
 * Checked by corr_create():
 *   abi_version == CORR_ABI_VERSION and struct_size == sizeof(corr_config)
 *                                              (else CORR_ERR_ABI)
 *   1 <= n_station <= 128, and every configured device owns at most 1024
 *       baselines under the split (the reference's per-device limit,
 *       corr-cuda/src/kernels.cu:474-483): n_station <= 44 on one device or
 *       under the time slice (every device owns every baseline); more stations
 *       when the baseline range or pair covering split them over devices
 *   n_freq a multiple of 2048 up to 32768, as the reference requires (a
 *       frame must be whole 4096-sample packets), or 512 or 1024 (the engine
 *       only needs a transform length it has a plan for). Multiples of 2048
 *       above 32768 return CORR_ERR_NOT_IMPL, everything else CORR_ERR_ARG.
 *   frames_per_slot >= 1, 1 <= chunk_frames <= frames_per_slot
 *   block_slots >= 2, rows_per_fetch >= 1
 *   the device ordinal(s) exist and are distinct; the split gives every
 *       device at least one baseline
 */
typedef struct corr_config {
    uint32_t abi_version;
    uint32_t struct_size;
    int32_t  device_id;       /* used when n_devices == 0                     */
    int32_t  n_station;       /* N inputs; N*(N+1)/2 baselines incl. autos    */
    int32_t  n_freq;          /* retained channels; frame = 2*n_freq samples  */
    int32_t  frames_per_slot; /* frames one staging slot holds per station    */
    int32_t  chunk_frames;    /* frames per host-to-device copy               */
    int32_t  block_slots;     /* slots in the staging ring                    */
    int32_t  rows_per_fetch;  /* rows held on the device between fetches      */
    int32_t  n_devices;       /* 0 = just device_id; else entries of devices  */
    int32_t  devices[CORR_MAX_DEVICES];
    int32_t  split_mode;      /* CORR_SPLIT_*                                 */
} corr_config;

/* One device's share (reference corr_cuda.h:209-219), 20 bytes. */
typedef struct corr_device_plan {
    int32_t device_id;
    int32_t n_station_resident;
    int32_t first_baseline;
    int32_t n_baseline;
    int32_t contiguous;
} corr_device_plan;

/* Cumulative counters for one device (reference corr_cuda.h:229-245), 72 bytes. */
typedef struct corr_device_stats {
    int32_t  device_id;
    uint64_t bytes_h2d;     /* staging bytes copied to the device           */
    uint64_t bytes_d2h;     /* visibility bytes copied back                 */
    uint64_t transfers;     /* host-to-device chunk copies issued           */
    uint64_t ns_accumulate; /* calling-thread ns inside each call, summed   */
    uint64_t ns_slot_free;
    uint64_t ns_row_end;
    uint64_t ns_rows_wait;
    uint64_t ns_fetch;
} corr_device_stats;

/*
 * One station's staging region (reference corr_cuda.h:262-294), 48 bytes.
 * `base` already points at the station. Frame f of slot s starts at
 *   base + s*slot_stride + f*frame_stride
 * and holds 2*n_freq two's-complement int8 samples. The validity mask of slot
 * s is `validity_bytes_per_slot` bytes at base + validity_offset +
 * s*validity_bytes_per_slot: bit f (LSB first, byte f/8) set means frame f is
 * present. A clear bit makes the device treat the frame as all zeros. The mask
 * starts all-zero and corr_row_slot_free() clears it again.
 */
typedef struct corr_staging {
    int8_t *base;
    size_t  frame_stride;            /* 2*n_freq                               */
    size_t  slot_stride;             /* frames_per_slot*frame_stride           */
    size_t  total_bytes;             /* this station's extent, samples + mask  */
    size_t  validity_offset;         /* block_slots*slot_stride                */
    size_t  validity_bytes_per_slot; /* ceil(frames_per_slot/8)                */
} corr_staging;

/* Library banner; contains "abi=7" (reference corr_cuda.h:301). */
const char *corr_abi_banner(void);

/* Thread-local message of the last failure on this thread, "" if none
   (reference corr_cuda.h:307). Never NULL. */
const char *corr_last_error(void);

/* Validate, allocate staging and device state, zero the row stack
   (reference corr_cuda.h:317). *out_ctx is NULL on failure. */
corr_status corr_create(const corr_config *cfg, void **out_ctx);

/* Drain and free a context; NULL is a no-op (reference corr_cuda.h:320). */
corr_status corr_destroy(void *ctx);

/* Where station `station` writes (reference corr_cuda.h:326). */
corr_status corr_staging_info(void *ctx, int32_t station, corr_staging *out);

/*
 * Queue slot `slot_seq % block_slots` (frames 0..frames-1 of every station) for
 * correlation into the active row (reference corr_cuda.h:356). Returns once
 * queued. CORR_ERR_ARG for a negative sequence or frames outside
 * [1, frames_per_slot]; CORR_ERR_BUSY if the slot was submitted and not freed.
 */
corr_status corr_row_accumulate(void *ctx, int64_t slot_seq, int32_t frames);

/* Block until the slot's host-to-device copy is done, clear its mask, hand it
   back (reference corr_cuda.h:371). CORR_ERR_STATE if it was not submitted. */
corr_status corr_row_slot_free(void *ctx, int64_t slot_seq);

/* Callback form of the release (reference corr_cuda.h:399-412). `cb(user)` runs
   on a CUDA thread once the copy is done and may only signal; the caller then
   completes the release with corr_row_slot_free_finish(). */
typedef void (*corr_notify_fn)(void *user);
corr_status corr_row_slot_free_submit(void *ctx, int64_t slot_seq,
                                      corr_notify_fn cb, void *user);
corr_status corr_row_slot_free_finish(void *ctx, int64_t slot_seq);

/* Close the active row, dividing it by `frames` (the caller's count, not the
   valid-frame count). CORR_ERR_ARG for 0, CORR_ERR_BUSY when rows_per_fetch
   rows are already waiting to be fetched (reference corr_cuda.h:428). */
corr_status corr_row_end(void *ctx, uint64_t frames);

/* Block until every closed row is scaled (reference corr_cuda.h:434). */
corr_status corr_rows_wait(void *ctx);

/* Callback form of corr_rows_wait (reference corr_cuda.h:445). */
corr_status corr_rows_wait_submit(void *ctx, corr_notify_fn cb, void *user);

/* 0 when the closed rows are done, CORR_ERR_BUSY while running, an error when
   they failed (reference corr_cuda.h:452). */
corr_status corr_rows_ready(void *ctx);

/* Closed rows waiting to be fetched, in [0, rows_per_fetch]
   (reference corr_cuda.h:459). */
corr_status corr_rows_pending(void *ctx, int32_t *out_pending);

/*
 * Copy the closed rows to `out` and clear them (reference corr_cuda.h:487).
 * out_bytes >= rows_per_fetch*n_baseline*n_freq*8. Layout
 * out[(row*n_baseline + baseline)*n_freq + bin], complex64, real first; bin 0
 * is DC, the Nyquist bin is dropped, no FFT normalisation, already divided by
 * the row's frame count. *out_rows = rows written (0 is valid).
 */
corr_status corr_rows_fetch(void *ctx, void *out, size_t out_bytes, int32_t *out_rows);

/* Callback form of the fetch (reference corr_cuda.h:511): *out_rows is set on
   return, `cb(user)` fires once the bytes are in `out`. */
corr_status corr_rows_fetch_submit(void *ctx, void *out, size_t out_bytes,
                                   int32_t *out_rows, corr_notify_fn cb, void *user);

/* 0 when the last fetch completed, CORR_ERR_BUSY while in flight
   (reference corr_cuda.h:520). */
corr_status corr_rows_fetch_ready(void *ctx);

/* n_station*(n_station+1)/2, or -1 for n_station < 1 (reference corr_cuda.h:529). */
int32_t corr_n_baseline(int32_t n_station);

/* Baseline table, row-major over j <= k: out_jk[2i] = j, out_jk[2i+1] = k;
   out_len must equal 2*corr_n_baseline(n_station) (reference corr_cuda.h:542). */
corr_status corr_baseline_pairs(int32_t n_station, int32_t *out_jk, int32_t out_len);

/* Device introspection (reference corr_cuda.h:561-584). */
int32_t corr_n_devices(void *ctx);
corr_status corr_device_plan_get(void *ctx, int32_t device_index, corr_device_plan *out);
corr_status corr_device_stations(void *ctx, int32_t device_index,
                                 int32_t *out_stations, int32_t out_len);
corr_status corr_device_baselines(void *ctx, int32_t device_index,
                                  int32_t *out_baselines, int32_t out_len);
corr_status corr_device_stats_get(void *ctx, int32_t device_index, corr_device_stats *out);

/* Page-locked host buffer for fetches, and its release (reference corr_cuda.h:603-604). */
corr_status corr_host_alloc(size_t bytes, void **out);
void corr_host_free(void *p);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* CORR_CUDA_H */
