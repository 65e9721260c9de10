/*
 * corr_gb300.h -- extensions of the GB300 engine beyond the reference ABI.
 *
 * None of these has a counterpart in the reference's public header; they expose
 * what the reference keeps internal (corr-cuda/src/gpu_internal.h, the per-chunk
 * work of gpu_accumulate at corr-cuda/src/kernels.cu:684-857) so that callers
 * holding data already in device memory -- benchmarks, a batching front end, a
 * multi-integration replay -- can drive the F- and X-engines without going
 * through the pinned staging ring. The same kernels run behind corr_cuda.h.
 *
 * All device pointers are plain CUDA device addresses; `stream` is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).
 */

#ifndef CORR_GB300_H
#define CORR_GB300_H

#include "corr_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* X-engine forms. */
#define CORR_X_PLAIN_FP32    0 /* FP32 SIMT complex multiply-accumulate (default)     */
#define CORR_X_TC_FP16       1 /* tcgen05: FP16 spectra, per-channel power-of-two
                                  scale, FP32 accumulation in tensor memory          */
#define CORR_X_TC_FP16_SPLIT 2 /* as CORR_X_TC_FP16 with a hi/lo split product that
                                  recovers about 22 bits of the spectra               */

/* Select the X-engine of an ABI context. Allowed only while no row holds data
   (after corr_create, or right after a fetch). */
corr_status corr_set_xengine(void *ctx, int32_t mode);

typedef struct corrx_params {
    uint32_t struct_size; /* sizeof(corrx_params)                                 */
    int32_t  n_station;   /* 1..128 (the tensor X-engines: 1..64)                 */
    int32_t  n_freq;      /* 512, 1024, or a multiple of 2048 up to 32768          */
    int32_t  max_frames;  /* frames per F/X pass; sizes the spectra buffer
                             (max_frames*n_station*n_freq*8 bytes)               */
    int32_t  xmode;       /* CORR_X_*                                             */
    int32_t  device_id;   /* CUDA ordinal                                         */
} corrx_params;

/* Create / destroy a device-resident engine (spectra buffer, twiddle tables,
   watchdog flag). */
corr_status corrx_create(const corrx_params *p, void **out_eng);
corr_status corrx_destroy(void *eng);

/*
 * acc[b*n_freq + c] += sum over frames f < `frames` of Y_j[f][c]*conj(Y_k[f][c])
 * for every baseline b = (j,k), j <= k, in corr_baseline_pairs() order.
 *
 * Frame f of station s is 2*n_freq int8 samples at
 *   d_samples + s*station_stride + f*frame_stride            (16-byte aligned)
 * If d_mask is not NULL, frame f of station s is treated as all zeros unless bit
 * (mask_bit0 + f) of the bit string at d_mask + s*mask_station_stride is set
 * (LSB first), exactly as the staging validity mask is read.
 * d_acc holds n_baseline*n_freq complex64 (FP32 re, im), or complex128 for an
 * engine with the FP64 accumulator (corrx_set_accumulator), must not alias, and
 * must be 16-byte aligned.
 */
corr_status corrx_accumulate(void *eng, const int8_t *d_samples, size_t station_stride,
                             size_t frame_stride, const uint8_t *d_mask,
                             size_t mask_station_stride, int32_t mask_bit0, int32_t frames,
                             void *d_acc, void *stream);

/*
 * corrx_accumulate with packet-granular loss: the samples of frame f of station s
 * are taken in 1024-sample packets, and packet p counts as all zeros unless bit p
 * of the 32-bit word d_pmask[s*pmask_station_stride + pmask_frame0 + f] is set
 * (bit 0 = the frame's first 1024 samples). A frame with no packet left is
 * skipped like a frame whose d_mask bit is clear (d_mask may be NULL). No
 * counterpart in the reference, whose receive side zero-fills whole frames; its
 * ABI path keeps that rule. 2*n_freq <= 32768 (at most 32 packets per frame).
 */
corr_status corrx_accumulate_packets(void *eng, const int8_t *d_samples, size_t station_stride,
                                     size_t frame_stride, const uint8_t *d_mask,
                                     size_t mask_station_stride, int32_t mask_bit0,
                                     const uint32_t *d_pmask, size_t pmask_station_stride,
                                     int32_t pmask_frame0, int32_t frames, void *d_acc,
                                     void *stream);

/* d_acc *= 1.0f/(float)frames over n_baseline*n_freq complex values (in double
   precision for an engine with the FP64 accumulator). */
corr_status corrx_scale(void *eng, void *d_acc, uint64_t frames, void *stream);

/*
 * Accumulator precision of an engine. Every X-engine launch sums its frames in
 * FP32 (registers or tensor memory) and adds that partial sum into d_acc once.
 * CORRX_ACC_FP32 (the default): d_acc holds complex64, as the reference's row
 * (corr-cuda/src/kernels.cu:252-264 accumulates complex64 across chunks).
 * CORRX_ACC_FP64: d_acc holds complex128 (16 bytes per visibility), so a row
 * summed over many launches keeps the precision of one launch; corrx_dump
 * turns it into complex64. Applies to every later corrx_accumulate*,
 * corrx_run_xengine, corrx_scale and batch created from the engine. The ABI
 * contexts of corr_cuda.h always integrate in complex128 and hand back
 * complex64 rows.
 */
#define CORRX_ACC_FP32 0
#define CORRX_ACC_FP64 1
corr_status corrx_set_accumulator(void *eng, int32_t precision);

/* d_out (complex64, n_baseline*n_freq) = d_acc * (1/frames), rounded once from
   the accumulator's precision; d_out may equal d_acc for an FP32 accumulator.
   Both 16-byte aligned. */
corr_status corrx_dump(void *eng, const void *d_acc, uint64_t frames, void *d_out,
                       void *stream);

/*
 * Device ordinals of ABI contexts created after this call: configured device i
 * (corr_config.devices[i], or device_id) runs on CUDA device physical[i]
 * (i < n); n = 0 restores the identity. Process-wide. Meant for tests: several
 * configured devices may share one GPU, each with its own buffers, streams and
 * share of the work, so the multi-device paths (time slice, baseline range,
 * pair covering) run on a one-GPU machine exactly as they would on several.
 * No counterpart in the reference.
 */
corr_status corrx_set_device_map(const int32_t *physical, int32_t n);

/*
 * The placement corr_create would make for `cfg` on device index
 * `device_index` (what corr_device_plan_get, corr_device_stations and
 * corr_device_baselines report for it), computed on the host alone: no device
 * is touched, so it works on a machine without a GPU. out_local receives, for
 * each reported baseline, its index among the device's own baselines (j <= k
 * over its stations, row-major). Any array may be NULL; a shorter array than
 * the plan is CORR_ERR_ARG. Splits (CORR_SPLIT_*):
 *   time slice     -- every device: every station, every baseline (a partial
 *                     row over the slots with slot_seq % n_devices == index);
 *   baseline range -- every device: every station, a contiguous range of
 *                     n_baseline/n_devices baselines (+1 for the first
 *                     n_baseline % n_devices devices);
 *   pair covering  -- the stations are cut into m contiguous groups, m the
 *                     largest with m(m-1)/2 <= n_devices; device d holds the
 *                     d-th pair of groups (cyclically), and each baseline goes
 *                     to the least-loaded device holding both its stations.
 * No counterpart in the reference, whose planner runs inside corr_create.
 */
corr_status corrx_plan_query(const corr_config *cfg, int32_t device_index,
                             corr_device_plan *out, int32_t *out_stations,
                             int32_t stations_len, int32_t *out_baselines,
                             int32_t baselines_len, int32_t *out_local, int32_t local_len);

/* Synchronise the engine's device and report a tripped device watchdog
   (CORR_ERR_INTERNAL) or a CUDA error. */
corr_status corrx_check(void *eng);

/*
 * Tile shapes of an engine. ytile is the spectra layout between the F- and
 * X-engines: n_freq = one contiguous row per (frame, station); a smaller power
 * of two = channel tiles of that width holding every frame and station (any
 * width for the plain X-engine; for the tensor forms only ytile = xct, where a
 * stage is one contiguous block). xct and xkt are the tensor X-engine's
 * channels per CTA tile (2, 4, 8) and frames per pipeline stage (16, 32, 64);
 * the plain X-engine ignores them. corrx_create picks contiguous rows and the
 * widest feasible tensor tile with 32-frame stages (16 if none fits).
 */
typedef struct corrx_tiles {
    uint32_t struct_size; /* sizeof(corrx_tiles)                                   */
    int32_t  ytile;
    int32_t  xct;
    int32_t  xkt;
    int32_t  fplan;       /* F-engine FFT plan: 0 (three passes; four at the
                             lengths that are not powers of two), or at n_freq
                             16384 also 1 (four passes, twice the threads) and,
                             with FP16 spectra (CORR_X_TC_FP16) only, 2 (the
                             DFT stages as tcgen05 matrix products; faster, with
                             about 1.5x the FP16 path's error; set explicitly,
                             corrx_autotune keeps to plans 0 and 1)              */
    float    ms_fengine;  /* corrx_autotune: F-engine ms per max_frames pass       */
    float    ms_xengine;  /* corrx_autotune: X-engine ms per max_frames pass       */
} corrx_tiles;

corr_status corrx_get_tiles(void *eng, corrx_tiles *out);
/* CORR_ERR_ARG for an infeasible shape; the spectra buffer's previous contents
   become meaningless (run the F-engine again). */
corr_status corrx_set_tiles(void *eng, const corrx_tiles *t);
/* Time FFT plans 0 and 1 and every feasible (ytile, xct, xkt) on this device --
   F- and X-engine passes of min(max_frames, 1024) synthetic frames (temporary
   device buffers of that many frames plus one row) -- keep the fastest F-engine
   plan and X-engine tile and report them in *out (may be NULL). Plan 2 (less
   precise) is never chosen here; corrx_set_tiles selects it. Synchronises
   `stream`. */
corr_status corrx_autotune(void *eng, void *stream, corrx_tiles *out);

/* corrx_autotune for the engine inside an ABI context; allowed only while no
   row holds data, like corr_set_xengine. */
corr_status corr_autotune(void *ctx, corrx_tiles *out);
/* corrx_get_tiles / corrx_set_tiles for the engine inside an ABI context (set
   only while no row holds data), e.g. to choose FFT plan 2 for the FP16 form.
   corr_set_xengine resets an FFT plan that the new mode cannot use to plan 0. */
corr_status corr_get_tiles(void *ctx, corrx_tiles *out);
corr_status corr_set_tiles(void *ctx, const corrx_tiles *t);

/* The two halves of corrx_accumulate, for timing and profiling each kernel on
   its own. corrx_run_fengine transforms `frames` (<= max_frames) frames into the
   engine's spectra buffer; corrx_run_xengine correlates the first `frames`
   frames of that buffer into d_acc. */
corr_status corrx_run_fengine(void *eng, const int8_t *d_samples, size_t station_stride,
                              size_t frame_stride, const uint8_t *d_mask,
                              size_t mask_station_stride, int32_t mask_bit0, int32_t frames,
                              void *stream);
corr_status corrx_run_xengine(void *eng, int32_t frames, void *d_acc, void *stream);

/* Watchdog self-test: launches one block that waits on an mbarrier nothing will
   ever complete, with a budget of `budget_cycles` clock cycles. The wait runs
   out, the kernel records the timeout in the engine's watchdog flag and returns;
   corrx_check() then reports CORR_ERR_INTERNAL and clears the flag. Exists so
   the timeout path of every bounded wait can be exercised without hanging a GPU. */
corr_status corrx_selftest_watchdog(void *eng, int64_t budget_cycles, void *stream);

/*
 * Batched integration blocks in one CUDA graph. No counterpart in the reference
 * (whose host drives one row at a time through corr_row_accumulate/row_end).
 *
 * corrx_batch_create captures, for every block i, the whole life of one
 * integration into a single graph:
 *   clear row i of d_rows (n_baseline*n_freq complex64 per block)
 *   F/X passes over frames [block_first[i], block_first[i] + block_frames[i])
 *   scale by 1/block_frames[i]
 *   copy row i to h_rows (pinned host, may be NULL) on a side stream
 * with a GPU timestamp at each block's start and after its dump.
 * corrx_batch_launch replays the graph on `stream` (one launch for all blocks);
 * corrx_batch_block_ms waits for the last launch and reports each block's
 * latency from its start to its row being on the host (or computed, without
 * h_rows); CORR_ERR_STATE before any launch. block_first/block_frames are host arrays
 * read at creation; samples/mask follow corrx_accumulate's conventions and must
 * stay valid for the batch's lifetime.
 */
corr_status corrx_batch_create(void *eng, const int8_t *d_samples, size_t station_stride,
                               size_t frame_stride, const uint8_t *d_mask,
                               size_t mask_station_stride, const int64_t *block_first,
                               const int32_t *block_frames, int32_t n_blocks, void *d_rows,
                               void *h_rows, void **out_batch);
/* corrx_batch_create with a choice of engine per block: block i runs on
   engines[block_engine[i]] (host arrays read at creation). The engines must share
   device, n_station and n_freq; each keeps its own spectra buffer and tiles --
   e.g. the FP16 tensor form for blocks long enough to meet a precision target
   and the split form for the short ones. */
corr_status corrx_batch_create_mixed(void *const *engines, int32_t n_engines,
                                     const int32_t *block_engine, const int8_t *d_samples,
                                     size_t station_stride, size_t frame_stride,
                                     const uint8_t *d_mask, size_t mask_station_stride,
                                     const int64_t *block_first, const int32_t *block_frames,
                                     int32_t n_blocks, void *d_rows, void *h_rows,
                                     void **out_batch);
/* corrx_batch_create_mixed with packet-granular loss (corrx_accumulate_packets'
   rule): frame f of station s keeps the 1024-sample packets whose bits are set
   in d_pmask[s*pmask_station_stride + f], f counted like block_first. d_mask may
   be NULL; block_engine may be NULL with one engine. */
corr_status corrx_batch_create_packets(void *const *engines, int32_t n_engines,
                                       const int32_t *block_engine, const int8_t *d_samples,
                                       size_t station_stride, size_t frame_stride,
                                       const uint8_t *d_mask, size_t mask_station_stride,
                                       const uint32_t *d_pmask, size_t pmask_station_stride,
                                       const int64_t *block_first, const int32_t *block_frames,
                                       int32_t n_blocks, void *d_rows, void *h_rows,
                                       void **out_batch);
corr_status corrx_batch_launch(void *batch, void *stream);
corr_status corrx_batch_block_ms(void *batch, float *out_ms, int32_t n);
corr_status corrx_batch_destroy(void *batch);

/*
 * corrx_accumulate without any device allocation. No counterpart in the
 * reference. For callers that may not call cudaMalloc: a host that owns all
 * device memory through its own pool and does not let libraries allocate, a
 * real-time loop where an allocation (and the device synchronisation it can
 * imply) would break a deadline, a process whose device-memory budget is fixed
 * up front. The spectra between the F- and X-engine live in a fixed 64 MiB
 * device array inside the library (held by every GPU that loads it until exit),
 * so one call covers at most 64 MiB / (n_station * n_freq * e) frames, e = 4
 * bytes per bin for CORR_X_TC_FP16 and 8 for the other forms (42 or 21 frames at
 * 24 inputs and n_freq 16384); more is rejected with CORR_ERR_ARG before
 * anything is launched. Same arguments and result as corrx_accumulate (d_acc +=
 * visibilities, complex64), plus the geometry and X-engine that an engine would
 * otherwise carry. The first call on a device sets that device up with it
 * current (looks up the arrays' addresses and copies the twiddle tables of every
 * transform length, synchronously): make it before any stream capture. All
 * calls share the spectra array: calls whose kernels overlap on the GPU race,
 * calls ordered on one stream do not. Nothing in it needs to start at zero.
 */
corr_status corrx_accumulate_noalloc(int32_t n_station, int32_t n_freq, int32_t xmode,
                                     const int8_t *d_samples, size_t station_stride,
                                     size_t frame_stride, const uint8_t *d_mask,
                                     size_t mask_station_stride, int32_t mask_bit0,
                                     int32_t frames, void *d_acc, void *stream);

/*
 * The tensor X-engine's geometry for a tile shape, as the kernel will use it
 * (no device work; for callers that plan shared memory or TMEM around it, and
 * for checking the kernel's index arithmetic on a machine without a GPU).
 * ok = 0: the shape is not feasible for n_station (everything else zero).
 * form: 0 split stacked, 1 split wide, 2 FP16 paired, 3 FP16 wide. Operand
 * region r starts at r*region_stride + skew(r) bytes into an operand stage,
 * skew(r) = ((r&1) | ((r&2)<<1) | ((r&4)>>1)) * 16; row `row`, 8-frame group kq
 * of a region lies at (row/8)*sbo + kq*128 + (row%8)*16 from its start.
 */
typedef struct corrx_tc_geom {
    uint32_t struct_size;  /* sizeof(corrx_tc_geom)                                  */
    int32_t  ok, form, elem, R, nb, regions, sbo, region_stride;
    int32_t  op_stage, ld_stage, n_op, n_ld, acc_cols, n_acc, tmem_cols, items, smem;
} corrx_tc_geom;

corr_status corrx_tc_geometry(int32_t n_station, int32_t split, int32_t ct, int32_t kt,
                              corrx_tc_geom *out);

/*
 * The row orders and operand offsets of FFT plan 2 (the tensor-core F-engine at
 * n_freq 16384), exactly as its kernel computes them; no device work. Fills
 *   b_of_row[512]      stage-1 row -> b (n = 512 a + b)
 *   row2[32 * 16]      [k1 * 16 + d] -> stage-2 row
 *   row3[32 * 32]      [k1 * 32 + k2a] -> stage-3 row
 *   off12[512 * 32]    [row * 32 + e] -> byte offset of complex element e of a
 *                      stage-1/2 operand row
 *   off3[1024 * 16]    [row * 16 + e] -> the same for the stage-3 operand
 * (any pointer may be NULL to skip it).
 */
corr_status corrx_tc_fft_maps(int32_t *b_of_row, int32_t *row2, int32_t *row3, uint32_t *off12,
                              uint32_t *off3);

/*
 * On-device synthetic front end: the traffic of the reference's test transmitter
 * (corr-rs/src/bin/replay.rs), assembled into frames and a validity mask the way
 * the receive side does it (corr-rs/src/assemble.rs), written straight into
 * device memory or into the pinned staging ring.
 *
 * Packets: an 8-byte counter c and SAMPLES_PER_PACKET = 4096 int8 samples
 * (corr-rs/src/config.rs:26). Frame id = c / P, P = 2*n_freq/4096 packets per
 * frame, the packet's samples at byte (c % P)*4096 of the frame. Patterns
 * (replay.rs:212-265), station s, sample k of the packet:
 *   ZERO    0
 *   COUNTER x = c*0x9E3779B97F4A7C15 + s*0x12345678; per sample x ^= x<<13,
 *           x ^= x>>7, x ^= x<<17, sample = (x>>3) % 9 - 4
 *   PRNG    splitmix64-style hash of the absolute sample index c*4096 + k - d_s
 *           plus seed, sample = (h>>8) % 9 - 4 (replay.rs:212-226); d_s is the
 *           station's sample delay (times the ladder step, below)
 *   SINE    round(4*sin(phase + k*tone*2pi/4096)), phase = (c + seed*s)*tone*2pi,
 *           evaluated in IEEE double without contraction
 * Station s sends counters start_counter + counter_offset[s] + n for
 * n < n_packets (0 = no end). Packet n is missing if gap_at <= n < gap_at +
 * gap_len, or if the loss hash of (c, s) falls below drop_rate (replay.rs:
 * 414-424). Ladder (ladder_frames > 0): the delay of station s in frame F is
 * sample_delay[s]*k, k = 1 + (F - origin)/ladder_frames for F >= origin else 1,
 * capped at ladder_steps when that is > 0, origin = the first multiple of
 * ladder_frames at or after frame (start_counter*4096)/(2*n_freq). The time-based
 * stall of replay.rs (a station silent for some seconds) is not modelled.
 *
 * corrx_frontend_fill writes frames [frame0, frame0 + frames) of stations
 * station0 .. station0 + n_station - 1 (station indices as the transmitter numbers
 * them, which select sample_delay[], counter_offset[] and enter the patterns and
 * the loss hash): station station0 + s, frame f at samples + s*station_stride +
 * f*frame_stride (any alignment; 16-byte aligned frames are written fastest;
 * bytes of frames whose bit is clear hold the pattern, which the engines never
 * read), and validity bit f (LSB first) of the
 * bit string at mask + s*mask_station_stride: set iff all P packets of the frame
 * were sent and not lost, as the receive side sets it; the bits after `frames`
 * in the last byte are cleared. Either pointer may be NULL to skip that output;
 * both may be device memory or pinned host memory (the staging ring, one call
 * per station as corr_staging_info describes it). n_freq must be a multiple of
 * 2048 (whole packets per frame), station0 + n_station <= 64.
 */
enum { CORRX_PATTERN_ZERO = 0, CORRX_PATTERN_COUNTER = 1, CORRX_PATTERN_PRNG = 2,
       CORRX_PATTERN_SINE = 3 };
#define CORRX_FRONTEND_MAX_STATIONS 64

typedef struct corrx_frontend {
    uint32_t struct_size;     /* sizeof(corrx_frontend)                            */
    int32_t  pattern;         /* CORRX_PATTERN_*             (replay --pattern)     */
    uint64_t seed;            /*                             (replay --seed)        */
    double   tone;            /* SINE: cycles per sample     (replay --tone)        */
    uint64_t start_counter;   /* first counter               (replay --start-counter) */
    uint64_t n_packets;       /* packets per station, 0 = unbounded (duration*rate) */
    double   drop_rate;       /* in [0, 1)                   (replay --drop-rate)   */
    uint64_t gap_at;          /*                             (replay --gap-at)      */
    uint64_t gap_len;         /*                             (replay --gap-len)     */
    uint64_t ladder_frames;   /* 0 = no ladder               (replay --ladder-frames) */
    uint64_t ladder_steps;    /* 0 = no cap                  (replay --ladder-steps) */
    int64_t  sample_delay[CORRX_FRONTEND_MAX_STATIONS];   /* --sample-delay, or
                                 --delay-stride * s, resolved per station          */
    uint64_t counter_offset[CORRX_FRONTEND_MAX_STATIONS]; /* replay --offset        */
} corrx_frontend;

corr_status corrx_frontend_fill(const corrx_frontend *fe, int32_t station0, int32_t n_station,
                                int32_t n_freq, int64_t frame0, int32_t frames, int8_t *samples,
                                size_t station_stride, size_t frame_stride, uint8_t *mask,
                                size_t mask_station_stride, void *stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* CORR_GB300_H */
