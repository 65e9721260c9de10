/*
 * corr_writer.h -- the correlator's output file sets, written natively.
 *
 * The reference's host writes every fetched row with corr-rs/src/writer.rs; this
 * is that writer's on-disk format and rules behind a C ABI, so a host that links
 * libcorr_cuda.so can hand rows straight from corr_rows_fetch to a writer thread
 * in the same library. Layout of a set (writer.rs:1-22), with <P> = file_prefix
 * and <T> = the local time of the set's first row in file_prefix_format
 * ("%Y%m%d-%H%M%S" by default):
 *
 *   <P><station_j><station_k>-<T>.bin   complex64[ntime][n_freq], one per baseline (j <= k)
 *   <P><T>-time.bin                     int64 little-endian Unix ms, one per row
 *   <P><T>-time.txt                     local "YYYY-mm-DD HH:MM:SS.mmm", one line per row
 *   <P><T>-blocks.csv                   row_index,station,first_frame_id,n_cum,valid,zero_filled
 *                                       (one line per station per row, no header)
 *   <P><T>-metadata.yaml                geometry, conventions, the set's identity,
 *                                       stations and each baseline's file name
 *
 * Rules kept (writer.rs:24-47): every file is a whole number of rows (a resumed
 * set is truncated back to the shortest file's row count, and the text sidecar
 * is rebuilt from time.bin); a row's spectra are written before its sidecars; a
 * set that already holds rows is never reused as a new set. With daily_files, a
 * row whose local day is later than the set's closes the set and opens the next
 * (set_kind rollover); an earlier day keeps the current set (writer.rs:1652-1659).
 *
 * Threading: corrw_write_row copies the row into one of queue_rows buffers and
 * returns; a writer thread writes it. A full queue drops the whole row (counted
 * in corrw_stats.rows_dropped) or blocks, as queue_full says (writer.rs:1485-1556).
 * queue_rows = 0 writes in the calling thread. One thread drives a writer.
 *
 * Status codes: CORR_ERR_ARG bad parameters or row shape; CORR_ERR_ABI
 * struct_size; CORR_ERR_STATE a set conflict (tag in use, config_hash differs
 * from the set being resumed, no such set); CORR_ERR_INTERNAL an I/O error (the
 * message names the file and errno), after which the writer only reports it.
 */

#ifndef CORR_WRITER_H
#define CORR_WRITER_H

#include "corr_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { CORRW_SET_AUTO = 0,     /* append to the latest set of today, else open a new one */
       CORRW_SET_NEW = 1,      /* always open a new set (second_set if today has one)    */
       CORRW_SET_EXPLICIT = 2  /* append to the set named by set_tag                     */ };
enum { CORRW_QUEUE_DROP = 0, CORRW_QUEUE_BLOCK = 1 };

typedef struct corrw_station {
    const char *name;        /* used in the baseline file names                      */
    const char *group_ip;    /* metadata only; NULL leaves group_ip/dest_port/board out */
    int32_t     dest_port;
    const char *board;
} corrw_station;

typedef struct corrw_params {
    uint32_t struct_size;         /* sizeof(corrw_params)                             */
    int32_t  n_station;           /* 1..64                                            */
    int32_t  n_freq;
    uint32_t n_cum;               /* frames per row                                   */
    uint32_t frames_per_slot;     /* metadata                                         */
    uint32_t rows_per_fetch;      /* metadata                                         */
    uint64_t sample_rate_hz;      /* metadata; frame rate = sample_rate / (2 n_freq)  */
    int32_t  data_shift_count;    /* metadata                                         */
    int32_t  daily_files;         /* 1: a set per local day; 0: one set per open      */
    int32_t  set_policy;          /* CORRW_SET_* (daily_files only)                   */
    int32_t  queue_full;          /* CORRW_QUEUE_*                                    */
    uint32_t queue_rows;          /* rows in flight; 0 = synchronous writes           */
    uint32_t fsync_every_rows;    /* >= 1                                             */
    const char *dir;              /* created if missing                               */
    const char *file_prefix;      /* NULL = ""                                        */
    const char *file_prefix_format; /* strftime; NULL = "%Y%m%d-%H%M%S"               */
    const char *config_version;   /* metadata                                         */
    const char *config_hash;      /* metadata; must match to resume a set             */
    const char *set_tag;          /* CORRW_SET_EXPLICIT                               */
    const corrw_station *stations; /* n_station entries                               */
} corrw_params;

typedef struct corrw_resume {
    uint32_t struct_size;
    uint32_t has_next_frame_id;   /* 1 when a resumed set has rows                    */
    uint64_t rows_written;        /* complete rows kept in the resumed set            */
    uint64_t truncated_rows;      /* rows of spectra cut back to match the sidecars   */
    uint64_t next_frame_id;       /* first frame of the last row + n_cum              */
} corrw_resume;

typedef struct corrw_stats {
    uint32_t struct_size;
    uint32_t sets_opened;         /* by this writer (rollovers included)              */
    uint64_t rows_written;        /* rows on disk, all sets of this writer, incl. resumed */
    uint64_t rows_dropped;        /* full queue with CORRW_QUEUE_DROP                 */
    uint64_t max_queued;
    char     set_tag[256];        /* the set being written ("" before the first row)  */
} corrw_stats;

corr_status corrw_open(const corrw_params *p, void **out_writer, corrw_resume *resume);
/* row: n_baseline * n_freq complex64, baseline-major (the layout corr_rows_fetch
   writes for one row); valid_frames: n_station counts of frames each station
   delivered in this row (blocks.csv). */
corr_status corrw_write_row(void *w, const void *row, size_t row_bytes, int64_t row_ms,
                            uint64_t row_index, uint64_t first_frame_id,
                            const uint64_t *valid_frames);
/* Wait until every queued row is in the files (not fsynced). */
corr_status corrw_sync(void *w);
corr_status corrw_stats_get(void *w, corrw_stats *out);
/* Write what is queued, fsync every file, stop the thread and free the writer. */
corr_status corrw_close(void *w);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* CORR_WRITER_H */
