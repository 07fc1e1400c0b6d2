/*
 * h264r_server.h — continuous-batching server on top of the reconstruction
 * engine (include/h264r.h).
 *
 * No counterpart in the reference, which decodes one bitstream at a time in
 * a single thread (H264VideoDecoder.cpp:83-140).  A server serves many
 * streams of different sizes on one GPU:
 *   - a stream asks to be opened; it is admitted when its device-resident
 *     DPB fits the context's memory budget (h264r_cfg.dpb_budget_bytes),
 *     otherwise it waits, in arrival order, until finished streams free
 *     their DPBs;
 *   - the host parser pushes each picture's records as soon as they are
 *     complete; the records are copied into the stream's syntax queue in
 *     device memory;
 *   - a scheduler thread keeps forming batches from whatever is ready: the
 *     next dependency group of every admitted stream goes into one fused
 *     launch sequence (h264r_submit_batch_device), so pictures that arrive
 *     while others are on the GPU join the next batch and their work
 *     overlaps on the device;
 *   - each finished picture is reported with its latency, from the push of
 *     its records to its planes being ready (copied to the caller's host
 *     buffer when one was given).
 * Every call returns 0 or a negative H264R_ERR_* code.
 */
#ifndef H264R_SERVER_H
#define H264R_SERVER_H

#include "h264r.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct h264r_server h264r_server;

typedef struct h264r_server_cfg {
    uint32_t max_batch_pictures; /* pictures per launch (0: the context's limit) */
    uint32_t queue_depth;        /* pictures a stream may hold in device memory
                                    (uploaded or in flight), 0: 4             */
    uint32_t flags;              /* reserved, 0                               */
    uint32_t lanes;              /* batch chains over disjoint stream sets
                                    (streams split by id; 0: 6, at most 8)    */
} h264r_server_cfg;

/* One finished picture. */
typedef struct h264r_server_done {
    int32_t  stream;       /* stream id from h264r_server_open                */
    int32_t  status;       /* 0, or the error that ended the stream           */
    uint64_t tag;          /* the tag given to h264r_server_push              */
    double   latency_ms;   /* push of the records -> planes ready (host clock)*/
} h264r_server_done;

typedef struct h264r_server_stats {
    uint64_t pictures_done;
    uint64_t streams_open;      /* admitted and not finished                  */
    uint64_t streams_waiting;   /* waiting for DPB memory                     */
    uint64_t streams_done;
    uint64_t batches;           /* launch sequences                           */
    uint64_t batch_pictures;    /* pictures in them                           */
    uint64_t dpb_bytes_in_use;
    uint64_t dpb_bytes_peak;
    uint64_t waiting_peak;      /* most streams waiting at once               */
    double   p50_ms, p99_ms, max_ms;  /* latency of the finished pictures     */
} h264r_server_stats;

/* Start a server (and its scheduler thread) on a context. */
int h264r_server_create(h264r_ctx *ctx, const h264r_server_cfg *cfg, h264r_server **out);
/* Finish all pushed work, close every stream and stop the scheduler. */
int h264r_server_destroy(h264r_server *srv);

/* Ask for a stream; *stream_id is valid at once, the stream is admitted
 * when its DPB fits the budget.  Fails with H264R_ERR_BUDGET only when the
 * DPB alone exceeds the whole budget. */
int h264r_server_open(h264r_server *srv, const h264r_stream_cfg *cfg, int *stream_id);

/* Queue one picture of a stream, in decoding order.  Consecutive pictures
 * with the same dependency_group reference none of each other and may share
 * a launch.  The records (host memory) are validated and copied before the
 * call returns.  out_planes: host buffer for the decoded Y, Cb, Cr planes
 * (width*height*3/2 bytes, pinned for speed) or NULL. */
int h264r_server_push(h264r_server *srv, int stream_id, const h264r_picture *pic, int dependency_group, uint64_t tag,
                      uint8_t *out_planes);

/* No more pictures for this stream; it is closed (DPB freed) once its last
 * picture is done. */
int h264r_server_end(h264r_server *srv, int stream_id);

/* Up to max finished pictures into done[]; waits up to wait_ms for the
 * first.  Returns the number written (>= 0) or an error code. */
int h264r_server_poll(h264r_server *srv, h264r_server_done *done, int max, int wait_ms);

/* Pictures pushed to the stream and not yet reported by h264r_server_poll. */
int h264r_server_pending(h264r_server *srv, int stream_id);

int h264r_server_get_stats(h264r_server *srv, h264r_server_stats *out);

#ifdef __cplusplus
}
#endif

#endif /* H264R_SERVER_H */
