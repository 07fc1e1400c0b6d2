/*
 * h264r.h — C ABI of the GB300 H.264 macroblock-reconstruction engine.
 *
 * The host side (entropy decoding, slice headers, reference lists, motion
 * vector derivation, DPB bookkeeping) stays serial on the CPU and emits, per
 * decoded picture, the compact records declared here.  The engine turns the
 * records into decoded samples on the GPU:
 *   8.5  dequantisation and 4x4 / 8x8 / DC inverse transforms
 *   8.4.2 quarter-sample luma and eighth-sample chroma motion compensation
 *        with default / explicit / implicit weighted prediction
 *   8.3  intra prediction (4x4, 8x8, 16x16, chroma, I_PCM)
 *   8.7  deblocking
 *
 * It replaces, for that path, the per-macroblock reconstruction calls the
 * reference decoder makes from its slice-data loop
 * (h264_video_decoder_demo/H264SliceData.cpp:222-227, 333-338, 389-487) and
 * the per-picture deblocking call
 * (h264_video_decoder_demo/H264PictureBase.cpp:707 ->
 *  H264PictureDeblockingFilterProcess.cpp:76).
 *
 * Conventions follow the reference decoder: every entry point returns 0 on
 * success and a negative error code on failure (CommonFunction.h:40-47);
 * h264r_last_error() gives a one-line reason.  No call traps or hangs: device
 * side waits are bounded and surface as H264R_ERR_DEVICE_TIMEOUT.
 *
 * All integer fields are little-endian host order; structures are packed to
 * the sizes asserted below so that the same bytes can be copied to the GPU.
 */
#ifndef H264R_H
#define H264R_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define H264R_ABI_VERSION 1

/* ---- error codes ------------------------------------------------------ */
#define H264R_OK                 0
#define H264R_ERR_INVALID_ARG   -1   /* null pointer, size out of range        */
#define H264R_ERR_BAD_RECORD    -2   /* record field out of range (validator)  */
#define H264R_ERR_UNSUPPORTED   -3   /* coding tool outside the engine's scope */
#define H264R_ERR_CUDA          -4   /* CUDA runtime error                      */
#define H264R_ERR_NO_MEMORY     -5   /* device/pinned allocation failed         */
#define H264R_ERR_BUDGET        -6   /* admission refused: DPB memory budget    */
#define H264R_ERR_DEVICE_TIMEOUT -7  /* a bounded device-side wait expired      */
#define H264R_ERR_BUSY          -8   /* no free slot / queue full               */
#define H264R_ERR_TOO_LARGE     -9   /* exceeds a fixed maximum size            */
#define H264R_ERR_IO           -10   /* a file could not be written             */

/* ---- macroblock record ------------------------------------------------- */
/* mb type classes (derived from mb_type / MbPartPredMode, 7.4.5)          */
#define H264R_MB_INTER   0   /* P/B, including P_Skip and B_Skip          */
#define H264R_MB_I4x4    1
#define H264R_MB_I8x8    2
#define H264R_MB_I16x16  3
#define H264R_MB_IPCM    4
#define H264R_MB_NONE    5   /* not decoded (its slice was lost): samples
                                stay zero; see the deblocking stop rule    */

/* h264r_mb.flags */
#define H264R_MBF_T8x8        0x01  /* transform_size_8x8_flag               */
#define H264R_MBF_FIELD       0x02  /* mb_field_decoding_flag (MBAFF)        */
#define H264R_MBF_CIP         0x04  /* constrained_intra_pred_flag           */

#define H264R_NONE 0xFFFFFFFFu

/*
 * One record per macroblock, indexed by mbAddr (raster order for non-MBAFF
 * pictures, pair order for MBAFF).  Restates the reconstruction-relevant
 * subset of CH264MacroBlock (H264MacroBlock.h:110-252): 18,200 bytes there,
 * 32 bytes here plus the variable-size motion / coefficient payloads.
 */
typedef struct h264r_mb {
    uint8_t  type;          /* H264R_MB_*                                    */
    uint8_t  flags;         /* H264R_MBF_*                                   */
    uint8_t  qpy;           /* QPY, 0..51 (8-bit video: QP'Y == QPY)         */
    uint8_t  i16_mode;      /* Intra16x16PredMode 0..3                       */
    uint8_t  chroma_mode;   /* intra_chroma_pred_mode 0..3                   */
    uint8_t  nz8x8;         /* bit b: 8x8 luma block b has non-zero levels   */
    uint16_t nz4x4;         /* bit b: 4x4 luma block b (luma4x4BlkIdx order)
                               has non-zero levels                           */
    uint16_t slice;         /* slice number within the picture               */
    uint16_t reserved;
    uint32_t ipred[2];      /* Intra4x4PredMode[16] (4 bits each, block 0 in
                               the low nibble of ipred[0]) or
                               Intra8x8PredMode[4] in ipred[0] bits 0..15     */
    uint32_t coef;          /* byte offset into the coefficient pool, or
                               H264R_NONE when the MB has no levels          */
    uint32_t aux;           /* inter: byte offset into the motion pool;
                               I_PCM: index of its 384-byte sample block      */
    uint32_t reserved2;
} h264r_mb;

/*
 * Coefficient payload of one macroblock, at h264r_mb.coef (4-byte aligned):
 *   uint32 mask        which blocks are present:
 *                        bits 0..15  4x4 luma block (luma4x4BlkIdx) levels
 *                                    (Intra16x16: the AC list, scan pos 1..15)
 *                        bits 0..3   8x8 luma block (when H264R_MBF_T8x8)
 *                        bit  16     Intra16x16 luma DC
 *                        bits 17,18  Cb / Cr chroma DC (4:2:0: 4 levels)
 *                        bits 19..22 Cb AC blocks 0..3 (scan pos 1..15)
 *                        bits 23..26 Cr AC blocks 0..3
 *   uint16 sig[...]    per present block, in mask bit order: one significance
 *                      word (bit i = scan position i non-zero), four words
 *                      for an 8x8 block (positions 0..63)
 *   (pad to 4 bytes)
 *   int16  level[...]  the non-zero levels, block after block, ascending scan
 *                      position
 * Levels are in coded scan order (zig-zag, or field scan for field MBs), as
 * the reference stores them in LumaLevel4x4 / LumaLevel8x8 /
 * Intra16x16DCLevel / Intra16x16ACLevel / ChromaDCLevel / ChromaACLevel.
 */
#define H264R_CM_LUMA_DC  (1u << 16)
#define H264R_CM_CB_DC    (1u << 17)
#define H264R_CM_CR_DC    (1u << 18)
#define H264R_CM_CB_AC0   19
#define H264R_CM_CR_AC0   23

/*
 * Motion payload of one inter macroblock, at h264r_mb.aux (4-byte aligned):
 *   uint16 shape       bits 0..1: 0 16x16, 1 16x8, 2 8x16, 3 8x8
 *                      bits 2+2q..3+2q: sub-partition of 8x8 quadrant q
 *                                       (0 8x8, 1 8x4, 2 4x8, 3 4x4)
 *   uint16 count       number of h264r_part entries that follow
 *   h264r_part part[count]   ordered by (mbPartIdx, subMbPartIdx)
 * B_Skip / B_Direct_16x16 / B_Direct_8x8 quadrants are described as 4x4
 * sub-partitions, which is how the reference predicts them
 * (H264InterPrediction.cpp:475-486).
 */
typedef struct h264r_part {
    int16_t  mv[2][2];      /* [list][x,y] luma motion vector, 1/4 sample    */
    int8_t   ref[2];        /* motion-compensation reference per list, -1 if
                               the list is unused; bits 0..4 DPB slot,
                               bit 5 field reference, bit 6 bottom field      */
    int8_t   dref[2];       /* reference identity used by the deblocking
                               filter's bS rules, -1 for none: the picture-
                               level list entry the reference compares
                               (H264PictureDeblockingFilterProcess.cpp:
                               1175-1178), which can differ from ref[]      */
    uint16_t wt;            /* index into the picture's weight table         */
    uint16_t reserved;
} h264r_part;

#define H264R_REF_SLOT(r)   ((r) & 31)
#define H264R_REF_FIELD     0x20
#define H264R_REF_BOTTOM    0x40

/* Weighted-prediction parameters of one partition (8.4.2.3, 8.4.3). */
typedef struct h264r_weight {
    int8_t   weighted;      /* 0: default prediction 8.4.2.3.1;
                               1: weighted prediction 8.4.2.3.2             */
    int8_t   log_wd[3];     /* logWD for Y, Cb, Cr                           */
    int16_t  w0[3], w1[3];  /* weights                                       */
    int16_t  o0[3], o1[3];  /* offsets (already scaled by bit depth)        */
    int16_t  reserved[2];
} h264r_weight;

/* Per-slice parameters used by reconstruction and deblocking. */
typedef struct h264r_slice {
    int8_t   chroma_qp_offset[2];   /* chroma_qp_index_offset,
                                       second_chroma_qp_index_offset        */
    int8_t   filter_offset_a;       /* FilterOffsetA = alpha offset << 1     */
    int8_t   filter_offset_b;       /* FilterOffsetB                         */
    uint8_t  disable_deblocking_filter_idc;
    uint8_t  slice_type;            /* 0 P, 1 B, 2 I, 3 SP, 4 SI             */
    uint8_t  reserved[2];
} h264r_slice;

#define H264R_STRUCT_FRAME   0
#define H264R_STRUCT_TOP     1
#define H264R_STRUCT_BOTTOM  2

/* One decoded picture's worth of records (host or device pointers). */
typedef struct h264r_picture {
    uint16_t width_mbs;        /* PicWidthInMbs                              */
    uint16_t height_mbs;       /* FrameHeightInMbs                           */
    uint8_t  structure;        /* H264R_STRUCT_*: a field picture (TOP /
                                  BOTTOM) writes its field's lines of
                                  dst_slot, reads fields only (its own slot's
                                  other field allowed), num_mbs is half the
                                  frame's, mbaff 0                           */
    uint8_t  mbaff;            /* MbaffFrameFlag                             */
    uint8_t  dst_slot;         /* DPB slot that receives the samples         */
    uint8_t  deblock;          /* 1: run the 8.7 deblocking filter           */
    uint16_t num_slices;
    uint16_t num_weights;
    uint32_t num_mbs;          /* PicSizeInMbs                               */
    uint32_t motion_bytes;
    uint32_t coef_bytes;
    uint32_t num_pcm;
    uint8_t  scaling4x4[6][16];/* ScalingList4x4, coded (zig-zag) order      */
    uint8_t  scaling8x8[6][64];/* ScalingList8x8                             */
    const h264r_mb     *mbs;
    const h264r_slice  *slices;
    const h264r_weight *weights;
    const uint8_t      *motion;
    const uint8_t      *coef;
    const uint8_t      *pcm;    /* 384 bytes per I_PCM MB: 256 Y, 64 Cb, 64 Cr */
} h264r_picture;

/* ---- engine objects ----------------------------------------------------- */
typedef struct h264r_ctx h264r_ctx;
typedef struct h264r_stream h264r_stream;

typedef struct h264r_cfg {
    int      device;             /* CUDA device ordinal                      */
    uint64_t dpb_budget_bytes;   /* admission budget for all stream DPBs;
                                    0 = 90% of free device memory            */
    uint32_t max_batch_pictures; /* pictures per batched launch (0: 64)      */
    uint32_t flags;              /* H264R_CFG_*                              */
} h264r_cfg;

/* h264r_cfg.flags: device-resident records are complete in device memory
 * when h264r_submit_*_device is called (they are not produced by work still
 * queued on the streams).  The boundary strengths of a batch are then derived
 * on the stream's side stream as soon as the call is made, ahead of the
 * batches queued before it.  (Host-resident records are uploaded by the
 * engine itself and get this ordering without the flag.) */
#define H264R_CFG_DEVICE_RECORDS_READY 0x1u

typedef struct h264r_stream_cfg {
    uint16_t width_mbs;
    uint16_t height_mbs;         /* frame height in MBs                      */
    uint16_t dpb_slots;          /* number of picture buffers (<= 32)        */
    uint16_t reserved;
} h264r_stream_cfg;

/*
 * Create / destroy an engine context on one GPU.
 * Replaces: the reference's per-decoder state set up in
 * CH264VideoDecoder::open (H264VideoDecoder.cpp:56-80).
 */
int  h264r_ctx_create(const h264r_cfg *cfg, h264r_ctx **out);
int  h264r_ctx_destroy(h264r_ctx *ctx);
const char *h264r_last_error(const h264r_ctx *ctx);

/*
 * Open a stream: allocate its device-resident DPB (dpb_slots pictures in the
 * reference's single-allocation Y/Cb/Cr layout, H264PictureBase.cpp:162-181).
 * Replaces: CH264PicturesGOP's 16 CH264Picture buffers
 * (H264PicturesGOP.cpp:27-50).  Fails with H264R_ERR_BUDGET when the DPB
 * would exceed the context's memory budget.
 */
int  h264r_stream_open(h264r_ctx *ctx, const h264r_stream_cfg *cfg, h264r_stream **out);
int  h264r_stream_close(h264r_stream *s);
/* Make an idle stream ready for a new bitstream of the same geometry, as a
 * freshly opened one: its picture buffers are cleared again (queued on its
 * CUDA stream, like the clear at open) and its pending output copies are
 * waited for.  The stream must have no launch in flight.  A server reuses
 * streams this way instead of closing and opening them per request.  No
 * counterpart in the reference, which decodes one bitstream per decoder. */
int  h264r_stream_reset(h264r_stream *s);
uint64_t h264r_stream_dpb_bytes(const h264r_stream_cfg *cfg);

/*
 * Reconstruct one picture from host-resident records: copies the records to
 * the device (through pinned staging), runs inter + intra reconstruction and
 * deblocking into DPB slot pic->dst_slot, and returns once the work is
 * enqueued on the stream.  Replaces the reconstruction dispatch of
 * CH264SliceData::slice_data (H264SliceData.cpp:389-487, skip paths 222-227
 * and 333-338) plus CH264PictureBase::Deblocking_filter_process
 * (H264PictureDeblockingFilterProcess.cpp:76).
 */
int  h264r_submit_picture(h264r_stream *s, const h264r_picture *pic);

/*
 * Same as h264r_submit_picture, but every pointer in pic (mbs, slices,
 * weights, motion, coef, pcm) is already device memory.  Used when the
 * records are staged on the GPU ahead of time.
 */
int  h264r_submit_picture_device(h264r_stream *s, const h264r_picture *pic);

/*
 * Batched reconstruction: n independent pictures (of any streams in the same
 * context; no picture may reference another picture of the same batch) in
 * one fused launch sequence.  Pointers are device memory.  The batch runs on
 * the CUDA stream of streams[0] after the work already queued on the other
 * member streams, and their later work waits for it; batches over disjoint
 * sets of streams with different first members therefore overlap.
 */
int  h264r_submit_batch_device(h264r_ctx *ctx, int n, h264r_stream *const *streams,
                               const h264r_picture *pics);
/*
 * The same on a CUDA stream of the caller's, with no ordering against the
 * member streams' own CUDA streams: all earlier work that touches the
 * members' picture buffers (earlier batches, the clear of a stream opened
 * or reset, output copies) must be queued on cuda_stream or ordered before
 * it.  A server that runs every batch of a set of streams on one CUDA stream
 * saves the per-member event plumbing this way.  No counterpart in the
 * reference (one bitstream, one thread).
 */
int  h264r_submit_batch_device_on(h264r_ctx *ctx, void *cuda_stream, int n, h264r_stream *const *streams,
                                  const h264r_picture *pics);

/*
 * Batched reconstruction from host-resident records: the records of all n
 * pictures are packed into pinned staging memory and copied to the device
 * in one transfer, then reconstructed in one fused launch sequence (same
 * rules as h264r_submit_batch_device).
 */
int  h264r_submit_batch(h264r_ctx *ctx, int n, h264r_stream *const *streams, const h264r_picture *pics);

/*
 * Algorithmic bytes of one picture per engine stage, for roofline
 * accounting: out[0] inter stage (records read + reference samples + 384
 * output bytes per inter / I_PCM MB), out[1] intra stage (records + 384 per
 * intra MB), out[2] deblocking (768 per MB + 32 record bytes), out[3] all
 * record bytes.  Reference samples per partition and list:
 * (w + 5*[xFrac!=0]) * (h + 5*[yFrac!=0]) luma plus
 * 2 * (w/2 + [xFracC!=0]) * (h/2 + [yFracC!=0]) chroma.  Host pointers.
 */
int  h264r_picture_bytes(const h264r_picture *pic, uint64_t out[4]);

/*
 * Copy a decoded picture (DPB slot) to host planes at coded size: luma
 * width_mbs*16 x height_mbs*16, chroma half in each direction.  Replaces the
 * borrowed CH264Picture the reference hands to its output callback
 * (H264VideoDecoder.cpp:383-435).  Enqueued; call h264r_stream_sync before
 * reading the planes.
 */
int  h264r_output(h264r_stream *s, int slot, uint8_t *y, uint8_t *cb, uint8_t *cr);
/*
 * As h264r_output, on the stream's own copy stream: the copy starts when the
 * work enqueued on the stream so far is done and overlaps the stream's later
 * launches; a later launch (or h264r_load_slot) that writes the same slot
 * waits for the copy.  Host planes should be pinned for the copy to be
 * asynchronous; call h264r_stream_sync before reading them.
 */
int  h264r_output_async(h264r_stream *s, int slot, uint8_t *y, uint8_t *cb, uint8_t *cr);
/* As h264r_output_async, on a CUDA stream of the caller's that is already
 * ordered after the picture's batch (a later launch writing the slot still
 * waits for the copy).  Replaces, like h264r_output, the reference's hand-off
 * of a decoded picture (H264VideoDecoder.cpp:383-435), for callers that order
 * their own streams. */
int  h264r_output_async_on(h264r_stream *s, int slot, uint8_t *y, uint8_t *cb, uint8_t *cr, void *cuda_stream);
/*
 * Decoded picture (DPB slot) as BGR24 rows of row_bytes bytes (at least
 * 3*width, a multiple of 4, like the reference's bitmap rows), top-down, or
 * bottom-up when flip != 0: the reference's conversion for its BMP output
 * and its player (CH264PictureBase::convertYuv420pToBgr24 /
 * convertYuv420pToBgr24FlipLines, H264PictureBase.cpp:440-499), computed on
 * the GPU.  dst: host memory (h264r_output_bgr24, enqueued: call
 * h264r_stream_sync before reading) or 4-byte aligned device memory
 * (h264r_output_bgr24_device).
 */
int  h264r_output_bgr24(h264r_stream *s, int slot, uint8_t *dst, uint32_t row_bytes, int flip);
int  h264r_output_bgr24_device(h264r_stream *s, int slot, void *dst, uint32_t row_bytes, int flip);
/* 24-bit BMP file of top-down BGR24 rows, written bottom-up with the
 * reference's 54-byte header (CH264PictureBase::saveBmp,
 * H264PictureBase.cpp:554-600).  Host only. */
int  h264r_write_bmp(const char *path, const uint8_t *bgr, uint32_t width, uint32_t height, uint32_t row_bytes);
/* Planar YUV 4:2:0 file at coded size (CH264PictureBase::writeYUV,
 * H264PictureBase.cpp:651-665).  Host only. */
int  h264r_write_yuv(const char *path, const uint8_t *y, const uint8_t *cb, const uint8_t *cr, uint32_t width, uint32_t height);
/* Upload host planes into a DPB slot (initial state / tests). */
int  h264r_load_slot(h264r_stream *s, int slot, const uint8_t *y, const uint8_t *cb, const uint8_t *cr);
/* Device address of a DPB slot's Y plane (Cb, Cr follow contiguously). */
int  h264r_slot_device_ptr(h264r_stream *s, int slot, void **dev_y);
int  h264r_stream_sync(h264r_stream *s);
int  h264r_ctx_sync(h264r_ctx *ctx);
/* The CUDA stream the engine enqueues this stream's work on (cudaStream_t). */
void *h264r_stream_cuda_stream(h264r_stream *s);
/* The stream's copy stream, which h264r_output_async enqueues on
 * (cudaStream_t): an event recorded on it after h264r_output_async marks the
 * copy as done. */
void *h264r_stream_output_cuda_stream(h264r_stream *s);
/* The context's own CUDA stream (used by h264r_ctx_sync), cudaStream_t. */
void *h264r_ctx_cuda_stream(h264r_ctx *ctx);

/*
 * Deblock one picture in place without allocating any device memory.
 * No counterpart in the reference: it exists for callers that cannot let a
 * library allocate on the GPU — processes that hand all device memory to a
 * pool of their own up front, and real-time decode loops that must not stall
 * other streams (cudaMalloc and cudaFree synchronise the device).
 *
 * pic: records of a reconstructed picture, every pointer device memory (as
 *      for h264r_submit_picture_device); pic->deblock is ignored.
 * planes: device address of the picture's samples, Y then Cb then Cr
 *      contiguous at coded size (the engine's DPB slot layout), 16-byte
 *      aligned; filtered in place.  cuda_stream: the cudaStream_t to run on (0: legacy default).
 * The scratch it needs (bS table, wavefront counters) is one static device
 * array compiled into the library, sized for pictures of at most
 * H264R_NOALLOC_MAX_MBS macroblocks and H264R_NOALLOC_MAX_MB_ROWS MB rows
 * (1920x1088 fits); larger pictures return H264R_ERR_TOO_LARGE.  Every GPU
 * that loads the library holds that array (about 2.1 MB) until the process
 * exits.  The first call on a device resolves the array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call
 * before any stream capture.  All calls in a process share the one array:
 * calls that overlap on the GPU race and corrupt each other, so do not run
 * two at once.  The call waits for its stream and returns 0 or the device
 * error (H264R_ERR_DEVICE_TIMEOUT / H264R_ERR_BAD_RECORD).
 */
#define H264R_NOALLOC_MAX_MBS     8192
#define H264R_NOALLOC_MAX_MB_ROWS 256
int  h264r_deblock_picture_noalloc(const h264r_picture *pic, uint8_t *planes, void *cuda_stream);

/* Validate a picture's records on the host (ranges, offsets, payload sizes).
 * Returns 0 or H264R_ERR_BAD_RECORD / H264R_ERR_UNSUPPORTED. */
int  h264r_validate_picture(const h264r_picture *pic, int dpb_slots);

/* The context's CUDA device, DPB memory budget (bytes) and batch limit. */
int      h264r_ctx_device(const h264r_ctx *ctx);
uint64_t h264r_ctx_dpb_budget(const h264r_ctx *ctx);
int      h264r_ctx_max_batch(const h264r_ctx *ctx);

/* Number of engine kernels launched so far by this context. */
uint64_t h264r_ctx_kernel_launches(const h264r_ctx *ctx);

/* Device timing of the engine's kernels, measured with CUDA events on the
 * stream each kernel runs on.  h264r_ctx_set_timing(ctx, 1) clears the
 * totals and starts recording; h264r_ctx_last_timing waits for the recorded
 * launches and returns the summed milliseconds since then: t[0] inter,
 * t[1] intra, t[2] deblocking (bS + filter); *launches receives the number
 * of launch sequences summed. */
int  h264r_ctx_set_timing(h264r_ctx *ctx, int enable);
int  h264r_ctx_last_timing(h264r_ctx *ctx, float t[3], int *launches);
/* The same totals per kernel: t[0] k_inter, t[1] k_intra, t[2] k_bs,
 * t[3] the deblocking filter kernels.  While timing is on, k_bs runs in line
 * on the batch's stream (not beside k_inter / k_intra), so that with one
 * launch sequence in flight at a time each kernel is timed alone. */
int  h264r_ctx_kernel_timing(h264r_ctx *ctx, float t[4], int *launches);
/* Host time of the context's h264r_submit_batch calls since it was created,
 * in seconds: s[0] waiting for a free launch slot (the GPU behind), s[1]
 * validating and packing the records on the host workers, s[2] upload and
 * kernel launches; s[3] receives the number of threads that pack. */
int  h264r_ctx_host_stats(h264r_ctx *ctx, double s[4]);

/*
 * Failure-path tests.  The reference's error convention is to print and
 * return a negative code (RETURN_IF_FAILED, CommonFunction.h:40-47); the
 * engine's device-side equivalent is a bounded wait that records
 * H264R_ERR_DEVICE_TIMEOUT and returns.  This makes such a wait run out on
 * purpose, without a fault or a hang:
 *   spin_limit           iterations a device wait may spin before it gives
 *                        up (0: the default, ~seconds)
 *   withhold_first_rows  non-zero: later launches do not hand out the first
 *                        tickets of the intra and deblocking wavefronts, so
 *                        the first picture's first row (block of rows) never
 *                        runs and the rows below it wait on progress that is
 *                        never published; with a small spin_limit the
 *                        launch ends with every kernel returned, and
 *                        h264r_stream_sync / h264r_ctx_sync report
 *                        H264R_ERR_DEVICE_TIMEOUT once
 * h264r_ctx_set_wait_test(ctx, 0, 0) restores normal operation; the context
 * stays usable.  Not for production use.
 */
int  h264r_ctx_set_wait_test(h264r_ctx *ctx, uint64_t spin_limit, int withhold_first_rows);

/* ---- launch shapes, captured launch graphs, autotuner ------------------ */
/*
 * No counterpart in the reference, which reconstructs one macroblock at a
 * time on one CPU thread.  The tuning of a launch sequence:
 *   inter_mbs_per_cta      k_inter: MBs (one warp each) per thread block,
 *                          2, 4 or 8 (0: 4)
 *   deblock_pairs_per_cta  frame-picture deblocking: MB-row pairs (one warp
 *                          each) per thread block, 4 or 8 (0: 8)
 *   graphs                 non-zero: a launch sequence (descriptor upload,
 *                          k_bs beside k_inter / k_intra, deblocking) whose
 *                          shape a launch buffer has seen before is captured
 *                          once as a CUDA graph and replayed from then on;
 *                          not while kernel timing is on
 * Decoded samples do not depend on the tuning.  A context starts with the
 * defaults {4, 8, 0}; h264r_ctx_set_tuning changes them for every batch
 * without an autotuned entry.  Entries are keyed by the batch's picture
 * geometry mix (the multiset of width x height x MBAFF of its pictures).
 * Returns H264R_ERR_INVALID_ARG for a shape outside the lists above.
 */
typedef struct h264r_tuning {
    int32_t inter_mbs_per_cta;
    int32_t deblock_pairs_per_cta;
    int32_t graphs;
    int32_t reserved;
} h264r_tuning;

int  h264r_ctx_set_tuning(h264r_ctx *ctx, const h264r_tuning *t);
/* The tuning a batch of these n pictures would launch with (n = 0: the
 * context's default). */
int  h264r_ctx_get_tuning(h264r_ctx *ctx, int n, const h264r_picture *pics, h264r_tuning *out);
/* Set the tuning of the geometry mix of these n pictures, e.g. one that an
 * earlier autotuner run found and the caller kept (only the pictures'
 * width_mbs, height_mbs and mbaff are read). */
int  h264r_ctx_set_mix_tuning(h264r_ctx *ctx, int n, const h264r_picture *pics, const h264r_tuning *t);
/*
 * Autotuner: runs the batch (as h264r_submit_batch_device) under every
 * launch shape and graph setting, reps times each after warm-up runs,
 * times each setting on the host clock from the first submission to the
 * end of the last (a synchronised throughput measurement on streams[0]'s
 * CUDA stream), in three rounds over all settings in turn, each setting
 * keeping its best round.  It keeps the fastest for the batch's geometry
 * mix, unless that is less than 3 % faster than the mix's current tuning
 * (which then stays).  The
 * batch must be one that can run again with the same result: its pictures
 * reference none of its own destination slots, which holds for every
 * dependency group.  *best / *best_ms (either may be NULL) receive the
 * choice and its milliseconds per batch.
 */
int  h264r_autotune_batch_device(h264r_ctx *ctx, int n, h264r_stream *const *streams, const h264r_picture *pics,
                                 int reps, h264r_tuning *best, float *best_ms);
/* Launch sequences replayed from captured graphs, and graphs instantiated,
 * so far by this context. */
uint64_t h264r_ctx_graph_replays(const h264r_ctx *ctx);
uint64_t h264r_ctx_graphs_captured(const h264r_ctx *ctx);

#ifdef __cplusplus
}
#endif

#endif /* H264R_H */
