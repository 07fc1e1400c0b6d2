/*
 * h264r_decoder.h — whole-stream decoding on one GPU: the host front end
 * (include/h264r_parser.h) feeding the reconstruction engine
 * (include/h264r.h), with decoded pictures handed to a callback in output
 * order.
 *
 * Replaces CH264VideoDecoder (H264VideoDecoder.h:25-42,
 * H264VideoDecoder.cpp): set_output_frame_callback_functuin -> set_callback,
 * open(url) -> h264r_decoder_open, do_callback's reorder buffer -> the
 * parser's output order.  The callback convention is the reference's
 * (H264VideoDecoder.cpp:383-435, 369-374): one call per output picture in
 * output order with error_code 0, then one final call with frame == NULL
 * and error_code H264R_DECODE_FILE_END; a non-zero return from a picture
 * call stops the decode (the final call still comes).  Include
 * include/compat/H264VideoDecoder.h for the reference's C++ class itself.
 *
 * Host-side scope is the parser's: CAVLC progressive streams (see
 * h264r_parser.h); other streams fail with H264R_ERR_UNSUPPORTED.
 */
#ifndef H264R_DECODER_H
#define H264R_DECODER_H

#include <stddef.h>
#include <stdint.h>

#include "h264r.h"

#ifdef __cplusplus
extern "C" {
#endif

/* error_code of the callback, as H264_DECODE_ERROR_CODE (H264CommonFunc.h:477-484) */
#define H264R_DECODE_UNKNOWN          0
#define H264R_DECODE_FILE_END         1
#define H264R_DECODE_OPEN_FILE_FAILED 2

typedef struct h264r_decoder h264r_decoder;

/* One output picture.  Valid only during the callback. */
typedef struct h264r_frame {
    const uint8_t *y, *cb, *cr;  /* planes at coded size, host memory        */
    int32_t  width, height;      /* luma samples (coded size)                 */
    int32_t  poc;                /* PicOrderCnt                               */
    int32_t  output_count;       /* pictures output before this one           */
    uint32_t decode_index;       /* position in decoding order (m_PicNumCnt)  */
    uint8_t  slice_type;         /* slice_type % 5 of its first slice         */
    uint8_t  reserved[3];
    int32_t  slot;               /* engine DPB slot holding it (GPU-side use) */
    h264r_stream *stream;        /* engine stream of the decoder              */
} h264r_frame;

typedef int (*h264r_frame_callback)(const h264r_frame *frame, void *user, int error_code);

int  h264r_decoder_create(h264r_ctx *ctx, h264r_decoder **out);
int  h264r_decoder_destroy(h264r_decoder *d);
const char *h264r_decoder_last_error(const h264r_decoder *d);
int  h264r_decoder_set_callback(h264r_decoder *d, h264r_frame_callback cb, void *user);

/* Bytes of an Annex B stream, any chunking: pictures are reconstructed on
 * the GPU as they complete; a due picture is copied to host memory beside the
 * stream's later pictures and handed out once the copy is done (at the
 * latest by h264r_decoder_flush), so parsing is not held up by the GPU.  The
 * picture's slot is not overwritten before its callback has returned. */
int  h264r_decoder_push(h264r_decoder *d, const uint8_t *data, size_t size);
/* End of the stream: the remaining pictures, then the final callback.
 * Returns that callback's return value (or a negative error). */
int  h264r_decoder_flush(h264r_decoder *d);
/* Whole file: push + flush (CH264VideoDecoder::open).  A file that cannot
 * be read gets one callback (NULL, user, H264R_DECODE_OPEN_FILE_FAILED) and
 * returns H264R_ERR_IO. */
int  h264r_decoder_open(h264r_decoder *d, const char *path);

/* Pictures reconstructed / handed out so far. */
uint32_t h264r_decoder_decoded(const h264r_decoder *d);
uint32_t h264r_decoder_output(const h264r_decoder *d);

#ifdef __cplusplus
}
#endif

#endif /* H264R_DECODER_H */
