/*
 * h264r_order.h — output order of decoded pictures (host only).
 *
 * The reference hands decoded pictures to its output callback through a
 * bounded reorder buffer (CH264PicturesGOP::getOneOutPicture,
 * H264PicturesGOP.cpp:89-168), driven once per decoded picture by
 * CH264VideoDecoder::do_callback (H264VideoDecoder.cpp:383-435): an IDR
 * picture first flushes the buffer in POC order; with a depth of 0 every
 * picture goes out at once; otherwise pictures are held until the buffer is
 * full, after which each new picture either goes out itself (when its POC is
 * below every held one) or takes the place of the held picture with the
 * lowest POC, which goes out.  The end of the stream flushes the rest
 * (H264VideoDecoder.cpp:353-367).  This is that logic for the engine's DPB
 * slots: the caller names each picture by a tag (for instance its slot) and
 * copies out (h264r_output) the pictures it returns.
 */
#ifndef H264R_ORDER_H
#define H264R_ORDER_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct h264r_order h264r_order;

/* max_num_reorder_frames: 0..16, from the SPS VUI, or
 * h264r_order_infer_depth when the VUI has none. */
int h264r_order_create(int max_num_reorder_frames, h264r_order **out);
int h264r_order_destroy(h264r_order *q);

/* A picture finished decoding (decoding order).  Writes the tags of the
 * pictures to output now, in output order, to out[] (cap >= depth + 1) and
 * returns how many (or a negative error code).  idr != 0: the picture is an
 * IDR picture, so every held picture goes out first. */
int h264r_order_push(h264r_order *q, uint64_t tag, int32_t poc, int idr, uint64_t *out, int cap);

/* End of the stream: the tags of every held picture, in output order. */
int h264r_order_flush(h264r_order *q, uint64_t *out, int cap);

/* 1 while the picture waits for output (its DPB slot must not be reused). */
int h264r_order_holds(const h264r_order *q, uint64_t tag);

/* The depth the reference infers when the VUI gives none (H264SPS.cpp:365-396):
 * 0 for the intra profiles with constraint_set3_flag, else
 * min(MaxDpbMbs(level) / (width_mbs * frame_height_mbs), 16) from Table A-1. */
int h264r_order_infer_depth(int profile_idc, int constraint_set3_flag, int level_idc, int width_mbs, int frame_height_mbs);

#ifdef __cplusplus
}
#endif

#endif /* H264R_ORDER_H */
