/*
 * h264r_oracle.h — CPU restatement of the reference decoder's macroblock
 * reconstruction (test infrastructure: the checker the GPU engine is held
 * to, never the engine itself).
 */
#ifndef H264R_ORACLE_H
#define H264R_ORACLE_H

#include <stdint.h>
#include "../include/h264r.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Bytes of one DPB picture buffer (Y, Cb, Cr contiguous) plus a zero guard
 * that absorbs the reference's field-reference over-reads. */
uint64_t h264o_slot_bytes(int width_mbs, int height_mbs);

/*
 * Reconstruct one picture into dpb[pic->dst_slot] exactly as the reference
 * decoder does: the buffer is cleared (CH264PictureBase::reset), every
 * macroblock is reconstructed in decoding order, and, when pic->deblock is
 * set, the 8.7 filter runs over the picture.  When pre is not NULL the
 * pre-deblocking planes are copied there.  dpb[i] must hold
 * h264o_slot_bytes() bytes for every slot the records reference.
 * Returns 0, or a negative H264R_ERR_* code.
 */
int h264o_reconstruct(const h264r_picture *pic, uint8_t *const *dpb, int nslots, uint8_t *pre);

/* Only the deblocking pass, in place on dpb[pic->dst_slot]. */
int h264o_deblock(const h264r_picture *pic, uint8_t *const *dpb, int nslots);

/* YUV 4:2:0 planes (Y, Cb, Cr contiguous, coded size) to BGR24 rows of
 * row_bytes bytes, bottom-up when flip (CH264PictureBase::
 * convertYuv420pToBgr24 / convertYuv420pToBgr24FlipLines,
 * H264PictureBase.cpp:440-499). */
void h264o_bgr24(int width, int height, const uint8_t *yuv, uint8_t *bgr, int row_bytes, int flip);

#ifdef __cplusplus
}
#endif

#endif
