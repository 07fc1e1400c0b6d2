/*
 * dumpfmt.h — on-disk container for reconstruction records plus the
 * reference decoder's own sample planes (test infrastructure only).
 *
 * A dump file is a sequence of pictures in decoding order:
 *   file header:  char magic[8] = "H264RDMP"; uint32 version (=1); uint32 0
 *   per picture:  h264r_dump_pic header, then
 *                 h264r_mb[num_mbs], h264r_slice[num_slices],
 *                 h264r_weight[num_weights], motion[motion_bytes],
 *                 coef[coef_bytes], pcm[num_pcm * 384],
 *                 pre-deblock planes  (plane_bytes, if flags & 1),
 *                 post-deblock planes (plane_bytes, if flags & 2)
 * Planes are the reference's single Y/Cb/Cr allocation at coded size
 * (H264PictureBase.cpp:162-181): W*H luma, then (W/2)*(H/2) Cb, then Cr.
 * Used by the oracle checker, the golden-fixture generator and the tests.
 */
#ifndef H264R_DUMPFMT_H
#define H264R_DUMPFMT_H

#include <stdint.h>

#define H264R_DUMP_MAGIC   "H264RDMP"
#define H264R_DUMP_VERSION 1
#define H264R_DUMP_PIC_TAG 0x31434950u /* "PIC1" */

#define H264R_DUMP_HAS_PRE   1u
#define H264R_DUMP_HAS_POST  2u

typedef struct h264r_dump_pic {
    uint32_t tag;             /* H264R_DUMP_PIC_TAG                        */
    uint16_t width_mbs, height_mbs;
    uint8_t  structure, mbaff, dst_slot, deblock;
    uint16_t num_slices, num_weights;
    uint32_t num_mbs, motion_bytes, coef_bytes, num_pcm;
    uint8_t  scaling4x4[6][16];
    uint8_t  scaling8x8[6][64];
    int32_t  poc;             /* PicOrderCnt, informational                */
    int32_t  pic_num_cnt;     /* decode counter, informational             */
    uint32_t flags;           /* H264R_DUMP_HAS_*                          */
    uint32_t plane_bytes;     /* bytes of one plane set                    */
} h264r_dump_pic;

#endif
