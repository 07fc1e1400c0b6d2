/*
 * h264r_writer.h — seeded H.264 bitstream writer (CAVLC, progressive frames).
 *
 * No counterpart in the reference decoder, which only reads streams.  It
 * writes Annex B streams of random but valid syntax with the shapes and value
 * distributions of the benchmark configurations, so that the reference
 * decoder itself can decode the very content the engine is measured on:
 * SPS / PPS / slice headers (7.3.2.1, 7.3.2.2, 7.3.3, pred_weight_table
 * 7.3.3.2), CAVLC slice data with skip runs, I_PCM, Intra 4x4 / 8x8 / 16x16,
 * P and B partitions down to 4x4, direct prediction, explicit or implicit
 * weighted prediction and 8x8 transforms (7.3.4, 7.3.5, 9.2), progressive
 * or MBAFF frames (frame / field MB pairs, mb_field_decoding_flag).
 *
 * The writer chooses syntax elements, not samples: target motion vectors,
 * intra prediction modes, reference indices, coded block patterns, QP and
 * coefficient levels are drawn from the configuration, and the values that
 * are coded relative to a prediction (mvd, prev_intra4x4_pred_mode_flag /
 * rem_intra4x4_pred_mode, CAVLC nC) are derived by running the library's own
 * front end (include/h264r_parser.h) on the stream as it is written.  Intra
 * modes are drawn only from the modes whose neighbouring samples are
 * available; explicit bi-predictive weights keep every pairwise sum within
 * the range 8.4.2.3 allows; explicit weighting never meets a list-1-only
 * partition (the writer avoids it, also for direct blocks).
 *
 * MBAFF: a pair whose two MBs are skipped takes the field flag the decoder
 * infers (left pair, else the pair above, else frame); field MBs index the
 * fields of the reference frames (twice the entries).
 *
 * Deterministic for a given configuration on every host (own generator, no
 * floating point).  Host only.
 */
#ifndef H264R_WRITER_H
#define H264R_WRITER_H

#include <stddef.h>
#include <stdint.h>

#include "h264r.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct h264r_writer_cfg {
    uint32_t seed;
    uint16_t width_mbs;         /* PicWidthInMbs                               */
    uint16_t height_mbs;        /* frame height in MBs                         */
    uint16_t num_pictures;
    uint8_t  profile_idc;       /* 66 Baseline (4x4 transforms, no B) or 100 High */
    uint8_t  level_idc;         /* 0: the smallest level whose DPB holds 4 frames */
    uint8_t  gop_length;        /* an I picture every gop_length pictures (display
                                   order); 0: only the first                   */
    uint8_t  b_pictures;        /* B pictures between anchors (0: I/P only)     */
    uint8_t  num_refs;          /* max_num_ref_frames (1..15): the length of list
                                   0 once as many reference pictures exist;
                                   list 1 of B slices up to 2                  */
    uint8_t  transform8x8;      /* High: transform_8x8_mode_flag               */
    uint8_t  weighted;          /* 0 none; 1 explicit (P and B); 2 implicit B   */
    uint8_t  direct_spatial;    /* B_Skip / B_Direct: 1 spatial, 0 temporal (the
                                   reference decoder divides by zero in temporal
                                   direct prediction of inter co-located blocks,
                                   so streams for it use spatial)             */
    uint8_t  min_partition;     /* 0 16x16, 1 16x8 / 8x16, 2 8x8, 3 down to 4x4
                                   (P; B quadrants stay 8x8 or direct: the
                                   reference decoder fails B sub_mb_type > 3) */
    uint8_t  intra_percent;     /* intra MBs in P and B pictures               */
    uint8_t  skip_percent;      /* P_Skip / B_Skip MBs                         */
    uint8_t  edge_mv_percent;   /* partitions whose reference block lies past a
                                   picture edge                                */
    uint8_t  qp_min, qp_max;    /* QPY of each coded MB (mb_qp_delta)          */
    uint8_t  filter_offset_max; /* slice alpha / beta offsets (div2) uniform in
                                   [-max, max]                                 */
    uint8_t  coef_density;      /* percent: coded 8x8 luma blocks / chroma      */
    uint8_t  slices;            /* slices per picture (1..)                    */
    uint8_t  pcm_permille;      /* I_PCM MBs per thousand intra MBs            */
    uint8_t  chroma_qp_offset_max; /* chroma_qp_index_offset (and the second one,
                                   High) uniform in [-max, max]                */
    uint8_t  mbaff;             /* 1: MBAFF frames (High): MB pairs coded as
                                   two frame MBs or two field MBs; height_mbs
                                   even; bottom field POC one above the top   */
    uint8_t  field_percent;     /* MBAFF: MB pairs coded as field MBs          */
    uint8_t  reserved;
    uint16_t mv_range;          /* MV components uniform in [-mv_range, mv_range]
                                   quarter samples                            */
    uint16_t reserved2;
} h264r_writer_cfg;

/* Write a whole stream: *data receives a buffer of *size bytes (Annex B, SPS
 * and PPS first) to be released with h264r_writer_free.  Returns 0, or
 * H264R_ERR_INVALID_ARG for a configuration outside the ranges above. */
int  h264r_write_stream(const h264r_writer_cfg *cfg, uint8_t **data, size_t *size);
void h264r_writer_free(uint8_t *data);
/* Why the last h264r_write_stream call of this thread failed. */
const char *h264r_writer_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* H264R_WRITER_H */
