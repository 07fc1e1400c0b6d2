/*
 * h264r_synth.h — seeded synthetic picture records for benchmarks and
 * parity tests (no counterpart in the reference, which only decodes
 * bitstreams).  The generator emits, in decoding order, the records a
 * conforming host parser would emit for a stream with the requested coding
 * tools: I/P/B pictures, 16x16..4x4 partitions, several reference pictures,
 * explicit or implicit weighted prediction, 4x4/8x8 transforms, intra modes
 * drawn from the modes whose neighbours are available, random QP and
 * deblocking offsets.  Same seed, same records, on any host.
 */
#ifndef H264R_SYNTH_H
#define H264R_SYNTH_H

#include "h264r.h"

#ifdef __cplusplus
extern "C" {
#endif

#define H264R_SYNTH_GOP_IPPP 0   /* I then P pictures                       */
#define H264R_SYNTH_GOP_IBBP 1   /* I/P anchors every 3rd picture, 2 B between */

#define H264R_SYNTH_WP_NONE     0
#define H264R_SYNTH_WP_EXPLICIT 1 /* P and B: explicit weights              */
#define H264R_SYNTH_WP_IMPLICIT 2 /* P explicit, B implicit                  */

typedef struct h264r_synth_cfg {
    uint32_t seed;
    uint16_t width_mbs, height_mbs;
    uint16_t num_pictures;      /* pictures in the stream                    */
    uint16_t gop_length;        /* I every gop_length pictures (display)     */
    uint8_t  gop_kind;          /* H264R_SYNTH_GOP_*                         */
    uint8_t  num_refs;          /* 1..4 reference pictures for P            */
    uint8_t  transform8x8;      /* allow 8x8 transforms (High profile)       */
    uint8_t  weighted;          /* H264R_SYNTH_WP_*                          */
    uint8_t  min_partition;     /* 0: 16x16 only, 1: 16x8/8x16, 2: 8x8, 3: 4x4 */
    uint8_t  intra_percent;     /* intra MBs in P/B pictures                 */
    uint8_t  skip_percent;      /* skipped MBs in P/B pictures               */
    uint8_t  qp_min, qp_max;    /* per-MB QPY range                          */
    uint8_t  edge_mv_percent;   /* MVs pointing beyond the picture edges     */
    int16_t  mv_range;          /* MVs uniform in [-mv_range, mv_range] qpel */
    int8_t   filter_offset_max; /* slice alpha/beta offsets in [-max, max]   */
    uint8_t  coef_density;      /* 0..100: share of coded 4x4 blocks        */
    uint8_t  mbaff;             /* 1: MBAFF frames (frame/field MB pairs)     */
    uint8_t  field_percent;     /* MBAFF: MB pairs coded as field MBs         */
    uint8_t  slice_rows;        /* 0: one slice per picture; N: a new slice
                                   every N MB rows (MB-pair rows for MBAFF),
                                   each with its own QP offsets, filter
                                   offsets and deblocking mode (0, 1 or 2)    */
    uint8_t  cip_percent;       /* P/B pictures coded with
                                   constrained_intra_pred_flag               */
    uint8_t  paff_percent;      /* frames coded as two field pictures (PAFF:
                                   top then bottom, in the frame's slot;
                                   height_mbs even), the others as frames
                                   (MBAFF frames when mbaff is set)          */
} h264r_synth_cfg;

typedef struct h264r_synth h264r_synth;

int h264r_synth_create(const h264r_synth_cfg *cfg, h264r_synth **out);
/* DPB slots the generated stream needs. */
int h264r_synth_dpb_slots(const h264r_synth *g);
/* Next picture in decoding order.  The record pointers stay valid until the
 * next call or h264r_synth_destroy.  Returns 0, or 1 at the end of stream.
 * *dependency_group receives a number that is equal for consecutive
 * pictures that reference none of each other (they may share a batch). */
int h264r_synth_next(h264r_synth *g, h264r_picture *pic, int *dependency_group);
int h264r_synth_destroy(h264r_synth *g);

#ifdef __cplusplus
}
#endif

#endif
