/*
 * h264r_parser.h — host-side H.264 front end: Annex B byte stream in,
 * per-picture reconstruction records (include/h264r.h) out.
 *
 * It is the part of the reference decoder that stays on the CPU in front of
 * the engine: NAL units, parameter sets and slice headers
 * (CH264NalUnit / CH264SPS / CH264PPS / CH264SliceHeader), CAVLC and CABAC slice data
 * (CH264SliceData::slice_data, H264SliceData.cpp; CH264MacroBlock,
 * H264MacroBlock.cpp; CH264ResidualBlockCavlc), intra prediction mode
 * derivation (8.3.1.1 / 8.3.2.1), motion vector and reference index
 * derivation (8.4.1: P_Skip, median / directional prediction, spatial and
 * temporal direct; H264InterPrediction.cpp:671-2001), prediction weights
 * (8.4.2.3), picture order counts (8.2.1), reference picture lists (8.2.4)
 * and marking (8.2.5; H264RefPicList.cpp), and the reference's output order
 * (include/h264r_order.h).  Each completed picture comes out as the records
 * the engine reconstructs, with the DPB slot it writes and the slots that
 * are due for output after it.
 *
 * Scope: frame pictures, progressive or MBAFF (frame / field MB pairs),
 * 4:2:0, 8 bits, CAVLC or CABAC, one slice group, I / P / B slices.  Field
 * pictures (PAFF), SP/SI slices, slice groups and other chroma formats return
 * H264R_ERR_UNSUPPORTED.
 *
 * Host only.  A parser object is used by one thread at a time; parsers share
 * no state, so several streams parse in parallel on their own threads.
 */
#ifndef H264R_PARSER_H
#define H264R_PARSER_H

#include <stddef.h>
#include <stdint.h>

#include "h264r.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct h264r_parser h264r_parser;

/* One completed picture, in decoding order.  Every pointer stays valid until
 * the next h264r_parser_next / feed / end call on the same parser. */
typedef struct h264r_parsed {
    h264r_picture pic;          /* records; pic.dst_slot = its DPB slot      */
    int32_t  poc;               /* PicOrderCnt                               */
    uint32_t index;             /* position in decoding order (0-based)      */
    uint8_t  idr;               /* IdrPicFlag                                */
    uint8_t  reference;         /* nal_ref_idc != 0                          */
    uint8_t  slice_type;        /* slice_type % 5 of its first slice         */
    uint8_t  reserved;
    uint32_t num_output;        /* DPB slots to output once this picture is
                                   reconstructed, in output order            */
    const uint8_t *output_slots;
    const int32_t *output_poc;  /* their PicOrderCnt                         */
    const uint32_t *output_index; /* their decoding-order index              */
} h264r_parsed;

int  h264r_parser_create(h264r_parser **out);
int  h264r_parser_destroy(h264r_parser *p);
const char *h264r_parser_last_error(const h264r_parser *p);

/* Bytes of an Annex B stream, in any chunking. */
int  h264r_parser_feed(h264r_parser *p, const uint8_t *data, size_t size);
/* End of the stream: the last picture completes with deblock = 0 (the
 * reference's flush does not deblock it, H264VideoDecoder.cpp:352-367) and
 * every held picture becomes due for output. */
int  h264r_parser_end(h264r_parser *p);
/* Next completed picture: 1 when *out was filled, 0 when none is ready,
 * negative on a stream error (the parser then stops). */
int  h264r_parser_next(h264r_parser *p, h264r_parsed *out);

/* Geometry of the active sequence once the first picture started (0 before):
 * MB width / frame height, and the DPB slots the parser uses (its references
 * plus the output reorder depth plus the picture being decoded, plus one
 * spare).  A new picture takes the slot that has been free longest, so that
 * pictures that do not depend on each other use different slots. */
int  h264r_parser_geometry(const h264r_parser *p, int *width_mbs, int *height_mbs, int *dpb_slots);

/* CAVLC table probes: decode a 16-bit window (first code bit = bit 15)
 * exactly as the parser does.  out[0] = code length in bits, then the
 * decoded values (coeff_token: TrailingOnes, TotalCoeff; total_zeros /
 * run_before: the value).  Return 0, or -1 when no code word matches.  For
 * tests that compare the tables with other decoders. */
int  h264r_probe_coeff_token(int nC, uint32_t window16, int out[3]);
int  h264r_probe_total_zeros(int max_coeff, int total_coeff, uint32_t window16, int out[2]);
int  h264r_probe_run_before(int zeros_left, uint32_t window16, int out[2]);
/* coded_block_pattern of me(v) code_num (4:2:0), or -1 */
int  h264r_probe_cbp(uint32_t code_num, int intra);
/* CABAC probes: the context initialisation values (m, n) the parser uses
 * (Tables 9-12 to 9-33) for model 0 (I slices) or 1 + cabac_init_idc and
 * ctxIdx 0..459; and one decision of its arithmetic decoding engine
 * (9.3.3.2.1) from a context state, range and offset, renormalising with
 * zero bits.  out: binVal, pStateIdx, valMPS, codIRange, codIOffset after
 * it. */
int  h264r_probe_cabac_init(int model, int ctx_idx, int out[2]);
int  h264r_probe_cabac_decision(int p_state, int val_mps, int range, int offset, int out[5]);

#ifdef __cplusplus
}
#endif

#endif /* H264R_PARSER_H */
