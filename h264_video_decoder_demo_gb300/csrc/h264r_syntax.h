// h264r_syntax.h — parameter sets and slice headers (7.3.2.1, 7.3.2.2, 7.3.3)
// for the host-side parser.  Host only.
#pragma once

#include <cstdint>
#include <vector>

#include "h264r_bits.h"

namespace h264r {

enum { kSliceP = 0, kSliceB = 1, kSliceI = 2, kSliceSP = 3, kSliceSI = 4 };

struct Sps {
    bool valid = false;
    int profile_idc = 0, constraint_set3 = 0, level_idc = 0, id = 0;
    int chroma_format_idc = 1, bit_depth_luma = 8, bit_depth_chroma = 8;
    int transform_bypass = 0;
    bool scaling_present = false;
    uint8_t sl4[6][16], sl8[6][64];  // coded (zig-zag) order
    int log2_max_frame_num = 4, poc_type = 0, log2_max_poc_lsb = 4;
    int delta_pic_order_always_zero = 0, offset_for_non_ref_pic = 0, offset_for_top_to_bottom_field = 0;
    std::vector<int> offset_for_ref_frame;
    int max_num_ref_frames = 0, gaps_allowed = 0;
    int width_mbs = 0, height_map_units = 0, frame_mbs_only = 1, mbaff = 0, direct_8x8_inference = 0;
    int frame_height_mbs() const { return (2 - frame_mbs_only) * height_map_units; }
    // VUI bitstream restriction
    bool has_reorder = false;
    int max_num_reorder_frames = 0, max_dec_frame_buffering = 0;
};

struct Pps {
    bool valid = false;
    int id = 0, sps_id = 0, cabac = 0, bottom_field_pic_order_present = 0, num_slice_groups = 1;
    int num_ref_idx_default[2] = {1, 1};
    int weighted_pred = 0, weighted_bipred_idc = 0, pic_init_qp = 26, pic_init_qs = 26;
    int chroma_qp_offset[2] = {0, 0};
    int deblocking_control = 0, constrained_intra_pred = 0, redundant_pic_cnt_present = 0;
    int transform_8x8_mode = 0;
    bool scaling_present = false;
    bool sl_present[12];
    uint8_t sl4[6][16], sl8[6][64];
};

struct RefMod {
    int idc;   // modification_of_pic_nums_idc
    int value; // abs_diff_pic_num_minus1 or long_term_pic_num
};

struct Mmco {
    int op, diff_pic_nums_minus1, long_term_pic_num, long_term_frame_idx, max_long_term_frame_idx_plus1;
};

struct PredWeights {
    int luma_log2 = 0, chroma_log2 = 0;
    // [list][refIdx]: weight, offset; chroma [.][.][Cb/Cr]
    int lw[2][32], lo[2][32], cw[2][32][2], co[2][32][2];
    bool lflag[2][32], cflag[2][32];
};

struct SliceHeader {
    int nal_ref_idc = 0, nal_unit_type = 0, idr = 0;
    int first_mb = 0, slice_type = 0, raw_slice_type = 0, pps_id = 0;
    int frame_num = 0, field_pic = 0, bottom_field = 0, idr_pic_id = 0;
    int poc_lsb = 0, delta_poc_bottom = 0, delta_poc[2] = {0, 0}, redundant_pic_cnt = 0;
    int direct_spatial = 0, num_ref_idx_active[2] = {0, 0};
    std::vector<RefMod> mods[2];
    bool weights_present = false;
    PredWeights pw;
    int no_output_of_prior_pics = 0, long_term_reference = 0, adaptive_marking = 0;
    std::vector<Mmco> mmcos;
    int cabac_init_idc = 0, slice_qp_delta = 0, sp_for_switch = 0, slice_qs_delta = 0;
    int disable_deblocking_filter_idc = 0, alpha_offset_div2 = 0, beta_offset_div2 = 0;
    int mbaff = 0;  // MbaffFrameFlag
};

// Parse functions return 0 or a negative H264R_ERR_* code; `why` receives a
// short reason on failure.
int parse_sps(BitReader &br, Sps &sps, const char **why);
int parse_pps(BitReader &br, const Sps *sps_table, Pps &pps, const char **why);
int parse_slice_header(BitReader &br, int nal_unit_type, int nal_ref_idc, const Sps *sps_table, const Pps *pps_table,
                       SliceHeader &sh, const char **why);

}  // namespace h264r
