// h264r_syntax.cpp — sequence / picture parameter sets and slice headers
// (7.3.2.1.1, 7.3.2.2, 7.3.3, E.1.1), restated from the syntax tables; the
// reference parses the same syntax in CH264SPS::seq_parameter_set_data
// (H264SPS.cpp), CH264PPS::pic_parameter_set_rbsp (H264PPS.cpp) and
// CH264SliceHeader::slice_header (H264SliceHeader.cpp).
#include "h264r_syntax.h"

#include <cstring>

#include "../../include/h264r.h"

namespace h264r {

namespace {

// Table 7-3 / 7-4 default scaling lists, in coded (zig-zag) order
const uint8_t kDefault4x4Intra[16] = {6, 13, 13, 20, 20, 20, 28, 28, 28, 28, 32, 32, 32, 37, 37, 42};
const uint8_t kDefault4x4Inter[16] = {10, 14, 14, 20, 20, 20, 24, 24, 24, 24, 27, 27, 27, 30, 30, 34};
const uint8_t kDefault8x8Intra[64] = {6,  10, 10, 13, 11, 13, 16, 16, 16, 16, 18, 18, 18, 18, 18, 23,
                                      23, 23, 23, 23, 23, 25, 25, 25, 25, 25, 25, 25, 27, 27, 27, 27,
                                      27, 27, 27, 27, 29, 29, 29, 29, 29, 29, 29, 31, 31, 31, 31, 31,
                                      31, 33, 33, 33, 33, 33, 36, 36, 36, 36, 38, 38, 38, 40, 40, 42};
const uint8_t kDefault8x8Inter[64] = {9,  13, 13, 15, 13, 15, 17, 17, 17, 17, 19, 19, 19, 19, 19, 21,
                                      21, 21, 21, 21, 21, 22, 22, 22, 22, 22, 22, 22, 24, 24, 24, 24,
                                      24, 24, 24, 24, 25, 25, 25, 25, 25, 25, 25, 27, 27, 27, 27, 27,
                                      27, 28, 28, 28, 28, 28, 30, 30, 30, 30, 32, 32, 32, 33, 33, 35};

#define FAIL(msg)            \
    do {                     \
        if (why) *why = msg; \
        return H264R_ERR_BAD_RECORD; \
    } while (0)
#define UNSUPPORTED(msg)     \
    do {                     \
        if (why) *why = msg; \
        return H264R_ERR_UNSUPPORTED; \
    } while (0)

// scaling_list( ) (7.3.2.1.1.1); returns useDefaultScalingMatrixFlag
bool scaling_list(BitReader &br, uint8_t *list, int size)
{
    int last = 8, next = 8;
    bool use_default = false;
    for (int j = 0; j < size; j++) {
        if (next != 0) {
            const int delta = br.se();
            next = (last + delta + 256) % 256;
            use_default = j == 0 && next == 0;
        }
        list[j] = (uint8_t)(next == 0 ? last : next);
        last = list[j];
    }
    return use_default;
}

const uint8_t *default_list(int i) { return i < 3 ? kDefault4x4Intra : i < 6 ? kDefault4x4Inter : (i % 2 == 0 ? kDefault8x8Intra : kDefault8x8Inter); }

// the lists of one parameter set: present[i] from the bitstream, absent ones
// by fall-back rule A (SPS, fallback == nullptr) or B (PPS, fallback = the
// SPS lists), Table 7-2
void read_lists(BitReader &br, int count, uint8_t (*sl4)[16], uint8_t (*sl8)[64], const uint8_t (*fb4)[16],
                const uint8_t (*fb8)[64], bool *present_out)
{
    for (int i = 0; i < 12; i++) {
        const bool present = i < count ? br.flag() : false;
        if (present_out) present_out[i] = present;
        uint8_t *dst = i < 6 ? sl4[i] : sl8[i - 6];
        const int size = i < 6 ? 16 : 64;
        if (present) {
            if (scaling_list(br, dst, size)) memcpy(dst, default_list(i), size);
            continue;
        }
        if (i == 0 || i == 3 || i == 6 || i == 7) {  // the heads of the fall-back chains
            if (fb4) memcpy(dst, i < 6 ? fb4[i] : fb8[i - 6], size);
            else memcpy(dst, default_list(i), size);
        } else if (i < 6) {
            memcpy(dst, sl4[i - 1], 16);
        } else {
            memcpy(dst, sl8[i - 8], 64);  // 4:4:4 chroma 8x8 lists: two back
        }
    }
}

void skip_hrd(BitReader &br)
{
    const uint32_t cpb_cnt = br.ue() + 1;
    br.u(4);
    br.u(4);
    for (uint32_t i = 0; i < cpb_cnt && !br.err; i++) {
        br.ue();
        br.ue();
        br.u(1);
    }
    br.u(5);
    br.u(5);
    br.u(5);
    br.u(5);
}

void parse_vui(BitReader &br, Sps &sps)
{
    if (br.flag()) {  // aspect_ratio_info_present_flag
        if (br.u(8) == 255) {
            br.u(16);
            br.u(16);
        }
    }
    if (br.flag()) br.u(1);  // overscan
    if (br.flag()) {         // video_signal_type_present_flag
        br.u(3);
        br.u(1);
        if (br.flag()) br.u(24);
    }
    if (br.flag()) {  // chroma_loc_info_present_flag
        br.ue();
        br.ue();
    }
    if (br.flag()) {  // timing_info_present_flag
        br.u(16);
        br.u(16);
        br.u(16);
        br.u(16);
        br.u(1);
    }
    const bool nal_hrd = br.flag();
    if (nal_hrd) skip_hrd(br);
    const bool vcl_hrd = br.flag();
    if (vcl_hrd) skip_hrd(br);
    if (nal_hrd || vcl_hrd) br.u(1);  // low_delay_hrd_flag
    br.u(1);                          // pic_struct_present_flag
    if (br.flag()) {                  // bitstream_restriction_flag
        br.u(1);
        br.ue();
        br.ue();
        br.ue();
        br.ue();
        sps.max_num_reorder_frames = (int)br.ue();
        sps.max_dec_frame_buffering = (int)br.ue();
        sps.has_reorder = !br.err;
    }
}

}  // namespace

int parse_sps(BitReader &br, Sps &sps, const char **why)
{
    Sps s;
    s.profile_idc = (int)br.u(8);
    const uint32_t cflags = br.u(8);
    s.constraint_set3 = (cflags >> 4) & 1;
    s.level_idc = (int)br.u(8);
    s.id = (int)br.ue();
    if (s.id > 31) FAIL("seq_parameter_set_id out of range");
    for (int i = 0; i < 6; i++) memset(s.sl4[i], 16, 16);
    for (int i = 0; i < 6; i++) memset(s.sl8[i], 16, 64);
    const int p = s.profile_idc;
    if (p == 100 || p == 110 || p == 122 || p == 244 || p == 44 || p == 83 || p == 86 || p == 118 || p == 128 ||
        p == 138 || p == 139 || p == 134 || p == 135) {
        s.chroma_format_idc = (int)br.ue();
        if (s.chroma_format_idc == 3) br.u(1);
        s.bit_depth_luma = 8 + (int)br.ue();
        s.bit_depth_chroma = 8 + (int)br.ue();
        s.transform_bypass = (int)br.u(1);
        if (br.flag()) {
            s.scaling_present = true;
            read_lists(br, s.chroma_format_idc != 3 ? 8 : 12, s.sl4, s.sl8, nullptr, nullptr, nullptr);
        }
    }
    s.log2_max_frame_num = 4 + (int)br.ue();
    s.poc_type = (int)br.ue();
    if (s.poc_type == 0) {
        s.log2_max_poc_lsb = 4 + (int)br.ue();
    } else if (s.poc_type == 1) {
        s.delta_pic_order_always_zero = (int)br.u(1);
        s.offset_for_non_ref_pic = br.se();
        s.offset_for_top_to_bottom_field = br.se();
        const uint32_t n = br.ue();
        if (n > 255) FAIL("num_ref_frames_in_pic_order_cnt_cycle out of range");
        for (uint32_t i = 0; i < n; i++) s.offset_for_ref_frame.push_back(br.se());
    } else if (s.poc_type != 2) {
        FAIL("pic_order_cnt_type out of range");
    }
    s.max_num_ref_frames = (int)br.ue();
    s.gaps_allowed = (int)br.u(1);
    s.width_mbs = (int)br.ue() + 1;
    s.height_map_units = (int)br.ue() + 1;
    s.frame_mbs_only = (int)br.u(1);
    if (!s.frame_mbs_only) s.mbaff = (int)br.u(1);
    s.direct_8x8_inference = (int)br.u(1);
    if (br.flag()) {  // frame_cropping_flag: output is at coded size
        br.ue();
        br.ue();
        br.ue();
        br.ue();
    }
    if (br.flag()) parse_vui(br, s);
    if (br.err) FAIL("truncated sequence parameter set");
    if (s.max_num_ref_frames > 16 || s.log2_max_frame_num > 16 || s.log2_max_poc_lsb > 16) FAIL("SPS field out of range");
    if (s.chroma_format_idc != 1) UNSUPPORTED("chroma format other than 4:2:0");
    if (s.bit_depth_luma != 8 || s.bit_depth_chroma != 8) UNSUPPORTED("bit depth other than 8");
    if (s.transform_bypass) UNSUPPORTED("transform bypass");
    if (s.width_mbs > 1024 || s.frame_height_mbs() > 1024) FAIL("picture size out of range");
    s.valid = true;
    sps = s;
    return H264R_OK;
}

int parse_pps(BitReader &br, const Sps *sps_table, Pps &pps, const char **why)
{
    Pps q;
    q.id = (int)br.ue();
    q.sps_id = (int)br.ue();
    if (q.id > 255 || q.sps_id > 31) FAIL("parameter set id out of range");
    const Sps &sps = sps_table[q.sps_id];
    if (!sps.valid) FAIL("picture parameter set refers to an unknown SPS");
    q.cabac = (int)br.u(1);
    q.bottom_field_pic_order_present = (int)br.u(1);
    q.num_slice_groups = (int)br.ue() + 1;
    if (q.num_slice_groups > 1) UNSUPPORTED("slice groups (FMO)");
    q.num_ref_idx_default[0] = (int)br.ue() + 1;
    q.num_ref_idx_default[1] = (int)br.ue() + 1;
    q.weighted_pred = (int)br.u(1);
    q.weighted_bipred_idc = (int)br.u(2);
    q.pic_init_qp = 26 + br.se();
    q.pic_init_qs = 26 + br.se();
    q.chroma_qp_offset[0] = br.se();
    q.deblocking_control = (int)br.u(1);
    q.constrained_intra_pred = (int)br.u(1);
    q.redundant_pic_cnt_present = (int)br.u(1);
    q.chroma_qp_offset[1] = q.chroma_qp_offset[0];
    for (int i = 0; i < 12; i++) q.sl_present[i] = false;
    if (br.more_rbsp_data()) {
        q.transform_8x8_mode = (int)br.u(1);
        if (br.flag()) {
            q.scaling_present = true;
            read_lists(br, 6 + (sps.chroma_format_idc != 3 ? 2 : 6) * q.transform_8x8_mode, q.sl4, q.sl8, sps.sl4, sps.sl8,
                       q.sl_present);
            // second_chroma_qp_index_offset follows the scaling lists for
            // every PPS in 7.3.2.2; the reference reads it only inside the
            // pic_scaling_matrix_present_flag branch (H264PPS.cpp:206-227)
            // and otherwise keeps chroma_qp_index_offset, which is followed
            // here so that Cr is reconstructed as the reference does
            q.chroma_qp_offset[1] = br.se();
        }
    }
    if (br.err) FAIL("truncated picture parameter set");
    if (q.num_ref_idx_default[0] > 32 || q.num_ref_idx_default[1] > 32 || q.weighted_bipred_idc > 2 ||
        q.pic_init_qp < 0 || q.pic_init_qp > 51 || q.chroma_qp_offset[0] < -12 || q.chroma_qp_offset[0] > 12 ||
        q.chroma_qp_offset[1] < -12 || q.chroma_qp_offset[1] > 12)
        FAIL("PPS field out of range");
    if (!q.scaling_present) {  // the sequence lists (flat when the SPS has none)
        memcpy(q.sl4, sps.sl4, sizeof(q.sl4));
        memcpy(q.sl8, sps.sl8, sizeof(q.sl8));
    }
    q.valid = true;
    pps = q;
    return H264R_OK;
}

namespace {

int parse_weights(BitReader &br, SliceHeader &sh, int nlists, const char **why)
{
    PredWeights &w = sh.pw;
    w.luma_log2 = (int)br.ue();
    w.chroma_log2 = (int)br.ue();
    if (w.luma_log2 > 7 || w.chroma_log2 > 7) FAIL("weight denominator out of range");
    for (int l = 0; l < nlists; l++) {
        for (int i = 0; i < sh.num_ref_idx_active[l]; i++) {
            w.lflag[l][i] = br.flag();
            w.lw[l][i] = 1 << w.luma_log2;
            w.lo[l][i] = 0;
            if (w.lflag[l][i]) {
                w.lw[l][i] = br.se();
                w.lo[l][i] = br.se();
            }
            w.cflag[l][i] = br.flag();
            for (int c = 0; c < 2; c++) {
                w.cw[l][i][c] = 1 << w.chroma_log2;
                w.co[l][i][c] = 0;
            }
            if (w.cflag[l][i]) {
                for (int c = 0; c < 2; c++) {
                    w.cw[l][i][c] = br.se();
                    w.co[l][i][c] = br.se();
                }
            }
        }
    }
    sh.weights_present = true;
    return H264R_OK;
}

}  // namespace

int parse_slice_header(BitReader &br, int nal_unit_type, int nal_ref_idc, const Sps *sps_table, const Pps *pps_table,
                       SliceHeader &sh, const char **why)
{
    SliceHeader h;
    h.nal_unit_type = nal_unit_type;
    h.nal_ref_idc = nal_ref_idc;
    h.idr = nal_unit_type == 5;
    h.first_mb = (int)br.ue();
    h.raw_slice_type = (int)br.ue();
    if (h.raw_slice_type > 9) FAIL("slice_type out of range");
    h.slice_type = h.raw_slice_type % 5;
    h.pps_id = (int)br.ue();
    if (h.pps_id > 255 || !pps_table[h.pps_id].valid) FAIL("slice refers to an unknown PPS");
    const Pps &pps = pps_table[h.pps_id];
    const Sps &sps = sps_table[pps.sps_id];
    h.frame_num = (int)br.u(sps.log2_max_frame_num);
    if (!sps.frame_mbs_only) {
        h.field_pic = (int)br.u(1);
        if (h.field_pic) h.bottom_field = (int)br.u(1);
    }
    if (h.field_pic) UNSUPPORTED("field pictures (PAFF)");
    h.mbaff = sps.mbaff && !h.field_pic;
    if (h.idr) h.idr_pic_id = (int)br.ue();
    if (sps.poc_type == 0) {
        h.poc_lsb = (int)br.u(sps.log2_max_poc_lsb);
        if (pps.bottom_field_pic_order_present && !h.field_pic) h.delta_poc_bottom = br.se();
    }
    if (sps.poc_type == 1 && !sps.delta_pic_order_always_zero) {
        h.delta_poc[0] = br.se();
        if (pps.bottom_field_pic_order_present && !h.field_pic) h.delta_poc[1] = br.se();
    }
    if (pps.redundant_pic_cnt_present) h.redundant_pic_cnt = (int)br.ue();
    if (h.slice_type == kSliceB) h.direct_spatial = (int)br.u(1);
    if (h.slice_type == kSliceP || h.slice_type == kSliceSP || h.slice_type == kSliceB) {
        h.num_ref_idx_active[0] = pps.num_ref_idx_default[0];
        h.num_ref_idx_active[1] = h.slice_type == kSliceB ? pps.num_ref_idx_default[1] : 0;
        if (br.flag()) {
            h.num_ref_idx_active[0] = (int)br.ue() + 1;
            if (h.slice_type == kSliceB) h.num_ref_idx_active[1] = (int)br.ue() + 1;
        }
        if (h.num_ref_idx_active[0] > 32 || h.num_ref_idx_active[1] > 32) FAIL("num_ref_idx_active out of range");
    }
    // ref_pic_list_modification( )
    if (h.slice_type != kSliceI && h.slice_type != kSliceSI) {
        for (int l = 0; l < (h.slice_type == kSliceB ? 2 : 1); l++) {
            if (br.flag()) {
                for (int n = 0; n < 66; n++) {
                    RefMod m;
                    m.idc = (int)br.ue();
                    if (m.idc == 3) break;
                    if (m.idc > 5 || br.err) FAIL("modification_of_pic_nums_idc out of range");
                    m.value = (int)br.ue();
                    h.mods[l].push_back(m);
                }
            }
        }
    }
    if ((pps.weighted_pred && (h.slice_type == kSliceP || h.slice_type == kSliceSP)) ||
        (pps.weighted_bipred_idc == 1 && h.slice_type == kSliceB)) {
        const int rc = parse_weights(br, h, h.slice_type == kSliceB ? 2 : 1, why);
        if (rc) return rc;
    }
    if (nal_ref_idc != 0) {  // dec_ref_pic_marking( )
        if (h.idr) {
            h.no_output_of_prior_pics = (int)br.u(1);
            h.long_term_reference = (int)br.u(1);
        } else {
            h.adaptive_marking = (int)br.u(1);
            if (h.adaptive_marking) {
                for (int n = 0; n < 66; n++) {
                    Mmco m = {0, 0, 0, 0, 0};
                    m.op = (int)br.ue();
                    if (m.op == 0) break;
                    if (m.op > 6 || br.err) FAIL("memory_management_control_operation out of range");
                    if (m.op == 1 || m.op == 3) m.diff_pic_nums_minus1 = (int)br.ue();
                    if (m.op == 2) m.long_term_pic_num = (int)br.ue();
                    if (m.op == 3 || m.op == 6) m.long_term_frame_idx = (int)br.ue();
                    if (m.op == 4) m.max_long_term_frame_idx_plus1 = (int)br.ue();
                    h.mmcos.push_back(m);
                }
            }
        }
    }
    if (pps.cabac && h.slice_type != kSliceI && h.slice_type != kSliceSI) h.cabac_init_idc = (int)br.ue();
    h.slice_qp_delta = br.se();
    if (h.slice_type == kSliceSP || h.slice_type == kSliceSI) {
        if (h.slice_type == kSliceSP) h.sp_for_switch = (int)br.u(1);
        h.slice_qs_delta = br.se();
    }
    if (pps.deblocking_control) {
        h.disable_deblocking_filter_idc = (int)br.ue();
        if (h.disable_deblocking_filter_idc > 2) FAIL("disable_deblocking_filter_idc out of range");
        if (h.disable_deblocking_filter_idc != 1) {
            h.alpha_offset_div2 = br.se();
            h.beta_offset_div2 = br.se();
        }
    }
    if (br.err) FAIL("truncated slice header");
    const int qp = pps.pic_init_qp + h.slice_qp_delta;
    if (qp < 0 || qp > 51) FAIL("SliceQPY out of range");
    if (h.slice_type == kSliceSP || h.slice_type == kSliceSI) UNSUPPORTED("SP / SI slices");
    sh = h;
    return H264R_OK;
}

}  // namespace h264r
