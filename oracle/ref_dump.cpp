/*
 * ref_dump.cpp — test harness around the UNMODIFIED reference decoder
 * (jfu222/h264_video_decoder_demo), linked from its own object files.
 *
 * It decodes an Annex-B stream with CH264VideoDecoder::open
 * (H264VideoDecoder.cpp:56) and intercepts every call of
 * CH264PictureBase::Deblocking_filter_process (made from
 * end_decode_the_picture_and_get_a_new_empty_picture,
 * H264PictureBase.cpp:707) with the linker's --wrap option.  At that point
 * the picture is fully reconstructed but not yet deblocked, so the harness
 * serialises:
 *   - the reconstruction records (include/h264r.h) restated from the
 *     picture's CH264MacroBlock array (H264MacroBlock.h:110-252),
 *   - the reference's pre-deblock planes,
 *   - after calling the real filter, the post-deblock planes.
 * The records are what the GPU engine consumes; the planes are the golden
 * outputs its oracle and kernels must reproduce byte for byte.
 *
 * Usage: ref_dump <in.h264> <out.dmp> [max_pictures] [--no-planes] [--bmp <dir>]
 *                 [--order <file>] [--yuv <file>] (--yuv: every output picture's planes)
 * Test infrastructure only; never part of the engine.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <map>
#include <algorithm>

#include "H264VideoDecoder.h"
#include "H264Picture.h"
#include "H264PictureBase.h"
#include "H264MacroBlock.h"

#include "../include/h264r.h"
#include "dumpfmt.h"

static FILE *g_out = NULL;
static int g_pictures = 0;
static int g_max_pictures = 1 << 30;
static int g_write_planes = 1;
static const char *g_bmp_dir = NULL;  // --bmp: the reference's BMP of every dumped picture
static FILE *g_order = NULL;         // --order: decoding order (POC, IdrPicFlag, reorder depth) and output order
static FILE *g_yuv = NULL;           // --yuv: every output picture's planes, in output order
static int g_unsupported = 0;
static int g_verbose = 1;

extern "C" int __real__ZN16CH264PictureBase25Deblocking_filter_processEv(CH264PictureBase *self);

static int slot_of(CH264PictureBase *pic, CH264Picture *p)
{
    if (p == NULL) return -1;
    for (int i = 0; i < 16; i++)
        if (pic->m_dpb[i] == p) return i;
    return 62; /* pointer outside the DPB: distinct identity */
}

/* shape codes of an inter MB (see h264r.h "Motion payload"):
   macroblock partition 16x16/16x8/8x16/8x8 -> 0..3 */
static int part_code(H264_MB_TYPE t)
{
    int w = 0, h = 0;
    if (CH264MacroBlock::getMbPartWidthAndHeight(t, w, h) != 0) return -1;
    if (w == 16 && h == 16) return 0;
    if (w == 16 && h == 8) return 1;
    if (w == 8 && h == 16) return 2;
    if (w == 8 && h == 8) return 3;
    return -1;
}

/* sub-macroblock partition 8x8/8x4/4x8/4x4 -> 0..3 */
static int sub_code(H264_MB_TYPE t)
{
    int w = 0, h = 0;
    if (CH264MacroBlock::getMbPartWidthAndHeight(t, w, h) != 0) return -1;
    if (w == 8 && h == 8) return 0;
    if (w == 8 && h == 4) return 1;
    if (w == 4 && h == 8) return 2;
    if (w == 4 && h == 4) return 3;
    return -1;
}

/* entry index covering 4x4 block (bx, by) for a shape code */
static int entry_of_block(int shape, int bx, int by)
{
    int mp = shape & 3;
    if (mp == 0) return 0;
    if (mp == 1) return by >> 1;
    if (mp == 2) return bx >> 1;
    int q = (by >> 1) * 2 + (bx >> 1), base = 0;
    for (int i = 0; i < q; i++) {
        int sc = (shape >> (2 + 2 * i)) & 3;
        base += (sc == 0) ? 1 : (sc == 3 ? 4 : 2);
    }
    int sc = (shape >> (2 + 2 * q)) & 3, sx = bx & 1, sy = by & 1;
    if (sc == 0) return base;
    if (sc == 1) return base + sy;
    if (sc == 2) return base + sx;
    return base + sy * 2 + sx;
}

static void put(const void *p, size_t n) { fwrite(p, 1, n, g_out); }

static void dump_picture(CH264PictureBase *pic, const uint8_t *pre, const uint8_t *post, size_t plane_bytes)
{
    CH264SliceHeader &sh = pic->m_h264_slice_header;
    const int n = pic->PicSizeInMbs;
    std::vector<h264r_mb> mbs(n);
    std::vector<h264r_slice> slices;
    std::map<int, int> slice_index;
    std::vector<h264r_weight> weights;
    std::vector<uint8_t> motion, coef, pcm;
    h264r_weight wdef;
    memset(&wdef, 0, sizeof(wdef));
    weights.push_back(wdef); /* index 0: default prediction */

    auto add_weight = [&](const h264r_weight &w) -> uint16_t {
        for (size_t i = 0; i < weights.size(); i++)
            if (memcmp(&weights[i], &w, sizeof(w)) == 0) return (uint16_t)i;
        weights.push_back(w);
        return (uint16_t)(weights.size() - 1);
    };

    const int slice_type = sh.slice_type % 5;

    for (int addr = 0; addr < n; addr++) {
        CH264MacroBlock &mb = pic->m_mbs[addr];
        h264r_mb r;
        memset(&r, 0, sizeof(r));
        r.coef = H264R_NONE;
        r.aux = H264R_NONE;

        if (mb.m_mb_pred_mode == Intra_4x4) r.type = H264R_MB_I4x4;
        else if (mb.m_mb_pred_mode == Intra_8x8) r.type = H264R_MB_I8x8;
        else if (mb.m_mb_pred_mode == Intra_16x16) r.type = H264R_MB_I16x16;
        else if (mb.m_name_of_mb_type == I_PCM) r.type = H264R_MB_IPCM;
        else if (mb.m_name_of_mb_type == MB_TYPE_NA) r.type = H264R_MB_NONE;
        else r.type = H264R_MB_INTER;

        if (mb.transform_size_8x8_flag) r.flags |= H264R_MBF_T8x8;
        if (mb.mb_field_decoding_flag && sh.MbaffFrameFlag) r.flags |= H264R_MBF_FIELD;
        if (mb.constrained_intra_pred_flag) r.flags |= H264R_MBF_CIP;
        if (mb.TransformBypassModeFlag) g_unsupported |= 1;
        r.qpy = (uint8_t)mb.QPY;
        r.i16_mode = (uint8_t)mb.Intra16x16PredMode;
        r.chroma_mode = (uint8_t)mb.intra_chroma_pred_mode;
        for (int b = 0; b < 16; b++)
            if (mb.mb_luma_4x4_non_zero_count_coeff[b] > 0) r.nz4x4 |= (uint16_t)(1u << b);
        for (int b = 0; b < 4; b++)
            if (mb.mb_luma_8x8_non_zero_count_coeff[b] > 0) r.nz8x8 |= (uint8_t)(1u << b);

        if (slice_index.find(mb.slice_number) == slice_index.end()) {
            h264r_slice s;
            memset(&s, 0, sizeof(s));
            s.chroma_qp_offset[0] = (int8_t)sh.m_pps.chroma_qp_index_offset;
            s.chroma_qp_offset[1] = (int8_t)sh.m_pps.second_chroma_qp_index_offset;
            s.filter_offset_a = (int8_t)mb.FilterOffsetA;
            s.filter_offset_b = (int8_t)mb.FilterOffsetB;
            s.disable_deblocking_filter_idc = (uint8_t)mb.disable_deblocking_filter_idc;
            s.slice_type = (uint8_t)(mb.m_slice_type % 5);
            slice_index[mb.slice_number] = (int)slices.size();
            slices.push_back(s);
        }
        r.slice = (uint16_t)slice_index[mb.slice_number];

        if (r.type == H264R_MB_I4x4) {
            for (int b = 0; b < 16; b++)
                r.ipred[b >> 3] |= (uint32_t)(mb.Intra4x4PredMode[b] & 15) << (4 * (b & 7));
        } else if (r.type == H264R_MB_I8x8) {
            for (int b = 0; b < 4; b++)
                r.ipred[0] |= (uint32_t)(mb.Intra8x8PredMode[b] & 15) << (4 * b);
        }

        /* ---- coefficient payload ---- */
        {
            uint32_t mask = 0;
            std::vector<uint16_t> sig;
            std::vector<int16_t> lv;
            auto block16 = [&](const int32_t *v, int off, int npos, int bit) {
                /* v[k] holds scan position k+off, k = 0..npos-1 */
                uint16_t s = 0;
                std::vector<int16_t> vals;
                for (int k = 0; k < npos; k++) {
                    if (v[k] != 0) {
                        s |= (uint16_t)(1u << (k + off));
                        vals.push_back((int16_t)v[k]);
                    }
                }
                if (s) {
                    mask |= 1u << bit;
                    sig.push_back(s);
                    lv.insert(lv.end(), vals.begin(), vals.end());
                }
            };
            /* blocks in mask-bit order: luma 0..15, DC 16, chroma DC 17/18,
               chroma AC 19..26 */
            if (r.type != H264R_MB_IPCM && r.type != H264R_MB_NONE) {
                if (r.flags & H264R_MBF_T8x8) {
                    for (int b = 0; b < 4; b++) {
                        uint16_t s4[4] = {0, 0, 0, 0};
                        std::vector<int16_t> vals;
                        for (int k = 0; k < 64; k++)
                            if (mb.LumaLevel8x8[b][k] != 0) {
                                s4[k >> 4] |= (uint16_t)(1u << (k & 15));
                                vals.push_back((int16_t)mb.LumaLevel8x8[b][k]);
                            }
                        if (!vals.empty()) {
                            mask |= 1u << b;
                            sig.insert(sig.end(), s4, s4 + 4);
                            lv.insert(lv.end(), vals.begin(), vals.end());
                        }
                    }
                } else if (r.type == H264R_MB_I16x16) {
                    for (int b = 0; b < 16; b++)
                        block16(mb.Intra16x16ACLevel[b], 1, 15, b);
                } else {
                    for (int b = 0; b < 16; b++)
                        block16(mb.LumaLevel4x4[b], 0, 16, b);
                }
                if (r.type == H264R_MB_I16x16)
                    block16(mb.Intra16x16DCLevel, 0, 16, 16);
                block16(mb.ChromaDCLevel[0], 0, 4, 17);
                block16(mb.ChromaDCLevel[1], 0, 4, 18);
                for (int b = 0; b < 4; b++)
                    block16(mb.ChromaACLevel[0][b], 1, 15, H264R_CM_CB_AC0 + b);
                for (int b = 0; b < 4; b++)
                    block16(mb.ChromaACLevel[1][b], 1, 15, H264R_CM_CR_AC0 + b);
            }
            if (mask) {
                while (coef.size() & 3) coef.push_back(0);
                r.coef = (uint32_t)coef.size();
                const uint8_t *pm = (const uint8_t *)&mask;
                coef.insert(coef.end(), pm, pm + 4);
                const uint8_t *ps = (const uint8_t *)sig.data();
                coef.insert(coef.end(), ps, ps + 2 * sig.size());
                while (coef.size() & 3) coef.push_back(0);
                const uint8_t *pl = (const uint8_t *)lv.data();
                coef.insert(coef.end(), pl, pl + 2 * lv.size());
            }
        }

        /* ---- I_PCM samples ---- */
        if (r.type == H264R_MB_IPCM) {
            r.aux = (uint32_t)(pcm.size() / 384);
            for (int i = 0; i < 256; i++) pcm.push_back((uint8_t)mb.pcm_sample_luma[i]);
            for (int i = 0; i < 128; i++) pcm.push_back((uint8_t)mb.pcm_sample_chroma[i]);
        }

        /* ---- motion payload ---- */
        if (r.type == H264R_MB_INTER) {
            H264_MB_TYPE t = mb.m_name_of_mb_type;
            int shape;
            if (t == B_Skip || t == B_Direct_16x16) {
                shape = 3 | (3 << 2) | (3 << 4) | (3 << 6) | (3 << 8);
            } else {
                int pc = part_code(t);
                if (pc < 0) { g_unsupported |= 2; pc = 0; if (g_verbose) fprintf(stderr, "unsupported mb type %d at %d\n", (int)t, addr); }
                shape = pc;
                if (pc == 3) {
                    for (int q = 0; q < 4; q++) {
                        int sc = (mb.m_name_of_sub_mb_type[q] == B_Direct_8x8) ? 3 : sub_code(mb.m_name_of_sub_mb_type[q]);
                        if (sc < 0) { g_unsupported |= 4; sc = 0; if (g_verbose) fprintf(stderr, "unsupported sub type %d at %d\n", (int)mb.m_name_of_sub_mb_type[q], addr); }
                        shape |= sc << (2 + 2 * q);
                    }
                }
            }
            /* entries in (mbPartIdx, subMbPartIdx) order */
            std::vector<std::pair<int, int>> ent;
            int mbpc = shape & 3;
            int nparts = (mbpc == 0) ? 1 : (mbpc == 3 ? 4 : 2);
            for (int mp = 0; mp < nparts; mp++) {
                int nsub = 1;
                if (mbpc == 3) {
                    int sc = (shape >> (2 + 2 * mp)) & 3;
                    nsub = (sc == 0) ? 1 : (sc == 3 ? 4 : 2);
                }
                for (int sp = 0; sp < nsub; sp++) ent.push_back(std::make_pair(mp, sp));
            }
            /* cross-check the entry order against the reference's own
               6.4.13.4 mapping, used by its deblocking filter */
            for (int by = 0; by < 4; by++)
                for (int bx = 0; bx < 4; bx++) {
                    int mp = 0, sp = 0;
                    pic->Derivation_process_for_macroblock_and_sub_macroblock_partition_indices(
                        t, mb.m_name_of_sub_mb_type, bx * 4, by * 4, mp, sp);
                    int e = entry_of_block(shape, bx, by);
                    if (t != MB_TYPE_NA && (e >= (int)ent.size() || ent[e] != std::make_pair(mp, sp))) {
                        g_unsupported |= 8;
                        if (g_verbose) fprintf(stderr, "partition map mismatch type %d at %d\n", (int)t, addr);
                    }
                }
            while (motion.size() & 3) motion.push_back(0);
            r.aux = (uint32_t)motion.size();
            uint16_t hdr[2] = {(uint16_t)shape, (uint16_t)ent.size()};
            const uint8_t *ph = (const uint8_t *)hdr;
            motion.insert(motion.end(), ph, ph + 4);
            const int field = (r.flags & H264R_MBF_FIELD) ? 1 : 0;
            const int mb_bottom = addr & 1; /* MBAFF: bottom MB of the pair */
            for (size_t e = 0; e < ent.size(); e++) {
                int mp = ent[e].first, sp = ent[e].second;
                h264r_part p;
                memset(&p, 0, sizeof(p));
                int refIdx[2] = {mb.m_RefIdxL0[mp], mb.m_RefIdxL1[mp]};
                int pf[2] = {mb.m_PredFlagL0[mp], mb.m_PredFlagL1[mp]};
                p.mv[0][0] = (int16_t)mb.m_MvL0[mp][sp][0];
                p.mv[0][1] = (int16_t)mb.m_MvL0[mp][sp][1];
                p.mv[1][0] = (int16_t)mb.m_MvL1[mp][sp][0];
                p.mv[1][1] = (int16_t)mb.m_MvL1[mp][sp][1];
                for (int l = 0; l < 2; l++) {
                    CH264Picture **list = (l == 0) ? pic->m_RefPicList0 : pic->m_RefPicList1;
                    p.ref[l] = -1;
                    if (pf[l]) {
                        if (!field) {
                            p.ref[l] = (int8_t)slot_of(pic, list[refIdx[l]]);
                        } else {
                            int s = slot_of(pic, list[refIdx[l] / 2]);
                            int same = (refIdx[l] % 2) == 0;
                            int bottom = same ? mb_bottom : !mb_bottom;
                            p.ref[l] = (int8_t)(s | H264R_REF_FIELD | (bottom ? H264R_REF_BOTTOM : 0));
                        }
                    }
                    p.dref[l] = (int8_t)((refIdx[l] >= 0) ? slot_of(pic, list[refIdx[l]]) : -1);
                }
                /* weights, exactly as Inter_prediction_process derives them
                   (H264InterPrediction.cpp:521-546) and dispatches them
                   (Weighted_sample_prediction_process, 2526-2613) */
                h264r_weight w;
                memset(&w, 0, sizeof(w));
                int use_wp = (sh.m_pps.weighted_pred_flag == 1 && (slice_type == 0 || slice_type == 3)) ||
                             (sh.m_pps.weighted_bipred_idc > 0 && slice_type == 1);
                if (use_wp) {
                    int32_t v[15] = {0, 1, 1, 0, 0, 0, 1, 1, 0, 0, 0, 1, 1, 0, 0};
                    pic->CurrMbAddr = addr;
                    pic->Derivation_process_for_prediction_weights(refIdx[0], refIdx[1], pf[0], pf[1],
                        v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10], v[11], v[12], v[13], v[14]);
                    int weighted = 0;
                    if (pf[0] && (slice_type == 0 || slice_type == 3))
                        weighted = sh.m_pps.weighted_pred_flag == 1;
                    else if ((pf[0] || pf[1]) && slice_type == 1) {
                        if (sh.m_pps.weighted_bipred_idc == 1) weighted = 1;
                        else if (sh.m_pps.weighted_bipred_idc == 2) weighted = pf[0] && pf[1];
                    }
                    if (weighted) {
                        w.weighted = 1;
                        for (int c = 0; c < 3; c++) {
                            w.log_wd[c] = (int8_t)v[5 * c + 0];
                            w.w0[c] = (int16_t)v[5 * c + 1];
                            w.w1[c] = (int16_t)v[5 * c + 2];
                            w.o0[c] = (int16_t)v[5 * c + 3];
                            w.o1[c] = (int16_t)v[5 * c + 4];
                        }
                    }
                }
                p.wt = add_weight(w);
                const uint8_t *pp = (const uint8_t *)&p;
                motion.insert(motion.end(), pp, pp + sizeof(p));
            }
        }
        mbs[addr] = r;
    }

    h264r_dump_pic h;
    memset(&h, 0, sizeof(h));
    h.tag = H264R_DUMP_PIC_TAG;
    h.width_mbs = (uint16_t)pic->PicWidthInMbs;
    h.height_mbs = (uint16_t)(pic->PicHeightInMbs * ((pic->m_picture_coded_type == H264_PICTURE_CODED_TYPE_FRAME) ? 1 : 2));
    h.structure = (pic->m_picture_coded_type == H264_PICTURE_CODED_TYPE_TOP_FIELD) ? H264R_STRUCT_TOP :
                  (pic->m_picture_coded_type == H264_PICTURE_CODED_TYPE_BOTTOM_FIELD) ? H264R_STRUCT_BOTTOM : H264R_STRUCT_FRAME;
    h.mbaff = (uint8_t)sh.MbaffFrameFlag;
    h.dst_slot = (uint8_t)slot_of(pic, pic->m_parent);
    h.deblock = 1;
    h.num_slices = (uint16_t)slices.size();
    h.num_weights = (uint16_t)weights.size();
    h.num_mbs = (uint32_t)n;
    h.motion_bytes = (uint32_t)motion.size();
    h.coef_bytes = (uint32_t)coef.size();
    h.num_pcm = (uint32_t)(pcm.size() / 384);
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 16; k++) h.scaling4x4[i][k] = (uint8_t)sh.ScalingList4x4[i][k];
    for (int i = 0; i < 6; i++)
        for (int k = 0; k < 64; k++) h.scaling8x8[i][k] = (uint8_t)sh.ScalingList8x8[i][k];
    h.poc = pic->PicOrderCnt;
    h.pic_num_cnt = pic->m_PicNumCnt;
    h.flags = g_write_planes ? (H264R_DUMP_HAS_PRE | H264R_DUMP_HAS_POST) : 0;
    h.plane_bytes = (uint32_t)plane_bytes;
    put(&h, sizeof(h));
    put(mbs.data(), sizeof(h264r_mb) * mbs.size());
    put(slices.data(), sizeof(h264r_slice) * slices.size());
    put(weights.data(), sizeof(h264r_weight) * weights.size());
    put(motion.data(), motion.size());
    put(coef.data(), coef.size());
    put(pcm.data(), pcm.size());
    if (g_write_planes) {
        put(pre, plane_bytes);
        put(post, plane_bytes);
    }
}

extern "C" int __wrap__ZN16CH264PictureBase25Deblocking_filter_processEv(CH264PictureBase *self)
{
    if (g_order) {  // a completed picture, in decoding order (all but the stream's last)
        const CH264SliceHeader &sh = self->m_h264_slice_header;
        fprintf(g_order, "D %d %d %d\n", self->PicOrderCnt, (int)sh.m_nal_unit.IdrPicFlag, (int)sh.m_sps.m_vui.max_num_reorder_frames);
    }
    if (g_out == NULL || g_pictures >= g_max_pictures || self->m_picture_coded_type != H264_PICTURE_CODED_TYPE_FRAME)
        return __real__ZN16CH264PictureBase25Deblocking_filter_processEv(self);
    size_t plane_bytes = (size_t)self->PicWidthInSamplesL * self->PicHeightInSamplesL +
                         2 * (size_t)self->PicWidthInSamplesC * self->PicHeightInSamplesC;
    std::vector<uint8_t> pre(self->m_pic_buff_luma, self->m_pic_buff_luma + plane_bytes);
    int ret = __real__ZN16CH264PictureBase25Deblocking_filter_processEv(self);
    std::vector<uint8_t> post(self->m_pic_buff_luma, self->m_pic_buff_luma + plane_bytes);
    dump_picture(self, pre.data(), post.data(), plane_bytes);
    if (g_bmp_dir) {
        // the reference's own output path for this picture (YUV420P -> BGR24 -> BMP)
        char path[4096];
        snprintf(path, sizeof(path), "%s/pic_%03d.bmp", g_bmp_dir, g_pictures);
        self->saveToBmpFile(path);
    }
    g_pictures++;
    return ret;
}

static int on_frame(CH264Picture *out, void *user, int err)
{
    (void)user;
    (void)err;
    if (out == NULL) return -1;
    if (g_order) fprintf(g_order, "O %d\n", out->m_picture_frame.PicOrderCnt);
    if (g_yuv) {
        const CH264PictureBase &f = out->m_picture_frame;
        fwrite(f.m_pic_buff_luma, 1, (size_t)f.PicWidthInSamplesL * f.PicHeightInSamplesL, g_yuv);
        fwrite(f.m_pic_buff_cb, 1, (size_t)f.PicWidthInSamplesC * f.PicHeightInSamplesC, g_yuv);
        fwrite(f.m_pic_buff_cr, 1, (size_t)f.PicWidthInSamplesC * f.PicHeightInSamplesC, g_yuv);
    }
    return (g_pictures >= g_max_pictures) ? -1 : 0;
}

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: %s <in.h264> <out.dmp> [max_pictures] [--no-planes] [--bmp <dir>] [--order <file>] [--yuv <file>]\n", argv[0]);
        return 2;
    }
    for (int i = 3; i < argc; i++) {
        if (strcmp(argv[i], "--no-planes") == 0) g_write_planes = 0;
        else if (strcmp(argv[i], "--bmp") == 0 && i + 1 < argc) g_bmp_dir = argv[++i];
        else if (strcmp(argv[i], "--order") == 0 && i + 1 < argc) {
            g_order = fopen(argv[++i], "w");
            if (!g_order) { perror("fopen"); return 1; }
        }
        else if (strcmp(argv[i], "--yuv") == 0 && i + 1 < argc) {
            g_yuv = fopen(argv[++i], "wb");
            if (!g_yuv) { perror("fopen"); return 1; }
        }
        else g_max_pictures = atoi(argv[i]);
    }
    g_out = fopen(argv[2], "wb");
    if (!g_out) { perror("fopen"); return 1; }
    fwrite(H264R_DUMP_MAGIC, 1, 8, g_out);
    uint32_t v[2] = {H264R_DUMP_VERSION, 0};
    fwrite(v, 4, 2, g_out);

    CH264VideoDecoder dec;
    dec.init();
    dec.set_output_frame_callback_functuin(on_frame, NULL);
    dec.open(argv[1]);
    fclose(g_out);
    if (g_order) fclose(g_order);
    if (g_yuv) fclose(g_yuv);
    fprintf(stderr, "ref_dump: %d pictures, unsupported-flags=0x%x\n", g_pictures, g_unsupported);
    return g_unsupported ? 3 : 0;
}
