// h264r_parser.cpp — host-side front end (include/h264r_parser.h): NAL units,
// slice data (CAVLC), the derivations that turn syntax into reconstruction
// records (intra modes 8.3.1.1 / 8.3.2.1, motion vectors 8.4.1, weights
// 8.4.2.3), picture order counts (8.2.1), reference lists (8.2.4), marking
// (8.2.5), DPB slots and output order.  Restated from the standard; the
// reference's counterparts are named at each step.
#include "h264r_parser_impl.h"

namespace h264r {
namespace pimpl {

// CABAC readers of the prediction syntax (h264r_cabac.cpp)
int cabac_sub_mb_type(MbDecoder &d, bool is_b);
int cabac_ref_idx(MbDecoder &d, int l, int x, int y);
int cabac_mvd(MbDecoder &d, int l, int comp, int x, int y);

// P mb_type 0..4 and B mb_type 1..21: partition shape (0 16x16, 1 16x8,
// 2 8x16) and prediction lists per partition (bit 0 L0, bit 1 L1)
struct InterType {
    int shape, pred0, pred1;
};

InterType b_type(int t)
{
    if (t >= 1 && t <= 3) return {0, t, 0};
    static const int pairs[9][2] = {{1, 1}, {2, 2}, {1, 2}, {2, 1}, {1, 3}, {2, 3}, {3, 1}, {3, 2}, {3, 3}};
    const int j = (t - 4) / 2;
    return {(t % 2 == 0) ? 1 : 2, pairs[j][0], pairs[j][1]};
}

// sub_mb_type: record sub shape (0 8x8, 1 8x4, 2 4x8, 3 4x4), lists
struct SubType {
    int shape, pred;
};

SubType p_sub(int t) { return {t, 1}; }
SubType b_sub(int t)
{
    if (t == 0) return {3, 0};  // direct: 4x4 blocks
    if (t <= 3) return {0, t};
    static const SubType s[9] = {{1, 1}, {2, 1}, {1, 2}, {2, 2}, {1, 3}, {2, 3}, {3, 1}, {3, 2}, {3, 3}};
    return s[t - 4];
}

void sub_geom(int shape, int sp, int &x, int &y, int &w, int &h)
{
    switch (shape) {
    case 0: x = 0; y = 0; w = 8; h = 8; break;
    case 1: x = 0; y = 4 * sp; w = 8; h = 4; break;
    case 2: x = 4 * sp; y = 0; w = 4; h = 8; break;
    default: x = 4 * (sp & 1); y = 4 * (sp >> 1); w = 4; h = 4; break;
    }
}

int MbDecoder::inter_pred(int mb_type, bool is_b, h264r_mb &r, bool &no_sub_lt8)
{
    no_sub_lt8 = true;
    // a field MB of an MBAFF frame indexes fields: twice the entries, and
    // ref_idx is present even with one frame in the list (7.3.5.1)
    const int nref[2] = {ref_limit(0), ref_limit(1)};
    const bool ref_present[2] = {nref[0] > 1 || fld, nref[1] > 1 || fld};
    parts.clear();
    int shape = 0;
    // read the syntax first (mb_pred / sub_mb_pred, 7.3.5.1 / 7.3.5.2)
    const bool b8x8 = is_b ? mb_type == 22 : (mb_type == 3 || mb_type == 4);
    for (int i = 0; i < 16; i++) decoded4x4[i] = false;
    spatial_ready = false;
    if (!b8x8) {
        InterType t = is_b ? b_type(mb_type) : InterType{mb_type == 0 ? 0 : mb_type, 1, 1};
        const int np = t.shape == 0 ? 1 : 2;
        const int pred[2] = {t.pred0, np == 2 ? t.pred1 : 0};
        int ref[2][2] = {{-1, -1}, {-1, -1}}, mvd[2][2][2] = {};
        // 4x4 blocks (x0 .. x0 + w4, y0 .. y0 + h4) that partition p covers
        auto cover = [&](int p, int &x0, int &y0, int &w4, int &h4) {
            x0 = t.shape == 2 ? 2 * p : 0;
            y0 = t.shape == 1 ? 2 * p : 0;
            w4 = t.shape == 2 ? 2 : 4;
            h4 = t.shape == 1 ? 2 : 4;
        };
        if (cab)
            for (int p = 0; p < np; p++) {
                int x0, y0, w4, h4;
                cover(p, x0, y0, w4, h4);
                for (int j = y0; j < y0 + h4; j++)
                    for (int i = x0; i < x0 + w4; i++) predl_cur[j * 4 + i] = (uint8_t)pred[p];
            }
        for (int l = 0; l < 2; l++)
            for (int p = 0; p < np; p++)
                if (pred[p] & (1 << l)) {
                    int x0, y0, w4, h4;
                    cover(p, x0, y0, w4, h4);
                    if (cab) ref[p][l] = ref_present[l] ? cabac_ref_idx(*this, l, 4 * x0, 4 * y0) : 0;
                    else ref[p][l] = ref_present[l] ? (int)br.te(nref[l] - 1) : 0;
                    if (ref[p][l] >= nref[l] || !ref_pic(l, ref[p][l]))
                        return P.fail(H264R_ERR_BAD_RECORD, "ref_idx names no picture (MB %d)", addr);
                    if (cab)
                        for (int j = y0; j < y0 + h4; j++)
                            for (int i = x0; i < x0 + w4; i++) refsyn_cur[l][j * 4 + i] = (int8_t)ref[p][l];
                }
        for (int l = 0; l < 2; l++)
            for (int p = 0; p < np; p++)
                if (pred[p] & (1 << l)) {
                    if (cab) {
                        int x0, y0, w4, h4;
                        cover(p, x0, y0, w4, h4);
                        mvd[p][l][0] = cabac_mvd(*this, l, 0, 4 * x0, 4 * y0);
                        mvd[p][l][1] = cabac_mvd(*this, l, 1, 4 * x0, 4 * y0);
                        for (int j = y0; j < y0 + h4; j++)
                            for (int i = x0; i < x0 + w4; i++) {
                                mvd_cur[l][j * 4 + i][0] = (int16_t)mvd[p][l][0];
                                mvd_cur[l][j * 4 + i][1] = (int16_t)mvd[p][l][1];
                            }
                    } else {
                        mvd[p][l][0] = br.se();
                        mvd[p][l][1] = br.se();
                    }
                }
        shape = t.shape;
        for (int p = 0; p < np; p++) {
            const int x = t.shape == 2 ? 8 * p : 0, y = t.shape == 1 ? 8 * p : 0;
            const int w = t.shape == 2 ? 8 : 16, h = t.shape == 1 ? 8 : 16;
            Blk b;
            for (int l = 0; l < 2; l++) {
                b.ref[l] = (int8_t)ref[p][l];
                b.mv[l][0] = b.mv[l][1] = 0;
                if (ref[p][l] >= 0) {
                    int m[2];
                    mvp(x, y, w, t.shape, p, l, ref[p][l], m);
                    b.mv[l][0] = (int16_t)(m[0] + mvd[p][l][0]);
                    b.mv[l][1] = (int16_t)(m[1] + mvd[p][l][1]);
                }
            }
            set_blocks(x, y, w, h, b);
            parts.push_back({p, 0, x, y, w, h});
        }
    } else {
        int sub[4];
        SubType st[4];
        for (int q = 0; q < 4; q++) {
            sub[q] = cab ? cabac_sub_mb_type(*this, is_b) : (int)br.ue();
            if (sub[q] > (is_b ? 12 : 3)) return P.fail(H264R_ERR_BAD_RECORD, "sub_mb_type out of range (MB %d)", addr);
            st[q] = is_b ? b_sub(sub[q]) : p_sub(sub[q]);
            // noSubMbPartSizeLessThan8x8Flag (7.3.5)
            if (is_b && sub[q] == 0) {
                if (!sps.direct_8x8_inference) no_sub_lt8 = false;
            } else if (st[q].shape != 0) {
                no_sub_lt8 = false;
            }
        }
        const bool ref0 = !is_b && mb_type == 4;  // P_8x8ref0
        int ref[4][2], mvd[4][4][2][2] = {};
        if (cab)
            for (int q = 0; q < 4; q++) {
                const int qx = (q & 1) * 2, qy = (q >> 1) * 2;
                const uint8_t pl = (uint8_t)st[q].pred;  // 0 for B_Direct_8x8
                for (int j = qy; j < qy + 2; j++)
                    for (int i = qx; i < qx + 2; i++) predl_cur[j * 4 + i] = pl;
            }
        for (int l = 0; l < 2; l++)
            for (int q = 0; q < 4; q++) {
                ref[q][l] = -1;
                if (st[q].pred & (1 << l)) {
                    const int qx = (q & 1) * 8, qy = (q >> 1) * 8;
                    if (cab) ref[q][l] = (!ref0 && ref_present[l]) ? cabac_ref_idx(*this, l, qx, qy) : 0;
                    else ref[q][l] = (!ref0 && ref_present[l]) ? (int)br.te(nref[l] - 1) : 0;
                    if (ref[q][l] >= nref[l] || !ref_pic(l, ref[q][l]))
                        return P.fail(H264R_ERR_BAD_RECORD, "ref_idx names no picture (MB %d)", addr);
                    if (cab)
                        for (int j = qy / 4; j < qy / 4 + 2; j++)
                            for (int i = qx / 4; i < qx / 4 + 2; i++) refsyn_cur[l][j * 4 + i] = (int8_t)ref[q][l];
                }
            }
        for (int l = 0; l < 2; l++)
            for (int q = 0; q < 4; q++)
                if (st[q].pred & (1 << l)) {
                    const int ns = st[q].shape == 0 ? 1 : (st[q].shape == 3 ? 4 : 2);
                    for (int s = 0; s < ns; s++) {
                        if (cab) {
                            int sx, sy, w, h;
                            sub_geom(st[q].shape, s, sx, sy, w, h);
                            const int x = (q & 1) * 8 + sx, y = (q >> 1) * 8 + sy;
                            mvd[q][s][l][0] = cabac_mvd(*this, l, 0, x, y);
                            mvd[q][s][l][1] = cabac_mvd(*this, l, 1, x, y);
                            for (int j = y >> 2; j < (y + h) >> 2; j++)
                                for (int i = x >> 2; i < (x + w) >> 2; i++) {
                                    mvd_cur[l][j * 4 + i][0] = (int16_t)mvd[q][s][l][0];
                                    mvd_cur[l][j * 4 + i][1] = (int16_t)mvd[q][s][l][1];
                                }
                        } else {
                            mvd[q][s][l][0] = br.se();
                            mvd[q][s][l][1] = br.se();
                        }
                    }
                }
        shape = 3;
        for (int q = 0; q < 4; q++) {
            shape |= st[q].shape << (2 + 2 * q);
            const int qx = (q & 1) * 8, qy = (q >> 1) * 8;
            if (is_b && sub[q] == 0) {  // B_Direct_8x8: four 4x4 blocks
                for (int s = 0; s < 4; s++) {
                    const int x = qx + 4 * (s & 1), y = qy + 4 * (s >> 1);
                    Blk b;
                    if (direct_block(x >> 2, y >> 2, b)) return -1;
                    set_blocks(x, y, 4, 4, b);
                    parts.push_back({q, s, x, y, 4, 4});
                }
                continue;
            }
            const int ns = st[q].shape == 0 ? 1 : (st[q].shape == 3 ? 4 : 2);
            for (int s = 0; s < ns; s++) {
                int sx, sy, w, h;
                sub_geom(st[q].shape, s, sx, sy, w, h);
                const int x = qx + sx, y = qy + sy;
                Blk b;
                for (int l = 0; l < 2; l++) {
                    b.ref[l] = (int8_t)ref[q][l];
                    b.mv[l][0] = b.mv[l][1] = 0;
                    if (ref[q][l] >= 0) {
                        int m[2];
                        mvp(x, y, w, 0, 0, l, ref[q][l], m);
                        b.mv[l][0] = (int16_t)(m[0] + mvd[q][s][l][0]);
                        b.mv[l][1] = (int16_t)(m[1] + mvd[q][s][l][1]);
                    }
                }
                set_blocks(x, y, w, h, b);
                parts.push_back({q, s, x, y, w, h});
            }
        }
    }
    if (br.err) return P.fail(H264R_ERR_BAD_RECORD, "truncated prediction syntax (MB %d)", addr);
    emit_motion(shape, parts, r);
    return 0;
}

// motion payload of the record: shape, then one h264r_part per partition
void MbDecoder::emit_motion(int shape, const std::vector<PartRec> &parts, h264r_mb &r)
{
    std::vector<uint8_t> &m = P.motion;
    while (m.size() & 3) m.push_back(0);
    r.aux = (uint32_t)m.size();
    const uint16_t hdr[2] = {(uint16_t)shape, (uint16_t)parts.size()};
    m.insert(m.end(), (const uint8_t *)hdr, (const uint8_t *)hdr + 4);
    for (const PartRec &pr : parts) {
        const Blk &b = blk[(pr.y >> 2) * 4 + (pr.x >> 2)];
        h264r_part p;
        memset(&p, 0, sizeof(p));
        for (int l = 0; l < 2; l++) {
            p.mv[l][0] = b.mv[l][0];
            p.mv[l][1] = b.mv[l][1];
            p.ref[l] = -1;
            p.dref[l] = b.ref[l];  // refIdx for now: the picture-level list resolves it at the end
            if (b.ref[l] >= 0) {
                const Pic *rp = ref_pic(l, b.ref[l]);
                p.ref[l] = (int8_t)rp->slot;
                if (fld) p.ref[l] = (int8_t)(rp->slot | H264R_REF_FIELD | (ref_bottom(b.ref[l]) ? H264R_REF_BOTTOM : 0));
            }
        }
        p.wt = weight_index(b.ref[0], b.ref[1]);
        const size_t off = m.size();
        m.insert(m.end(), (const uint8_t *)&p, (const uint8_t *)&p + sizeof(p));
        P.dref_parts.push_back((uint32_t)off);
    }
}

// motion of the finished MB into the neighbour state
void MbDecoder::store_motion()
{
    for (int l = 0; l < 2; l++)
        for (int i = 0; i < 16; i++) {
            const int r = blk[i].ref[l];  // -1 .. 31 (the entry was checked when parsed)
            cur->ref[l][i] = (int8_t)r;
            cur->mv[l][i][0] = blk[i].mv[l][0];
            cur->mv[l][i][1] = blk[i].mv[l][1];
            cur->refpic[l][i] = uid[l][(fld && r >= 0 ? r >> 1 : r) + 1];
        }
}

// residual( 0, 15 ) (7.3.5.3) with CAVLC blocks; fills the coefficient
// payload parts and the TotalCoeff state
int MbDecoder::residual(int cls, int cbp, bool t8, uint32_t &mask, std::vector<uint16_t> &sig, std::vector<int16_t> &lv,
                        h264r_mb &r)
{
    const int cbp_luma = cbp & 15, cbp_chroma = cbp >> 4;
    int tc = 0;
    // a block's significance word and its levels in scan order, as the
    // block decoder returns them
    auto put_sparse = [&](uint16_t s, const int16_t *v, int n, int bit) {
        if (!s) return;
        mask |= 1u << bit;
        sig.push_back(s);
        lv.insert(lv.end(), v, v + n);
    };
    const bool i16 = cls == H264R_MB_I16x16;
    uint16_t dc_sig = 0;
    int16_t dc_lev[16];
    int dc_n = 0;
    bool have_dc = false;
    int16_t lev[16];
    uint16_t bsig = 0;
    // r.nz4x4 / nz8x8 follow the blocks as they are parsed, so that a MB
    // whose residual fails keeps the counts reached, as the reference's does
    r.nz4x4 = 0;
    r.nz8x8 = 0;
    for (int b = 0; b < 16; b++) cur->tc[b] = 0;
    if (i16) {
        if (cavlc_residual_sparse(br, nc_luma(0), 0, 15, 16, 0, dc_sig, dc_lev, tc)) return -1;
        dc_n = tc;
        have_dc = true;
        // the reference keeps the DC block's TotalCoeff as block 0's count
        // until an AC block 0 replaces it (H264MacroBlock.cpp residual_luma);
        // no other MB takes block 0 as a neighbour, so parsing is unaffected
        cur->tc[0] = (uint8_t)tc;
        if (tc) r.nz4x4 = 1;
    }
    // 8x8 transform: coefficient k of 4x4 block b4 is 8x8 scan index
    // 4k + b4; the set indices per 8x8 block, and the levels at them
    uint64_t m64[4] = {0, 0, 0, 0};
    int16_t v64[4][64];
    for (int b8 = 0; b8 < 4; b8++) {
        for (int b4 = 0; b4 < 4; b4++) {
            const int b = b8 * 4 + b4;
            if (!(cbp_luma & (1 << b8))) continue;
            if (i16) {
                if (cavlc_residual_sparse(br, nc_luma(b), 0, 14, 15, 1, bsig, lev, tc)) return -1;
                put_sparse(bsig, lev, tc, b);
            } else if (t8) {
                if (cavlc_residual_sparse(br, nc_luma(b), 0, 15, 16, 0, bsig, lev, tc)) return -1;
                uint32_t bits = bsig;
                for (int j = 0; bits; j++) {
                    const int k = __builtin_ctz(bits);
                    bits &= bits - 1;
                    const int idx = 4 * k + b4;
                    m64[b8] |= 1ull << idx;
                    v64[b8][idx] = lev[j];
                }
            } else {
                if (cavlc_residual_sparse(br, nc_luma(b), 0, 15, 16, 0, bsig, lev, tc)) return -1;
                put_sparse(bsig, lev, tc, b);
            }
            cur->tc[b] = (uint8_t)tc;
            r.nz4x4 = (uint16_t)((r.nz4x4 & ~(1u << b)) | (tc ? 1u << b : 0u));
            if (tc) r.nz8x8 |= (uint8_t)(1u << b8);
        }
    }
    if (t8) {
        for (int b8 = 0; b8 < 4; b8++) {
            if (!m64[b8]) continue;
            mask |= 1u << b8;
            for (int w = 0; w < 4; w++) sig.push_back((uint16_t)(m64[b8] >> (16 * w)));
            for (uint64_t bits = m64[b8]; bits; bits &= bits - 1) lv.push_back(v64[b8][__builtin_ctzll(bits)]);
        }
    }
    if (have_dc) put_sparse(dc_sig, dc_lev, dc_n, 16);
    // chroma DC then AC (4:2:0)
    uint16_t cdc_sig[2] = {0, 0};
    int16_t cdc_lev[2][4];
    int cdc_n[2] = {0, 0};
    for (int cc = 0; cc < 2; cc++) {
        if ((cbp_chroma & 3) && cavlc_residual_sparse(br, -1, 0, 3, 4, 0, cdc_sig[cc], cdc_lev[cc], tc)) return -1;
        if (cbp_chroma & 3) cdc_n[cc] = tc;
    }
    put_sparse(cdc_sig[0], cdc_lev[0], cdc_n[0], 17);
    put_sparse(cdc_sig[1], cdc_lev[1], cdc_n[1], 18);
    for (int cc = 0; cc < 2; cc++)
        for (int b = 0; b < 4; b++) {
            cur->tcc[cc][b] = 0;
            if (!(cbp_chroma & 2)) continue;
            if (cavlc_residual_sparse(br, nc_chroma(cc, b), 0, 14, 15, 1, bsig, lev, tc)) return -1;
            cur->tcc[cc][b] = (uint8_t)tc;
            put_sparse(bsig, lev, tc, (cc ? H264R_CM_CR_AC0 : H264R_CM_CB_AC0) + b);
        }
    return 0;
}

int MbDecoder::decode()
{
    h264r_mb r;
    memset(&r, 0, sizeof(r));
    r.coef = H264R_NONE;
    r.aux = H264R_NONE;
    r.slice = (uint16_t)sc.index;
    if (pps.constrained_intra_pred) r.flags |= H264R_MBF_CIP;
    const int st = sc.sh.slice_type;
    uint32_t mb_type = br.ue();
    bool is_intra_type = true;
    uint32_t itype = mb_type;
    if (st == kSliceP) {
        if (mb_type < 5) is_intra_type = false;
        else itype = mb_type - 5;
    } else if (st == kSliceB) {
        if (mb_type < 23) is_intra_type = false;
        else itype = mb_type - 23;
    }
    if (is_intra_type && itype > 25) return P.fail(H264R_ERR_BAD_RECORD, "mb_type %u out of range (MB %d)", mb_type, addr);
    for (int i = 0; i < 16; i++) {
        cur->ipm4[i] = 2;
        cur->tc[i] = 0;
    }
    for (int i = 0; i < 4; i++) cur->ipm8[i] = 2;
    memset(cur->tcc, 0, sizeof(cur->tcc));
    for (int i = 0; i < 16; i++) {
        blk[i].ref[0] = blk[i].ref[1] = -1;
        blk[i].mv[0][0] = blk[i].mv[0][1] = blk[i].mv[1][0] = blk[i].mv[1][1] = 0;
    }
    if (is_intra_type && itype == 25) {  // I_PCM
        while (!br.byte_aligned()) br.u(1);
        r.type = H264R_MB_IPCM;
        cur->cls = H264R_MB_IPCM;
        r.aux = (uint32_t)(P.pcm.size() / 384);
        for (int i = 0; i < 384; i++) P.pcm.push_back((uint8_t)br.u(8));
        // non-zero counts stay 0 (see total_of: the reference's nN of an I_PCM MB)
        r.qpy = (uint8_t)qp;
        if (br.err) return P.fail(H264R_ERR_BAD_RECORD, "truncated I_PCM (MB %d)", addr);
        P.rec[addr] = r;
        return 0;
    }
    int cbp = 0;
    bool t8 = false;
    int cls;
    if (is_intra_type) {
        if (itype == 0) {  // I_NxN
            if (pps.transform_8x8_mode) t8 = br.flag();
            cls = t8 ? H264R_MB_I8x8 : H264R_MB_I4x4;
            cur->cls = (uint8_t)cls;
            if (!t8) {
                int flag[16], rem[16];
                for (int b = 0; b < 16; b++) {
                    flag[b] = (int)br.u(1);
                    rem[b] = flag[b] ? 0 : (int)br.u(3);
                }
                for (int b = 0; b < 16; b++) {
                    cur->ipm4[b] = (int8_t)derive_mode(kBlkX[b] * 4, kBlkY[b] * 4, false, flag[b], rem[b]);
                    r.ipred[b >> 3] |= (uint32_t)(cur->ipm4[b] & 15) << (4 * (b & 7));
                }
            } else {
                int flag[4], rem[4];
                for (int b = 0; b < 4; b++) {
                    flag[b] = (int)br.u(1);
                    rem[b] = flag[b] ? 0 : (int)br.u(3);
                }
                for (int b = 0; b < 4; b++) {
                    cur->ipm8[b] = (int8_t)derive_mode((b & 1) * 8, (b >> 1) * 8, true, flag[b], rem[b]);
                    r.ipred[0] |= (uint32_t)(cur->ipm8[b] & 15) << (4 * b);
                    for (int k = 0; k < 4; k++) cur->ipm4[b * 4 + k] = cur->ipm8[b];
                }
            }
            const uint32_t cm = br.ue();
            if (cm > 3) return P.fail(H264R_ERR_BAD_RECORD, "intra_chroma_pred_mode out of range (MB %d)", addr);
            r.chroma_mode = (uint8_t)cm;
            const uint32_t code = br.ue();
            cbp = cbp_from_code(code, true);
            if (cbp < 0) return P.fail(H264R_ERR_BAD_RECORD, "coded_block_pattern out of range (MB %d)", addr);
        } else {  // I_16x16
            cls = H264R_MB_I16x16;
            cur->cls = (uint8_t)cls;
            r.i16_mode = (uint8_t)((itype - 1) % 4);
            cbp = (((itype - 1) / 4) % 3) << 4 | (itype >= 13 ? 15 : 0);
            const uint32_t cm = br.ue();
            if (cm > 3) return P.fail(H264R_ERR_BAD_RECORD, "intra_chroma_pred_mode out of range (MB %d)", addr);
            r.chroma_mode = (uint8_t)cm;
        }
        r.type = (uint8_t)cls;
        // an intra MB has no motion: list entries stay unused
    } else {
        cls = H264R_MB_INTER;
        cur->cls = H264R_MB_INTER;
        r.type = H264R_MB_INTER;
        const bool is_b = st == kSliceB;
        bool no_sub_lt8 = true;
        if (is_b && mb_type == 0) {  // B_Direct_16x16
            for (int i = 0; i < 16; i++) decoded4x4[i] = false;
            spatial_ready = false;
            parts.clear();
            for (int q = 0; q < 4; q++)
                for (int s = 0; s < 4; s++) {
                    const int x = (q & 1) * 8 + 4 * (s & 1), y = (q >> 1) * 8 + 4 * (s >> 1);
                    Blk b;
                    if (direct_block(x >> 2, y >> 2, b)) return -1;
                    set_blocks(x, y, 4, 4, b);
                    parts.push_back({q, s, x, y, 4, 4});
                }
            emit_motion(3 | (3 << 2) | (3 << 4) | (3 << 6) | (3 << 8), parts, r);
            if (!sps.direct_8x8_inference) no_sub_lt8 = false;
        } else {
            if (inter_pred((int)mb_type, is_b, r, no_sub_lt8)) return -1;
        }
        const uint32_t code = br.ue();
        cbp = cbp_from_code(code, false);
        if (cbp < 0) return P.fail(H264R_ERR_BAD_RECORD, "coded_block_pattern out of range (MB %d)", addr);
        if ((cbp & 15) && pps.transform_8x8_mode && no_sub_lt8 &&
            (!(is_b && mb_type == 0) || sps.direct_8x8_inference))
            t8 = br.flag();
    }
    if (t8) r.flags |= H264R_MBF_T8x8;
    uint32_t mask = 0;
    sig.clear();
    lv.clear();
    if ((cbp & 15) || (cbp >> 4) || cls == H264R_MB_I16x16) {
        int dq = br.se();
        dq = clip3(-26, 25, dq);
        qp = (qp + dq + 52) % 52;
        if (residual(cls, cbp, t8, mask, sig, lv, r)) {
            // the reference stops the slice here but has already set up this
            // MB: it is predicted without residual, with QPY still 0
            r.qpy = 0;
            r.coef = H264R_NONE;
            if (cls == H264R_MB_INTER) store_motion();
            P.rec[addr] = r;
            return P.fail(H264R_ERR_BAD_RECORD, "residual syntax error (MB %d)", addr);
        }
    }
    r.qpy = (uint8_t)qp;
    if (mask) {
        std::vector<uint8_t> &c = P.coef;
        while (c.size() & 3) c.push_back(0);
        r.coef = (uint32_t)c.size();
        c.insert(c.end(), (const uint8_t *)&mask, (const uint8_t *)&mask + 4);
        c.insert(c.end(), (const uint8_t *)sig.data(), (const uint8_t *)sig.data() + 2 * sig.size());
        while (c.size() & 3) c.push_back(0);
        c.insert(c.end(), (const uint8_t *)lv.data(), (const uint8_t *)lv.data() + 2 * lv.size());
    }
    if (br.err) return P.fail(H264R_ERR_BAD_RECORD, "truncated macroblock (MB %d)", addr);
    if (cls == H264R_MB_INTER) store_motion();
    P.rec[addr] = r;
    return 0;
}

}  // namespace pimpl
}  // namespace h264r

namespace h264r {
namespace pimpl {

// P_Skip / B_Skip (8.4.1.1, 8.4.1.2): motion only, QPY unchanged
int decode_skip(MbDecoder &d, h264r_mb &r)
{
    memset(&r, 0, sizeof(r));
    r.coef = H264R_NONE;
    r.aux = H264R_NONE;
    r.type = H264R_MB_INTER;
    r.slice = (uint16_t)d.sc.index;
    if (d.pps.constrained_intra_pred) r.flags |= H264R_MBF_CIP;
    r.qpy = (uint8_t)d.qp;
    MbState *cur = d.cur;
    cur->cls = H264R_MB_INTER;
    cur->skip = true;
    cur->cbp = 0;
    cur->t8 = false;
    cur->direct16 = d.sc.sh.slice_type == kSliceB;
    cur->chroma_mode = 0;
    cur->cbf_dc = 0;
    cur->cbf_ac[0] = cur->cbf_ac[1] = cur->cbf_ac[2] = 0;
    memset(cur->predl, 0, sizeof(cur->predl));
    memset(cur->mvd, 0, sizeof(cur->mvd));
    for (int i = 0; i < 16; i++) {
        cur->ipm4[i] = 2;
        cur->tc[i] = 0;
        d.decoded4x4[i] = false;
    }
    for (int i = 0; i < 4; i++) cur->ipm8[i] = 2;
    memset(cur->tcc, 0, sizeof(cur->tcc));
    std::vector<PartRec> &parts = d.parts;
    parts.clear();
    if (d.sc.sh.slice_type == kSliceB) {
        d.spatial_ready = false;
        for (int q = 0; q < 4; q++)
            for (int s = 0; s < 4; s++) {
                const int x = (q & 1) * 8 + 4 * (s & 1), y = (q >> 1) * 8 + 4 * (s >> 1);
                Blk b;
                if (d.direct_block(x >> 2, y >> 2, b)) return -1;
                d.set_blocks(x, y, 4, 4, b);
                parts.push_back({q, s, x, y, 4, 4});
            }
        d.emit_motion(3 | (3 << 2) | (3 << 4) | (3 << 6) | (3 << 8), parts, r);
    } else {
        const MbDecoder::Nb A = d.nb_motion(-1, 0, 0), B = d.nb_motion(0, -1, 0);
        Blk b;
        b.ref[0] = 0;
        b.ref[1] = -1;
        b.mv[0][0] = b.mv[0][1] = b.mv[1][0] = b.mv[1][1] = 0;
        const bool zero = !A.avail || !B.avail || (A.ref == 0 && A.mv[0] == 0 && A.mv[1] == 0) ||
                          (B.ref == 0 && B.mv[0] == 0 && B.mv[1] == 0);
        if (!zero) {
            int m[2];
            d.mvp(0, 0, 16, 0, 0, 0, 0, m);
            b.mv[0][0] = (int16_t)m[0];
            b.mv[0][1] = (int16_t)m[1];
        }
        d.set_blocks(0, 0, 16, 16, b);
        parts.push_back({0, 0, 0, 0, 16, 16});
        d.emit_motion(0, parts, r);
    }
    d.store_motion();
    return 0;
}

}  // namespace pimpl
}  // namespace h264r

// slice_data( ) (7.3.4) of a CABAC slice: cabac_alignment_one_bit, then per
// MB mb_skip_flag, macroblock_layer( ) and end_of_slice_flag
// (CH264SliceData::slice_data, H264SliceData.cpp:64-534)
int h264r_parser::decode_slice_cabac(SliceCtx &sc, BitReader &br)
{
    if (cur_mbaff) return decode_slice_mbaff(sc, br, true);
    const int num_mbs = (int)mbs.size();
    MbDecoder d(*this, sc, br);
    Cabac cab;
    cab.br = &br;
    d.cab = &cab;
    int addr = sc.sh.first_mb;
    if (addr >= num_mbs) return fail(H264R_ERR_BAD_RECORD, "first_mb_in_slice %d out of range", addr);
    while (!br.byte_aligned()) br.u(1);
    cab.init_contexts(sc.sh.slice_type, sc.sh.cabac_init_idc, sc.pps->pic_init_qp + sc.sh.slice_qp_delta);
    cab.init_engine();
    const bool skips = sc.sh.slice_type != kSliceI;
    for (;;) {
        if (addr >= num_mbs) return fail(H264R_ERR_BAD_RECORD, "slice data past the picture end");
        if (mbs[addr].slice >= 0) return fail(H264R_ERR_BAD_RECORD, "MB %d decoded twice", addr);
        d.addr = addr;
        d.mbx = addr % width_mbs;
        d.cur = &mbs[addr];
        d.cur->slice = sc.index;
        d.cur->skip = false;
        bool skip = false;
        if (skips) {
            // the skip flag's context reads the neighbours only
            skip = d.cab->decision((sc.sh.slice_type == kSliceB ? 24 : 11) + cabac_skip_inc(d)) != 0;
        }
        if (skip) {
            if (decode_skip(d, rec[addr])) return failed ? H264R_ERR_BAD_RECORD : fail(H264R_ERR_BAD_RECORD, "skip MB %d", addr);
            d.prev_qp_nz = false;
        } else if (d.decode_cabac()) {
            return H264R_ERR_BAD_RECORD;
        }
        if (br.err) return fail(H264R_ERR_BAD_RECORD, "truncated CABAC slice data (MB %d)", addr);
        addr++;
        if (cab.terminate()) break;  // end_of_slice_flag
    }
    return H264R_OK;
}

// slice_data( ) (7.3.4) of an MBAFF frame, CAVLC or CABAC: MB pairs, each
// with its mb_field_decoding_flag, in the order and with the inference the
// reference decoder uses (CH264SliceData::slice_data,
// H264SliceData.cpp:163-521):
//   - the flag is read before the first coded MB of a pair (the top MB, or
//     the bottom one when the top is skipped); a skipped top MB takes the
//     bottom's flag, so it is decoded once that is known: in CAVLC the flag
//     follows a skip run that ends on a top MB, in CABAC the bottom's
//     mb_skip_flag (and then the flag) is decoded right after the top's;
//   - a pair with both MBs skipped infers the flag from the left pair of the
//     slice, else the pair above, else frame;
//   - CABAC: the contexts of a top MB's mb_skip_flag see the flag of the
//     pair decoded last (the pair above for the first pair of a row), the
//     inference of 7.4.4 as the reference applies it.
int h264r_parser::decode_slice_mbaff(SliceCtx &sc, BitReader &br, bool cabac)
{
    const int num_mbs = (int)mbs.size(), W = width_mbs;
    MbDecoder d(*this, sc, br);
    d.mbaff = true;
    Cabac cab;
    if (cabac) {
        cab.br = &br;
        d.cab = &cab;
        while (!br.byte_aligned()) br.u(1);
        cab.init_contexts(sc.sh.slice_type, sc.sh.cabac_init_idc, sc.pps->pic_init_qp + sc.sh.slice_qp_delta);
        cab.init_engine();
    }
    int addr = 2 * sc.sh.first_mb;
    if (addr >= num_mbs) return fail(H264R_ERR_BAD_RECORD, "first_mb_in_slice %d out of range", sc.sh.first_mb);
    const bool skips = sc.sh.slice_type != kSliceI;
    bool field = false;             // mb_field_decoding_flag as the slice decodes it
    bool prev_skipped = false;      // prevMbSkipped
    bool flag_read = false;         // the current pair's flag was read ahead
    int bottom_skip = 0;            // CABAC: the bottom MB's mb_skip_flag, decoded ahead
    // 7.4.4 inference for a pair whose MBs are both skipped
    auto infer = [&](int a) {
        const int pair = a >> 1;
        if (pair % W > 0 && mbs[a - 2].slice == sc.index) return mbs[a - 2].field;
        if (pair >= W && mbs[a - 2 * W].slice == sc.index) return mbs[a - 2 * W].field;
        return false;
    };
    auto enter = [&](int a) -> int {
        if (a >= num_mbs) return fail(H264R_ERR_BAD_RECORD, "slice data past the picture end");
        if (mbs[a].slice >= 0) return fail(H264R_ERR_BAD_RECORD, "MB %d decoded twice", a);
        mbs[a].slice = sc.index;
        mbs[a].skip = false;
        mbs[a].field = field;
        d.set_mb(a);
        return 0;
    };
    auto skip_mb = [&](int a) -> int {
        mbs[a].field = field;
        d.set_mb(a);
        if (decode_skip(d, rec[a])) return failed ? H264R_ERR_BAD_RECORD : fail(H264R_ERR_BAD_RECORD, "skip MB %d", a);
        if (field) rec[a].flags |= H264R_MBF_FIELD;
        d.prev_qp_nz = false;
        return 0;
    };
    auto coded_mb = [&](int a) -> int {
        mbs[a].field = field;
        d.set_mb(a);
        if (cabac ? d.decode_cabac() : d.decode()) return H264R_ERR_BAD_RECORD;
        if (field) rec[a].flags |= H264R_MBF_FIELD;
        return 0;
    };
    bool more = true;
    while (more) {
        bool skipped = false;
        if (skips && !cabac) {
            const uint32_t run = br.ue();
            if (br.err) return fail(H264R_ERR_BAD_RECORD, "truncated mb_skip_run");
            prev_skipped = run > 0;
            for (uint32_t i = 0; i < run; i++) {
                if (int rc = enter(addr)) return rc;
                if ((addr & 1) == 0) {
                    if (i == run - 1) {
                        // the bottom MB is coded: its flag follows the run
                        field = br.u(1) != 0;
                        flag_read = true;
                    } else {
                        field = infer(addr);
                    }
                }
                if (int rc = skip_mb(addr)) return rc;
                addr++;
            }
            if (run > 0) more = br.more_rbsp_data();
            if (!more) break;
        } else if (skips) {
            if (int rc = enter(addr)) return rc;
            if ((addr & 1) == 0) {
                const int pair = addr >> 1;
                // the flag the contexts of this pair's mb_skip_flag see
                if (pair % W == 0 && pair >= W) field = mbs[addr - 2 * W].slice == sc.index ? mbs[addr - 2 * W].field : false;
                mbs[addr].field = field;
                d.set_mb(addr);
            }
            int sk;
            if ((addr & 1) && prev_skipped) {
                sk = bottom_skip;
            } else {
                sk = cab.decision((sc.sh.slice_type == kSliceB ? 24 : 11) + cabac_skip_inc(d));
            }
            if (sk) {
                skipped = true;
                if ((addr & 1) == 0) {
                    // the bottom MB's mb_skip_flag, and its flag if it is coded,
                    // decide the pair's kind before the top MB is decoded
                    mbs[addr].skip = true;
                    if (addr + 1 >= num_mbs) return fail(H264R_ERR_BAD_RECORD, "MBAFF pair past the picture end");
                    mbs[addr + 1].slice = sc.index;
                    mbs[addr + 1].skip = false;
                    mbs[addr + 1].field = field;
                    d.set_mb(addr + 1);
                    bottom_skip = cab.decision((sc.sh.slice_type == kSliceB ? 24 : 11) + cabac_skip_inc(d));
                    mbs[addr + 1].slice = -1;  // entered again in its turn
                    if (!bottom_skip) {
                        field = cab.decision(70 + cabac_field_inc(d)) != 0;
                        flag_read = true;
                    } else {
                        field = infer(addr);
                    }
                }
                if (int rc = skip_mb(addr)) return rc;
            }
        }
        if (!skipped) {
            if (!skips || !cabac) {
                if (int rc = enter(addr)) return rc;
            }
            if ((addr & 1) == 0 || prev_skipped) {
                if (!flag_read) {
                    if (cabac) {
                        d.set_mb(addr);
                        field = cab.decision(70 + cabac_field_inc(d)) != 0;
                    } else {
                        field = br.u(1) != 0;
                    }
                }
                flag_read = false;
            }
            if (int rc = coded_mb(addr)) return rc;
        }
        // prevMbSkipped: in CABAC the MB just decoded; in CAVLC the last run
        if (cabac && skips) prev_skipped = skipped;
        if (br.err) return fail(H264R_ERR_BAD_RECORD, "truncated slice data (MB %d)", addr);
        if (cabac) {
            if ((addr & 1) == 0) more = true;
            else more = !cab.terminate();
        } else {
            more = br.more_rbsp_data();
        }
        addr++;
    }
    return H264R_OK;
}

// slice_data( ) (7.3.4), CAVLC
int h264r_parser::decode_slice(SliceCtx &sc, BitReader &br)
{
    if (sc.pps->cabac) return decode_slice_cabac(sc, br);
    if (cur_mbaff) return decode_slice_mbaff(sc, br, false);
    const int num_mbs = (int)mbs.size();
    MbDecoder d(*this, sc, br);
    int addr = sc.sh.first_mb;
    if (addr >= num_mbs) return fail(H264R_ERR_BAD_RECORD, "first_mb_in_slice %d out of range", addr);
    const bool skips = sc.sh.slice_type != kSliceI;
    bool more = true;
    while (more) {
        if (skips) {
            const uint32_t run = br.ue();
            if (br.err) return fail(H264R_ERR_BAD_RECORD, "truncated mb_skip_run");
            for (uint32_t i = 0; i < run; i++) {
                if (addr >= num_mbs) return fail(H264R_ERR_BAD_RECORD, "mb_skip_run past the picture end");
                if (mbs[addr].slice >= 0) return fail(H264R_ERR_BAD_RECORD, "MB %d decoded twice", addr);
                d.addr = addr;
                d.mbx = addr % width_mbs;
                d.cur = &mbs[addr];
                d.cur->slice = sc.index;
                d.cur->skip = false;
                if (decode_skip(d, rec[addr])) return failed ? H264R_ERR_BAD_RECORD : fail(H264R_ERR_BAD_RECORD, "skip MB %d", addr);
                addr++;
            }
            if (run > 0) more = br.more_rbsp_data();
        }
        if (more) {
            if (addr >= num_mbs) return fail(H264R_ERR_BAD_RECORD, "slice data past the picture end");
            if (mbs[addr].slice >= 0) return fail(H264R_ERR_BAD_RECORD, "MB %d decoded twice", addr);
            d.addr = addr;
            d.mbx = addr % width_mbs;
            d.cur = &mbs[addr];
            d.cur->slice = sc.index;
            d.cur->skip = false;
            if (d.decode()) return H264R_ERR_BAD_RECORD;
            addr++;
            more = br.more_rbsp_data();
        }
    }
    return H264R_OK;
}

// ---------------------------------------------------------------- POC (8.2.1)
void h264r_parser::compute_poc(const SliceHeader &sh, const Sps &s)
{
    const int max_frame_num = 1 << s.log2_max_frame_num;
    if (s.poc_type == 0) {
        if (sh.idr) {
            prev_poc_msb = prev_poc_lsb = 0;
        } else if (prev_ref_mmco5) {
            prev_poc_msb = 0;
            prev_poc_lsb = prev_ref_bottom_field ? 0 : prev_ref_top_poc;
        }
        const int max_lsb = 1 << s.log2_max_poc_lsb;
        int msb;
        if (sh.poc_lsb < prev_poc_lsb && prev_poc_lsb - sh.poc_lsb >= max_lsb / 2) msb = prev_poc_msb + max_lsb;
        else if (sh.poc_lsb > prev_poc_lsb && sh.poc_lsb - prev_poc_lsb > max_lsb / 2) msb = prev_poc_msb - max_lsb;
        else msb = prev_poc_msb;
        cur.top_poc = msb + sh.poc_lsb;
        cur.bottom_poc = cur.top_poc + sh.delta_poc_bottom;
        if (sh.nal_ref_idc) {  // becomes prevPicOrderCntMsb / Lsb for the next picture
            pending_msb = msb;
            pending_lsb = sh.poc_lsb;
        }
    } else {
        if (sh.idr) frame_num_offset = 0;
        else {
            const int prev_off = prev_mmco5 ? 0 : prev_frame_num_offset;
            frame_num_offset = prev_frame_num > sh.frame_num ? prev_off + max_frame_num : prev_off;
        }
        if (s.poc_type == 1) {
            const int cycle = (int)s.offset_for_ref_frame.size();
            int abs_frame_num = cycle != 0 ? frame_num_offset + sh.frame_num : 0;
            if (sh.nal_ref_idc == 0 && abs_frame_num > 0) abs_frame_num--;
            int expected = 0;
            if (abs_frame_num > 0) {
                int delta_cycle = 0;
                for (int i = 0; i < cycle; i++) delta_cycle += s.offset_for_ref_frame[i];
                const int cnt = (abs_frame_num - 1) / cycle, in_cycle = (abs_frame_num - 1) % cycle;
                expected = cnt * delta_cycle;
                for (int i = 0; i <= in_cycle; i++) expected += s.offset_for_ref_frame[i];
            }
            if (sh.nal_ref_idc == 0) expected += s.offset_for_non_ref_pic;
            cur.top_poc = expected + sh.delta_poc[0];
            cur.bottom_poc = cur.top_poc + s.offset_for_top_to_bottom_field + sh.delta_poc[1];
        } else {
            int t = 0;
            if (!sh.idr) t = sh.nal_ref_idc == 0 ? 2 * (frame_num_offset + sh.frame_num) - 1 : 2 * (frame_num_offset + sh.frame_num);
            cur.top_poc = cur.bottom_poc = t;
        }
    }
    cur.poc = std::min(cur.top_poc, cur.bottom_poc);
}

// ---------------------------------------------------------------- lists (8.2.4)
int h264r_parser::build_lists(SliceCtx &sc)
{
    const SliceHeader &sh = sc.sh;
    const Sps &s = *sc.sps;
    const int max_frame_num = 1 << s.log2_max_frame_num;
    sc.list[0].clear();
    sc.list[1].clear();
    if (sh.slice_type == kSliceI) return H264R_OK;
    std::vector<Pic *> shorts, longs;
    for (Pic &p : dpb) {
        if (p.short_ref) {
            p.frame_num_wrap = p.frame_num > sh.frame_num ? p.frame_num - max_frame_num : p.frame_num;
            shorts.push_back(&p);
        } else if (p.long_ref) {
            longs.push_back(&p);
        }
    }
    std::stable_sort(longs.begin(), longs.end(), [](const Pic *a, const Pic *b) { return a->long_term_frame_idx < b->long_term_frame_idx; });
    std::vector<Pic *> init[2];
    if (sh.slice_type == kSliceP) {
        std::vector<Pic *> st = shorts;
        std::stable_sort(st.begin(), st.end(), [](const Pic *a, const Pic *b) { return a->frame_num_wrap > b->frame_num_wrap; });
        init[0] = st;
        init[0].insert(init[0].end(), longs.begin(), longs.end());
    } else {
        // CH264PictureBase::Initialisation_process_for_reference_picture_lists_for_B_slices_in_frames
        // (H264RefPicList.cpp:830-1015): POC <= current on the L0 side
        std::vector<Pic *> before, after;
        for (Pic *p : shorts) (p->poc > cur.poc ? after : before).push_back(p);
        std::stable_sort(before.begin(), before.end(), [](const Pic *a, const Pic *b) { return a->poc > b->poc; });
        std::stable_sort(after.begin(), after.end(), [](const Pic *a, const Pic *b) { return a->poc < b->poc; });
        init[0] = before;
        init[0].insert(init[0].end(), after.begin(), after.end());
        init[0].insert(init[0].end(), longs.begin(), longs.end());
        init[1] = after;
        init[1].insert(init[1].end(), before.begin(), before.end());
        init[1].insert(init[1].end(), longs.begin(), longs.end());
        if (init[1].size() > 1 && init[1] == init[0]) std::swap(init[1][0], init[1][1]);
        if (init[0].empty()) return fail(H264R_ERR_BAD_RECORD, "B slice without reference pictures");
    }
    const int nlists = sh.slice_type == kSliceB ? 2 : 1;
    for (int l = 0; l < nlists; l++) {
        const int n = sh.num_ref_idx_active[l];
        std::vector<Pic *> list = init[l];
        list.resize(n, nullptr);
        // modification (8.2.4.3)
        const int cur_pic_num = sh.frame_num, max_pic_num = max_frame_num;
        int pred = cur_pic_num, idx = 0;
        for (const RefMod &m : sh.mods[l]) {
            if (idx >= n) return fail(H264R_ERR_BAD_RECORD, "too many reference list modifications");
            Pic *target = nullptr;
            if (m.idc == 0 || m.idc == 1) {
                const int d = m.value + 1;
                int no_wrap;
                if (m.idc == 0) {
                    no_wrap = pred - d;
                    if (no_wrap < 0) no_wrap += max_pic_num;
                } else {
                    no_wrap = pred + d;
                    if (no_wrap >= max_pic_num) no_wrap -= max_pic_num;
                }
                pred = no_wrap;
                const int pic_num = no_wrap > cur_pic_num ? no_wrap - max_pic_num : no_wrap;
                for (Pic *p : shorts)
                    if (p->frame_num_wrap == pic_num) target = p;
                if (!target) return fail(H264R_ERR_BAD_RECORD, "modification names a missing short-term picture");
            } else if (m.idc == 2) {
                for (Pic *p : longs)
                    if (p->long_term_frame_idx == m.value) target = p;
                if (!target) return fail(H264R_ERR_BAD_RECORD, "modification names a missing long-term picture");
            } else {
                return fail(H264R_ERR_UNSUPPORTED, "modification_of_pic_nums_idc %d", m.idc);
            }
            // insert target at idx, drop its later duplicate
            list.insert(list.begin() + idx, target);
            idx++;
            int w = idx;
            for (int k = idx; k < (int)list.size(); k++)
                if (list[k] != target) list[w++] = list[k];
            list.resize(std::max(w, n));
            list.resize(n);
        }
        sc.list[l] = list;
        if (n < 1 || !list[0]) return fail(H264R_ERR_BAD_RECORD, "reference list %d is empty", l);
    }
    return H264R_OK;
}

// ---------------------------------------------------------------- marking (8.2.5)
int h264r_parser::mark_references(const SliceHeader &sh, const Sps &s)
{
    const int max_frame_num = 1 << s.log2_max_frame_num;
    cur.mmco5 = false;
    if (sh.idr) {
        for (Pic &p : dpb) p.short_ref = p.long_ref = false;
        if (sh.long_term_reference) {
            cur.long_ref = true;
            cur.long_term_frame_idx = 0;
            max_long_term_frame_idx = 0;
        } else {
            cur.short_ref = true;
            max_long_term_frame_idx = kNoLongTerm;
        }
        return H264R_OK;
    }
    bool cur_long = false;
    if (sh.adaptive_marking) {
        for (Pic &p : dpb)
            if (p.short_ref) p.frame_num_wrap = p.frame_num > sh.frame_num ? p.frame_num - max_frame_num : p.frame_num;
        for (const Mmco &m : sh.mmcos) {
            if (m.op == 1 || m.op == 3) {
                const int pic_num_x = sh.frame_num - (m.diff_pic_nums_minus1 + 1);
                Pic *t = nullptr;
                for (Pic &p : dpb)
                    if (p.short_ref && p.frame_num_wrap == pic_num_x) t = &p;
                if (!t) continue;
                if (m.op == 1) {
                    t->short_ref = false;
                } else {
                    for (Pic &p : dpb)
                        if (p.long_ref && p.long_term_frame_idx == m.long_term_frame_idx) p.long_ref = false;
                    t->short_ref = false;
                    t->long_ref = true;
                    t->long_term_frame_idx = m.long_term_frame_idx;
                }
            } else if (m.op == 2) {
                for (Pic &p : dpb)
                    if (p.long_ref && p.long_term_frame_idx == m.long_term_pic_num) p.long_ref = false;
            } else if (m.op == 4) {
                max_long_term_frame_idx = m.max_long_term_frame_idx_plus1 - 1;
                for (Pic &p : dpb)
                    if (p.long_ref && p.long_term_frame_idx > max_long_term_frame_idx) p.long_ref = false;
            } else if (m.op == 5) {
                for (Pic &p : dpb) p.short_ref = p.long_ref = false;
                max_long_term_frame_idx = kNoLongTerm;
                cur.mmco5 = true;
            } else if (m.op == 6) {
                for (Pic &p : dpb)
                    if (p.long_ref && p.long_term_frame_idx == m.long_term_frame_idx) p.long_ref = false;
                cur.long_ref = true;
                cur.long_term_frame_idx = m.long_term_frame_idx;
                cur_long = true;
            }
        }
    } else {
        // sliding window (8.2.5.3)
        int n_short = 0, n_long = 0;
        for (Pic &p : dpb) {
            n_short += p.short_ref;
            n_long += p.long_ref;
        }
        if (n_short + n_long >= std::max(s.max_num_ref_frames, 1) && n_short > 0) {
            // the smallest FrameNumWrap as last derived: the reference derives
            // it only while building the lists of a P or B slice
            // (H264RefPicList.cpp:339-349) and compares those stored values
            // (H264RefPicList.cpp:1660-1676), so a picture decoded after the
            // last list construction still has its initial 0 (build_lists
            // keeps frame_num_wrap the same way)
            Pic *oldest = nullptr;
            for (Pic &p : dpb)
                if (p.short_ref && (!oldest || p.frame_num_wrap < oldest->frame_num_wrap)) oldest = &p;
            oldest->short_ref = false;
        }
    }
    if (!cur_long) cur.short_ref = true;
    if (cur.mmco5) {  // the picture counts as frame_num 0 with its POC rebased (8.2.1)
        const int t = cur.poc;
        cur.top_poc -= t;
        cur.bottom_poc -= t;
        cur.poc = 0;
        cur.frame_num = 0;
    }
    return H264R_OK;
}

int h264r_parser::alloc_slot()
{
    // the free slot that has been free longest: consecutive pictures land in
    // different slots, so pictures that do not reference each other (B
    // pictures between two anchors) can be reconstructed in one batch
    int best = -1;
    for (int i = 0; i < (int)slot_uid.size(); i++)
        if (slot_uid[i] < 0 && (best < 0 || slot_freed[i] < slot_freed[best])) best = i;
    return best;
}

// first slice of a new picture
int h264r_parser::start_picture(const SliceHeader &sh, const Sps &s, const Pps &q)
{
    (void)q;
    if (!active_sps) {
        active_sps = &s;
        width_mbs = s.width_mbs;
        height_mbs = s.frame_height_mbs();
        reorder_depth = s.has_reorder ? s.max_num_reorder_frames
                                      : h264r_order_infer_depth(s.profile_idc, s.constraint_set3, s.level_idc, width_mbs, height_mbs);
        if (reorder_depth < 0) reorder_depth = 0;
        if (reorder_depth > 16) reorder_depth = 16;
        // references + pictures held for output + the picture being decoded,
        // and one spare slot: with it the B pictures between two anchors and
        // the next anchor land in slots no picture they depend on uses, so
        // the batched entry points can reconstruct them together
        dpb_slots = std::min(32, std::max(s.max_num_ref_frames, 1) + reorder_depth + 2);
        slot_uid.assign(dpb_slots, -1);
        slot_freed.assign(dpb_slots, -1);
        slot_poc.assign(dpb_slots, 0);
        slot_index.assign(dpb_slots, 0);
        if (h264r_order_create(reorder_depth, &order)) return fail(H264R_ERR_INVALID_ARG, "reorder depth");
    } else if (s.width_mbs != width_mbs || s.frame_height_mbs() != height_mbs) {
        return fail(H264R_ERR_UNSUPPORTED, "picture size change within the stream");
    }
    cur_mbaff = sh.mbaff != 0;
    cur = Pic();
    cur.uid = next_uid++;
    // FrameNum of the picture as a reference: the reference decoder assigns
    // it (from frame_num) only while it builds reference lists, i.e. in P and
    // B slices (H264RefPicList.cpp:334, reached from H264RefPicList.cpp:284
    // for P / B slices only); a picture of I slices keeps FrameNum 0, so a
    // non-IDR I picture sorts last in P lists and is the first one the
    // sliding window drops.  begin_slice sets it for P / B slices.
    cur.frame_num = 0;
    compute_poc(sh, s);
    const int slot = alloc_slot();
    if (slot < 0) return fail(H264R_ERR_BUSY, "no free DPB slot");
    cur.slot = slot;
    slot_uid[slot] = cur.uid;
    slot_poc[slot] = cur.poc;
    slot_index[slot] = decoded;
    const int n = width_mbs * height_mbs;
    // every reader of a neighbour's state checks that it was decoded in the
    // same slice (slice >= 0) first, so only that mark is reset per picture
    if ((int)mbs.size() != n) mbs.assign(n, MbState());
    else
        for (MbState &m : mbs) {
            m.slice = -1;
            m.field = false;
        }
    h264r_mb none;
    memset(&none, 0, sizeof(none));
    none.type = H264R_MB_NONE;
    none.coef = H264R_NONE;
    none.aux = H264R_NONE;
    rec.assign(n, none);
    rec_slices.clear();
    rec_weights.assign(1, h264r_weight());
    memset(&rec_weights[0], 0, sizeof(h264r_weight));
    motion.clear();
    coef.clear();
    pcm.clear();
    dref_parts.clear();
    num_slices = 0;
    first_sh = sh;
    first_slice_type = (uint8_t)sh.slice_type;
    in_pic = true;
    return H264R_OK;
}

// the current picture is complete: records out, marking, DPB, output order
int h264r_parser::finish_picture(bool last)
{
    if (!in_pic) return H264R_OK;
    in_pic = false;
    const SliceHeader &sh = first_sh;
    const Sps &s = *active_sps;
    // deblocking identity of every part: the last slice's lists
    for (uint32_t off : dref_parts) {
        h264r_part p;
        memcpy(&p, &motion[off], sizeof(p));
        for (int l = 0; l < 2; l++) {
            const int ri = p.dref[l];
            p.dref[l] = -1;
            if (ri >= 0 && ri < (int)last_list[l].size() && last_list[l][ri]) p.dref[l] = (int8_t)last_list[l][ri]->slot;
        }
        memcpy(&motion[off], &p, sizeof(p));
    }
    // co-located motion for later direct prediction; the co-located picture
    // is a reference picture (RefPicList1[0]), so non-reference pictures keep
    // none (a missing one reads as intra, as before any motion exists)
    const int n = (int)mbs.size();
    cur.motion.reset();
    if (sh.nal_ref_idc) {
    // a buffer no picture holds any more is reused (every entry is rewritten)
    std::shared_ptr<Motion> mo;
    for (auto &m : motion_pool)
        if (m.use_count() == 1) {
            mo = m;
            break;
        }
    if (!mo) {
        mo = std::make_shared<Motion>();
        motion_pool.push_back(mo);
    }
    mo->intra.resize(n);
    mo->field.assign(n, 0);
    mo->mv.resize((size_t)n * 2 * 16 * 2);
    mo->ref.resize((size_t)n * 2 * 16);
    mo->refpic.resize((size_t)n * 2 * 16);
    // per MB the [list][4x4 block] arrays have the MB state's layout: one
    // copy each (intra and undecoded MBs: no motion, references -1)
    static_assert(sizeof(MbState::mv) == 2 * 16 * 2 * sizeof(int16_t) && sizeof(MbState::ref) == 32 &&
                      sizeof(MbState::refpic) == 32 * sizeof(int32_t),
                  "co-located motion layout");
    for (int a = 0; a < n; a++) {
        const MbState &m = mbs[a];
        const bool inter = m.slice >= 0 && m.cls == H264R_MB_INTER;
        mo->intra[a] = inter ? 0 : (m.slice >= 0 && m.cls == H264R_MB_IPCM ? 2 : 1);
        mo->field[a] = cur_mbaff && m.field ? 1 : 0;
        int16_t *mv = &mo->mv[(size_t)a * 64];
        int8_t *ref = &mo->ref[(size_t)a * 32];
        int32_t *rp = &mo->refpic[(size_t)a * 32];
        if (inter) {
            memcpy(mv, m.mv, sizeof(m.mv));
            memcpy(ref, m.ref, sizeof(m.ref));
            memcpy(rp, m.refpic, sizeof(m.refpic));
        } else {
            memset(mv, 0, sizeof(m.mv));
            memset(ref, 0xFF, sizeof(m.ref));
            memset(rp, 0xFF, sizeof(m.refpic));  // -1 in every int32
        }
    }
    cur.motion = mo;
    }
    // marking, then POC state for the next picture
    if (sh.nal_ref_idc) {
        const int rc = mark_references(sh, s);
        if (rc) return rc;
        prev_ref_mmco5 = cur.mmco5;
        prev_ref_bottom_field = 0;
        prev_ref_top_poc = cur.top_poc;
        if (s.poc_type == 0) {
            prev_poc_msb = cur.mmco5 ? 0 : pending_msb;
            prev_poc_lsb = cur.mmco5 ? cur.top_poc : pending_lsb;
        }
    }
    prev_mmco5 = cur.mmco5;
    prev_frame_num_offset = frame_num_offset;
    prev_frame_num = cur.mmco5 ? 0 : sh.frame_num;
    // records out
    Done d;
    d.mbs.swap(rec);
    d.slices.swap(rec_slices);
    d.weights.swap(rec_weights);
    d.motion.swap(motion);
    d.coef.swap(coef);
    d.pcm.swap(pcm);
    memset(&d.pic, 0, sizeof(d.pic));
    d.pic.width_mbs = (uint16_t)width_mbs;
    d.pic.height_mbs = (uint16_t)height_mbs;
    d.pic.structure = H264R_STRUCT_FRAME;
    d.pic.mbaff = cur_mbaff ? 1 : 0;
    d.pic.dst_slot = (uint8_t)cur.slot;
    d.pic.deblock = last ? 0 : 1;
    const Pps &q = pps[sh.pps_id];
    for (int i = 0; i < 6; i++) memcpy(d.pic.scaling4x4[i], q.sl4[i], 16);
    for (int i = 0; i < 6; i++) memcpy(d.pic.scaling8x8[i], q.sl8[i], 64);
    d.poc = cur.poc;
    d.index = decoded++;
    d.idr = (uint8_t)sh.idr;
    d.reference = sh.nal_ref_idc != 0;
    d.slice_type = first_slice_type;
    // output order (CH264VideoDecoder::do_callback through the reorder buffer)
    uint64_t outs[40];
    int k = h264r_order_push(order, (uint64_t)cur.slot, cur.poc, sh.idr, outs, 40);
    if (k < 0) return fail(k, "output order");
    if (last) {
        const int k2 = h264r_order_flush(order, outs + k, 40 - k);
        if (k2 < 0) return fail(k2, "output order flush");
        k += k2;
    }
    for (int i = 0; i < k; i++) {
        const int sl = (int)outs[i];
        d.out_slots.push_back((uint8_t)sl);
        d.out_poc.push_back(slot_poc[sl]);
        d.out_index.push_back(slot_index[sl]);
    }
    // the picture joins the DPB; free what is neither referenced nor held
    dpb.push_back(cur);
    for (auto it = dpb.begin(); it != dpb.end();) {
        if (!it->is_ref() && !h264r_order_holds(order, (uint64_t)it->slot)) {
            slot_uid[it->slot] = -1;
            slot_freed[it->slot] = (int64_t)decoded;
            it = dpb.erase(it);
        } else {
            ++it;
        }
    }
    done.push_back(std::move(d));
    return H264R_OK;
}

// ---------------------------------------------------------------- NAL units
int h264r_parser::process_nal(const uint8_t *p, size_t n)
{
    if (n < 1) return H264R_OK;
    const int type = p[0] & 31;
    const char *why = nullptr;
    BitReader br;
    if (type == 7 || type == 8) {
        nal_to_rbsp(p + 1, n - 1, rbsp);
        br.reset(rbsp.data(), rbsp.size());
    }
    if (type == 7) {
        Sps s;
        const int rc = parse_sps(br, s, &why);
        if (rc) return fail(rc, "SPS: %s", why ? why : "error");
        if (active_sps && s.id == active_sps->id && (s.width_mbs != width_mbs || s.frame_height_mbs() != height_mbs))
            return fail(H264R_ERR_UNSUPPORTED, "picture size change within the stream");
        sps[s.id] = s;
        return H264R_OK;
    }
    if (type == 8) {
        Pps q;
        const int rc = parse_pps(br, sps, q, &why);
        if (rc) return fail(rc, "PPS: %s", why ? why : "error");
        pps[q.id] = q;
        return H264R_OK;
    }
    if (type == 2 || type == 3 || type == 4) return fail(H264R_ERR_UNSUPPORTED, "data partitioning");
    if (type != 1 && type != 5) return H264R_OK;  // SEI, AUD, filler and others carry no picture data here
    SliceCtx sc;
    BitReader sbr;
    const int rb = begin_slice(p, n, sc, sbr);
    if (rb <= 0) return rb;
    const int r3 = decode_slice(sc, sbr);
    if (r3 == H264R_ERR_BAD_RECORD) {
        // the reference skips the rest of a slice that fails to decode and
        // goes on with the next one (H264VideoDecoder.cpp:136): its MBs
        // from the failing one on stay undecoded
        slice_errors++;
        failed = false;
        for (MbState &m : mbs)
            if (m.slice == sc.index && rec[&m - mbs.data()].type == H264R_MB_NONE) m.slice = -1;
        return H264R_OK;
    }
    return r3;
}

int h264r_parser::begin_slice(const uint8_t *p, size_t n, SliceCtx &sc, BitReader &br)
{
    if (n < 1) return fail(H264R_ERR_BAD_RECORD, "empty slice NAL unit");
    const int nal_ref_idc = (p[0] >> 5) & 3, type = p[0] & 31;
    nal_to_rbsp(p + 1, n - 1, rbsp);
    br.reset(rbsp.data(), rbsp.size());
    const char *why = nullptr;
    const int rc = parse_slice_header(br, type, nal_ref_idc, sps, pps, sc.sh, &why);
    if (rc) return fail(rc, "slice header: %s", why ? why : "error");
    sc.pps = &pps[sc.sh.pps_id];
    sc.sps = &sps[sc.pps->sps_id];
    if (sc.sh.redundant_pic_cnt > 0) return 0;  // redundant slices are not decoded
    // first VCL NAL unit of a new primary picture (7.4.1.2.4)
    bool first = !in_pic;
    if (in_pic) {
        const SliceHeader &a = first_sh;
        const SliceHeader &b = sc.sh;
        first = a.frame_num != b.frame_num || a.pps_id != b.pps_id || (a.nal_ref_idc == 0) != (b.nal_ref_idc == 0) ||
                a.poc_lsb != b.poc_lsb || a.delta_poc_bottom != b.delta_poc_bottom || a.delta_poc[0] != b.delta_poc[0] ||
                a.delta_poc[1] != b.delta_poc[1] || a.idr != b.idr || (a.idr && b.idr && a.idr_pic_id != b.idr_pic_id);
    }
    if (first) {
        int r2 = finish_picture(false);
        if (r2) return r2;
        r2 = start_picture(sc.sh, *sc.sps, *sc.pps);
        if (r2) return r2;
    }
    sc.index = num_slices++;
    if (sc.sh.slice_type != kSliceI && sc.sh.slice_type != kSliceSI) cur.frame_num = sc.sh.frame_num;
    h264r_slice rs;
    memset(&rs, 0, sizeof(rs));
    rs.chroma_qp_offset[0] = (int8_t)sc.pps->chroma_qp_offset[0];
    rs.chroma_qp_offset[1] = (int8_t)sc.pps->chroma_qp_offset[1];
    rs.filter_offset_a = (int8_t)(sc.sh.alpha_offset_div2 * 2);
    rs.filter_offset_b = (int8_t)(sc.sh.beta_offset_div2 * 2);
    rs.disable_deblocking_filter_idc = (uint8_t)sc.sh.disable_deblocking_filter_idc;
    rs.slice_type = (uint8_t)sc.sh.slice_type;
    rec_slices.push_back(rs);
    const int r3 = build_lists(sc);
    if (r3) return r3;
    last_list[0] = sc.list[0];
    last_list[1] = sc.list[1];
    return 1;
}

// ---------------------------------------------------------------- C API
namespace {

// start code positions in buf: returns the offset of the next 00 00 01 at or after `from`, or npos
size_t find_start(const std::vector<uint8_t> &b, size_t from)
{
    for (size_t i = from; i + 2 < b.size(); i++)
        if (b[i] == 0 && b[i + 1] == 0 && b[i + 2] == 1) return i;
    return std::string::npos;
}

int drain(h264r_parser *p, bool at_end)
{
    size_t s = find_start(p->buf, 0);
    if (s == std::string::npos) {
        if (at_end) p->buf.clear();
        return H264R_OK;
    }
    size_t consumed = s;
    while (true) {
        const size_t begin = s + 3;
        size_t next = find_start(p->buf, begin);
        size_t end;
        if (next == std::string::npos) {
            if (!at_end) break;
            end = p->buf.size();
        } else {
            end = next;
        }
        // trailing zero bytes belong to the next start code (zero_byte) or are trailing_zero_8bits
        size_t e = end;
        while (e > begin && p->buf[e - 1] == 0) e--;
        if (e > begin) {
            const int rc = p->process_nal(p->buf.data() + begin, e - begin);
            if (rc) return rc;
        }
        consumed = end;
        if (next == std::string::npos) break;
        s = next;
    }
    p->buf.erase(p->buf.begin(), p->buf.begin() + (ptrdiff_t)consumed);
    return H264R_OK;
}

}  // namespace

extern "C" int h264r_parser_create(h264r_parser **out)
{
    if (!out) return H264R_ERR_INVALID_ARG;
    h264r_parser *p = new (std::nothrow) h264r_parser();
    if (!p) return H264R_ERR_NO_MEMORY;
    *out = p;
    return H264R_OK;
}

extern "C" int h264r_parser_destroy(h264r_parser *p)
{
    if (!p) return H264R_ERR_INVALID_ARG;
    delete p;
    return H264R_OK;
}

extern "C" const char *h264r_parser_last_error(const h264r_parser *p) { return p ? p->err.c_str() : "null parser"; }

extern "C" int h264r_parser_feed(h264r_parser *p, const uint8_t *data, size_t size)
{
    if (!p || (!data && size)) return H264R_ERR_INVALID_ARG;
    if (p->failed) return H264R_ERR_BAD_RECORD;
    if (p->ended) return p->fail(H264R_ERR_INVALID_ARG, "feed after end of stream");
    p->buf.insert(p->buf.end(), data, data + size);
    return drain(p, false);
}

extern "C" int h264r_parser_end(h264r_parser *p)
{
    if (!p) return H264R_ERR_INVALID_ARG;
    if (p->failed) return H264R_ERR_BAD_RECORD;
    if (p->ended) return H264R_OK;
    int rc = drain(p, true);
    if (rc) return rc;
    p->ended = true;
    return p->finish_picture(true);
}

extern "C" int h264r_parser_next(h264r_parser *p, h264r_parsed *out)
{
    if (!p || !out) return H264R_ERR_INVALID_ARG;
    if (p->done.empty()) return p->failed ? H264R_ERR_BAD_RECORD : 0;
    p->current_out = std::move(p->done.front());
    p->done.pop_front();
    h264r_parser::Done &d = p->current_out;
    memset(out, 0, sizeof(*out));
    out->pic = d.pic;
    out->pic.num_slices = (uint16_t)d.slices.size();
    out->pic.num_weights = (uint16_t)d.weights.size();
    out->pic.num_mbs = (uint32_t)d.mbs.size();
    out->pic.motion_bytes = (uint32_t)d.motion.size();
    out->pic.coef_bytes = (uint32_t)d.coef.size();
    out->pic.num_pcm = (uint32_t)(d.pcm.size() / 384);
    out->pic.mbs = d.mbs.data();
    out->pic.slices = d.slices.data();
    out->pic.weights = d.weights.data();
    out->pic.motion = d.motion.data();
    out->pic.coef = d.coef.data();
    out->pic.pcm = d.pcm.data();
    out->poc = d.poc;
    out->index = d.index;
    out->idr = d.idr;
    out->reference = d.reference;
    out->slice_type = d.slice_type;
    out->num_output = (uint32_t)d.out_slots.size();
    out->output_slots = d.out_slots.data();
    out->output_poc = d.out_poc.data();
    out->output_index = d.out_index.data();
    return 1;
}

extern "C" int h264r_parser_geometry(const h264r_parser *p, int *width_mbs, int *height_mbs, int *dpb_slots)
{
    if (!p) return H264R_ERR_INVALID_ARG;
    if (width_mbs) *width_mbs = p->width_mbs;
    if (height_mbs) *height_mbs = p->height_mbs;
    if (dpb_slots) *dpb_slots = p->dpb_slots;
    return H264R_OK;
}
