// h264r_parser_impl.h — internals of the host-side front end shared by the
// parser (h264r_parser.cpp) and the seeded bitstream writer
// (h264r_writer.cpp): decoder state, the macroblock decoder and its
// derivations.  Host only; not an interface of the library.
#pragma once

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <string>
#include <vector>

#include "../../include/h264r_order.h"
#include "../../include/h264r_parser.h"
#include "h264r_bits.h"
#include "h264r_syntax.h"

namespace h264r {

int cavlc_residual_block(BitReader &br, int nC, int start, int end, int max_coeff, int *coeff, int &total);
int cavlc_residual_sparse(BitReader &br, int nC, int start, int end, int max_coeff, int off, uint16_t &sig, int16_t *lev,
                          int &total);
int cbp_from_code(uint32_t code, bool intra);

namespace pimpl {

constexpr int kNoLongTerm = -1;

// luma4x4BlkIdx -> 4x4 block position (in 4-sample units), 6.4.3
inline constexpr uint8_t kBlkX[16] = {0, 1, 0, 1, 2, 3, 2, 3, 0, 1, 0, 1, 2, 3, 2, 3};
inline constexpr uint8_t kBlkY[16] = {0, 0, 1, 1, 0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 3, 3};

inline int blk_of(int x4, int y4) { return 8 * (y4 >> 1) + 4 * (x4 >> 1) + 2 * (y4 & 1) + (x4 & 1); }
inline int clip3(int lo, int hi, int v) { return v < lo ? lo : (v > hi ? hi : v); }
inline int median3(int a, int b, int c) { return std::max(std::min(a, b), std::min(std::max(a, b), c)); }

// ---------------------------------------------------------------- pictures
// Motion of a decoded picture, kept while it is a reference (co-located
// data for direct prediction, 8.4.1.2.1).
struct Motion {
    std::vector<uint8_t> intra;   // per MB: 1 intra or undecoded, 2 I_PCM
    std::vector<uint8_t> field;   // per MB: field MB of an MBAFF frame
    std::vector<int16_t> mv;      // [mb][list][4x4 raster][2]
    std::vector<int8_t> ref;      // [mb][list][4x4 raster], -1: list unused
    std::vector<int32_t> refpic;  // [mb][list][4x4 raster]: uid of the reference picture
};

struct Pic {
    int uid = -1, slot = -1;
    int frame_num = 0, frame_num_wrap = 0, long_term_frame_idx = 0;
    bool short_ref = false, long_ref = false;
    int poc = 0, top_poc = 0, bottom_poc = 0;
    bool mmco5 = false;
    std::shared_ptr<Motion> motion;
    bool is_ref() const { return short_ref || long_ref; }
};

// Neighbour state of one MB of the picture being decoded.
struct MbState {
    int slice = -1;  // slice number, -1 while not decoded
    uint8_t cls = 0; // H264R_MB_*
    bool skip = false;
    bool field = false;  // MBAFF: mb_field_decoding_flag of the MB's pair
    uint8_t tc[16];        // TotalCoeff per luma4x4BlkIdx
    uint8_t tcc[2][4];     // chroma AC TotalCoeff
    int8_t ipm4[16];       // Intra4x4PredMode per luma4x4BlkIdx
    int8_t ipm8[4];        // Intra8x8PredMode
    int16_t mv[2][16][2];  // per 4x4 block, raster order
    int8_t ref[2][16];
    int32_t refpic[2][16];
    // syntax the CABAC contexts of later MBs read (9.3.3.1.1)
    uint8_t cbp = 0;          // coded_block_pattern: luma bits 0..3, chroma << 4
    bool t8 = false;          // transform_size_8x8_flag
    bool direct16 = false;    // B_Skip or B_Direct_16x16
    uint8_t chroma_mode = 0;  // intra_chroma_pred_mode
    uint8_t cbf_dc = 0;       // coded_block_flag of the DC blocks: bit 0 luma, 1 Cb, 2 Cr
    uint16_t cbf_ac[3] = {0, 0, 0};  // coded_block_flag of the luma 4x4 blocks (8x8 blocks
                                     // in bits 0..3 when t8) and the Cb / Cr AC blocks
    uint8_t predl[16];        // per 4x4 block: lists its partition predicts from (bit 0
                              // L0, bit 1 L1; 0 for direct, skipped and intra MBs)
    int16_t mvd[2][16][2];    // mvd_lX per 4x4 block (0 where none was coded)
    bool intra() const { return cls != H264R_MB_INTER && cls != H264R_MB_NONE; }
};

// CABAC arithmetic decoding engine and context states (9.3.1.2, 9.3.3.2)
struct Cabac {
    BitReader *br = nullptr;
    uint32_t range = 510, offset = 0;
    uint8_t state[460], mps[460];
    void init_contexts(int slice_type, int cabac_init_idc, int qp);
    void init_engine()
    {
        range = 510;
        offset = br->u(9);
    }
    int decision(int ctx);
    int bypass()
    {
        offset = (offset << 1) | br->u(1);
        if (offset >= range) {
            offset -= range;
            return 1;
        }
        return 0;
    }
    int terminate()
    {
        range -= 2;
        if (offset >= range) return 1;
        while (range < 256) {
            range <<= 1;
            offset = (offset << 1) | br->u(1);
        }
        return 0;
    }
};

struct SliceCtx {
    SliceHeader sh;
    const Sps *sps = nullptr;
    const Pps *pps = nullptr;
    std::vector<Pic *> list[2];
    int index = 0;  // slice number within the picture
};

// one 4x4 block's motion during the MB derivation
struct Blk {
    int16_t mv[2][2];
    int8_t ref[2];
};

struct PartRec {
    int mp, sp;         // mbPartIdx, subMbPartIdx
    int x, y, w, h;     // luma samples within the MB
};

}  // namespace pimpl

}  // namespace h264r

using namespace h264r;
using namespace h264r::pimpl;

struct h264r_parser {
    std::string err;
    // byte stream
    std::vector<uint8_t> buf;  // unconsumed input
    bool ended = false, failed = false;
    // parameter sets
    Sps sps[32];
    Pps pps[256];
    const Sps *active_sps = nullptr;
    int width_mbs = 0, height_mbs = 0, dpb_slots = 0, reorder_depth = 0;
    // DPB
    std::deque<Pic> dpb;       // decoded pictures still referenced or awaiting output
    int next_uid = 0;
    uint32_t decoded = 0;
    h264r_order *order = nullptr;
    std::vector<int> slot_uid;  // slot -> uid of its picture, -1 free
    std::vector<int64_t> slot_freed;  // slot -> pictures decoded when it was freed (-1: never used)
    // POC state
    int prev_poc_msb = 0, prev_poc_lsb = 0, prev_frame_num_offset = 0, prev_frame_num = 0, prev_ref_frame_num = 0;
    bool prev_ref_mmco5 = false, prev_mmco5 = false;
    int prev_ref_bottom_field = 0, prev_ref_top_poc = 0;
    int max_long_term_frame_idx = kNoLongTerm;
    // current picture
    bool in_pic = false;
    bool cur_mbaff = false;  // MbaffFrameFlag of the current picture
    SliceHeader first_sh;  // first slice of the current picture
    Pic cur;
    int frame_num_offset = 0;
    int pending_msb = 0, pending_lsb = 0;
    std::vector<MbState> mbs;
    std::vector<h264r_mb> rec;
    std::vector<h264r_slice> rec_slices;
    std::vector<h264r_weight> rec_weights;
    std::vector<uint8_t> motion, coef, pcm;
    std::vector<uint32_t> dref_parts;  // motion offsets of the parts whose dref still holds a refIdx
    std::vector<std::shared_ptr<Motion>> motion_pool;  // co-located motion buffers, reused
    std::vector<Pic *> last_list[2];
    int num_slices = 0;
    uint32_t slice_errors = 0;  // slices skipped after a syntax error
    uint8_t first_slice_type = 0;
    // completed pictures waiting for h264r_parser_next
    struct Done {
        h264r_picture pic;
        std::vector<h264r_mb> mbs;
        std::vector<h264r_slice> slices;
        std::vector<h264r_weight> weights;
        std::vector<uint8_t> motion, coef, pcm;
        int32_t poc;
        uint32_t index;
        uint8_t idr, reference, slice_type;
        std::vector<uint8_t> out_slots;
        std::vector<int32_t> out_poc;
        std::vector<uint32_t> out_index;
    };
    std::deque<Done> done;
    Done current_out;  // storage behind the last h264r_parser_next result
    // slot -> (poc, index) of the picture it holds, for output reporting
    std::vector<int32_t> slot_poc;
    std::vector<uint32_t> slot_index;
    std::vector<uint8_t> rbsp;

    ~h264r_parser()
    {
        if (order) h264r_order_destroy(order);
    }

    int fail(int code, const char *fmt, ...)
    {
        char m[256];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(m, sizeof(m), fmt, ap);
        va_end(ap);
        err = m;
        failed = true;
        return code;
    }

    // ---- NAL units
    int process_nal(const uint8_t *p, size_t n);
    // a slice NAL unit up to its slice data: header, picture boundary,
    // slice record and reference lists; 1 with sc / br ready for
    // decode_slice, 0 for a slice that is not decoded, or an error code
    int begin_slice(const uint8_t *p, size_t n, SliceCtx &sc, BitReader &br);
    int start_picture(const SliceHeader &sh, const Sps &s, const Pps &q);
    int finish_picture(bool last);
    int decode_slice(SliceCtx &sc, BitReader &br);
    int decode_slice_cabac(SliceCtx &sc, BitReader &br);
    int decode_slice_mbaff(SliceCtx &sc, BitReader &br, bool cabac);
    int build_lists(SliceCtx &sc);
    void compute_poc(const SliceHeader &sh, const Sps &s);
    int mark_references(const SliceHeader &sh, const Sps &s);
    int alloc_slot();
};

namespace h264r {
namespace pimpl {

// ---------------------------------------------------------------- MB layer
// Macroblock-level decoding context: parses one MB, derives its prediction
// parameters and writes its record.
struct MbDecoder {
    h264r_parser &P;
    SliceCtx &sc;
    BitReader &br;
    const Sps &sps;
    const Pps &pps;
    int W, addr = 0, qp = 0;
    int mbx = 0;  // MB (pair, in MBAFF frames) column of addr, set with addr
    MbState *cur = nullptr;
    // MBAFF frames: MBs come in pairs (addr 2p top, 2p + 1 bottom) and a
    // pair is two frame MBs or two field MBs (mb_field_decoding_flag)
    bool mbaff = false;
    bool fld = false;   // the current MB is a field MB of an MBAFF frame
    bool bot = false;   // the current MB is the bottom MB of its pair
    bool decoded4x4[16];  // motion of this 4x4 block already derived
    Blk blk[16];          // motion of the current MB (raster)
    // per-MB scratch, reused across the slice's MBs
    std::vector<PartRec> parts;
    std::vector<uint16_t> sig;
    std::vector<int16_t> lv;
    // uid of the slice's list entry refIdx at [list][refIdx + 1] (-1 for
    // refIdx -1 and for missing entries)
    int32_t uid[2][33];

    MbDecoder(h264r_parser &p, SliceCtx &s, BitReader &b)
        : P(p), sc(s), br(b), sps(*s.sps), pps(*s.pps), W(p.width_mbs)
    {
        qp = pps.pic_init_qp + s.sh.slice_qp_delta;
        for (int l = 0; l < 2; l++)
            for (int i = 0; i < 33; i++)
                uid[l][i] = (i > 0 && i - 1 < (int)s.list[l].size() && s.list[l][i - 1]) ? s.list[l][i - 1]->uid : -1;
    }

    // the current MB: address, column, state; fld from the MB's state
    void set_mb(int a)
    {
        addr = a;
        mbx = mbaff ? (a >> 1) % W : a % W;
        cur = &P.mbs[a];
        bot = mbaff && (a & 1);
        fld = mbaff && cur->field;
    }

    // reference indices of the current MB: a field MB of an MBAFF frame
    // indexes the fields of the list's frames (8.4.2.1): refIdx >> 1 is the
    // frame, an even refIdx its field of the MB's parity, an odd one the other
    int ref_limit(int l) const { return fld ? 2 * sc.sh.num_ref_idx_active[l] : sc.sh.num_ref_idx_active[l]; }
    const Pic *ref_pic(int l, int ref) const
    {
        const int i = fld ? ref >> 1 : ref;
        return i >= 0 && i < (int)sc.list[l].size() ? sc.list[l][i] : nullptr;
    }
    bool ref_bottom(int ref) const { return (ref & 1) ? !bot : bot; }
    // PicOrderCnt of what refIdx names, and of the current picture or field
    int ref_poc(int l, int ref) const
    {
        const Pic *p = ref_pic(l, ref);
        return !fld ? p->poc : (ref_bottom(ref) ? p->bottom_poc : p->top_poc);
    }
    int cur_poc() const { return !fld ? P.cur.poc : (bot ? P.cur.bottom_poc : P.cur.top_poc); }

    // decoded MB of this slice (or the current MB itself)
    bool usable(int n) const { return n >= 0 && (n == addr || P.mbs[n].slice == sc.index); }

    // 6.4.12.2 (Table 6-4): the MB of an MBAFF frame holding luma or chroma
    // location (xN, yN) relative to the current MB, or -1; (xW, yW) inside it
    int nb_mb_mbaff(int xN, int yN, int maxW, int maxH, int &xW, int &yW) const
    {
        const int pair = addr >> 1, px = pair % W;
        auto pr = [&](int q, bool ok) { return ok && q >= 0 && usable(2 * q) ? 2 * q : -1; };
        const int A = pr(pair - 1, px > 0), B = pr(pair - W, true), C = pr(pair - W + 1, px + 1 < W),
                  D = pr(pair - W - 1, px > 0);
        auto frm = [&](int n) { return !P.mbs[n].field; };
        const bool frame = !fld, top = !bot;
        int n = -1, yM = 0;
        if (xN < 0 && yN < 0) {
            if (frame) {
                if (top) { if (D >= 0) { n = D + 1; yM = yN; } }
                else if (A >= 0) {
                    if (frm(A)) { n = A; yM = yN; } else { n = A + 1; yM = (yN + maxH) >> 1; }
                }
            } else {
                if (top) {
                    if (D >= 0) { if (frm(D)) { n = D + 1; yM = 2 * yN; } else { n = D; yM = yN; } }
                } else if (D >= 0) { n = D + 1; yM = yN; }
            }
        } else if (xN < 0 && yN < maxH) {
            if (A >= 0) {
                if (frame) {
                    if (top) {
                        if (frm(A)) { n = A; yM = yN; } else { n = (yN % 2 == 0) ? A : A + 1; yM = yN >> 1; }
                    } else {
                        if (frm(A)) { n = A + 1; yM = yN; } else { n = (yN % 2 == 0) ? A : A + 1; yM = (yN + maxH) >> 1; }
                    }
                } else {
                    if (top) {
                        if (frm(A)) {
                            if (yN < maxH / 2) { n = A; yM = yN << 1; } else { n = A + 1; yM = (yN << 1) - maxH; }
                        } else { n = A; yM = yN; }
                    } else {
                        if (frm(A)) {
                            if (yN < maxH / 2) { n = A; yM = (yN << 1) + 1; } else { n = A + 1; yM = (yN << 1) + 1 - maxH; }
                        } else { n = A + 1; yM = yN; }
                    }
                }
            }
        } else if (xN < maxW && yN < 0) {
            if (frame) {
                if (top) { if (B >= 0) { n = B + 1; yM = yN; } }
                else { n = addr - 1; yM = yN; }
            } else {
                if (top) {
                    if (B >= 0) { if (frm(B)) { n = B + 1; yM = 2 * yN; } else { n = B; yM = yN; } }
                } else if (B >= 0) { n = B + 1; yM = yN; }
            }
        } else if (xN < maxW && yN < maxH) {
            n = addr; yM = yN;
        } else if (xN >= maxW && yN < 0) {
            if (frame) {
                if (top) { if (C >= 0) { n = C + 1; yM = yN; } }
            } else {
                if (top) {
                    if (C >= 0) { if (frm(C)) { n = C + 1; yM = 2 * yN; } else { n = C; yM = yN; } }
                } else if (C >= 0) { n = C + 1; yM = yN; }
            }
        }
        if (n < 0) return -1;
        xW = (xN + maxW) & (maxW - 1);
        yW = (yM + maxH) & (maxH - 1);
        return n;
    }

    // ---- neighbours (6.4.12.1): the MB holding luma location (xN, yN)
    // relative to the current MB, or -1; (xW, yW) inside it
    int nb_mb(int xN, int yN, int maxW, int maxH, int &xW, int &yW) const
    {
        if (mbaff) return nb_mb_mbaff(xN, yN, maxW, maxH, xW, yW);
        int n;
        const int x = mbx;
        if (xN < 0 && yN < 0) n = x > 0 ? addr - W - 1 : -1;
        else if (xN < 0 && yN < maxH) n = x > 0 ? addr - 1 : -1;
        else if (xN < maxW && yN < 0) n = addr - W;
        else if (xN < maxW && yN < maxH) n = addr;
        else if (xN >= maxW && yN < 0) n = x + 1 < W ? addr - W + 1 : -1;
        else return -1;
        if (n < 0) return -1;
        if (n != addr && P.mbs[n].slice != sc.index) return -1;  // not yet decoded or another slice
        xW = (xN + maxW) & (maxW - 1);  // maxW, maxH: 16 or 8
        yW = (yN + maxH) & (maxH - 1);
        return n;
    }

    // ---- intra prediction modes (8.3.1.1 Intra4x4PredMode, 8.3.2.1 Intra8x8PredMode;
    // CH264PictureBase::getIntra4x4PredMode / getIntra8x8PredMode, H264PictureBase.cpp:773-1058)
    int pred_mode_nb(int xN, int yN, bool for8x8, bool isA, int &dcflag) const
    {
        int xW = 0, yW = 0;
        const int n = nb_mb(xN, yN, 16, 16, xW, yW);
        if (n < 0) {
            dcflag = 1;
            return 2;
        }
        const MbState &m = P.mbs[n];
        if (!m.intra() && pps.constrained_intra_pred) dcflag = 1;
        if (m.cls == H264R_MB_I4x4) {
            const int b = blk_of(xW >> 2, yW >> 2);
            if (!for8x8) return m.ipm4[b];
            // 8x8 block of the neighbour, n = 1 for A, 2 for B
            return m.ipm4[(b >> 2) * 4 + (isA ? 1 : 2)];
        }
        if (m.cls == H264R_MB_I8x8) return m.ipm8[blk_of(xW >> 2, yW >> 2) >> 2];
        return 2;
    }

    int derive_mode(int x, int y, bool for8x8, int prev_flag, int rem) const
    {
        int dc = 0;
        int a = pred_mode_nb(x - 1, y, for8x8, true, dc);
        int b = pred_mode_nb(x, y - 1, for8x8, false, dc);
        if (dc) a = b = 2;
        const int pred = std::min(a, b);
        if (prev_flag) return pred;
        return rem < pred ? rem : rem + 1;
    }

    // ---- CAVLC nC (9.2.1)
    int total_of(int n, bool chroma, int comp, int b) const
    {
        const MbState &m = P.mbs[n];
        if (m.skip) return 0;
        // 9.2.1 gives an I_PCM neighbour nN = 16; the reference compares the
        // MB's type number (25) with its enum value of I_PCM (26,
        // H264ResidualBlockCavlc.cpp:497 / 532, H264CommonFunc.h:183-210), so
        // the test never holds and it reads the PCM MB's non-zero counts,
        // which it leaves at zero: an I_PCM neighbour counts as 0 here too
        return chroma ? m.tcc[comp][b] : m.tc[b];
    }

    int nc_luma(int b) const
    {
        const int x = kBlkX[b] * 4, y = kBlkY[b] * 4;
        int xW = 0, yW = 0;
        const int na = nb_mb(x - 1, y, 16, 16, xW, yW);
        const int nA = na >= 0 ? total_of(na, false, 0, blk_of(xW >> 2, yW >> 2)) : 0;
        const int nbm = nb_mb(x, y - 1, 16, 16, xW, yW);
        const int nB = nbm >= 0 ? total_of(nbm, false, 0, blk_of(xW >> 2, yW >> 2)) : 0;
        if (na >= 0 && nbm >= 0) return (nA + nB + 1) >> 1;
        return na >= 0 ? nA : (nbm >= 0 ? nB : 0);
    }

    int nc_chroma(int comp, int b) const
    {
        const int x = (b & 1) * 4, y = (b >> 1) * 4;
        int xW = 0, yW = 0;
        const int na = nb_mb(x - 1, y, 8, 8, xW, yW);
        const int nA = na >= 0 ? total_of(na, true, comp, (yW >> 2) * 2 + (xW >> 2)) : 0;
        const int nbm = nb_mb(x, y - 1, 8, 8, xW, yW);
        const int nB = nbm >= 0 ? total_of(nbm, true, comp, (yW >> 2) * 2 + (xW >> 2)) : 0;
        if (na >= 0 && nbm >= 0) return (nA + nB + 1) >> 1;
        return na >= 0 ? nA : (nbm >= 0 ? nB : 0);
    }

    // ---- motion neighbours (6.4.11.7, 8.4.1.3.2)
    struct Nb {
        bool avail;
        int ref;
        int mv[2];
    };

    Nb nb_motion(int xN, int yN, int list) const
    {
        Nb r = {false, -1, {0, 0}};
        int xW = 0, yW = 0;
        const int n = nb_mb(xN, yN, 16, 16, xW, yW);
        if (n < 0) return r;
        const int bi = (yW >> 2) * 4 + (xW >> 2);
        if (n == addr) {
            // 6.4.11.7 marks a partition of the current MB that is not yet
            // decoded as not available (C is then replaced by D); the
            // reference leaves that rule out (commented out at
            // H264InterPrediction.cpp:3158-3165) and reads the partition's
            // motion as stored so far: the MB record is cleared per picture
            // and a partition's prediction flags and vectors are written only
            // once it is derived (H264InterPrediction.cpp:592-603), so such a
            // C neighbour is available with no prediction from this list.  It
            // happens for sub-macroblock partitions whose top-right
            // neighbour lies in the next 8x8 quadrant (8x4 / 4x4 partitions
            // in the lower half of quadrants 0 and 2).
            r.avail = true;
            if (!decoded4x4[bi]) return r;
            r.ref = blk[bi].ref[list];
            if (r.ref >= 0) {
                r.mv[0] = blk[bi].mv[list][0];
                r.mv[1] = blk[bi].mv[list][1];
            }
            return r;
        }
        const MbState &m = P.mbs[n];
        r.avail = true;
        if (m.intra()) return r;
        r.ref = m.ref[list][bi];
        if (r.ref >= 0) {
            r.mv[0] = m.mv[list][bi][0];
            r.mv[1] = m.mv[list][bi][1];
            // 8.4.1.3.2: a neighbour of the other kind (frame / field MB of
            // an MBAFF frame) in the current MB's units; '/' truncates
            if (fld && !m.field) {
                r.mv[1] = r.mv[1] / 2;
                r.ref *= 2;
            } else if (!fld && m.field && mbaff) {
                r.mv[1] *= 2;
                r.ref /= 2;
            }
        }
        return r;
    }

    // 8.4.1.3: mvpLX of the partition at (x, y) of width w; shape: 0
    // 16x16 / other, 1 16x8, 2 8x16 (directional rules), part: mbPartIdx
    void mvp(int x, int y, int w, int shape, int part, int list, int ref, int out[2]) const
    {
        Nb A = nb_motion(x - 1, y, list), B = nb_motion(x, y - 1, list), C = nb_motion(x + w, y - 1, list);
        if (!C.avail) C = nb_motion(x - 1, y - 1, list);
        if (shape == 1) {
            if (part == 0 && B.ref == ref) { out[0] = B.mv[0]; out[1] = B.mv[1]; return; }
            if (part == 1 && A.ref == ref) { out[0] = A.mv[0]; out[1] = A.mv[1]; return; }
        } else if (shape == 2) {
            if (part == 0 && A.ref == ref) { out[0] = A.mv[0]; out[1] = A.mv[1]; return; }
            if (part == 1 && C.ref == ref) { out[0] = C.mv[0]; out[1] = C.mv[1]; return; }
        }
        if (!B.avail && !C.avail && A.avail) B = C = A;
        const int match = (A.ref == ref) + (B.ref == ref) + (C.ref == ref);
        if (match == 1) {
            const Nb &s = A.ref == ref ? A : (B.ref == ref ? B : C);
            out[0] = s.mv[0];
            out[1] = s.mv[1];
            return;
        }
        out[0] = median3(A.mv[0], B.mv[0], C.mv[0]);
        out[1] = median3(A.mv[1], B.mv[1], C.mv[1]);
    }

    void set_blocks(int x, int y, int w, int h, const Blk &b)
    {
        for (int j = y >> 2; j < (y + h) >> 2; j++)
            for (int i = x >> 2; i < (x + w) >> 2; i++) {
                blk[j * 4 + i] = b;
                decoded4x4[j * 4 + i] = true;
            }
    }

    // ---- direct prediction (8.4.1.2)
    struct Col {
        int mv[2];
        int ref;      // refIdxCol, -1 for intra
        int refpic;   // uid of the picture it refers to
    };

    Col colocated(int bi) const
    {
        Col c = {{0, 0}, -1, -1};
        const Pic *col = sc.list[1].empty() ? nullptr : sc.list[1][0];
        if (!col || !col->motion) return c;
        const Motion &m = *col->motion;
        int mb = addr;
        if (mbaff && !m.field.empty()) {
            // Table 8-8 for an MBAFF frame and an MBAFF co-located frame
            // (H264InterPrediction.cpp:1173-1215): the co-located pair's kind
            // picks the MB and the row yM of the co-located block
            const int xCol = (bi & 3) * 4, yCol = (bi >> 2) * 4;
            int yM = yCol;
            const bool col_field = m.field[addr] != 0;
            if (!fld && col_field) {
                const int top = std::abs(col->top_poc - P.cur.poc), bottom = std::abs(col->bottom_poc - P.cur.poc);
                mb = 2 * (addr / 2) + (top < bottom ? 0 : 1);
                yM = 8 * (addr % 2) + 4 * (yCol / 8);
            } else if (fld && !col_field) {
                mb = 2 * (addr / 2) + yCol / 8;
                yM = (2 * yCol) % 16;
            }
            bi = (yM >> 2) * 4 + (xCol >> 2);
        }
        if (m.intra[mb] == 2 && sc.sh.direct_spatial) {
            // an I_PCM co-located MB: the reference's intra test does not
            // cover I_PCM (prediction mode Intra_NA), so it reads the MB's
            // cleared motion as list 1, refIdxCol 0 and mvCol (0, 0)
            // (H264InterPrediction.cpp:1230-1253), which sets colZeroFlag
            c.ref = 0;
            return c;
        }
        if (m.intra[mb]) return c;
        int l = 0;
        if (m.ref[(mb * 2 + 0) * 16 + bi] < 0) l = 1;
        const size_t o = (size_t)(mb * 2 + l) * 16 + bi;
        c.ref = m.ref[o];
        c.mv[0] = m.mv[o * 2];
        c.mv[1] = m.mv[o * 2 + 1];
        c.refpic = m.refpic[o];
        return c;
    }

    // spatial direct: MB-level reference indices and predictors (8.4.1.2.2)
    bool spatial_ready = false;
    int sp_ref[2];
    int sp_mv[2][2];
    bool sp_zero = false;

    void spatial_setup()
    {
        if (spatial_ready) return;
        spatial_ready = true;
        for (int l = 0; l < 2; l++) {
            Nb A = nb_motion(-1, 0, l), B = nb_motion(0, -1, l), C = nb_motion(16, -1, l);
            if (!C.avail) C = nb_motion(-1, -1, l);
            auto minpos = [](int a, int b) { return (a >= 0 && b >= 0) ? std::min(a, b) : std::max(a, b); };
            sp_ref[l] = minpos(A.ref, minpos(B.ref, C.ref));
        }
        sp_zero = sp_ref[0] < 0 && sp_ref[1] < 0;
        if (sp_zero) sp_ref[0] = sp_ref[1] = 0;
        for (int l = 0; l < 2; l++) {
            sp_mv[l][0] = sp_mv[l][1] = 0;
            if (sp_ref[l] >= 0 && !sp_zero) mvp(0, 0, 16, 0, 0, l, sp_ref[l], sp_mv[l]);
        }
    }

    // direct motion of the 4x4 block (bx, by) (raster units)
    int direct_block(int bx, int by, Blk &b)
    {
        const int q = (by >> 1) * 2 + (bx >> 1);
        const int cbx = sps.direct_8x8_inference ? ((q & 1) ? 3 : 0) : bx;
        const int cby = sps.direct_8x8_inference ? ((q & 2) ? 3 : 0) : by;
        const Col c = colocated(cby * 4 + cbx);
        if (sc.sh.direct_spatial) {
            spatial_setup();
            const Pic *l1 = sc.list[1][0];
            const bool colzero = l1 && l1->short_ref && c.ref == 0 && c.mv[0] >= -1 && c.mv[0] <= 1 && c.mv[1] >= -1 &&
                                 c.mv[1] <= 1;
            for (int l = 0; l < 2; l++) {
                b.ref[l] = (int8_t)sp_ref[l];
                if (sp_ref[l] < 0 || sp_zero || (sp_ref[l] == 0 && colzero)) {
                    b.mv[l][0] = b.mv[l][1] = 0;
                } else {
                    b.mv[l][0] = (int16_t)sp_mv[l][0];
                    b.mv[l][1] = (int16_t)sp_mv[l][1];
                }
            }
            return 0;
        }
        // temporal (8.4.1.2.3)
        int r0 = 0;
        if (c.ref >= 0) {
            r0 = -1;
            for (size_t i = 0; i < sc.list[0].size(); i++)
                if (sc.list[0][i] && sc.list[0][i]->uid == c.refpic) {
                    r0 = (int)i;
                    break;
                }
            if (r0 < 0) return P.fail(H264R_ERR_BAD_RECORD, "temporal direct: co-located reference not in RefPicList0 (MB %d)", addr);
        }
        const Pic *p0 = sc.list[0][r0], *p1 = sc.list[1][0];
        b.ref[0] = (int8_t)r0;
        b.ref[1] = 0;
        const int td = clip3(-128, 127, p1->poc - p0->poc);
        if (p0->long_ref || td == 0) {
            b.mv[0][0] = (int16_t)c.mv[0];
            b.mv[0][1] = (int16_t)c.mv[1];
            b.mv[1][0] = b.mv[1][1] = 0;
        } else {
            const int tb = clip3(-128, 127, P.cur.poc - p0->poc);
            const int tx = (16384 + std::abs(td / 2)) / td;
            const int dsf = clip3(-1024, 1023, (tb * tx + 32) >> 6);
            for (int k = 0; k < 2; k++) {
                b.mv[0][k] = (int16_t)((dsf * c.mv[k] + 128) >> 8);
                b.mv[1][k] = (int16_t)(b.mv[0][k] - c.mv[k]);
            }
        }
        return 0;
    }

    // ---- prediction weights (8.4.2.3), as the record's weight entry
    uint16_t weight_index(int ref0, int ref1)
    {
        const int st = sc.sh.slice_type;
        const bool pf0 = ref0 >= 0, pf1 = ref1 >= 0;
        h264r_weight w;
        memset(&w, 0, sizeof(w));
        bool weighted = false;
        if ((st == kSliceP || st == kSliceSP) && pps.weighted_pred && pf0) {
            weighted = true;
            const PredWeights &pw = sc.sh.pw;
            const int i0 = fld ? ref0 >> 1 : ref0;  // refIdxL0WP
            w.log_wd[0] = (int8_t)pw.luma_log2;
            w.log_wd[1] = w.log_wd[2] = (int8_t)pw.chroma_log2;
            w.w0[0] = (int16_t)pw.lw[0][i0];
            w.o0[0] = (int16_t)pw.lo[0][i0];
            for (int c = 0; c < 2; c++) {
                w.w0[1 + c] = (int16_t)pw.cw[0][i0][c];
                w.o0[1 + c] = (int16_t)pw.co[0][i0][c];
            }
        } else if (st == kSliceB && pps.weighted_bipred_idc == 1 && (pf0 || pf1)) {
            weighted = true;
            const PredWeights &pw = sc.sh.pw;
            w.log_wd[0] = (int8_t)pw.luma_log2;
            w.log_wd[1] = w.log_wd[2] = (int8_t)pw.chroma_log2;
            const int i0 = fld ? ref0 >> 1 : ref0, i1 = fld ? ref1 >> 1 : ref1;  // refIdxLXWP
            if (pf0) {
                w.w0[0] = (int16_t)pw.lw[0][i0];
                w.o0[0] = (int16_t)pw.lo[0][i0];
                for (int c = 0; c < 2; c++) {
                    w.w0[1 + c] = (int16_t)pw.cw[0][i0][c];
                    w.o0[1 + c] = (int16_t)pw.co[0][i0][c];
                }
            }
            if (pf1) {
                w.w1[0] = (int16_t)pw.lw[1][i1];
                w.o1[0] = (int16_t)pw.lo[1][i1];
                for (int c = 0; c < 2; c++) {
                    w.w1[1 + c] = (int16_t)pw.cw[1][i1][c];
                    w.o1[1 + c] = (int16_t)pw.co[1][i1][c];
                }
            }
        } else if (st == kSliceB && pps.weighted_bipred_idc == 2 && pf0 && pf1) {
            weighted = true;
            // field MBs of MBAFF frames: the POCs of the fields (8.4.2.3.1)
            const Pic *p0 = ref_pic(0, ref0), *p1 = ref_pic(1, ref1);
            int w0 = 32, w1 = 32;
            const int poc0 = ref_poc(0, ref0), poc1 = ref_poc(1, ref1);
            const int td = clip3(-128, 127, poc1 - poc0);
            if (td != 0 && !p0->long_ref && !p1->long_ref) {
                const int tb = clip3(-128, 127, cur_poc() - poc0);
                const int tx = (16384 + std::abs(td / 2)) / td;
                const int dsf = clip3(-1024, 1023, (tb * tx + 32) >> 6);
                if (!((dsf >> 2) < -64 || (dsf >> 2) > 128)) {
                    w0 = 64 - (dsf >> 2);
                    w1 = dsf >> 2;
                }
            }
            for (int c = 0; c < 3; c++) {
                w.log_wd[c] = 5;
                w.w0[c] = (int16_t)w0;
                w.w1[c] = (int16_t)w1;
            }
        }
        if (!weighted) return 0;
        w.weighted = 1;
        std::vector<h264r_weight> &t = P.rec_weights;
        for (size_t i = 0; i < t.size(); i++)
            if (memcmp(&t[i], &w, sizeof(w)) == 0) return (uint16_t)i;
        t.push_back(w);
        return (uint16_t)(t.size() - 1);
    }

    // ---- CABAC slice data (cab != nullptr): the syntax of the current MB
    // that the CABAC contexts of its later partitions and blocks read
    Cabac *cab = nullptr;
    int16_t mvd_cur[2][16][2];
    uint8_t predl_cur[16];
    int8_t refsyn_cur[2][16];
    bool prev_qp_nz = false;  // the previous MB of the slice had mb_qp_delta != 0

    int decode();
    int decode_cabac();
    int residual(int cls, int cbp, bool t8, uint32_t &mask, std::vector<uint16_t> &sig, std::vector<int16_t> &lv, h264r_mb &r);
    int inter_pred(int mb_type, bool is_b, h264r_mb &r, bool &no_sub_lt8);
    void emit_motion(int shape, const std::vector<PartRec> &parts, h264r_mb &r);
    void store_motion();
};

// P_Skip / B_Skip (8.4.1.1, 8.4.1.2): motion only, QPY unchanged
int decode_skip(MbDecoder &d, h264r_mb &r);
// ctxIdxInc of mb_skip_flag (9.3.3.1.1.1)
int cabac_skip_inc(MbDecoder &d);
// ctxIdxInc of mb_field_decoding_flag (9.3.3.1.1.2): field pairs left / above
int cabac_field_inc(MbDecoder &d);

}  // namespace pimpl
}  // namespace h264r
