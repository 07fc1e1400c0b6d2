// h264r_cabac.cpp — CABAC slice data for the host front end (9.3): the
// arithmetic decoding engine, context initialisation, the binarisations and
// context index derivations of every syntax element of 4:2:0 frame
// macroblocks, and the macroblock layer read through them.  The derivations
// (prediction, records) are the CAVLC path's own (h264r_parser.cpp); only the
// reading of the syntax differs.  The reference decoder's counterpart is
// CH264Cabac (H264Cabac.cpp) with its callers in CH264MacroBlock
// (H264MacroBlock.cpp) and CH264SliceData::slice_data (H264SliceData.cpp).
#include "h264r_parser_impl.h"

namespace h264r {
namespace pimpl {

namespace {

#include "h264r_cabac_init.inc"

// Table 9-44 rangeTabLPS [pStateIdx][qCodIRangeIdx]
const uint8_t kRangeLPS[64][4] = {
    {128, 176, 208, 240}, {128, 167, 197, 227}, {128, 158, 187, 216}, {123, 150, 178, 205}, {116, 142, 169, 195},
    {111, 135, 160, 185}, {105, 128, 152, 175}, {100, 122, 144, 166}, {95, 116, 137, 158},  {90, 110, 130, 150},
    {85, 104, 123, 142},  {81, 99, 117, 135},   {77, 94, 111, 128},   {73, 89, 105, 122},   {69, 85, 100, 116},
    {66, 80, 95, 110},    {62, 76, 90, 104},    {59, 72, 86, 99},     {56, 69, 81, 94},     {53, 65, 77, 89},
    {51, 62, 73, 85},     {48, 59, 69, 80},     {46, 56, 66, 76},     {43, 53, 63, 72},     {41, 50, 59, 69},
    {39, 48, 56, 65},     {37, 45, 54, 62},     {35, 43, 51, 59},     {33, 41, 48, 56},     {32, 39, 46, 53},
    {30, 37, 43, 50},     {29, 35, 41, 48},     {27, 33, 39, 45},     {26, 31, 37, 43},     {24, 30, 35, 41},
    {23, 28, 33, 39},     {22, 27, 32, 37},     {21, 26, 30, 35},     {20, 24, 29, 33},     {19, 23, 27, 31},
    {18, 22, 26, 30},     {17, 21, 25, 28},     {16, 20, 23, 27},     {15, 19, 22, 25},     {14, 18, 21, 24},
    {14, 17, 20, 23},     {13, 16, 19, 22},     {12, 15, 18, 21},     {12, 14, 17, 20},     {11, 14, 16, 19},
    {11, 13, 15, 18},     {10, 12, 15, 17},     {10, 12, 14, 16},     {9, 11, 13, 15},      {9, 11, 12, 14},
    {8, 10, 12, 14},      {8, 9, 11, 13},       {7, 9, 11, 12},       {7, 9, 10, 12},       {7, 8, 10, 11},
    {6, 8, 9, 11},        {6, 7, 9, 10},        {6, 7, 8, 9},         {2, 2, 2, 2},
};

// Table 9-45 transIdxLPS (transIdxMPS is min(pStateIdx + 1, 62), 63 stays)
const uint8_t kTransLPS[64] = {0,  0,  1,  2,  2,  4,  4,  5,  6,  7,  8,  9,  9,  11, 11, 12, 13, 13, 15, 15, 16, 16,
                               18, 18, 19, 19, 21, 21, 22, 22, 23, 24, 24, 25, 26, 26, 27, 27, 28, 29, 29, 30, 30, 30,
                               31, 32, 32, 33, 33, 33, 34, 34, 35, 35, 35, 36, 36, 36, 37, 37, 37, 38, 38, 63};

// Table 9-43: ctxIdxInc of significant_coeff_flag (frame coded) and of
// last_significant_coeff_flag for 8x8 blocks, by levelListIdx
const uint8_t kSig8x8Frame[63] = {0,  1,  2,  3,  4,  5,  5,  4,  4,  3,  3,  4,  4,  4,  5,  5,  4,  4,  4,  4,  3,
                                  3,  6,  7,  7,  7,  8,  9,  10, 9,  8,  7,  7,  6,  11, 12, 13, 11, 6,  7,  8,  9,
                                  14, 10, 9,  8,  6,  11, 12, 13, 11, 6,  9,  14, 10, 9,  11, 12, 13, 11, 14, 10, 12};
// ... and of significant_coeff_flag of field coded 8x8 blocks (field MBs of
// MBAFF frames), by levelListIdx
const uint8_t kSig8x8Field[63] = {0,  1,  1,  2,  2,  3,  3,  4,  5,  6,  7,  7,  7,  8,  4,  5,  6,  9,  10, 10, 8,
                                  11, 12, 11, 9,  9,  10, 10, 8,  11, 12, 11, 9,  9,  10, 10, 8,  11, 12, 11, 9,  9,
                                  10, 10, 8,  13, 13, 9,  9,  10, 10, 8,  13, 13, 9,  9,  10, 10, 14, 14, 14, 14, 14};
const uint8_t kLast8x8[63] = {0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2,
                              3, 3, 3, 3, 3, 3, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 5, 5, 5, 5, 6, 6, 6, 6, 7, 7, 7, 7, 8, 8, 8};

// ctxIdxBlockCatOffset (Table 9-40) of ctxBlockCat 0..4: coded_block_flag,
// significant / last_significant_coeff_flag, coeff_abs_level_minus1
const uint8_t kCbfCatOff[5] = {0, 4, 8, 12, 16};
const uint8_t kSigCatOff[5] = {0, 15, 29, 44, 47};
const uint8_t kAbsCatOff[5] = {0, 10, 20, 30, 39};

}  // namespace

void Cabac::init_contexts(int slice_type, int cabac_init_idc, int qp)
{
    const int model = slice_type == kSliceI ? 0 : 1 + cabac_init_idc;
    const int q = clip3(0, 51, qp);
    for (int i = 0; i < 460; i++) {
        const int m = kCabacInit[model][i][0], n = kCabacInit[model][i][1];
        const int pre = clip3(1, 126, ((m * q) >> 4) + n);
        if (pre <= 63) {
            state[i] = (uint8_t)(63 - pre);
            mps[i] = 0;
        } else {
            state[i] = (uint8_t)(pre - 64);
            mps[i] = 1;
        }
    }
}

int Cabac::decision(int ctx)
{
    const uint32_t lps = kRangeLPS[state[ctx]][(range >> 6) & 3];
    range -= lps;
    int bin;
    if (offset >= range) {
        bin = !mps[ctx];
        offset -= range;
        range = lps;
        if (state[ctx] == 0) mps[ctx] ^= 1;
        state[ctx] = kTransLPS[state[ctx]];
    } else {
        bin = mps[ctx];
        if (state[ctx] < 62) state[ctx]++;
    }
    while (range < 256) {
        range <<= 1;
        offset = (offset << 1) | br->u(1);
    }
    return bin;
}

namespace {

// ---------------------------------------------------------------- helpers
// the MB holding luma location (xN, yN) of the current MB, or -1
int nbmb(const MbDecoder &d, int xN, int yN, int &xW, int &yW) { return d.nb_mb(xN, yN, 16, 16, xW, yW); }


// mb_type of an intra MB (Table 9-36): I slices with the prefix context of
// 9.3.3.1.1.3 (offset 3), or the suffix of a P / B mb_type (offset 17 / 32).
// Returns the I mb_type 0..25.
int mb_type_i(MbDecoder &d, int off, bool in_i_slice)
{
    Cabac &c = *d.cab;
    int b0;
    if (in_i_slice) {
        int xW, yW;
        const int a = nbmb(d, -1, 0, xW, yW), b = nbmb(d, 0, -1, xW, yW);
        auto cond = [&](int n) {
            if (n < 0) return 0;
            const MbState &m = d.P.mbs[n];
            return (m.cls == H264R_MB_I4x4 || m.cls == H264R_MB_I8x8) ? 0 : 1;
        };
        b0 = c.decision(off + cond(a) + cond(b));
    } else {
        b0 = c.decision(off);
    }
    if (!b0) return 0;  // I_NxN
    if (c.terminate()) return 25;  // I_PCM
    const int luma = c.decision(off + (in_i_slice ? 3 : 1));
    const int ch1 = c.decision(off + (in_i_slice ? 4 : 2));
    int chroma = 0;
    if (ch1) chroma = c.decision(off + (in_i_slice ? 5 : 2)) ? 2 : 1;
    const int m1 = c.decision(off + (in_i_slice ? 6 : 3));
    const int m0 = c.decision(off + (in_i_slice ? 7 : 3));
    return 1 + (m1 * 2 + m0) + 4 * chroma + 12 * luma;
}

// mb_type of a B slice (Table 9-37); 23 + I type for intra MBs
int mb_type_b(MbDecoder &d)
{
    Cabac &c = *d.cab;
    int xW, yW;
    const int a = nbmb(d, -1, 0, xW, yW), b = nbmb(d, 0, -1, xW, yW);
    auto cond = [&](int n) { return n >= 0 && !d.P.mbs[n].skip && !d.P.mbs[n].direct16 ? 1 : 0; };
    if (!c.decision(27 + cond(a) + cond(b))) return 0;  // B_Direct_16x16
    if (!c.decision(30)) return 1 + c.decision(32);  // B_L0_16x16, B_L1_16x16
    int bits = c.decision(31) << 3;
    bits |= c.decision(32) << 2;
    bits |= c.decision(32) << 1;
    bits |= c.decision(32);
    if (bits < 8) return bits + 3;
    if (bits == 13) return 23 + mb_type_i(d, 32, false);
    if (bits == 14) return 11;  // B_L1_L0_8x16
    if (bits == 15) return 22;  // B_8x8
    bits = (bits << 1) | c.decision(32);
    return bits - 4;
}

// mb_type of a P slice; 5 + I type for intra MBs
int mb_type_p(MbDecoder &d)
{
    Cabac &c = *d.cab;
    if (c.decision(14)) return 5 + mb_type_i(d, 17, false);
    if (!c.decision(15)) return c.decision(16) ? 3 : 0;  // P_8x8 / P_L0_16x16
    return c.decision(17) ? 1 : 2;                       // 16x8 / 8x16
}

// mb_qp_delta (9.3.3.1.1.5, U binarisation of the mapped value)
int qp_delta(MbDecoder &d)
{
    Cabac &c = *d.cab;
    if (!c.decision(60 + (d.prev_qp_nz ? 1 : 0))) return 0;
    int k = 1;
    int ctx = 62;
    while (k < 104 && c.decision(ctx)) {
        ctx = 63;
        k++;
    }
    return (k & 1) ? (k + 1) / 2 : -(k / 2);
}

// intra_chroma_pred_mode (9.3.3.1.1.8, TU cMax 3)
int chroma_pred(MbDecoder &d)
{
    Cabac &c = *d.cab;
    int xW, yW;
    const int a = nbmb(d, -1, 0, xW, yW), b = nbmb(d, 0, -1, xW, yW);
    auto cond = [&](int n) {
        if (n < 0) return 0;
        const MbState &m = d.P.mbs[n];
        return (m.intra() && m.cls != H264R_MB_IPCM && m.chroma_mode != 0) ? 1 : 0;
    };
    if (!c.decision(64 + cond(a) + cond(b))) return 0;
    if (!c.decision(67)) return 1;
    return c.decision(67) ? 3 : 2;
}

// coded_block_pattern (9.3.3.1.1.4): four luma bins (FL), chroma TU cMax 2
int cbp(MbDecoder &d)
{
    Cabac &c = *d.cab;
    int luma = 0;
    for (int b8 = 0; b8 < 4; b8++) {
        const int x = (b8 & 1) * 8, y = (b8 >> 1) * 8;
        int cond[2];
        for (int k = 0; k < 2; k++) {
            const int xN = k ? x : x - 1, yN = k ? y - 1 : y;
            int xW = 0, yW = 0;
            const int n = nbmb(d, xN, yN, xW, yW);
            const int b8n = ((yW >> 3) << 1) | (xW >> 3);
            if (n < 0) {
                cond[k] = 0;
            } else if (n == d.addr) {
                cond[k] = ((luma >> b8n) & 1) ? 0 : 1;
            } else {
                const MbState &m = d.P.mbs[n];
                if (m.cls == H264R_MB_IPCM) cond[k] = 0;
                else if (!m.skip && ((m.cbp >> b8n) & 1)) cond[k] = 0;
                else cond[k] = 1;
            }
        }
        luma |= c.decision(73 + cond[0] + 2 * cond[1]) << b8;
    }
    int xW, yW;
    const int a = nbmb(d, -1, 0, xW, yW), b = nbmb(d, 0, -1, xW, yW);
    auto cc = [&](int n, int bin) {
        if (n < 0) return 0;
        const MbState &m = d.P.mbs[n];
        if (m.cls == H264R_MB_IPCM) return 1;
        if (m.skip) return 0;
        const int ch = m.cbp >> 4;
        return bin == 0 ? (ch != 0 ? 1 : 0) : (ch == 2 ? 1 : 0);
    };
    int chroma = 0;
    if (c.decision(77 + cc(a, 0) + 2 * cc(b, 0))) chroma = c.decision(77 + 4 + cc(a, 1) + 2 * cc(b, 1)) ? 2 : 1;
    return luma | (chroma << 4);
}

// transform_size_8x8_flag (9.3.3.1.1.10)
int t8_flag(MbDecoder &d)
{
    int xW, yW;
    const int a = nbmb(d, -1, 0, xW, yW), b = nbmb(d, 0, -1, xW, yW);
    const int inc = (a >= 0 && d.P.mbs[a].t8) + (b >= 0 && d.P.mbs[b].t8);
    return d.cab->decision(399 + inc);
}

// coded_block_flag context (9.3.3.1.1.9) of a block of ctxBlockCat cat:
// blk is the luma4x4BlkIdx (cat 1, 2) or chroma4x4BlkIdx (cat 4); comp 0
// luma, 1 Cb, 2 Cr
int cbf_inc(MbDecoder &d, int cat, int blk, int comp)
{
    const MbState &cur = *d.cur;
    const bool intra = cur.intra();
    int cond[2];
    for (int k = 0; k < 2; k++) {
        int xN, yN, maxW = 16, maxH = 16;
        if (cat == 0 || cat == 3) {
            xN = k ? 0 : -1;
            yN = k ? -1 : 0;
            if (cat == 3) maxW = maxH = 8;
        } else if (cat == 4) {
            maxW = maxH = 8;
            const int x = (blk & 1) * 4, y = (blk >> 1) * 4;
            xN = k ? x : x - 1;
            yN = k ? y - 1 : y;
        } else {
            const int x = kBlkX[blk] * 4, y = kBlkY[blk] * 4;
            xN = k ? x : x - 1;
            yN = k ? y - 1 : y;
        }
        int xW = 0, yW = 0;
        const int n = d.nb_mb(xN, yN, maxW, maxH, xW, yW);
        if (n < 0) {
            cond[k] = intra ? 1 : 0;
            continue;
        }
        const MbState &m = d.P.mbs[n];
        if (m.cls == H264R_MB_IPCM) {
            cond[k] = 1;
            continue;
        }
        int avail = 0, flag = 0;
        if (cat == 0) {
            if (m.cls == H264R_MB_I16x16) avail = 1, flag = m.cbf_dc & 1;
        } else if (cat == 1 || cat == 2) {
            const int bn = blk_of(xW >> 2, yW >> 2);
            if (!m.skip && ((m.cbp >> (bn >> 2)) & 1)) {
                avail = 1;
                flag = m.t8 ? (m.cbf_ac[0] >> (bn >> 2)) & 1 : (m.cbf_ac[0] >> bn) & 1;
            }
        } else if (cat == 3) {
            if (!m.skip && (m.cbp >> 4) != 0) avail = 1, flag = (m.cbf_dc >> comp) & 1;
        } else {
            const int bn = (yW >> 2) * 2 + (xW >> 2);
            if (!m.skip && (m.cbp >> 4) == 2) avail = 1, flag = (m.cbf_ac[comp] >> bn) & 1;
        }
        cond[k] = avail ? flag : 0;
    }
    return cond[0] + 2 * cond[1];
}

// residual_block_cabac( ) (7.3.5.3.3, 9.3.3.1.3) of a block of ctxBlockCat
// cat (0..4, or 5 for 8x8 luma) with max coefficients, the coded_block_flag
// context increment already derived (ignored for cat 5).  Field coded
// blocks (field MBs of MBAFF frames) take the field significance contexts
// (Table 9-34: 277 / 338, 436 / 451).  The levels go to lev[] in ascending
// scan position and their positions to *sig (16-bit word) or *sig64 (8x8).
// Returns the number of non-zero levels.
int block(Cabac &c, int cat, int cbf_ctx_inc, int max, int16_t *lev, uint16_t *sig, uint64_t *sig64, bool field)
{
    if (sig) *sig = 0;
    if (sig64) *sig64 = 0;
    if (cat != 5 && !c.decision(85 + kCbfCatOff[cat] + cbf_ctx_inc)) return 0;
    const int sig_base = cat == 5 ? (field ? 436 : 402) : (field ? 277 : 105) + kSigCatOff[cat];
    const int last_base = cat == 5 ? (field ? 451 : 417) : (field ? 338 : 166) + kSigCatOff[cat];
    const uint8_t *sig8 = field ? kSig8x8Field : kSig8x8Frame;
    const int abs_base = cat == 5 ? 426 : 227 + kAbsCatOff[cat];
    int pos[64];
    int n = 0;
    int num = max;
    for (int i = 0; i < num - 1; i++) {
        const int si = cat == 5 ? sig8[i] : (cat == 3 ? std::min(i, 2) : i);
        if (c.decision(sig_base + si)) {
            pos[n++] = i;
            const int li = cat == 5 ? kLast8x8[i] : (cat == 3 ? std::min(i, 2) : i);
            if (c.decision(last_base + li)) {
                num = i + 1;
                break;
            }
        }
    }
    if (num == max) pos[n++] = max - 1;  // the last position is significant when no last flag ended the scan
    // levels, highest scan position first
    int eq1 = 0, gt1 = 0;
    int16_t val[64];
    for (int k = n - 1; k >= 0; k--) {
        int a;
        const int inc0 = gt1 ? 0 : std::min(4, 1 + eq1);
        if (!c.decision(abs_base + inc0)) {
            a = 1;
        } else {
            const int inc = 5 + std::min(4 - (cat == 3 ? 1 : 0), gt1);
            int prefix = 1;
            while (prefix < 14 && c.decision(abs_base + inc)) prefix++;
            a = prefix + 1;
            if (prefix == 14) {  // Exp-Golomb k = 0 suffix
                int kk = 0;
                while (kk < 30 && c.bypass()) {
                    a += 1 << kk;
                    kk++;
                }
                while (kk-- > 0) a += c.bypass() << kk;
            }
        }
        if (a == 1) eq1++;
        else gt1++;
        val[k] = (int16_t)(c.bypass() ? -a : a);
    }
    for (int k = 0; k < n; k++) {
        if (sig64) *sig64 |= 1ull << pos[k];
        else *sig |= (uint16_t)(1u << pos[k]);
        lev[k] = val[k];
    }
    return n;
}

}  // namespace

// mb_skip_flag (9.3.3.1.1.1): neighbours A / B available and not skipped
int cabac_skip_inc(MbDecoder &d)
{
    int xW, yW;
    const int a = nbmb(d, -1, 0, xW, yW), b = nbmb(d, 0, -1, xW, yW);
    return (a >= 0 && !d.P.mbs[a].skip) + (b >= 0 && !d.P.mbs[b].skip);
}

// mb_field_decoding_flag (9.3.3.1.1.2): the left and upper MB pairs
// (6.4.10) of the slice that are field pairs
int cabac_field_inc(MbDecoder &d)
{
    const int pair = d.addr >> 1, W = d.W;
    const int a = pair % W > 0 ? 2 * (pair - 1) : -1, b = pair >= W ? 2 * (pair - W) : -1;
    const auto fieldpair = [&](int n) { return n >= 0 && d.P.mbs[n].slice == d.sc.index && d.P.mbs[n].field; };
    return fieldpair(a) + fieldpair(b);
}

// ---------------------------------------------------------------- motion syntax
int cabac_sub_mb_type(MbDecoder &d, bool is_b)
{
    Cabac &c = *d.cab;
    if (!is_b) {
        if (c.decision(21)) return 0;
        if (!c.decision(22)) return 1;
        return c.decision(23) ? 2 : 3;
    }
    if (!c.decision(36)) return 0;
    if (!c.decision(37)) return 1 + c.decision(39);
    int t = 3;
    if (c.decision(38)) {
        if (c.decision(39)) return 11 + c.decision(39);
        t += 4;
    }
    t += 2 * c.decision(39);
    t += c.decision(39);
    return t;
}

// the syntax of the neighbouring partition covering (xN, yN) relative to the
// current MB: lists its prediction uses, ref_idx and mvd (of list l); *field:
// the neighbour is a field MB of an MBAFF frame
static bool nb_syntax(const MbDecoder &d, int xN, int yN, int l, int &ref, int mvd[2], bool *field = nullptr)
{
    int xW = 0, yW = 0;
    const int n = d.nb_mb(xN, yN, 16, 16, xW, yW);
    ref = 0;
    mvd[0] = mvd[1] = 0;
    if (n < 0) return false;
    if (field) *field = n == d.addr ? d.fld : (d.mbaff && d.P.mbs[n].field);
    const int bi = (yW >> 2) * 4 + (xW >> 2);
    if (n == d.addr) {
        if (!(d.predl_cur[bi] & (1 << l))) return false;
        ref = d.refsyn_cur[l][bi];
        mvd[0] = d.mvd_cur[l][bi][0];
        mvd[1] = d.mvd_cur[l][bi][1];
        return true;
    }
    const MbState &m = d.P.mbs[n];
    if (m.skip || m.intra() || !(m.predl[bi] & (1 << l))) return false;
    ref = m.ref[l][bi];
    mvd[0] = m.mvd[l][bi][0];
    mvd[1] = m.mvd[l][bi][1];
    return true;
}

// ref_idx_lX of the partition at (x, y) (9.3.3.1.1.6, U binarisation); a
// field neighbour of a frame MB counts refIdx > 1 (its field index)
int cabac_ref_idx(MbDecoder &d, int l, int x, int y)
{
    Cabac &c = *d.cab;
    int ra, rb, mv[2];
    bool fa = false, fb = false;
    const bool na = nb_syntax(d, x - 1, y, l, ra, mv, &fa), nb = nb_syntax(d, x, y - 1, l, rb, mv, &fb);
    const int ca = na && ra > ((!d.fld && fa) ? 1 : 0);
    const int cb = nb && rb > ((!d.fld && fb) ? 1 : 0);
    if (!c.decision(54 + ca + 2 * cb)) return 0;
    int r = 1;
    int ctx = 58;
    while (r < 32 && c.decision(ctx)) {
        ctx = 59;
        r++;
    }
    return r;
}

// mvd_lX[comp] of the partition at (x, y) (9.3.3.1.1.7, UEG3 with uCoff 9)
int cabac_mvd(MbDecoder &d, int l, int comp, int x, int y)
{
    Cabac &c = *d.cab;
    int r, ma[2], mb[2];
    bool fa = false, fb = false;
    nb_syntax(d, x - 1, y, l, r, ma, &fa);
    nb_syntax(d, x, y - 1, l, r, mb, &fb);
    // vertical mvd of a neighbour of the other kind (MBAFF frame / field MB)
    // in the current MB's units
    auto scaled = [&](int v, bool f) {
        v = std::abs(v);
        if (comp == 1 && f != d.fld) v = d.fld ? v / 2 : v * 2;
        return v;
    };
    const int sum = scaled(ma[comp], fa) + scaled(mb[comp], fb);
    const int base = comp ? 47 : 40;
    if (!c.decision(base + (sum < 3 ? 0 : (sum <= 32 ? 1 : 2)))) return 0;
    int v = 1, ctx = 3;
    while (v < 9 && c.decision(base + ctx)) {
        if (v < 4) ctx++;
        v++;
    }
    if (v >= 9) {
        int k = 3;
        while (k < 24 && c.bypass()) {
            v += 1 << k;
            k++;
        }
        while (k-- > 0) v += c.bypass() << k;
    }
    return c.bypass() ? -v : v;
}

// ---------------------------------------------------------------- MB layer
// macroblock_layer( ) of a CABAC slice (7.3.5) into the record; mirrors
// MbDecoder::decode (CAVLC).  The CABAC state of the MB is kept for the
// contexts of later MBs.
int MbDecoder::decode_cabac()
{
    h264r_mb r;
    memset(&r, 0, sizeof(r));
    r.coef = H264R_NONE;
    r.aux = H264R_NONE;
    r.slice = (uint16_t)sc.index;
    if (pps.constrained_intra_pred) r.flags |= H264R_MBF_CIP;
    const int st = sc.sh.slice_type;
    Cabac &c = *cab;
    int mb_type, itype = 0;
    bool is_intra_type;
    if (st == kSliceI) {
        itype = mb_type_i(*this, 3, true);
        mb_type = itype;
        is_intra_type = true;
    } else if (st == kSliceP) {
        mb_type = mb_type_p(*this);
        is_intra_type = mb_type >= 5;
        itype = mb_type - 5;
    } else {
        mb_type = mb_type_b(*this);
        is_intra_type = mb_type >= 23;
        itype = mb_type - 23;
    }
    for (int i = 0; i < 16; i++) {
        cur->ipm4[i] = 2;
        cur->tc[i] = 0;
        cur->predl[i] = 0;
        predl_cur[i] = 0;
    }
    for (int i = 0; i < 4; i++) cur->ipm8[i] = 2;
    memset(cur->tcc, 0, sizeof(cur->tcc));
    memset(cur->mvd, 0, sizeof(cur->mvd));
    memset(mvd_cur, 0, sizeof(mvd_cur));
    memset(refsyn_cur, 0, sizeof(refsyn_cur));
    cur->cbp = 0;
    cur->t8 = false;
    cur->direct16 = false;
    cur->chroma_mode = 0;
    cur->cbf_dc = 0;
    cur->cbf_ac[0] = cur->cbf_ac[1] = cur->cbf_ac[2] = 0;
    for (int i = 0; i < 16; i++) {
        blk[i].ref[0] = blk[i].ref[1] = -1;
        blk[i].mv[0][0] = blk[i].mv[0][1] = blk[i].mv[1][0] = blk[i].mv[1][1] = 0;
    }
    if (is_intra_type && itype == 25) {  // I_PCM: samples byte-aligned, then the engine restarts
        while (!br.byte_aligned()) br.u(1);
        r.type = H264R_MB_IPCM;
        cur->cls = H264R_MB_IPCM;
        r.aux = (uint32_t)(P.pcm.size() / 384);
        for (int i = 0; i < 384; i++) P.pcm.push_back((uint8_t)br.u(8));
        r.qpy = (uint8_t)qp;
        prev_qp_nz = false;
        if (br.err) return P.fail(H264R_ERR_BAD_RECORD, "truncated I_PCM (MB %d)", addr);
        c.init_engine();
        P.rec[addr] = r;
        return 0;
    }
    int cbpv = 0;
    bool t8 = false;
    int cls;
    if (is_intra_type) {
        if (itype == 0) {  // I_NxN
            if (pps.transform_8x8_mode) t8 = t8_flag(*this) != 0;
            cls = t8 ? H264R_MB_I8x8 : H264R_MB_I4x4;
            cur->cls = (uint8_t)cls;
            const int nb = t8 ? 4 : 16;
            for (int b = 0; b < nb; b++) {
                const int flag = c.decision(68);
                int rem = 0;
                if (!flag) {
                    rem = c.decision(69);
                    rem |= c.decision(69) << 1;
                    rem |= c.decision(69) << 2;
                }
                if (!t8) {
                    cur->ipm4[b] = (int8_t)derive_mode(kBlkX[b] * 4, kBlkY[b] * 4, false, flag, rem);
                    r.ipred[b >> 3] |= (uint32_t)(cur->ipm4[b] & 15) << (4 * (b & 7));
                } else {
                    cur->ipm8[b] = (int8_t)derive_mode((b & 1) * 8, (b >> 1) * 8, true, flag, rem);
                    r.ipred[0] |= (uint32_t)(cur->ipm8[b] & 15) << (4 * b);
                    for (int k = 0; k < 4; k++) cur->ipm4[b * 4 + k] = cur->ipm8[b];
                }
            }
            r.chroma_mode = (uint8_t)chroma_pred(*this);
            cur->chroma_mode = r.chroma_mode;
            cbpv = cbp(*this);
        } else {  // I_16x16
            cls = H264R_MB_I16x16;
            cur->cls = (uint8_t)cls;
            r.i16_mode = (uint8_t)((itype - 1) % 4);
            cbpv = (((itype - 1) / 4) % 3) << 4 | (itype >= 13 ? 15 : 0);
            r.chroma_mode = (uint8_t)chroma_pred(*this);
            cur->chroma_mode = r.chroma_mode;
        }
        r.type = (uint8_t)cls;
    } else {
        cls = H264R_MB_INTER;
        cur->cls = H264R_MB_INTER;
        r.type = H264R_MB_INTER;
        const bool is_b = st == kSliceB;
        bool no_sub_lt8 = true;
        if (is_b && mb_type == 0) {  // B_Direct_16x16
            cur->direct16 = true;
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
            if (inter_pred(mb_type, is_b, r, no_sub_lt8)) return -1;
        }
        cbpv = cbp(*this);
        if ((cbpv & 15) && pps.transform_8x8_mode && no_sub_lt8 && (!(is_b && mb_type == 0) || sps.direct_8x8_inference))
            t8 = t8_flag(*this) != 0;
    }
    cur->cbp = (uint8_t)cbpv;
    cur->t8 = t8;
    if (t8) r.flags |= H264R_MBF_T8x8;
    uint32_t mask = 0;
    sig.clear();
    lv.clear();
    bool qp_nz = false;
    if ((cbpv & 15) || (cbpv >> 4) || cls == H264R_MB_I16x16) {
        int dq = qp_delta(*this);
        qp_nz = dq != 0;
        dq = clip3(-26, 25, dq);
        qp = (qp + dq + 52) % 52;
        // residual( 0, 15 ) (7.3.5.3)
        const int cbp_luma = cbpv & 15, cbp_chroma = cbpv >> 4;
        const bool i16 = cls == H264R_MB_I16x16;
        int16_t lev[64];
        uint16_t s16 = 0;
        r.nz4x4 = 0;
        r.nz8x8 = 0;
        auto put = [&](uint16_t s, const int16_t *v, int n, int bit) {
            if (!s) return;
            mask |= 1u << bit;
            sig.push_back(s);
            lv.insert(lv.end(), v, v + n);
        };
        uint16_t dc_sig = 0;
        int16_t dc_lev[16];
        int dc_n = 0;
        if (i16) {
            dc_n = block(c, 0, cbf_inc(*this, 0, 0, 0), 16, dc_lev, &dc_sig, nullptr, fld);
            if (dc_n) cur->cbf_dc |= 1;
            cur->tc[0] = (uint8_t)dc_n;  // as the reference keeps the DC count in block 0
            if (dc_n) r.nz4x4 = 1;
        }
        for (int b8 = 0; b8 < 4; b8++) {
            if (!(cbp_luma & (1 << b8))) continue;
            if (t8) {
                uint64_t s64 = 0;
                const int n = block(c, 5, 0, 64, lev, nullptr, &s64, fld);
                cur->cbf_ac[0] |= (uint16_t)(1u << b8);  // inferred coded_block_flag of an 8x8 block
                if (n) {
                    r.nz8x8 |= (uint8_t)(1u << b8);
                    mask |= 1u << b8;
                    for (int w = 0; w < 4; w++) sig.push_back((uint16_t)(s64 >> (16 * w)));
                    lv.insert(lv.end(), lev, lev + n);
                }
                continue;
            }
            for (int b4 = 0; b4 < 4; b4++) {
                const int b = b8 * 4 + b4;
                int n;
                if (i16) {
                    n = block(c, 1, cbf_inc(*this, 1, b, 0), 15, lev, &s16, nullptr, fld);
                    s16 = (uint16_t)(s16 << 1);  // AC list position k is scan position k + 1
                } else {
                    n = block(c, 2, cbf_inc(*this, 2, b, 0), 16, lev, &s16, nullptr, fld);
                }
                if (n) cur->cbf_ac[0] |= (uint16_t)(1u << b);
                cur->tc[b] = (uint8_t)n;
                r.nz4x4 = (uint16_t)((r.nz4x4 & ~(1u << b)) | (n ? 1u << b : 0u));
                if (n) r.nz8x8 |= (uint8_t)(1u << b8);
                put(s16, lev, n, b);
            }
        }
        if (dc_n) put(dc_sig, dc_lev, dc_n, 16);
        if (cbp_chroma & 3) {
            for (int cc = 0; cc < 2; cc++) {
                const int n = block(c, 3, cbf_inc(*this, 3, 0, 1 + cc), 4, lev, &s16, nullptr, fld);
                if (n) cur->cbf_dc |= (uint8_t)(2 << cc);
                put(s16, lev, n, 17 + cc);
            }
        }
        if (cbp_chroma & 2) {
            for (int cc = 0; cc < 2; cc++)
                for (int b = 0; b < 4; b++) {
                    int n = block(c, 4, cbf_inc(*this, 4, b, 1 + cc), 15, lev, &s16, nullptr, fld);
                    s16 = (uint16_t)(s16 << 1);
                    if (n) cur->cbf_ac[1 + cc] |= (uint16_t)(1u << b);
                    cur->tcc[cc][b] = (uint8_t)n;
                    put(s16, lev, n, (cc ? H264R_CM_CR_AC0 : H264R_CM_CB_AC0) + b);
                }
        }
        if (br.err) {
            r.qpy = 0;
            r.coef = H264R_NONE;
            if (cls == H264R_MB_INTER) store_motion();
            P.rec[addr] = r;
            return P.fail(H264R_ERR_BAD_RECORD, "truncated residual (MB %d)", addr);
        }
    }
    prev_qp_nz = qp_nz;
    r.qpy = (uint8_t)qp;
    if (mask) {
        std::vector<uint8_t> &cf = P.coef;
        while (cf.size() & 3) cf.push_back(0);
        r.coef = (uint32_t)cf.size();
        cf.insert(cf.end(), (const uint8_t *)&mask, (const uint8_t *)&mask + 4);
        cf.insert(cf.end(), (const uint8_t *)sig.data(), (const uint8_t *)sig.data() + 2 * sig.size());
        while (cf.size() & 3) cf.push_back(0);
        cf.insert(cf.end(), (const uint8_t *)lv.data(), (const uint8_t *)lv.data() + 2 * lv.size());
    }
    if (br.err) return P.fail(H264R_ERR_BAD_RECORD, "truncated macroblock (MB %d)", addr);
    if (cls == H264R_MB_INTER) {
        store_motion();
        memcpy(cur->mvd, mvd_cur, sizeof(mvd_cur));
        memcpy(cur->predl, predl_cur, sizeof(predl_cur));
    }
    P.rec[addr] = r;
    return 0;
}

}  // namespace pimpl
}  // namespace h264r

// ---- probes (tests compare the tables and the engine with other decoders)
extern "C" int h264r_probe_cabac_init(int model, int ctx_idx, int out[2])
{
    if (model < 0 || model > 3 || ctx_idx < 0 || ctx_idx >= 460 || !out) return H264R_ERR_INVALID_ARG;
    out[0] = h264r::pimpl::kCabacInit[model][ctx_idx][0];
    out[1] = h264r::pimpl::kCabacInit[model][ctx_idx][1];
    return 0;
}

extern "C" int h264r_probe_cabac_decision(int p_state, int val_mps, int range, int offset, int out[5])
{
    if (p_state < 0 || p_state > 63 || !out || range < 256 || range > 510 || offset < 0 || offset >= range)
        return H264R_ERR_INVALID_ARG;
    const uint8_t zeros[16] = {0};
    h264r::BitReader br(zeros, 16);
    h264r::pimpl::Cabac c;
    c.br = &br;
    c.state[0] = (uint8_t)p_state;
    c.mps[0] = (uint8_t)(val_mps & 1);
    c.range = (uint32_t)range;
    c.offset = (uint32_t)offset;
    out[0] = c.decision(0);
    out[1] = c.state[0];
    out[2] = c.mps[0];
    out[3] = (int)c.range;
    out[4] = (int)c.offset;
    return 0;
}
