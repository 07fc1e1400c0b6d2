// h264r_cavlc.cpp — CAVLC residual blocks (7.3.5.3.2, 9.2) and the me(v)
// coded_block_pattern mapping (9.1.2).  The code tables are the standard's
// Tables 9-4, 9-5 and 9-7 to 9-10, written here as bit strings per table
// row; they are turned into direct lookup tables once.  The reference
// decodes the same tables with if-chains (H264ResidualBlockCavlc.cpp:
// 580-3100, H264Golomb.cpp:120-330); tests/test_parser.py checks every
// table against those functions over all code words.
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/h264r.h"
#include "h264r_bits.h"

namespace h264r {

namespace {

// Table 9-5, coeff_token: [nC class][TotalCoeff][TrailingOnes]; classes
// 0 <= nC < 2, 2 <= nC < 4, 4 <= nC < 8, nC == -1 (4:2:0 chroma DC).
// (8 <= nC is the 6-bit fixed-length code, built in code.)
const char *const kCoeffToken[4][17][4] = {
    {{"1", 0, 0, 0},
     {"000101", "01", 0, 0},
     {"00000111", "000100", "001", 0},
     {"000000111", "00000110", "0000101", "00011"},
     {"0000000111", "000000110", "00000101", "000011"},
     {"00000000111", "0000000110", "000000101", "0000100"},
     {"0000000001111", "00000000110", "0000000101", "00000100"},
     {"0000000001011", "0000000001110", "00000000101", "000000100"},
     {"0000000001000", "0000000001010", "0000000001101", "0000000100"},
     {"00000000001111", "00000000001110", "0000000001001", "00000000100"},
     {"00000000001011", "00000000001010", "00000000001101", "0000000001100"},
     {"000000000001111", "000000000001110", "00000000001001", "00000000001100"},
     {"000000000001011", "000000000001010", "000000000001101", "00000000001000"},
     {"0000000000001111", "000000000000001", "000000000001001", "000000000001100"},
     {"0000000000001011", "0000000000001110", "0000000000001101", "000000000001000"},
     {"0000000000000111", "0000000000001010", "0000000000001001", "0000000000001100"},
     {"0000000000000100", "0000000000000110", "0000000000000101", "0000000000001000"}},
    {{"11", 0, 0, 0},
     {"001011", "10", 0, 0},
     {"000111", "00111", "011", 0},
     {"0000111", "001010", "001001", "0101"},
     {"00000111", "000110", "000101", "0100"},
     {"00000100", "0000110", "0000101", "00110"},
     {"000000111", "00000110", "00000101", "001000"},
     {"00000001111", "000000110", "000000101", "000100"},
     {"00000001011", "00000001110", "00000001101", "0000100"},
     {"000000001111", "00000001010", "00000001001", "000000100"},
     {"000000001011", "000000001110", "000000001101", "00000001100"},
     {"000000001000", "000000001010", "000000001001", "00000001000"},
     {"0000000001111", "0000000001110", "0000000001101", "000000001100"},
     {"0000000001011", "0000000001010", "0000000001001", "0000000001100"},
     {"0000000000111", "00000000001011", "0000000000110", "0000000001000"},
     {"00000000001001", "00000000001000", "00000000001010", "0000000000001"},
     {"00000000000111", "00000000000110", "00000000000101", "00000000000100"}},
    {{"1111", 0, 0, 0},
     {"001111", "1110", 0, 0},
     {"001011", "01111", "1101", 0},
     {"001000", "01100", "01110", "1100"},
     {"0001111", "01010", "01011", "1011"},
     {"0001011", "01000", "01001", "1010"},
     {"0001001", "001110", "001101", "1001"},
     {"0001000", "001010", "001001", "1000"},
     {"00001111", "0001110", "0001101", "01101"},
     {"00001011", "00001110", "0001010", "001100"},
     {"000001111", "00001010", "00001101", "0001100"},
     {"000001011", "000001110", "00001001", "00001100"},
     {"000001000", "000001010", "000001101", "00001000"},
     {"0000001101", "000000111", "000001001", "000001100"},
     {"0000001001", "0000001100", "0000001011", "0000001010"},
     {"0000000101", "0000001000", "0000000111", "0000000110"},
     {"0000000001", "0000000100", "0000000011", "0000000010"}},
    {{"01", 0, 0, 0},
     {"000111", "1", 0, 0},
     {"000100", "000110", "001", 0},
     {"000011", "0000011", "0000010", "000101"},
     {"000010", "00000011", "00000010", "0000000"}},
};

// Tables 9-7 / 9-8: total_zeros for 4x4 blocks, [TotalCoeff - 1][total_zeros]
const char *const kTotalZeros[15][16] = {
    {"1", "011", "010", "0011", "0010", "00011", "00010", "000011", "000010", "0000011", "0000010", "00000011",
     "00000010", "000000011", "000000010", "000000001"},
    {"111", "110", "101", "100", "011", "0101", "0100", "0011", "0010", "00011", "00010", "000011", "000010", "000001",
     "000000"},
    {"0101", "111", "110", "101", "0100", "0011", "100", "011", "0010", "00011", "00010", "000001", "00001", "000000"},
    {"00011", "111", "0101", "0100", "110", "101", "100", "0011", "011", "0010", "00010", "00001", "00000"},
    {"0101", "0100", "0011", "111", "110", "101", "100", "011", "0010", "00001", "0001", "00000"},
    {"000001", "00001", "111", "110", "101", "100", "011", "010", "0001", "001", "000000"},
    {"000001", "00001", "101", "100", "011", "11", "010", "0001", "001", "000000"},
    {"000001", "0001", "00001", "011", "11", "10", "010", "001", "000000"},
    {"000001", "000000", "0001", "11", "10", "001", "01", "00001"},
    {"00001", "00000", "001", "11", "10", "01", "0001"},
    {"0000", "0001", "001", "010", "1", "011"},
    {"0000", "0001", "01", "1", "001"},
    {"000", "001", "1", "01"},
    {"00", "01", "1"},
    {"0", "1"},
};

// Table 9-9 (a): total_zeros for 4:2:0 chroma DC, [TotalCoeff - 1][total_zeros]
const char *const kTotalZerosDc[3][4] = {{"1", "01", "001", "000"}, {"1", "01", "00", 0}, {"1", "0", 0, 0}};

// Table 9-10: run_before, [min(zerosLeft, 7) - 1][run_before]
const char *const kRunBefore[7][15] = {
    {"1", "0"},
    {"1", "01", "00"},
    {"11", "10", "01", "00"},
    {"11", "10", "01", "001", "000"},
    {"11", "10", "011", "010", "001", "000"},
    {"11", "000", "001", "011", "010", "101", "100"},
    {"111", "110", "101", "100", "011", "010", "001", "0001", "00001", "000001", "0000001", "00000001", "000000001",
     "0000000001", "00000000001"},
};

// Table 9-4 (ChromaArrayType 1 or 2): codeNum -> {Intra_4x4 / Intra_8x8, Inter}
const uint8_t kCbpMap[48][2] = {
    {47, 0},  {31, 16}, {15, 1},  {0, 2},   {23, 4},  {27, 8},  {29, 32}, {30, 3},  {7, 5},   {11, 10}, {13, 12}, {14, 15},
    {39, 47}, {43, 7},  {45, 11}, {46, 13}, {16, 14}, {3, 6},   {5, 9},   {10, 31}, {12, 35}, {19, 37}, {21, 42}, {26, 44},
    {28, 33}, {35, 34}, {37, 36}, {42, 40}, {44, 39}, {1, 43},  {2, 45},  {4, 46},  {8, 17},  {17, 18}, {18, 20}, {20, 24},
    {24, 19}, {6, 21},  {9, 26},  {22, 28}, {25, 23}, {32, 27}, {33, 29}, {34, 30}, {36, 22}, {40, 25}, {38, 38}, {41, 41},
};

// Direct lookup on the next `bits` bits: entry = length << 16 | value
// (0: no code word starts with these bits).
struct Vlc {
    int bits = 0;
    std::vector<uint32_t> lut;

    void add(const char *code, int value)
    {
        const int len = (int)strlen(code);
        uint32_t c = 0;
        for (int i = 0; i < len; i++) c = (c << 1) | (uint32_t)(code[i] == '1');
        const uint32_t first = c << (bits - len), n = 1u << (bits - len);
        for (uint32_t i = 0; i < n; i++) lut[first + i] = ((uint32_t)len << 16) | (uint32_t)value;
    }
    void init(int b)
    {
        bits = b;
        lut.assign((size_t)1 << b, 0);
    }
    // decoded value, or -1 when no code word matches
    int read(BitReader &br) const
    {
        const uint32_t e = lut[br.peek(bits)];
        if (!e) return -1;
        br.skip(e >> 16);
        return (int)(e & 0xFFFF);
    }
};

struct Tables {
    Vlc coeff_token[5];  // classes 0..2, 8 <= nC (3), nC == -1 (4); value TotalCoeff << 2 | TrailingOnes
    Vlc total_zeros[15], total_zeros_dc[3], run_before[7];
};

Tables build_tables()
{
    Tables t;
    {
        for (int c = 0; c < 3; c++) {
            t.coeff_token[c].init(16);
            for (int tc = 0; tc <= 16; tc++)
                for (int t1 = 0; t1 < 4; t1++)
                    if (kCoeffToken[c][tc][t1]) t.coeff_token[c].add(kCoeffToken[c][tc][t1], tc << 2 | t1);
        }
        t.coeff_token[3].init(6);
        t.coeff_token[3].add("000011", 0);
        for (int tc = 1; tc <= 16; tc++)
            for (int t1 = 0; t1 < 4 && t1 <= tc; t1++) {
                char code[7];
                const int v = ((tc - 1) << 2) | t1;
                for (int i = 0; i < 6; i++) code[i] = ((v >> (5 - i)) & 1) ? '1' : '0';
                code[6] = 0;
                t.coeff_token[3].add(code, tc << 2 | t1);
            }
        t.coeff_token[4].init(8);
        for (int tc = 0; tc <= 4; tc++)
            for (int t1 = 0; t1 < 4; t1++)
                if (kCoeffToken[3][tc][t1]) t.coeff_token[4].add(kCoeffToken[3][tc][t1], tc << 2 | t1);
        for (int i = 0; i < 15; i++) {
            t.total_zeros[i].init(9);
            for (int z = 0; z < 16; z++)
                if (kTotalZeros[i][z]) t.total_zeros[i].add(kTotalZeros[i][z], z);
        }
        for (int i = 0; i < 3; i++) {
            t.total_zeros_dc[i].init(3);
            for (int z = 0; z < 4; z++)
                if (kTotalZerosDc[i][z]) t.total_zeros_dc[i].add(kTotalZerosDc[i][z], z);
        }
        for (int i = 0; i < 7; i++) {
            t.run_before[i].init(11);
            for (int r = 0; r < 15; r++)
                if (kRunBefore[i][r]) t.run_before[i].add(kRunBefore[i][r], r);
        }
    }
    return t;
}

// built once when the library is loaded; read without a guard per code word
const Tables g_tables = build_tables();
inline const Tables &tables() { return g_tables; }

int nc_class(int nC) { return nC == -1 ? 4 : nC < 2 ? 0 : nC < 4 ? 1 : nC < 8 ? 2 : 3; }

}  // namespace

int cbp_from_code(uint32_t code, bool intra) { return code < 48 ? kCbpMap[code][intra ? 0 : 1] : -1; }

// coeff_token with nC (9.2.1): TotalCoeff and TrailingOnes, or -1
int cavlc_coeff_token(BitReader &br, int nC, int &total, int &t1)
{
    const int v = tables().coeff_token[nc_class(nC)].read(br);
    if (v < 0) return -1;
    total = v >> 2;
    t1 = v & 3;
    return 0;
}

int cavlc_total_zeros(BitReader &br, int max_coeff, int total)
{
    const Tables &t = tables();
    return max_coeff == 4 ? t.total_zeros_dc[total - 1].read(br) : t.total_zeros[total - 1].read(br);
}

int cavlc_run_before(BitReader &br, int zeros_left) { return tables().run_before[(zeros_left < 7 ? zeros_left : 7) - 1].read(br); }

// residual_block_cavlc( coeffLevel, startIdx, endIdx, maxNumCoeff ) (7.3.5.3.2,
// 9.2.2 - 9.2.4).  coeff[startIdx..endIdx] receive the levels (the rest of
// coeff[0..maxNumCoeff-1] zero); returns 0 or -1 on a syntax error.
// residual_block_cavlc (7.3.5.3.2) up to the levels and runs: level[i]
// and run[i] for i < total, highest frequency first (9.2.2 - 9.2.4)
static int cavlc_levels_runs(BitReader &br, int nC, int start, int end, int max_coeff, int *level, int *run, int &total)
{
    int t1 = 0;
    total = 0;
    if (cavlc_coeff_token(br, nC, total, t1)) return -1;
    if (total == 0) return 0;
    const int n = end - start + 1;
    if (total > n || t1 > total) return -1;
    int suffix_len = (total > 10 && t1 < 3) ? 1 : 0;
    for (int i = 0; i < total; i++) {
        if (i < t1) {
            level[i] = br.u(1) ? -1 : 1;
            continue;
        }
        // level_prefix: leading zero bits, then a one
        const uint32_t lead = br.peek(32);
        if (lead == 0) return -1;
        const int prefix = __builtin_clz(lead);
        br.skip((size_t)prefix + 1);
        if (br.err) return -1;
        int code = (prefix < 15 ? prefix : 15) << suffix_len;
        const int suffix_size = (prefix == 14 && suffix_len == 0) ? 4 : (prefix >= 15 ? prefix - 3 : suffix_len);
        if (suffix_size > 0) code += (int)br.u(suffix_size);
        if (prefix >= 15 && suffix_len == 0) code += 15;
        if (prefix >= 16) code += (1 << (prefix - 3)) - 4096;
        if (i == t1 && t1 < 3) code += 2;
        level[i] = (code % 2 == 0) ? (code + 2) >> 1 : (-code - 1) >> 1;
        if (suffix_len == 0) suffix_len = 1;
        const int a = level[i] < 0 ? -level[i] : level[i];
        if (a > (3 << (suffix_len - 1)) && suffix_len < 6) suffix_len++;
    }
    int zeros_left = 0;
    if (total < n) {
        zeros_left = cavlc_total_zeros(br, max_coeff, total);
        if (zeros_left < 0) return -1;
        if (total + zeros_left > n) return -1;
    }
    for (int i = 0; i < total - 1; i++) {
        if (zeros_left > 0) {
            run[i] = cavlc_run_before(br, zeros_left);
            if (run[i] < 0 || run[i] > zeros_left) return -1;
        } else {
            run[i] = 0;
        }
        zeros_left -= run[i];
    }
    run[total - 1] = zeros_left;
    return br.err ? -1 : 0;
}

int cavlc_residual_block(BitReader &br, int nC, int start, int end, int max_coeff, int *coeff, int &total)
{
    for (int i = 0; i < max_coeff; i++) coeff[i] = 0;
    int level[16], run[16];
    if (cavlc_levels_runs(br, nC, start, end, max_coeff, level, run, total)) return -1;
    int pos = -1;
    for (int i = total - 1; i >= 0; i--) {
        pos += run[i] + 1;
        coeff[start + pos] = level[i];
    }
    return 0;
}

int cavlc_residual_sparse(BitReader &br, int nC, int start, int end, int max_coeff, int off, uint16_t &sig, int16_t *lev,
                          int &total)
{
    sig = 0;
    int level[16], run[16];
    if (cavlc_levels_runs(br, nC, start, end, max_coeff, level, run, total)) return -1;
    int pos = -1;
    for (int i = total - 1; i >= 0; i--) {
        pos += run[i] + 1;
        sig |= (uint16_t)(1u << (start + pos + off));
        lev[total - 1 - i] = (int16_t)level[i];
    }
    return 0;
}

// ---------------------------------------------------------------- writing
// The inverse of the decoding above, for the seeded bitstream writer: the
// same code tables, read as bit strings.

static void put_code(BitWriter &bw, const char *code)
{
    for (const char *c = code; *c; c++) bw.u(1, *c == '1' ? 1u : 0u);
}

int cbp_to_code(int cbp, bool intra)
{
    for (int code = 0; code < 48; code++)
        if (kCbpMap[code][intra ? 0 : 1] == cbp) return code;
    return -1;
}

// residual_block_cavlc( ) of the levels coeff[start..end] (scan positions;
// max_coeff as in the syntax: 4 for 4:2:0 chroma DC, 15 for AC lists, 16
// otherwise).  Returns TotalCoeff, or -1 for a level outside the range the
// escape codes of a non-High profile carry.
int cavlc_write_block(BitWriter &bw, int nC, int start, int end, int max_coeff, const int *coeff)
{
    int level[16], run[16], total = 0;
    // highest frequency first; run[i] = zeros between level i and level i + 1
    int last = -1, hi = -1;
    for (int k = end; k >= start; k--) {
        if (!coeff[k]) continue;
        if (hi < 0) hi = k;
        level[total] = coeff[k];
        if (total > 0) run[total - 1] = last - k - 1;
        last = k;
        total++;
    }
    int t1 = 0;
    while (t1 < total && t1 < 3 && (level[t1] == 1 || level[t1] == -1)) t1++;
    // coeff_token
    if (nC == -1) {
        put_code(bw, kCoeffToken[3][total][t1]);
    } else if (nC >= 8) {
        if (total == 0) put_code(bw, "000011");
        else bw.u(6, (uint32_t)(((total - 1) << 2) | t1));
    } else {
        put_code(bw, kCoeffToken[nC < 2 ? 0 : (nC < 4 ? 1 : 2)][total][t1]);
    }
    if (total == 0) return 0;
    int suffix_len = (total > 10 && t1 < 3) ? 1 : 0;
    for (int i = 0; i < total; i++) {
        const int v = level[i];
        if (i < t1) {
            bw.u(1, v < 0 ? 1u : 0u);
            continue;
        }
        int code = v > 0 ? 2 * v - 2 : -2 * v - 1;
        if (i == t1 && t1 < 3) code -= 2;
        int prefix, ssize, suffix;
        if (suffix_len == 0) {
            if (code < 14) {
                prefix = code, ssize = 0, suffix = 0;
            } else if (code < 30) {
                prefix = 14, ssize = 4, suffix = code - 14;
            } else {
                prefix = 15, ssize = 12, suffix = code - 30;
            }
        } else if (code < (15 << suffix_len)) {
            prefix = code >> suffix_len, ssize = suffix_len, suffix = code & ((1 << suffix_len) - 1);
        } else {
            prefix = 15, ssize = 12, suffix = code - (15 << suffix_len);
        }
        if (suffix >= 4096) return -1;
        bw.u(prefix, 0);
        bw.u(1, 1);
        if (ssize) bw.u(ssize, (uint32_t)suffix);
        if (suffix_len == 0) suffix_len = 1;
        const int a = v < 0 ? -v : v;
        if (a > (3 << (suffix_len - 1)) && suffix_len < 6) suffix_len++;
    }
    // total_zeros: the zeros below the highest non-zero level
    int zeros = hi - start + 1 - total;
    if (total < end - start + 1)
        put_code(bw, max_coeff == 4 ? kTotalZerosDc[total - 1][zeros] : kTotalZeros[total - 1][zeros]);
    for (int i = 0; i < total - 1 && zeros > 0; i++) {
        put_code(bw, kRunBefore[(zeros < 7 ? zeros : 7) - 1][run[i]]);
        zeros -= run[i];
    }
    return total;
}

}  // namespace h264r

// ---- table probes (tests compare them with the reference's decoders)
extern "C" int h264r_probe_coeff_token(int nC, uint32_t window16, int out[3])
{
    uint8_t b[4] = {(uint8_t)(window16 >> 8), (uint8_t)window16, 0xFF, 0xFF};
    h264r::BitReader br(b, 4);
    int total = 0, t1 = 0;
    if (h264r::cavlc_coeff_token(br, nC, total, t1)) return -1;
    out[0] = (int)br.pos;
    out[1] = t1;
    out[2] = total;
    return 0;
}

extern "C" int h264r_probe_total_zeros(int max_coeff, int total_coeff, uint32_t window16, int out[2])
{
    if (total_coeff < 1 || total_coeff > (max_coeff == 4 ? 3 : 15)) return H264R_ERR_INVALID_ARG;
    uint8_t b[4] = {(uint8_t)(window16 >> 8), (uint8_t)window16, 0xFF, 0xFF};
    h264r::BitReader br(b, 4);
    const int z = h264r::cavlc_total_zeros(br, max_coeff, total_coeff);
    if (z < 0) return -1;
    out[0] = (int)br.pos;
    out[1] = z;
    return 0;
}

extern "C" int h264r_probe_run_before(int zeros_left, uint32_t window16, int out[2])
{
    if (zeros_left < 1) return H264R_ERR_INVALID_ARG;
    uint8_t b[4] = {(uint8_t)(window16 >> 8), (uint8_t)window16, 0xFF, 0xFF};
    h264r::BitReader br(b, 4);
    const int r = h264r::cavlc_run_before(br, zeros_left);
    if (r < 0) return -1;
    out[0] = (int)br.pos;
    out[1] = r;
    return 0;
}

extern "C" int h264r_probe_cbp(uint32_t code_num, int intra) { return h264r::cbp_from_code(code_num, intra != 0); }
