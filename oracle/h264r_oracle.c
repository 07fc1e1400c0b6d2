/*
 * h264r_oracle.c — CPU restatement of jfu222/h264_video_decoder_demo's
 * macroblock reconstruction, driven by the records of include/h264r.h.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU engine is held
 * to; the engine never links, calls or falls back to it.  It is pinned to the
 * reference by oracle/check_dump (pictures decoded by the unmodified reference
 * and dumped by oracle/ref_dump.cpp, bit-exact pre- and post-deblocking) and
 * by the golden fixtures in tests/golden.
 *
 * Every process cites the reference function it restates (paths are relative
 * to the reference's h264_video_decoder_demo/ directory).  The reference's
 * departures from the H.264 text are reproduced on purpose and marked
 * "quirk".  Scope: 8-bit 4:2:0 frames (progressive and MBAFF); field
 * pictures (PAFF) are rejected with H264R_ERR_UNSUPPORTED.
 */
#include "h264r_oracle.h"

#include <stdlib.h>
#include <string.h>

#define CLIP3(lo, hi, v) ((v) < (lo) ? (lo) : ((v) > (hi) ? (hi) : (v)))
#define ABS(v) ((v) < 0 ? -(v) : (v))
static inline int clip1(int v) { return CLIP3(0, 255, v); }

/* ------------------------------------------------------------------------ */
/* Tables of the H.264 text (the reference restates the same ones).         */

/* 4x4 zig-zag / field scan: scan index -> raster index (row*4+col),
   Inverse_scanning_process_for_4x4_transform_coefficients_and_scaling_lists
   (H264PictureBase.cpp:4542) */
static const uint8_t kZigzag4x4[16] = {0, 1, 4, 8, 5, 2, 3, 6, 9, 12, 13, 10, 7, 11, 14, 15};
static const uint8_t kField4x4[16] = {0, 4, 1, 8, 12, 5, 9, 13, 2, 6, 10, 14, 3, 7, 11, 15};
/* 8x8 zig-zag / field scan (H264PictureBase.cpp:4597) */
static const uint8_t kZigzag8x8[64] = {
    0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5,
    12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14, 21, 28,
    35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
    58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};
static const uint8_t kField8x8[64] = {
    0, 8, 16, 1, 9, 24, 32, 17, 2, 25, 40, 48, 56, 33, 10, 3,
    18, 41, 49, 57, 26, 11, 4, 19, 34, 42, 50, 58, 27, 12, 5, 20,
    35, 43, 51, 59, 28, 13, 6, 21, 36, 44, 52, 60, 29, 14, 22, 37,
    45, 53, 61, 30, 7, 15, 38, 46, 54, 62, 23, 31, 39, 47, 55, 63};

/* normAdjust4x4 / normAdjust8x8 (scaling_functions, H264PictureBase.cpp:4900-4951) */
static const int kV4[6][3] = {{10, 16, 13}, {11, 18, 14}, {13, 20, 16}, {14, 23, 18}, {16, 25, 20}, {18, 29, 23}};
static const int kV8[6][6] = {{20, 18, 32, 19, 25, 24}, {22, 19, 35, 21, 28, 26}, {26, 23, 42, 24, 33, 31},
                              {28, 25, 45, 26, 35, 33}, {32, 28, 51, 30, 40, 38}, {36, 32, 58, 34, 46, 43}};

/* Table 8-15, QPC as a function of qPI (get_chroma_quantisation_parameters,
   H264PictureBase.cpp:4773-4778) */
static const uint8_t kQpc[52] = {
    0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25,
    26, 27, 28, 29, 29, 30, 31, 32, 32, 33, 34, 34, 35, 35, 36, 36, 37, 37, 37, 38, 38, 38, 39, 39, 39, 39};

/* Table 8-16 alpha', beta' and Table 8-17 tC0'
   (H264PictureDeblockingFilterProcess.cpp:1330-1348, 1383-1409) */
static const uint8_t kAlpha[52] = {
    0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 4, 4, 5, 6, 7, 8, 9, 10, 12, 13,
    15, 17, 20, 22, 25, 28, 32, 36, 40, 45, 50, 56, 63, 71, 80, 90, 101, 113, 127, 144, 162, 182, 203, 226, 255, 255};
static const uint8_t kBeta[52] = {
    0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4,
    6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13, 14, 14, 15, 15, 16, 16, 17, 17, 18, 18};
static const uint8_t kTc0[3][52] = {
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1,
     1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 4, 5, 6, 6, 7, 8, 9, 10, 11, 13},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1,
     1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 5, 5, 6, 7, 8, 8, 10, 11, 12, 13, 15, 17},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1,
     1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 4, 5, 6, 6, 7, 8, 9, 10, 11, 13, 14, 16, 18, 20, 23, 25}};

/* luma4x4BlkIdx -> (x, y) in 4x4-block units (6.4.3) */
static const uint8_t kBlkX[16] = {0, 1, 0, 1, 2, 3, 2, 3, 0, 1, 0, 1, 2, 3, 2, 3};
static const uint8_t kBlkY[16] = {0, 0, 1, 1, 0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 3, 3};

/* ------------------------------------------------------------------------ */
/* A field picture (PAFF, structure TOP / BOTTOM) is reconstructed and
   filtered in a view of its field: W x H are the field's size, the planes
   start on the field's first line and step two frame lines (ys, cs), so MB
   geometry, neighbours (6.4.12.1) and filtering are those of a frame of the
   field's size.  Its MBs are field MBs all the same: field scans (8.5.6),
   field reference views, the chroma vector offset of Table 8-10 and the
   field rules of the bS derivation (8.7.2.1). */
typedef struct {
    const h264r_picture *pic;
    int wmb, hmb;          /* picture size in MBs (a field picture: its field) */
    int W, H, Wc, Hc;      /* picture size in samples */
    int fW, fH;            /* frame size in samples (the DPB slot layout) */
    int fpic;              /* 0 frame, 1 top field, 2 bottom field */
    int ys, cs;            /* row strides of the destination view */
    uint8_t *Y, *Cb, *Cr;  /* destination planes (a field picture: its first line) */
    uint8_t *const *dpb;
    int nslots;
} octx;

uint64_t h264o_slot_bytes(int width_mbs, int height_mbs)
{
    uint64_t W = (uint64_t)width_mbs * 16, H = (uint64_t)height_mbs * 16;
    return W * H * 3 / 2 + 4 * W + 64;
}

/* ---- macroblock geometry (6.4.1) ---------------------------------------- */
/* Inverse_macroblock_scanning_process (H264PictureBase.cpp:2503): luma
   origin of mbAddr, field MBs of an MBAFF pair start on row 0 / 1 of the pair
   and step 2 rows. */
static void mb_origin(const octx *c, int addr, int *x, int *y, int *dy)
{
    const h264r_mb *m = &c->pic->mbs[addr];
    if (!c->pic->mbaff) {
        *x = (addr % c->wmb) * 16;
        *y = (addr / c->wmb) * 16;
        *dy = 1;
    } else {
        int pair = addr >> 1;
        int x0 = (pair % c->wmb) * 16, y0 = (pair / c->wmb) * 32;
        *x = x0;
        if (m->flags & H264R_MBF_FIELD) {
            *y = y0 + (addr & 1);
            *dy = 2;
        } else {
            *y = y0 + (addr & 1) * 16;
            *dy = 1;
        }
    }
}

static int is_field_mb(const octx *c, int addr)
{
    return c->pic->mbaff && (c->pic->mbs[addr].flags & H264R_MBF_FIELD);
}

/* field scans and field rules: MBAFF field MBs and every MB of a field picture */
static int field_coded(const octx *c, int addr) { return is_field_mb(c, addr) || c->fpic != 0; }

static int is_intra_type(int t) { return t == H264R_MB_I4x4 || t == H264R_MB_I8x8 || t == H264R_MB_I16x16; }

/* ---- coefficient payload ------------------------------------------------ */
typedef struct {
    int32_t l4[16][16];   /* luma 4x4 lists (I16x16: AC in positions 1..15) */
    int32_t l8[4][64];    /* luma 8x8 lists */
    int32_t dc[16];       /* Intra16x16 DC list */
    int32_t cdc[2][4];    /* chroma DC (4:2:0) */
    int32_t cac[2][4][16];/* chroma AC lists (positions 1..15) */
} coefs;

static int parse_coef(const h264r_picture *pic, const h264r_mb *m, coefs *k)
{
    memset(k, 0, sizeof(*k));
    if (m->coef == H264R_NONE) return 0;
    if ((uint64_t)m->coef + 4 > pic->coef_bytes || (m->coef & 3)) return H264R_ERR_BAD_RECORD;
    const uint8_t *base = pic->coef + m->coef;
    uint32_t mask;
    memcpy(&mask, base, 4);
    if (mask >> 27) return H264R_ERR_BAD_RECORD;
    const int t8 = (m->flags & H264R_MBF_T8x8) != 0;
    int nwords = 0;
    for (int b = 0; b < 27; b++)
        if (mask & (1u << b)) nwords += (b < 4 && t8) ? 4 : 1;
    uint64_t vals_off = ((4 + 2 * (uint64_t)nwords) + 3) & ~3ull;
    if (m->coef + vals_off > pic->coef_bytes) return H264R_ERR_BAD_RECORD;
    const uint8_t *sigp = base + 4;
    const uint8_t *valp = base + vals_off;
    uint64_t vi = 0;
    int w = 0;
    for (int b = 0; b < 27; b++) {
        if (!(mask & (1u << b))) continue;
        int nw = (b < 4 && t8) ? 4 : 1;
        for (int q = 0; q < nw; q++) {
            uint16_t s;
            memcpy(&s, sigp + 2 * (w + q), 2);
            for (int i = 0; i < 16; i++) {
                if (!(s & (1u << i))) continue;
                int16_t v;
                if (m->coef + vals_off + 2 * (vi + 1) > pic->coef_bytes) return H264R_ERR_BAD_RECORD;
                memcpy(&v, valp + 2 * vi, 2);
                vi++;
                int pos = 16 * q + i;
                if (b < 16) {
                    if (t8) k->l8[b][pos] = v;
                    else k->l4[b][pos] = v;
                } else if (b == 16) k->dc[pos] = v;
                else if (b == 17 || b == 18) {
                    if (pos >= 4) return H264R_ERR_BAD_RECORD;
                    k->cdc[b - 17][pos] = v;
                } else if (b < 23) k->cac[0][b - 19][pos] = v;
                else k->cac[1][b - 23][pos] = v;
            }
        }
        w += nw;
    }
    return 0;
}

/* ---- scaling (8.5.9, scaling_functions, H264PictureBase.cpp:4852-4989) -- */
static int level_scale4(const octx *c, int list, int field, int m, int i, int j)
{
    const uint8_t *scan = field ? kField4x4 : kZigzag4x4;
    int ws = 16;
    for (int k = 0; k < 16; k++)
        if (scan[k] == i * 4 + j) { ws = c->pic->scaling4x4[list][k]; break; }
    int v = ((i & 1) == 0 && (j & 1) == 0) ? kV4[m][0] : (((i & 1) && (j & 1)) ? kV4[m][1] : kV4[m][2]);
    return ws * v;
}

static int level_scale8(const octx *c, int list, int field, int m, int i, int j)
{
    const uint8_t *scan = field ? kField8x8 : kZigzag8x8;
    int ws = 16;
    for (int k = 0; k < 64; k++)
        if (scan[k] == i * 8 + j) { ws = c->pic->scaling8x8[list][k]; break; }
    int v;
    if (i % 4 == 0 && j % 4 == 0) v = kV8[m][0];
    else if (i % 2 == 1 && j % 2 == 1) v = kV8[m][1];
    else if (i % 4 == 2 && j % 4 == 2) v = kV8[m][2];
    else if ((i % 4 == 0 && j % 2 == 1) || (i % 2 == 1 && j % 4 == 0)) v = kV8[m][3];
    else if ((i % 4 == 0 && j % 4 == 2) || (i % 4 == 2 && j % 4 == 0)) v = kV8[m][4];
    else v = kV8[m][5];
    return ws * v;
}

/* QP'C of one chroma component (get_chroma_quantisation_parameters,
   H264PictureBase.cpp:4748-4800), 8-bit video */
static int chroma_qp(int qpy, int offset)
{
    int qpi = CLIP3(0, 51, qpy + offset);
    return kQpc[qpi];
}

/* ---- inverse transforms ------------------------------------------------- */
/* 8.5.12 (H264PictureBase.cpp:4106-4266): scale the 4x4 list and transform.
   dc_pass: d[0][0] = c[0][0] (Intra16x16 luma, chroma). */
static void residual4x4(const octx *c, const int32_t *list, int field, int qp, int ls_list, int dc_pass,
                        int32_t dc_value, int32_t r[4][4])
{
    const uint8_t *scan = field ? kField4x4 : kZigzag4x4;
    int32_t cc[4][4] = {{0}}, d[4][4], f[4][4], h[4][4];
    for (int k = 0; k < 16; k++) cc[scan[k] >> 2][scan[k] & 3] = list[k];
    if (dc_pass) cc[0][0] = dc_value;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            if (i == 0 && j == 0 && dc_pass) {
                d[0][0] = cc[0][0];
            } else {
                int ls = level_scale4(c, ls_list, field, qp % 6, i, j);
                if (qp >= 24) d[i][j] = (cc[i][j] * ls) << (qp / 6 - 4);
                else d[i][j] = (cc[i][j] * ls + (1 << (3 - qp / 6))) >> (4 - qp / 6);
            }
        }
    for (int i = 0; i < 4; i++) {
        int e0 = d[i][0] + d[i][2], e1 = d[i][0] - d[i][2];
        int e2 = (d[i][1] >> 1) - d[i][3], e3 = d[i][1] + (d[i][3] >> 1);
        f[i][0] = e0 + e3; f[i][1] = e1 + e2; f[i][2] = e1 - e2; f[i][3] = e0 - e3;
    }
    for (int j = 0; j < 4; j++) {
        int g0 = f[0][j] + f[2][j], g1 = f[0][j] - f[2][j];
        int g2 = (f[1][j] >> 1) - f[3][j], g3 = f[1][j] + (f[3][j] >> 1);
        h[0][j] = g0 + g3; h[1][j] = g1 + g2; h[2][j] = g1 - g2; h[3][j] = g0 - g3;
    }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r[i][j] = (h[i][j] + 32) >> 6;
}

/* 8.5.13 (H264PictureBase.cpp:4270-4403) */
static void residual8x8(const octx *c, const int32_t *list, int field, int qp, int ls_list, int32_t r[8][8])
{
    const uint8_t *scan = field ? kField8x8 : kZigzag8x8;
    int32_t cc[8][8] = {{0}}, d[8][8], g[8][8], mm[8][8];
    for (int k = 0; k < 64; k++) cc[scan[k] >> 3][scan[k] & 7] = list[k];
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) {
            int ls = level_scale8(c, ls_list, field, qp % 6, i, j);
            if (qp >= 36) d[i][j] = (cc[i][j] * ls) << (qp / 6 - 6);
            else d[i][j] = (cc[i][j] * ls + (1 << (5 - qp / 6))) >> (6 - qp / 6);
        }
    for (int i = 0; i < 8; i++) {
        const int32_t *x = d[i];
        int e0 = x[0] + x[4];
        int e1 = -x[3] + x[5] - x[7] - (x[7] >> 1);
        int e2 = x[0] - x[4];
        int e3 = x[1] + x[7] - x[3] - (x[3] >> 1);
        int e4 = (x[2] >> 1) - x[6];
        int e5 = -x[1] + x[7] + x[5] + (x[5] >> 1);
        int e6 = x[2] + (x[6] >> 1);
        int e7 = x[3] + x[5] + x[1] + (x[1] >> 1);
        int f0 = e0 + e6, f1 = e1 + (e7 >> 2), f2 = e2 + e4, f3 = e3 + (e5 >> 2);
        int f4 = e2 - e4, f5 = (e3 >> 2) - e5, f6 = e0 - e6, f7 = e7 - (e1 >> 2);
        g[i][0] = f0 + f7; g[i][1] = f2 + f5; g[i][2] = f4 + f3; g[i][3] = f6 + f1;
        g[i][4] = f6 - f1; g[i][5] = f4 - f3; g[i][6] = f2 - f5; g[i][7] = f0 - f7;
    }
    for (int j = 0; j < 8; j++) {
        int x0 = g[0][j], x1 = g[1][j], x2 = g[2][j], x3 = g[3][j];
        int x4 = g[4][j], x5 = g[5][j], x6 = g[6][j], x7 = g[7][j];
        int e0 = x0 + x4;
        int e1 = -x3 + x5 - x7 - (x7 >> 1);
        int e2 = x0 - x4;
        int e3 = x1 + x7 - x3 - (x3 >> 1);
        int e4 = (x2 >> 1) - x6;
        int e5 = -x1 + x7 + x5 + (x5 >> 1);
        int e6 = x2 + (x6 >> 1);
        int e7 = x3 + x5 + x1 + (x1 >> 1);
        int f0 = e0 + e6, f1 = e1 + (e7 >> 2), f2 = e2 + e4, f3 = e3 + (e5 >> 2);
        int f4 = e2 - e4, f5 = (e3 >> 2) - e5, f6 = e0 - e6, f7 = e7 - (e1 >> 2);
        mm[0][j] = f0 + f7; mm[1][j] = f2 + f5; mm[2][j] = f4 + f3; mm[3][j] = f6 + f1;
        mm[4][j] = f6 - f1; mm[5][j] = f4 - f3; mm[6][j] = f2 - f5; mm[7][j] = f0 - f7;
    }
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) r[i][j] = (mm[i][j] + 32) >> 6;
}

/* 8.5.10 Intra16x16 DC (H264PictureBase.cpp:4993-5088) -> dcY[row][col] */
static void luma_dc(const octx *c, const int32_t *list, int field, int qp, int32_t dcY[4][4])
{
    const uint8_t *scan = field ? kField4x4 : kZigzag4x4;
    int32_t cc[4][4] = {{0}}, g[4][4], f[4][4];
    for (int k = 0; k < 16; k++) cc[scan[k] >> 2][scan[k] & 3] = list[k];
    for (int j = 0; j < 4; j++) {
        g[0][j] = cc[0][j] + cc[1][j] + cc[2][j] + cc[3][j];
        g[1][j] = cc[0][j] + cc[1][j] - cc[2][j] - cc[3][j];
        g[2][j] = cc[0][j] - cc[1][j] - cc[2][j] + cc[3][j];
        g[3][j] = cc[0][j] - cc[1][j] + cc[2][j] - cc[3][j];
    }
    for (int i = 0; i < 4; i++) {
        f[i][0] = g[i][0] + g[i][1] + g[i][2] + g[i][3];
        f[i][1] = g[i][0] + g[i][1] - g[i][2] - g[i][3];
        f[i][2] = g[i][0] - g[i][1] - g[i][2] + g[i][3];
        f[i][3] = g[i][0] - g[i][1] + g[i][2] - g[i][3];
    }
    int ls = level_scale4(c, 0, field, qp % 6, 0, 0);
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            if (qp >= 36) dcY[i][j] = (f[i][j] * ls) << (qp / 6 - 6);
            else dcY[i][j] = (f[i][j] * ls + (1 << (5 - qp / 6))) >> (6 - qp / 6);
        }
}

/* 8.5.11 chroma DC, 4:2:0 (H264PictureBase.cpp:3989-4044).  Quirk: the
   LevelScale4x4 used is the one last computed for the MB's luma (scaling
   list 0 for intra, 3 for inter), not the chroma list. */
static void chroma_dc(const octx *c, const int32_t *lv, int field, int qpc, int ls_list, int32_t dcC[4])
{
    int e00 = lv[0] + lv[2], e01 = lv[1] + lv[3], e10 = lv[0] - lv[2], e11 = lv[1] - lv[3];
    int f[4] = {e00 + e01, e00 - e01, e10 + e11, e10 - e11};
    int ls = level_scale4(c, ls_list, field, qpc % 6, 0, 0);
    for (int i = 0; i < 4; i++) dcC[i] = ((f[i] * ls) << (qpc / 6)) >> 5;
}

/* ---- sample access ------------------------------------------------------ */
static inline uint8_t *lum(const octx *c, int x, int y) { return c->Y + (size_t)y * c->ys + x; }
static inline uint8_t *chr(const octx *c, int pl, int x, int y)
{
    return (pl ? c->Cr : c->Cb) + (size_t)y * c->cs + x;
}

/* Luma / chroma residual of one MB, added to the prediction already in the
   picture: u = Clip1(pred + r), written back (8.5.14,
   Picture_construction_process_prior_to_deblocking_filter_process,
   H264PictureBase.cpp:4408-4538). */
static void add_block(uint8_t *p, int stride, const int32_t *r, int n)
{
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) p[(size_t)i * stride + j] = (uint8_t)clip1(p[(size_t)i * stride + j] + r[i * n + j]);
}

/* chroma residual of an MB: DC + AC for both components, added in place
   (transform_decoding_process_for_chroma_samples[_inter],
   H264PictureBase.cpp:3752-3940, H264InterPrediction.cpp:230-407) */
static void chroma_residual(const octx *c, int addr, const coefs *k, int ls_list)
{
    const h264r_mb *m = &c->pic->mbs[addr];
    const h264r_slice *s = &c->pic->slices[m->slice];
    int x, y, dy;
    mb_origin(c, addr, &x, &y, &dy);
    int field = is_field_mb(c, addr), sf = field_coded(c, addr);
    int xc = x / 2, yc = (y >> 4) * 8 + (y & 1);
    if (c->pic->mbaff && !field) yc = y / 2;
    for (int pl = 0; pl < 2; pl++) {
        int qpc = chroma_qp(m->qpy, s->chroma_qp_offset[pl]);
        int32_t dcC[4];
        chroma_dc(c, k->cdc[pl], sf, qpc, ls_list, dcC);
        for (int b = 0; b < 4; b++) {
            int32_t r[4][4];
            residual4x4(c, k->cac[pl][b], sf, qpc, ls_list, 1, dcC[b], r);
            int bx = (b & 1) * 4, by = (b >> 1) * 4;
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) {
                    uint8_t *p = chr(c, pl, xc + bx + j, yc + (by + i) * dy);
                    *p = (uint8_t)clip1(*p + r[i][j]);
                }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* 6.4.12 neighbouring locations, as the reference derives them
   (getMbAddrN_non_MBAFF_frames H264PictureBase.cpp:2878,
    getMbAddrN_MBAFF_frames 2984).  Returns mbAddrN or -1 and sets the
   location (xW, yW) inside it. */
static int avail_mb(const octx *c, int cur, int n)
{
    if (n < 0 || n > cur) return 0;
    return c->pic->mbs[n].slice == c->pic->mbs[cur].slice;
}

static int nb_loc_nonmbaff(const octx *c, int cur, int xN, int yN, int maxW, int maxH, int *xW, int *yW)
{
    int W = c->wmb, n = -1;
    if (xN < 0 && yN < 0) {
        n = cur - W - 1;
        if (cur % W == 0) n = -1;
    } else if (xN < 0 && yN < maxH) {
        n = cur - 1;
        if (cur % W == 0) n = -1;
    } else if (xN < maxW && yN < 0) {
        n = cur - W;
    } else if (xN < maxW && yN < maxH) {
        n = cur;
    } else if (xN >= maxW && yN < 0) {
        n = cur - W + 1;
        if ((cur + 1) % W == 0) n = -1;
    } else {
        return -1;
    }
    if (n != cur && !avail_mb(c, cur, n)) return -1;
    *xW = (xN + maxW) % maxW;
    *yW = (yN + maxH) % maxH;
    return n;
}

/* MBAFF neighbouring locations, Table 6-4 (getMbAddrN_MBAFF_frames,
   H264PictureBase.cpp:2984-3395).  An unavailable pair address is -2, so the
   unconditional "+1" entries of the table become -1 (not available). */
static int nb_loc_mbaff(const octx *c, int cur, int xN, int yN, int maxW, int maxH, int *xW, int *yW)
{
    const int W = c->wmb, pair = cur / 2;
    const h264r_mb *mbs = c->pic->mbs;
    int A = 2 * (pair - 1), B = 2 * (pair - W), C = 2 * (pair - W + 1), D = 2 * (pair - W - 1);
    if (A < 0 || A > cur || mbs[A].slice != mbs[cur].slice || pair % W == 0) A = -2;
    if (B < 0 || B > cur || mbs[B].slice != mbs[cur].slice) B = -2;
    if (C < 0 || C > cur || mbs[C].slice != mbs[cur].slice || (pair + 1) % W == 0) C = -2;
    if (D < 0 || D > cur || mbs[D].slice != mbs[cur].slice || pair % W == 0) D = -2;
#define FRM(a) (!(mbs[a].flags & H264R_MBF_FIELD))
    const int frame = FRM(cur), top = (cur % 2) == 0;
    int n = -1, yM = 0;
    if (xN < 0 && yN < 0) {
        if (frame) {
            if (top) { n = D + 1; yM = yN; }
            else if (A >= 0) {
                if (FRM(A)) { n = A; yM = yN; } else { n = A + 1; yM = (yN + maxH) >> 1; }
            }
        } else {
            if (top) {
                if (D >= 0) { if (FRM(D)) { n = D + 1; yM = 2 * yN; } else { n = D; yM = yN; } }
            } else { n = D + 1; yM = yN; }
        }
    } else if (xN < 0 && yN < maxH) {
        if (A >= 0) {
            if (frame) {
                if (top) {
                    if (FRM(A)) { n = A; yM = yN; } else { n = (yN % 2 == 0) ? A : A + 1; yM = yN >> 1; }
                } else {
                    if (FRM(A)) { n = A + 1; yM = yN; } else { n = (yN % 2 == 0) ? A : A + 1; yM = (yN + maxH) >> 1; }
                }
            } else {
                if (top) {
                    if (FRM(A)) {
                        if (yN < maxH / 2) { n = A; yM = yN << 1; } else { n = A + 1; yM = (yN << 1) - maxH; }
                    } else { n = A; yM = yN; }
                } else {
                    if (FRM(A)) {
                        if (yN < maxH / 2) { n = A; yM = (yN << 1) + 1; } else { n = A + 1; yM = (yN << 1) + 1 - maxH; }
                    } else { n = A + 1; yM = yN; }
                }
            }
        }
    } else if (xN < maxW && yN < 0) {
        if (frame) {
            if (top) { n = B + 1; yM = yN; } else { n = cur - 1; yM = yN; }
        } else {
            if (top) {
                if (B >= 0) { if (FRM(B)) { n = B + 1; yM = 2 * yN; } else { n = B; yM = yN; } }
            } else { n = B + 1; yM = yN; }
        }
    } else if (xN < maxW && yN < maxH) {
        n = cur; yM = yN;
    } else if (xN >= maxW && yN < 0) {
        if (frame) {
            if (top) { n = C + 1; yM = yN; } else n = -1;
        } else {
            if (top) {
                if (C >= 0) { if (FRM(C)) { n = C + 1; yM = 2 * yN; } else { n = C; yM = yN; } }
            } else { n = C + 1; yM = yN; }
        }
    }
#undef FRM
    if (n < 0) return -1;
    *xW = (xN + maxW) % maxW;
    *yW = (yM + maxH) % maxH;
    return n;
}

static int nb_loc(const octx *c, int cur, int xN, int yN, int maxW, int maxH, int *xW, int *yW)
{
    if (!c->pic->mbaff) return nb_loc_nonmbaff(c, cur, xN, yN, maxW, maxH, xW, yW);
    return nb_loc_mbaff(c, cur, xN, yN, maxW, maxH, xW, yW);
}

/* constructed sample p[x, y] relative to the current MB, or -1 when "not
   available for Intra prediction" (the per-mode sample collections of
   Intra_4x4/8x8/16x16/chroma_sample_prediction). */
static int intra_nb(const octx *c, int cur, int isChroma, int pl, int xN, int yN)
{
    int maxW = isChroma ? 8 : 16, maxH = isChroma ? 8 : 16;
    int xW, yW;
    int n = nb_loc(c, cur, xN, yN, maxW, maxH, &xW, &yW);
    if (n < 0) return -1;
    const h264r_mb *mn = &c->pic->mbs[n];
    if (n != cur && mn->type == H264R_MB_INTER && (mn->flags & H264R_MBF_CIP)) return -1;
    int x, y, dy;
    mb_origin(c, n, &x, &y, &dy);
    if (!isChroma) return *lum(c, x + xW, y + dy * yW);
    int xm = x / 2, ym;
    if (c->pic->mbaff) {
        ym = (y >> 4) * 8 + (y & 1);
        if (!is_field_mb(c, n)) ym = y / 2;
    } else {
        ym = y / 2;
    }
    return *chr(c, pl, xm + xW, ym + dy * yW);
}

/* ---- intra prediction --------------------------------------------------- */
/* 8.3.1.2 Intra_4x4_sample_prediction (H264PictureBase.cpp:1062-1419).
   pred[] receives the 16 samples; returns 0 when the mode's samples are not
   available, in which case the reference writes nothing and the cleared
   picture buffer (zeros) stays the prediction. */
static int pred4x4(const octx *c, int cur, int blk, int mode, uint8_t pred[16])
{
    int xO = kBlkX[blk] * 4, yO = kBlkY[blk] * 4;
    int P[5][9]; /* P[y+1][x+1] */
    for (int y = -1; y <= 3; y++)
        for (int x = -1; x <= 7; x++) P[y + 1][x + 1] = -1;
    for (int y = -1; y <= 3; y++) P[y + 1][0] = intra_nb(c, cur, 0, 0, xO - 1, yO + y);
    for (int x = 0; x <= 7; x++) {
        if (x > 3 && (blk == 3 || blk == 11)) P[0][x + 1] = -1;
        else P[0][x + 1] = intra_nb(c, cur, 0, 0, xO + x, yO - 1);
    }
#define p(x, y) P[(y) + 1][(x) + 1]
    if (p(4, -1) < 0 && p(5, -1) < 0 && p(6, -1) < 0 && p(7, -1) < 0 && p(3, -1) >= 0)
        for (int x = 4; x < 8; x++) p(x, -1) = p(3, -1);
    int top = p(0, -1) >= 0 && p(1, -1) >= 0 && p(2, -1) >= 0 && p(3, -1) >= 0;
    int top8 = top && p(4, -1) >= 0 && p(5, -1) >= 0 && p(6, -1) >= 0 && p(7, -1) >= 0;
    int left = p(-1, 0) >= 0 && p(-1, 1) >= 0 && p(-1, 2) >= 0 && p(-1, 3) >= 0;
    int corner = p(-1, -1) >= 0;
    for (int y = 0; y < 4; y++)
        for (int x = 0; x < 4; x++) {
            int v = 0;
            switch (mode) {
            case 0: if (!top) return 0; v = p(x, -1); break;
            case 1: if (!left) return 0; v = p(-1, y); break;
            case 2:
                if (top && left) v = (p(0, -1) + p(1, -1) + p(2, -1) + p(3, -1) + p(-1, 0) + p(-1, 1) + p(-1, 2) + p(-1, 3) + 4) >> 3;
                else if (left) v = (p(-1, 0) + p(-1, 1) + p(-1, 2) + p(-1, 3) + 2) >> 2;
                else if (top) v = (p(0, -1) + p(1, -1) + p(2, -1) + p(3, -1) + 2) >> 2;
                else v = 128;
                break;
            case 3:
                if (!top8) return 0;
                if (x == 3 && y == 3) v = (p(6, -1) + 3 * p(7, -1) + 2) >> 2;
                else v = (p(x + y, -1) + 2 * p(x + y + 1, -1) + p(x + y + 2, -1) + 2) >> 2;
                break;
            case 4:
                if (!(top && left && corner)) return 0;
                if (x > y) v = (p(x - y - 2, -1) + 2 * p(x - y - 1, -1) + p(x - y, -1) + 2) >> 2;
                else if (x < y) v = (p(-1, y - x - 2) + 2 * p(-1, y - x - 1) + p(-1, y - x) + 2) >> 2;
                else v = (p(0, -1) + 2 * p(-1, -1) + p(-1, 0) + 2) >> 2;
                break;
            case 5: {
                if (!(top && left && corner)) return 0;
                int z = 2 * x - y;
                if (z >= 0 && (z & 1) == 0) v = (p(x - (y >> 1) - 1, -1) + p(x - (y >> 1), -1) + 1) >> 1;
                else if (z >= 0) v = (p(x - (y >> 1) - 2, -1) + 2 * p(x - (y >> 1) - 1, -1) + p(x - (y >> 1), -1) + 2) >> 2;
                else if (z == -1) v = (p(-1, 0) + 2 * p(-1, -1) + p(0, -1) + 2) >> 2;
                else v = (p(-1, y - 1) + 2 * p(-1, y - 2) + p(-1, y - 3) + 2) >> 2;
                break;
            }
            case 6: {
                if (!(top && left && corner)) return 0;
                int z = 2 * y - x;
                if (z >= 0 && (z & 1) == 0) v = (p(-1, y - (x >> 1) - 1) + p(-1, y - (x >> 1)) + 1) >> 1;
                else if (z >= 0) v = (p(-1, y - (x >> 1) - 2) + 2 * p(-1, y - (x >> 1) - 1) + p(-1, y - (x >> 1)) + 2) >> 2;
                else if (z == -1) v = (p(-1, 0) + 2 * p(-1, -1) + p(0, -1) + 2) >> 2;
                else v = (p(x - 1, -1) + 2 * p(x - 2, -1) + p(x - 3, -1) + 2) >> 2;
                break;
            }
            case 7:
                if (!top8) return 0;
                if ((y & 1) == 0) v = (p(x + (y >> 1), -1) + p(x + (y >> 1) + 1, -1) + 1) >> 1;
                else v = (p(x + (y >> 1), -1) + 2 * p(x + (y >> 1) + 1, -1) + p(x + (y >> 1) + 2, -1) + 2) >> 2;
                break;
            case 8: {
                if (!left) return 0;
                int z = x + 2 * y;
                if (z <= 4 && (z & 1) == 0) v = (p(-1, y + (x >> 1)) + p(-1, y + (x >> 1) + 1) + 1) >> 1;
                else if (z < 5) v = (p(-1, y + (x >> 1)) + 2 * p(-1, y + (x >> 1) + 1) + p(-1, y + (x >> 1) + 2) + 2) >> 2;
                else if (z == 5) v = (p(-1, 2) + 3 * p(-1, 3) + 2) >> 2;
                else v = p(-1, 3);
                break;
            }
            default: return 0;
            }
            pred[y * 4 + x] = (uint8_t)v;
        }
#undef p
    return 1;
}

/* 8.3.2.2 Intra_8x8_sample_prediction with the reference sample filter
   8.3.2.2.1 (H264PictureBase.cpp:1423-1846) */
static int pred8x8(const octx *c, int cur, int blk, int mode, uint8_t pred[64])
{
    int xO = (blk & 1) * 8, yO = (blk >> 1) * 8;
    int P[9][17], Q[9][17];
    for (int y = 0; y < 9; y++)
        for (int x = 0; x < 17; x++) P[y][x] = Q[y][x] = -1;
#define p(x, y) P[(y) + 1][(x) + 1]
#define q(x, y) Q[(y) + 1][(x) + 1]
    for (int y = -1; y <= 7; y++) p(-1, y) = intra_nb(c, cur, 0, 0, xO - 1, yO + y);
    for (int x = 0; x <= 15; x++) p(x, -1) = intra_nb(c, cur, 0, 0, xO + x, yO - 1);
    {
        int all = 1;
        for (int x = 8; x < 16; x++) if (p(x, -1) >= 0) all = 0;
        if (all && p(7, -1) >= 0)
            for (int x = 8; x < 16; x++) p(x, -1) = p(7, -1);
    }
    int top16 = 1;
    for (int x = 0; x < 16; x++) if (p(x, -1) < 0) top16 = 0;
    if (top16) {
        q(0, -1) = (p(-1, -1) >= 0) ? (p(-1, -1) + 2 * p(0, -1) + p(1, -1) + 2) >> 2 : (3 * p(0, -1) + p(1, -1) + 2) >> 2;
        for (int x = 1; x <= 14; x++) q(x, -1) = (p(x - 1, -1) + 2 * p(x, -1) + p(x + 1, -1) + 2) >> 2;
        q(15, -1) = (p(14, -1) + 3 * p(15, -1) + 2) >> 2;
    }
    if (p(-1, -1) >= 0) {
        if (p(0, -1) < 0 || p(-1, 0) < 0) {
            if (p(0, -1) >= 0) q(-1, -1) = (3 * p(-1, -1) + p(0, -1) + 2) >> 2;
            else if (p(-1, 0) >= 0) q(-1, -1) = (3 * p(-1, -1) + p(-1, 0) + 2) >> 2;
            else q(-1, -1) = p(-1, -1);
        } else {
            q(-1, -1) = (p(0, -1) + 2 * p(-1, -1) + p(-1, 0) + 2) >> 2;
        }
    }
    int left8 = 1;
    for (int y = 0; y < 8; y++) if (p(-1, y) < 0) left8 = 0;
    if (left8) {
        q(-1, 0) = (p(-1, -1) >= 0) ? (p(-1, -1) + 2 * p(-1, 0) + p(-1, 1) + 2) >> 2 : (3 * p(-1, 0) + p(-1, 1) + 2) >> 2;
        for (int y = 1; y <= 6; y++) q(-1, y) = (p(-1, y - 1) + 2 * p(-1, y) + p(-1, y + 1) + 2) >> 2;
        q(-1, 7) = (p(-1, 6) + 3 * p(-1, 7) + 2) >> 2;
    }
#undef p
#define p(x, y) Q[(y) + 1][(x) + 1]
    int top = 1;
    for (int x = 0; x < 8; x++) if (p(x, -1) < 0) top = 0;
    int topr = top;
    for (int x = 8; x < 16; x++) if (p(x, -1) < 0) topr = 0;
    int left = 1;
    for (int y = 0; y < 8; y++) if (p(-1, y) < 0) left = 0;
    int corner = p(-1, -1) >= 0;
    for (int y = 0; y < 8; y++)
        for (int x = 0; x < 8; x++) {
            int v = 0;
            switch (mode) {
            case 0: if (!top) return 0; v = p(x, -1); break;
            case 1: if (!left) return 0; v = p(-1, y); break;
            case 2: {
                int st = 0, sl = 0;
                for (int i = 0; i < 8; i++) { st += top ? p(i, -1) : 0; sl += left ? p(-1, i) : 0; }
                if (top && left) v = (st + sl + 8) >> 4;
                else if (left) v = (sl + 4) >> 3;
                else if (top) v = (st + 4) >> 3;
                else v = 128;
                break;
            }
            case 3:
                if (!topr) return 0;
                if (x == 7 && y == 7) v = (p(14, -1) + 3 * p(15, -1) + 2) >> 2;
                else v = (p(x + y, -1) + 2 * p(x + y + 1, -1) + p(x + y + 2, -1) + 2) >> 2;
                break;
            case 4:
                if (!(top && left && corner)) return 0;
                if (x > y) v = (p(x - y - 2, -1) + 2 * p(x - y - 1, -1) + p(x - y, -1) + 2) >> 2;
                else if (x < y) v = (p(-1, y - x - 2) + 2 * p(-1, y - x - 1) + p(-1, y - x) + 2) >> 2;
                else v = (p(0, -1) + 2 * p(-1, -1) + p(-1, 0) + 2) >> 2;
                break;
            case 5: {
                if (!(top && left && corner)) return 0;
                int z = 2 * x - y;
                if (z >= 0 && (z & 1) == 0) v = (p(x - (y >> 1) - 1, -1) + p(x - (y >> 1), -1) + 1) >> 1;
                else if (z >= 0) v = (p(x - (y >> 1) - 2, -1) + 2 * p(x - (y >> 1) - 1, -1) + p(x - (y >> 1), -1) + 2) >> 2;
                else if (z == -1) v = (p(-1, 0) + 2 * p(-1, -1) + p(0, -1) + 2) >> 2;
                else v = (p(-1, y - 2 * x - 1) + 2 * p(-1, y - 2 * x - 2) + p(-1, y - 2 * x - 3) + 2) >> 2;
                break;
            }
            case 6: {
                if (!(top && left && corner)) return 0;
                int z = 2 * y - x;
                if (z >= 0 && (z & 1) == 0) v = (p(-1, y - (x >> 1) - 1) + p(-1, y - (x >> 1)) + 1) >> 1;
                else if (z >= 0) v = (p(-1, y - (x >> 1) - 2) + 2 * p(-1, y - (x >> 1) - 1) + p(-1, y - (x >> 1)) + 2) >> 2;
                else if (z == -1) v = (p(-1, 0) + 2 * p(-1, -1) + p(0, -1) + 2) >> 2;
                else v = (p(x - 2 * y - 1, -1) + 2 * p(x - 2 * y - 2, -1) + p(x - 2 * y - 3, -1) + 2) >> 2;
                break;
            }
            case 7:
                if (!topr) return 0;
                if ((y & 1) == 0) v = (p(x + (y >> 1), -1) + p(x + (y >> 1) + 1, -1) + 1) >> 1;
                else v = (p(x + (y >> 1), -1) + 2 * p(x + (y >> 1) + 1, -1) + p(x + (y >> 1) + 2, -1) + 2) >> 2;
                break;
            case 8: {
                if (!left) return 0;
                int z = x + 2 * y;
                if (z <= 12 && (z & 1) == 0) v = (p(-1, y + (x >> 1)) + p(-1, y + (x >> 1) + 1) + 1) >> 1;
                else if (z < 13) v = (p(-1, y + (x >> 1)) + 2 * p(-1, y + (x >> 1) + 1) + p(-1, y + (x >> 1) + 2) + 2) >> 2;
                else if (z == 13) v = (p(-1, 6) + 3 * p(-1, 7) + 2) >> 2;
                else v = p(-1, 7);
                break;
            }
            default: return 0;
            }
            pred[y * 8 + x] = (uint8_t)v;
        }
#undef p
#undef q
    return 1;
}

/* 8.3.3 Intra_16x16_sample_prediction (H264PictureBase.cpp:1847-2059) */
static int pred16x16(const octx *c, int cur, int mode, uint8_t pred[256])
{
    int top[16], left[16], corner = intra_nb(c, cur, 0, 0, -1, -1);
    int ta = 1, la = 1;
    for (int i = 0; i < 16; i++) {
        top[i] = intra_nb(c, cur, 0, 0, i, -1);
        left[i] = intra_nb(c, cur, 0, 0, -1, i);
        if (top[i] < 0) ta = 0;
        if (left[i] < 0) la = 0;
    }
    if (mode == 0) {
        if (!ta) return 0;
        for (int y = 0; y < 16; y++) for (int x = 0; x < 16; x++) pred[y * 16 + x] = (uint8_t)top[x];
    } else if (mode == 1) {
        if (!la) return 0;
        for (int y = 0; y < 16; y++) for (int x = 0; x < 16; x++) pred[y * 16 + x] = (uint8_t)left[y];
    } else if (mode == 2) {
        int st = 0, sl = 0, v;
        for (int i = 0; i < 16; i++) { st += top[i]; sl += left[i]; }
        if (ta && la) v = (st + sl + 16) >> 5;
        else if (la) v = (sl + 8) >> 4;
        else if (ta) v = (st + 8) >> 4;
        else v = 128;
        memset(pred, v, 256);
    } else if (mode == 3) {
        /* quirk: p[-1,-1] is not required; when unavailable its -1 marker
           enters H and V (H264PictureBase.cpp:2014-2030) */
        if (!(ta && la)) return 0;
        int H = 0, V = 0;
        for (int x = 0; x <= 7; x++) H += (x + 1) * (top[8 + x] - (6 - x >= 0 ? top[6 - x] : corner));
        for (int y = 0; y <= 7; y++) V += (y + 1) * (left[8 + y] - (6 - y >= 0 ? left[6 - y] : corner));
        int a = 16 * (left[15] + top[15]);
        int b = (5 * H + 32) >> 6, cc = (5 * V + 32) >> 6;
        for (int y = 0; y < 16; y++)
            for (int x = 0; x < 16; x++) pred[y * 16 + x] = (uint8_t)clip1((a + b * (x - 7) + cc * (y - 7) + 16) >> 5);
    } else {
        return 0;
    }
    return 1;
}

/* 8.3.4 chroma prediction, 4:2:0 (Intra_chroma_sample_prediction_for_YUV420_or_YUV422,
   H264PictureBase.cpp:2076-2385).  Quirk: Intra_Chroma_DC treats a
   neighbouring sample of value 0 as not available (it tests "> 0"). */
static int predchroma(const octx *c, int cur, int pl, int mode, uint8_t pred[64])
{
    int top[8], left[8], corner = intra_nb(c, cur, 1, pl, -1, -1);
    for (int i = 0; i < 8; i++) {
        top[i] = intra_nb(c, cur, 1, pl, i, -1);
        left[i] = intra_nb(c, cur, 1, pl, -1, i);
    }
    if (mode == 0) {
        for (int b = 0; b < 4; b++) {
            int xO = (b & 1) * 4, yO = (b >> 1) * 4;
            int t = top[xO] > 0 && top[xO + 1] > 0 && top[xO + 2] > 0 && top[xO + 3] > 0;
            int l = left[yO] > 0 && left[yO + 1] > 0 && left[yO + 2] > 0 && left[yO + 3] > 0;
            int st = t ? top[xO] + top[xO + 1] + top[xO + 2] + top[xO + 3] : 0;
            int sl = l ? left[yO] + left[yO + 1] + left[yO + 2] + left[yO + 3] : 0;
            int v;
            if ((xO == 0 && yO == 0) || (xO > 0 && yO > 0)) {
                if (t && l) v = (st + sl + 4) >> 3;
                else if (l) v = (sl + 2) >> 2;
                else if (t) v = (st + 2) >> 2;
                else v = 128;
            } else if (xO > 0) {
                if (t) v = (st + 2) >> 2;
                else if (l) v = (sl + 2) >> 2;
                else v = 128;
            } else {
                if (l) v = (sl + 2) >> 2;
                else if (t) v = (st + 2) >> 2;
                else v = 128;
            }
            for (int y = 0; y < 4; y++)
                for (int x = 0; x < 4; x++) pred[(yO + y) * 8 + xO + x] = (uint8_t)v;
        }
    } else if (mode == 1) {
        for (int y = 0; y < 8; y++) if (left[y] < 0) return 0;
        for (int y = 0; y < 8; y++) for (int x = 0; x < 8; x++) pred[y * 8 + x] = (uint8_t)left[y];
    } else if (mode == 2) {
        for (int x = 0; x < 8; x++) if (top[x] < 0) return 0;
        for (int y = 0; y < 8; y++) for (int x = 0; x < 8; x++) pred[y * 8 + x] = (uint8_t)top[x];
    } else if (mode == 3) {
        for (int x = 0; x < 8; x++) if (top[x] < 0) return 0;
        for (int y = 0; y < 8; y++) if (left[y] < 0) return 0;
        if (corner < 0) return 0;
        int H = 0, V = 0;
        for (int x = 0; x <= 3; x++) H += (x + 1) * (top[4 + x] - (2 - x >= 0 ? top[2 - x] : corner));
        for (int y = 0; y <= 3; y++) V += (y + 1) * (left[4 + y] - (2 - y >= 0 ? left[2 - y] : corner));
        int a = 16 * (left[7] + top[7]);
        int b = (34 * H + 32) >> 6, cc = (34 * V + 32) >> 6;
        for (int y = 0; y < 8; y++)
            for (int x = 0; x < 8; x++) pred[y * 8 + x] = (uint8_t)clip1((a + b * (x - 3) + cc * (y - 3) + 16) >> 5);
    } else {
        return 0;
    }
    return 1;
}

/* ---- intra macroblocks -------------------------------------------------- */
static int recon_intra(octx *c, int addr)
{
    const h264r_mb *m = &c->pic->mbs[addr];
    coefs k;
    int rc = parse_coef(c->pic, m, &k);
    if (rc) return rc;
    int x, y, dy;
    mb_origin(c, addr, &x, &y, &dy);
    int field = is_field_mb(c, addr), sf = field_coded(c, addr);
    int qp = m->qpy;
    if (m->type == H264R_MB_I4x4) {
        /* transform_decoding_process_for_4x4_luma_residual_blocks (3401) */
        for (int b = 0; b < 16; b++) {
            int mode = (m->ipred[b >> 3] >> (4 * (b & 7))) & 15;
            uint8_t pred[16];
            int bx = x + kBlkX[b] * 4, by = y + kBlkY[b] * 4 * dy;
            if (pred4x4(c, addr, b, mode, pred)) {
                for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) *lum(c, bx + j, by + i * dy) = pred[i * 4 + j];
            }
            int32_t r[4][4];
            residual4x4(c, k.l4[b], sf, qp, 0, 0, 0, r);
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) { uint8_t *p = lum(c, bx + j, by + i * dy); *p = (uint8_t)clip1(*p + r[i][j]); }
        }
    } else if (m->type == H264R_MB_I8x8) {
        /* transform_decoding_process_for_8x8_luma_residual_blocks (3651) */
        for (int b = 0; b < 4; b++) {
            int mode = (m->ipred[0] >> (4 * b)) & 15;
            uint8_t pred[64];
            int bx = x + (b & 1) * 8, by = y + (b >> 1) * 8 * dy;
            if (pred8x8(c, addr, b, mode, pred)) {
                for (int i = 0; i < 8; i++) for (int j = 0; j < 8; j++) *lum(c, bx + j, by + i * dy) = pred[i * 8 + j];
            }
            int32_t r[8][8];
            residual8x8(c, k.l8[b], sf, qp, 0, r);
            for (int i = 0; i < 8; i++)
                for (int j = 0; j < 8; j++) { uint8_t *p = lum(c, bx + j, by + i * dy); *p = (uint8_t)clip1(*p + r[i][j]); }
        }
    } else {
        /* transform_decoding_process_for_luma_samples_of_Intra_16x16 (3507) */
        int32_t dcY[4][4];
        luma_dc(c, k.dc, sf, qp, dcY);
        int32_t rmb[16][16];
        for (int b = 0; b < 16; b++) {
            int32_t r[4][4];
            residual4x4(c, k.l4[b], sf, qp, 0, 1, dcY[kBlkY[b]][kBlkX[b]], r);
            for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) rmb[kBlkY[b] * 4 + i][kBlkX[b] * 4 + j] = r[i][j];
        }
        uint8_t pred[256];
        if (pred16x16(c, addr, m->i16_mode, pred)) {
            for (int i = 0; i < 16; i++) for (int j = 0; j < 16; j++) *lum(c, x + j, y + i * dy) = pred[i * 16 + j];
        }
        for (int i = 0; i < 16; i++)
            for (int j = 0; j < 16; j++) { uint8_t *p = lum(c, x + j, y + i * dy); *p = (uint8_t)clip1(*p + rmb[i][j]); }
    }
    /* chroma: prediction, then residual (H264PictureBase.cpp:3752-3940) */
    int xc = x / 2, yc = c->pic->mbaff ? ((y >> 4) * 8 + (y & 1)) : y / 2;
    if (c->pic->mbaff && !field) yc = y / 2;
    for (int pl = 0; pl < 2; pl++) {
        uint8_t pred[64];
        if (predchroma(c, addr, pl, m->chroma_mode, pred)) {
            for (int i = 0; i < 8; i++) for (int j = 0; j < 8; j++) *chr(c, pl, xc + j, yc + i * dy) = pred[i * 8 + j];
        }
    }
    chroma_residual(c, addr, &k, 0);
    return 0;
}

static int recon_pcm(octx *c, int addr)
{
    const h264r_mb *m = &c->pic->mbs[addr];
    if (m->aux == H264R_NONE || m->aux >= c->pic->num_pcm) return H264R_ERR_BAD_RECORD;
    const uint8_t *s = c->pic->pcm + (size_t)m->aux * 384;
    int x, y, dy;
    mb_origin(c, addr, &x, &y, &dy);
    /* Sample_construction_process_for_I_PCM_macroblocks (H264PictureBase.cpp:2449) */
    for (int i = 0; i < 256; i++) *lum(c, x + (i % 16), y + dy * (i / 16)) = s[i];
    int xc = x / 2, yc = (y + 1) / 2;
    for (int i = 0; i < 64; i++) {
        *chr(c, 0, xc + (i % 8), yc + dy * (i / 8)) = s[256 + i];
        *chr(c, 1, xc + (i % 8), yc + dy * (i / 8)) = s[320 + i];
    }
    return 0;
}

/* ---- inter prediction --------------------------------------------------- */
/* motion payload lookup: entry index covering 4x4 block (bx, by) */
static int part_of_block(uint16_t shape, int bx, int by)
{
    int mp = shape & 3;
    if (mp == 0) return 0;
    if (mp == 1) return by >> 1;
    if (mp == 2) return bx >> 1;
    int q = (by >> 1) * 2 + (bx >> 1);
    int base = 0;
    for (int i = 0; i < q; i++) {
        int sc = (shape >> (2 + 2 * i)) & 3;
        base += (sc == 0) ? 1 : (sc == 3 ? 4 : 2);
    }
    int sc = (shape >> (2 + 2 * q)) & 3;
    int sx = bx & 1, sy = by & 1;
    if (sc == 0) return base;
    if (sc == 1) return base + sy;
    if (sc == 2) return base + sx;
    return base + sy * 2 + sx;
}

typedef struct {
    const uint8_t *y, *cb, *cr; /* plane origins (field: offset by parity) */
    int ystride, cstride;       /* row stride (field: doubled)              */
    int xmax, xmaxc;            /* clamp bounds used by the reference       */
} refplanes;

/* Reference plane view.  Frame references: the frame.  Field references of
   MBAFF field MBs: the frame's field view, whose PicWidthInSamples is the
   doubled stride (H264PictureBase.cpp:204-227); the reference clamps x to
   that doubled width (quirk, H264InterPrediction.cpp:2363, 2504-2507).
   Field pictures read fields only, clamped to the picture width as 8.4.2.2
   has it (the reference decodes no field picture to follow). */
static int ref_view(const octx *c, int ref, refplanes *rp)
{
    int slot = H264R_REF_SLOT(ref);
    if (slot >= c->nslots || !c->dpb[slot]) return H264R_ERR_BAD_RECORD;
    if (c->fpic && !(ref & H264R_REF_FIELD)) return H264R_ERR_BAD_RECORD;
    const int W = c->fW, H = c->fH, Wc = W / 2, Hc = H / 2;
    const uint8_t *base = c->dpb[slot];
    const uint8_t *cb = base + (size_t)W * H, *cr = cb + (size_t)Wc * Hc;
    if (ref & H264R_REF_FIELD) {
        int bot = (ref & H264R_REF_BOTTOM) ? 1 : 0;
        rp->y = base + bot * W;
        rp->cb = cb + bot * Wc;
        rp->cr = cr + bot * Wc;
        rp->ystride = 2 * W;
        rp->cstride = 2 * Wc;
        rp->xmax = c->fpic ? W - 1 : 2 * W - 1;
        rp->xmaxc = c->fpic ? Wc - 1 : 2 * Wc - 1;
    } else {
        rp->y = base; rp->cb = cb; rp->cr = cr;
        rp->ystride = W; rp->cstride = Wc;
        rp->xmax = W - 1; rp->xmaxc = Wc - 1;
    }
    return 0;
}

/* 8.4.2.2.1 Luma_sample_interpolation_process (H264InterPrediction.cpp:2344-2480) */
static int luma_sample(const refplanes *r, int ymax, int xi, int yi, int xf, int yf)
{
#define S(dx, dy) ((int)r->y[(size_t)CLIP3(0, ymax, yi + (dy)) * r->ystride + CLIP3(0, r->xmax, xi + (dx))])
#define TAP(a, b, c_, d, e, f) ((a) - 5 * (b) + 20 * (c_) + 20 * (d) - 5 * (e) + (f))
    int G = S(0, 0);
    if (xf == 0 && yf == 0) return G;
    int b1 = TAP(S(-2, 0), S(-1, 0), S(0, 0), S(1, 0), S(2, 0), S(3, 0));
    int h1 = TAP(S(0, -2), S(0, -1), S(0, 0), S(0, 1), S(0, 2), S(0, 3));
    int s1 = TAP(S(-2, 1), S(-1, 1), S(0, 1), S(1, 1), S(2, 1), S(3, 1));
    int m1 = TAP(S(1, -2), S(1, -1), S(1, 0), S(1, 1), S(1, 2), S(1, 3));
    int b = clip1((b1 + 16) >> 5), h = clip1((h1 + 16) >> 5), s = clip1((s1 + 16) >> 5), m = clip1((m1 + 16) >> 5);
    int j = 0;
    if ((xf == 2 && yf != 0) || (yf == 2 && xf != 0)) {
        int cc = TAP(S(-2, -2), S(-2, -1), S(-2, 0), S(-2, 1), S(-2, 2), S(-2, 3));
        int dd = TAP(S(-1, -2), S(-1, -1), S(-1, 0), S(-1, 1), S(-1, 2), S(-1, 3));
        int ee = TAP(S(2, -2), S(2, -1), S(2, 0), S(2, 1), S(2, 2), S(2, 3));
        int ff = TAP(S(3, -2), S(3, -1), S(3, 0), S(3, 1), S(3, 2), S(3, 3));
        int j1 = TAP(cc, dd, h1, m1, ee, ff);
        j = clip1((j1 + 512) >> 10);
    }
    int H_ = S(1, 0), M = S(0, 1);
#undef S
#undef TAP
    switch (xf * 4 + yf) {
    case 1: return (G + h + 1) >> 1;      /* d */
    case 2: return h;
    case 3: return (M + h + 1) >> 1;      /* n */
    case 4: return (G + b + 1) >> 1;      /* a */
    case 5: return (b + h + 1) >> 1;      /* e */
    case 6: return (h + j + 1) >> 1;      /* i */
    case 7: return (h + s + 1) >> 1;      /* p */
    case 8: return b;
    case 9: return (b + j + 1) >> 1;      /* f */
    case 10: return j;
    case 11: return (j + s + 1) >> 1;     /* q */
    case 12: return (H_ + b + 1) >> 1;    /* c */
    case 13: return (b + m + 1) >> 1;     /* g */
    case 14: return (j + m + 1) >> 1;     /* k */
    default: return (m + s + 1) >> 1;     /* r */
    }
}

/* 8.4.2.2.2 Chroma_sample_interpolation_process (H264InterPrediction.cpp:2485-2522) */
static int chroma_sample(const uint8_t *pl, int stride, int xmax, int ymax, int xi, int yi, int xf, int yf)
{
    int xa = CLIP3(0, xmax, xi), xb = CLIP3(0, xmax, xi + 1);
    int ya = CLIP3(0, ymax, yi), yb = CLIP3(0, ymax, yi + 1);
    int A = pl[(size_t)ya * stride + xa], B = pl[(size_t)ya * stride + xb];
    int C = pl[(size_t)yb * stride + xa], D = pl[(size_t)yb * stride + xb];
    return ((8 - xf) * (8 - yf) * A + xf * (8 - yf) * B + (8 - xf) * yf * C + xf * yf * D + 32) >> 6;
}

/* 8.4.2.3 weighted sample prediction (Weighted_sample_prediction_process,
   Default_..., _2: H264InterPrediction.cpp:2526-2829).  Quirk: with explicit
   weights and only list 1 in use, luma applies w0/o0 (2756-2771). */
static int weigh(const h264r_weight *w, int comp, int use0, int use1, int p0, int p1)
{
    if (!use0 && !use1) return 0;
    if (!w->weighted) {
        if (use0 && use1) return (p0 + p1 + 1) >> 1;
        return use0 ? p0 : p1;
    }
    int lw = w->log_wd[comp];
    if (use0 && use1)
        return clip1(((p0 * w->w0[comp] + p1 * w->w1[comp] + (1 << lw)) >> (lw + 1)) + ((w->o0[comp] + w->o1[comp] + 1) >> 1));
    int pv = use0 ? p0 : p1;
    int ww, oo;
    if (use0 || comp == 0) { ww = w->w0[comp]; oo = w->o0[comp]; }
    else { ww = w->w1[comp]; oo = w->o1[comp]; }
    if (lw >= 1) return clip1(((pv * ww + (1 << (lw - 1))) >> lw) + oo);
    return clip1(pv * ww + oo);
}

static int recon_inter(octx *c, int addr)
{
    const h264r_picture *pic = c->pic;
    const h264r_mb *m = &pic->mbs[addr];
    if (m->aux == H264R_NONE || (m->aux & 3) || (uint64_t)m->aux + 4 > pic->motion_bytes) return H264R_ERR_BAD_RECORD;
    uint16_t hdr[2];
    memcpy(hdr, pic->motion + m->aux, 4);
    uint16_t shape = hdr[0], count = hdr[1];
    if ((uint64_t)m->aux + 4 + (uint64_t)count * sizeof(h264r_part) > pic->motion_bytes) return H264R_ERR_BAD_RECORD;
    const h264r_part *parts = (const h264r_part *)(pic->motion + m->aux + 4);
    int x, y, dy;
    mb_origin(c, addr, &x, &y, &dy);
    const int field = is_field_mb(c, addr), sf = field_coded(c, addr);
    /* xAL/yAL in the (field) picture the MB predicts from
       (Inter_prediction_process, H264InterPrediction.cpp:574-580); a field
       picture's view is its field already */
    int yAL0 = field ? ((y - (y & 1)) / 2) : y;
    int ymax = field ? c->H / 2 - 1 : c->H - 1;
    int ymaxc = field ? c->Hc / 2 - 1 : c->Hc - 1;
    int bottom_mb = c->pic->mbaff ? (addr & 1) : (c->fpic == 2);
    int xc0 = x / 2, yc0 = field ? (((y >> 4) * 8 + (y & 1))) : y / 2;
    for (int b = 0; b < 16; b++) {
        int bx = b & 3, by = b >> 2; /* raster 4x4 */
        int e = part_of_block(shape, bx, by);
        if (e >= count) return H264R_ERR_BAD_RECORD;
        const h264r_part *p = &parts[e];
        if (p->wt >= pic->num_weights) return H264R_ERR_BAD_RECORD;
        const h264r_weight *w = &pic->weights[p->wt];
        int use[2] = {p->ref[0] >= 0, p->ref[1] >= 0};
        refplanes rp[2];
        int mvcy[2] = {0, 0};
        for (int l = 0; l < 2; l++) {
            if (!use[l]) continue;
            int rc = ref_view(c, p->ref[l], &rp[l]);
            if (rc) return rc;
            /* 8.4.1.4 chroma vector, Table 8-10 (H264InterPrediction.cpp:2006-2047) */
            mvcy[l] = p->mv[l][1];
            if (sf) {
                int refbot = (p->ref[l] & H264R_REF_BOTTOM) ? 1 : 0;
                if (!refbot && bottom_mb) mvcy[l] += 2;
                else if (refbot && !bottom_mb) mvcy[l] -= 2;
            }
        }
        int xAL = x + bx * 4, yAL = yAL0 + by * 4;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                int v[2] = {0, 0};
                for (int l = 0; l < 2; l++) {
                    if (!use[l]) continue;
                    int mvx = p->mv[l][0], mvy = p->mv[l][1];
                    v[l] = luma_sample(&rp[l], ymax, xAL + j + (mvx >> 2), yAL + i + (mvy >> 2), mvx & 3, mvy & 3);
                }
                *lum(c, x + bx * 4 + j, y + (by * 4 + i) * dy) = (uint8_t)weigh(w, 0, use[0], use[1], v[0], v[1]);
            }
        /* chroma 2x2 of this 4x4 */
        for (int pl = 0; pl < 2; pl++)
            for (int i = 0; i < 2; i++)
                for (int j = 0; j < 2; j++) {
                    int v[2] = {0, 0};
                    for (int l = 0; l < 2; l++) {
                        if (!use[l]) continue;
                        int mvx = p->mv[l][0], mvy = mvcy[l];
                        int xi = xAL / 2 + (mvx >> 3) + j, yi = yAL / 2 + (mvy >> 3) + i;
                        const uint8_t *plane = pl ? rp[l].cr : rp[l].cb;
                        v[l] = chroma_sample(plane, rp[l].cstride, rp[l].xmaxc, ymaxc, xi, yi, mvx & 7, mvy & 7);
                    }
                    *chr(c, pl, xc0 + bx * 2 + j, yc0 + (by * 2 + i) * dy) = (uint8_t)weigh(w, 1 + pl, use[0], use[1], v[0], v[1]);
                }
    }
    /* residual (H264InterPrediction.cpp:22-407); inter MBs always run it */
    coefs k;
    int rc = parse_coef(pic, m, &k);
    if (rc) return rc;
    if (m->coef == H264R_NONE) return 0;
    int qp = m->qpy;
    if (m->flags & H264R_MBF_T8x8) {
        for (int b = 0; b < 4; b++) {
            int32_t r[8][8];
            residual8x8(c, k.l8[b], sf, qp, 1, r);
            int bx = x + (b & 1) * 8, by = y + (b >> 1) * 8 * dy;
            for (int i = 0; i < 8; i++)
                for (int j = 0; j < 8; j++) { uint8_t *pp = lum(c, bx + j, by + i * dy); *pp = (uint8_t)clip1(*pp + r[i][j]); }
        }
    } else {
        for (int b = 0; b < 16; b++) {
            int32_t r[4][4];
            residual4x4(c, k.l4[b], sf, qp, 3, 0, 0, r);
            int bx = x + kBlkX[b] * 4, by = y + kBlkY[b] * 4 * dy;
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) { uint8_t *pp = lum(c, bx + j, by + i * dy); *pp = (uint8_t)clip1(*pp + r[i][j]); }
        }
    }
    chroma_residual(c, addr, &k, 3);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* 8.7 deblocking (H264PictureDeblockingFilterProcess.cpp)                  */

typedef struct {
    int mv[2][2];
    int pf[2];    /* PredFlagL0/L1 */
    int id[2];    /* reference identity, -1: none */
} blkmotion;

/* motion data the bS rules read for the 4x4 block containing (xq, yq) of
   MB addr (the reference reads m_MvLX / m_RefIdxLX / m_PredFlagLX through
   the 6.4.13.4 partition index, 1157-1178) */
static void get_motion(const octx *c, int addr, int xq, int yq, blkmotion *o)
{
    const h264r_mb *m = &c->pic->mbs[addr];
    memset(o, 0, sizeof(*o));
    o->id[0] = o->id[1] = -1;
    if (m->type != H264R_MB_INTER || m->aux == H264R_NONE) return;
    uint16_t hdr[2];
    memcpy(hdr, c->pic->motion + m->aux, 4);
    int e = part_of_block(hdr[0], xq >> 2, yq >> 2);
    if (e >= hdr[1]) return;
    const h264r_part *p = (const h264r_part *)(c->pic->motion + m->aux + 4) + e;
    for (int l = 0; l < 2; l++) {
        o->mv[l][0] = p->mv[l][0];
        o->mv[l][1] = p->mv[l][1];
        o->pf[l] = p->ref[l] >= 0;
        o->id[l] = p->dref[l];
    }
}

static int blk4(int x, int y) { return 8 * (y / 8) + 4 * (x / 8) + 2 * ((y % 8) / 4) + ((x % 8) / 4); }

/* returns bS, or -1 when the reference's bS derivation fails (it reaches
   the partition lookup of a macroblock that was never decoded) */
static int derive_bs(const octx *c, int mbP, int mbQ, int xp, int yp, int xq, int yq, int vertical)
{
    const h264r_picture *pic = c->pic;
    const h264r_mb *P = &pic->mbs[mbP], *Q = &pic->mbs[mbQ];
    const int mbaff = pic->mbaff, fpic = c->fpic != 0;
    /* every MB of a field picture is a field MB */
    int fP = ((P->flags & H264R_MBF_FIELD) && mbaff) || fpic, fQ = ((Q->flags & H264R_MBF_FIELD) && mbaff) || fpic;
    int mixed = mbaff && mbP != mbQ && fP != fQ;
    int intraP = is_intra_type(P->type), intraQ = is_intra_type(Q->type);
    int spP = pic->slices[P->slice].slice_type == 3 || pic->slices[P->slice].slice_type == 4;
    int spQ = pic->slices[Q->slice].slice_type == 3 || pic->slices[Q->slice].slice_type == 4;
    /* 994-1310 */
    if (mbP != mbQ) {
        if ((!fP && !fQ && (intraP || intraQ)) || (!fP && !fQ && (spP || spQ)) ||
            ((mbaff || fpic) && vertical && (intraP || intraQ)) || ((mbaff || fpic) && vertical && (spP || spQ)))
            return 4;
    }
    if ((!mixed && (intraP || intraQ)) || (!mixed && (spP || spQ)) ||
        (mixed && !vertical && (intraP || intraQ)) || (mixed && !vertical && (spP || spQ)))
        return 3;
    int bp4 = blk4(xp, yp), bq4 = blk4(xq, yq);
    int bp8 = 2 * (yp / 8) + (xp / 8), bq8 = 2 * (yq / 8) + (xq / 8);
    int nzP = (P->flags & H264R_MBF_T8x8) ? ((P->nz8x8 >> bp8) & 1) : ((P->nz4x4 >> bp4) & 1);
    int nzQ = (Q->flags & H264R_MBF_T8x8) ? ((Q->nz8x8 >> bq8) & 1) : ((Q->nz4x4 >> bq4) & 1);
    if (nzP || nzQ) return 2;
    if (P->type == H264R_MB_NONE || Q->type == H264R_MB_NONE) return -1;
    if (mixed) return 1;
    int mvy_lim = fQ ? 2 : 4;
    blkmotion a, b;
    get_motion(c, mbP, xp, yp, &a);
    get_motion(c, mbQ, xq, yq, &b);
#define DIFF(u, v) (ABS((u)[0] - (v)[0]) >= 4 || ABS((u)[1] - (v)[1]) >= mvy_lim)
    int r0p = a.id[0], r1p = a.id[1], r0q = b.id[0], r1q = b.id[1];
    int np = a.pf[0] + a.pf[1], nq = b.pf[0] + b.pf[1];
    if (!(((r0p == r0q && r1p == r1q) || (r0p == r1q && r1p == r0q)) && np == nq)) return 1;
    if (a.pf[0] && !a.pf[1] && b.pf[0] && !b.pf[1] && DIFF(a.mv[0], b.mv[0])) return 1;
    if (a.pf[0] && !a.pf[1] && !b.pf[0] && b.pf[1] && DIFF(a.mv[0], b.mv[1])) return 1;
    if (!a.pf[0] && a.pf[1] && b.pf[0] && !b.pf[1] && DIFF(a.mv[1], b.mv[0])) return 1;
    if (!a.pf[0] && a.pf[1] && !b.pf[0] && b.pf[1] && DIFF(a.mv[1], b.mv[1])) return 1;
    if (a.pf[0] && a.pf[1] && r0p != r1p && b.pf[0] && b.pf[1] &&
        ((r0q == r0p && r1q == r1p) || (r0q == r1p && r1q == r0p))) {
        if (r0q == r0p && (DIFF(a.mv[0], b.mv[0]) || DIFF(a.mv[1], b.mv[1]))) return 1;
        else if (r0q == r1p && (DIFF(a.mv[1], b.mv[0]) || DIFF(a.mv[0], b.mv[1]))) return 1;
    }
    /* quirk: the condition is parsed as (A || B) && C || D (1289-1298) */
    if (a.pf[0] && a.pf[1] && r0p == r1p && b.pf[0] && b.pf[1] && r0q == r1q && r0q == r0p) {
        if (((DIFF(a.mv[0], b.mv[0]) || DIFF(a.mv[1], b.mv[1])) && DIFF(a.mv[0], b.mv[1])) || DIFF(a.mv[1], b.mv[0]))
            return 1;
    }
#undef DIFF
    return 0;
}

/* 8.7.2.3 / 8.7.2.4 on one line of samples; p[0..3], q[0..3] in/out */
static void filter_line(int *p, int *q, int bS, int chromaEdge, int indexA, int alpha, int beta)
{
    int chromaStyle = chromaEdge;
    if (!(bS != 0 && ABS(p[0] - q[0]) < alpha && ABS(p[1] - p[0]) < beta && ABS(q[1] - q[0]) < beta)) return;
    int ap = ABS(p[2] - p[0]), aq = ABS(q[2] - q[0]);
    int np[3] = {p[0], p[1], p[2]}, nq[3] = {q[0], q[1], q[2]};
    if (bS < 4) {
        int tc0 = kTc0[bS - 1][indexA];
        int tc = chromaStyle ? tc0 + 1 : tc0 + (ap < beta) + (aq < beta);
        int delta = CLIP3(-tc, tc, ((((q[0] - p[0]) << 2) + (p[1] - q[1]) + 4) >> 3));
        np[0] = clip1(p[0] + delta);
        nq[0] = clip1(q[0] - delta);
        if (!chromaStyle && ap < beta) np[1] = (uint8_t)(p[1] + CLIP3(-tc0, tc0, (p[2] + ((p[0] + q[0] + 1) >> 1) - (p[1] << 1)) >> 1));
        if (!chromaStyle && aq < beta) nq[1] = (uint8_t)(q[1] + CLIP3(-tc0, tc0, (q[2] + ((p[0] + q[0] + 1) >> 1) - (q[1] << 1)) >> 1));
    } else {
        if (!chromaStyle && ap < beta && ABS(p[0] - q[0]) < ((alpha >> 2) + 2)) {
            np[0] = (p[2] + 2 * p[1] + 2 * p[0] + 2 * q[0] + q[1] + 4) >> 3;
            np[1] = (p[2] + p[1] + p[0] + q[0] + 2) >> 2;
            np[2] = (2 * p[3] + 3 * p[2] + p[1] + p[0] + q[0] + 4) >> 3;
        } else {
            np[0] = (2 * p[1] + p[0] + q[1] + 2) >> 2;
        }
        if (!chromaStyle && aq < beta && ABS(p[0] - q[0]) < ((alpha >> 2) + 2)) {
            nq[0] = (p[1] + 2 * p[0] + 2 * q[0] + 2 * q[1] + q[2] + 4) >> 3;
            nq[1] = (p[0] + q[0] + q[1] + q[2] + 2) >> 2;
            nq[2] = (2 * q[3] + 3 * q[2] + q[1] + q[0] + p[0] + 4) >> 3;
        } else {
            nq[0] = (2 * q[1] + q[0] + p[1] + 2) >> 2;
        }
    }
    for (int i = 0; i < 3; i++) { p[i] = np[i]; q[i] = nq[i]; }
}

typedef struct {
    octx *c;
    int stopped; /* the reference's filter returned early */
} dbctx;

/* 8.7.1 Filtering_process_for_block_edges (639-840) for one edge of MB cur:
   chroma: 0 luma, 1 Cb, 2 Cr; e: edge offset in samples of the component;
   mbN: mbAddrA/B of the reference (or -1); fieldMode: fieldModeInFrameFilteringFlag */
static void filter_edge(dbctx *d, int cur, int comp, int vertical, int e, int mbN, int fieldMode, int leftMbEdge)
{
    octx *c = d->c;
    if (d->stopped) return;
    const h264r_picture *pic = c->pic;
    const int chroma = comp != 0;
    const int nE = chroma ? 8 : 16;
    uint8_t *plane = comp == 0 ? c->Y : (comp == 1 ? c->Cb : c->Cr);
    const int stride = chroma ? c->cs : c->ys;
    const int ddy = 1 + fieldMode;
    int xI, yI, dyI;
    mb_origin(c, cur, &xI, &yI, &dyI);
    int xP = chroma ? xI / 2 : xI;
    int yP = chroma ? (yI + 1) / 2 : yI;
    const h264r_mb *Q = &pic->mbs[cur];
    const h264r_slice *sq = &pic->slices[Q->slice];
    for (int k = 0; k < nE; k++) {
        int xE = vertical ? e : k, yE = vertical ? k : e;
        size_t qi[4], pi[4];
        for (int i = 0; i < 4; i++) {
            if (vertical) {
                qi[i] = (size_t)(yP + ddy * yE) * stride + (xP + xE + i);
                pi[i] = (size_t)(yP + ddy * yE) * stride + (xP + xE - i - 1);
            } else {
                qi[i] = (size_t)(yP + ddy * (yE + i) - (yE % 2)) * stride + (xP + xE);
                pi[i] = (size_t)(yP + ddy * (yE - i - 1) - (yE % 2)) * stride + (xP + xE);
            }
        }
        /* p-side macroblock and the sample positions inside p / q MBs */
        int mbP = cur, xp0, yp0, xq0, yq0;
        if (vertical) {
            xp0 = xE - 1;
            if (xp0 < 0) {
                if (mbN >= 0) mbP = leftMbEdge ? mbN + (yE % 2) : mbN;
                xp0 += chroma ? 8 : 16;
            }
            yp0 = yE;
            xq0 = xE;
            yq0 = yE;
        } else {
            xp0 = xE;
            yp0 = (yE - 1) - (yE % 2);
            if (yp0 < 0) {
                if (mbN >= 0) mbP = mbN;
                yp0 += chroma ? 8 : 16;
            }
            xq0 = xE;
            yq0 = yE - (yE % 2);
        }
        int sx = chroma ? 2 : 1;
        int bS = derive_bs(c, mbP, cur, xp0 * sx, yp0 * sx, xq0 * sx, yq0 * sx, vertical);
        if (bS < 0) { d->stopped = 1; return; }
        const h264r_mb *P = &pic->mbs[mbP];
        int qPp, qPq;
        if (!chroma) {
            qPp = P->type == H264R_MB_IPCM ? 0 : P->qpy;
            qPq = Q->type == H264R_MB_IPCM ? 0 : Q->qpy;
        } else {
            /* get_chroma_quantisation_parameters2 with this picture's offsets */
            int off = pic->slices[Q->slice].chroma_qp_offset[comp - 1];
            qPp = chroma_qp(P->type == H264R_MB_IPCM ? 0 : P->qpy, off);
            qPq = chroma_qp(Q->type == H264R_MB_IPCM ? 0 : Q->qpy, off);
        }
        int qPav = (qPp + qPq + 1) >> 1;
        int indexA = CLIP3(0, 51, qPav + sq->filter_offset_a);
        int indexB = CLIP3(0, 51, qPav + sq->filter_offset_b);
        int alpha = kAlpha[indexA], beta = kBeta[indexB];
        int p[4], q[4];
        for (int i = 0; i < 4; i++) { p[i] = plane[pi[i]]; q[i] = plane[qi[i]]; }
        filter_line(p, q, bS, chroma, indexA, alpha, beta);
        for (int i = 0; i < 3; i++) { plane[qi[i]] = (uint8_t)q[i]; plane[pi[i]] = (uint8_t)p[i]; }
    }
}

/* Deblocking_filter_process (76-635) */
static int deblock_picture(octx *c)
{
    const h264r_picture *pic = c->pic;
    dbctx d = {c, 0};
    const int W = c->wmb;
    const int mbaff = pic->mbaff;
    for (int cur = 0; cur < (int)pic->num_mbs && !d.stopped; cur++) {
        const h264r_mb *m = &pic->mbs[cur];
        const h264r_slice *s = &pic->slices[m->slice];
        /* 6.4.11.1 neighbouring macroblocks A (-1, 0) and B (0, -1) */
        int xW, yW;
        int mbA = nb_loc(c, cur, -1, 0, 16, 16, &xW, &yW);
        int mbB = nb_loc(c, cur, 0, -1, 16, 16, &xW, &yW);
        int field = mbaff && (m->flags & H264R_MBF_FIELD);
        int idc = s->disable_deblocking_filter_idc;
        int internal = idc != 1;
        int left = !((!mbaff && cur % W == 0) || (mbaff && (cur >> 1) % W == 0) || idc == 1 || (idc == 2 && mbA < 0));
        int top = !((!mbaff && cur < W) || (mbaff && (cur >> 1) < W && field) ||
                    (mbaff && (cur >> 1) < W && !field && (cur % 2) == 0) || idc == 1 || (idc == 2 && mbB < 0));
        int t8 = (m->flags & H264R_MBF_T8x8) != 0;
        int leftMixed = mbaff && cur >= 2 && !field && (pic->mbs[cur - 2].flags & H264R_MBF_FIELD);
        int topDouble = mbaff && (cur % 2) == 0 && cur >= 2 * W && !field && (pic->mbs[cur - 2 * W + 1].flags & H264R_MBF_FIELD);
        /* luma */
        if (left) filter_edge(&d, cur, 0, 1, 0, mbA, field, leftMixed);
        if (internal) {
            if (!t8) filter_edge(&d, cur, 0, 1, 4, mbA, field, 0);
            filter_edge(&d, cur, 0, 1, 8, mbA, field, 0);
            if (!t8) filter_edge(&d, cur, 0, 1, 12, mbA, field, 0);
        }
        if (top) {
            if (topDouble) {
                filter_edge(&d, cur, 0, 0, 0, mbB - 1, 1, 0);
                filter_edge(&d, cur, 0, 0, 1, mbB, 1, 0);
            } else {
                filter_edge(&d, cur, 0, 0, 0, mbB, field, 0);
            }
        }
        if (internal) {
            if (!t8) filter_edge(&d, cur, 0, 0, 4, mbB, field, 0);
            filter_edge(&d, cur, 0, 0, 8, mbB, field, 0);
            if (!t8) filter_edge(&d, cur, 0, 0, 12, mbB, field, 0);
        }
        /* chroma (4:2:0) */
        if (left) {
            filter_edge(&d, cur, 1, 1, 0, mbA, field, leftMixed);
            filter_edge(&d, cur, 2, 1, 0, mbA, field, leftMixed);
        }
        if (internal) {
            filter_edge(&d, cur, 1, 1, 4, mbA, field, 0);
            filter_edge(&d, cur, 2, 1, 4, mbA, field, 0);
        }
        if (top) {
            if (topDouble) {
                filter_edge(&d, cur, 1, 0, 0, mbB, 1, 0);
                filter_edge(&d, cur, 2, 0, 0, mbB, 1, 0);
                filter_edge(&d, cur, 1, 0, 1, mbB, 1, 0);
                filter_edge(&d, cur, 2, 0, 1, mbB, 1, 0);
            } else {
                filter_edge(&d, cur, 1, 0, 0, mbB, field, 0);
                filter_edge(&d, cur, 2, 0, 0, mbB, field, 0);
            }
        }
        if (internal) {
            filter_edge(&d, cur, 1, 0, 4, mbB, field, 0);
            filter_edge(&d, cur, 2, 0, 4, mbB, field, 0);
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
static int setup(octx *c, const h264r_picture *pic, uint8_t *const *dpb, int nslots)
{
    if (!pic || !dpb) return H264R_ERR_INVALID_ARG;
    if (pic->structure > H264R_STRUCT_BOTTOM) return H264R_ERR_BAD_RECORD;
    if (pic->dst_slot >= nslots || !dpb[pic->dst_slot]) return H264R_ERR_INVALID_ARG;
    memset(c, 0, sizeof(*c));
    c->pic = pic;
    c->fpic = pic->structure;
    c->wmb = pic->width_mbs;
    c->hmb = c->fpic ? pic->height_mbs / 2 : pic->height_mbs;
    if (c->fpic && (pic->mbaff || (pic->height_mbs & 1))) return H264R_ERR_BAD_RECORD;
    if (pic->num_mbs != (uint32_t)c->wmb * c->hmb) return H264R_ERR_BAD_RECORD;
    if (pic->mbaff && (c->hmb & 1)) return H264R_ERR_BAD_RECORD;
    c->fW = c->wmb * 16;
    c->fH = pic->height_mbs * 16;
    c->W = c->fW;
    c->H = c->hmb * 16;
    c->Wc = c->W / 2;
    c->Hc = c->H / 2;
    const int bot = c->fpic == H264R_STRUCT_BOTTOM;
    c->ys = c->fpic ? 2 * c->fW : c->fW;
    c->cs = c->ys / 2;
    c->Y = dpb[pic->dst_slot] + (size_t)bot * c->fW;
    c->Cb = dpb[pic->dst_slot] + (size_t)c->fW * c->fH + (size_t)bot * (c->fW / 2);
    c->Cr = c->Cb + (size_t)(c->fW / 2) * (c->fH / 2);
    c->dpb = dpb;
    c->nslots = nslots;
    for (uint32_t i = 0; i < pic->num_mbs; i++) {
        if (pic->mbs[i].slice >= pic->num_slices) return H264R_ERR_BAD_RECORD;
        if (pic->mbs[i].type > H264R_MB_NONE || pic->mbs[i].qpy > 51) return H264R_ERR_BAD_RECORD;
    }
    return 0;
}

int h264o_reconstruct(const h264r_picture *pic, uint8_t *const *dpb, int nslots, uint8_t *pre)
{
    octx c;
    int rc = setup(&c, pic, dpb, nslots);
    if (rc) return rc;
    size_t planes = (size_t)c.fW * c.fH * 3 / 2;
    uint8_t *slot = dpb[pic->dst_slot];
    /* CH264PictureBase::reset clears a reused picture (H264PictureBase.cpp:44-60);
       a field picture clears its own field's lines */
    if (!c.fpic) {
        memset(slot, 0, planes);
    } else {
        for (int r = 0; r < c.H; r++) memset(c.Y + (size_t)r * c.ys, 0, (size_t)c.W);
        for (int r = 0; r < c.Hc; r++) {
            memset(c.Cb + (size_t)r * c.cs, 0, (size_t)c.Wc);
            memset(c.Cr + (size_t)r * c.cs, 0, (size_t)c.Wc);
        }
    }
    for (uint32_t a = 0; a < pic->num_mbs; a++) {
        const h264r_mb *m = &pic->mbs[a];
        switch (m->type) {
        case H264R_MB_INTER: rc = recon_inter(&c, (int)a); break;
        case H264R_MB_IPCM: rc = recon_pcm(&c, (int)a); break;
        case H264R_MB_NONE: rc = 0; break;
        default: rc = recon_intra(&c, (int)a); break;
        }
        if (rc) return rc;
    }
    if (pre) memcpy(pre, slot, planes);
    if (pic->deblock) rc = deblock_picture(&c);
    return rc;
}

int h264o_deblock(const h264r_picture *pic, uint8_t *const *dpb, int nslots)
{
    octx c;
    int rc = setup(&c, pic, dpb, nslots);
    if (rc) return rc;
    return deblock_picture(&c);
}

/* ---------------------------------------------------------------- output */
/* BT.601 limited-range integers with C division (truncation toward zero),
 * clipped, as H264PictureBase.cpp:457-463. */
void h264o_bgr24(int width, int height, const uint8_t *yuv, uint8_t *bgr, int row_bytes, int flip)
{
    const int W = width, H = height;
    for (int y = 0; y < H; y++) {
        uint8_t *row = bgr + (size_t)(flip ? H - 1 - y : y) * row_bytes;
        for (int x = 0; x < W; x++) {
            const int Y = yuv[(size_t)y * W + x];
            const int U = yuv[(size_t)H * W + (size_t)(y / 2) * (W / 2) + x / 2];
            const int V = yuv[(size_t)H * W + (size_t)H * W / 4 + (size_t)(y / 2) * (W / 2) + x / 2];
            const int b = (1164 * (Y - 16) + 2018 * (U - 128)) / 1000;
            const int g = (1164 * (Y - 16) - 813 * (V - 128) - 391 * (U - 128)) / 1000;
            const int r = (1164 * (Y - 16) + 1596 * (V - 128)) / 1000;
            row[3 * x + 0] = (uint8_t)(b < 0 ? 0 : b > 255 ? 255 : b);
            row[3 * x + 1] = (uint8_t)(g < 0 ? 0 : g > 255 ? 255 : g);
            row[3 * x + 2] = (uint8_t)(r < 0 ? 0 : r > 255 ? 255 : r);
        }
    }
}
