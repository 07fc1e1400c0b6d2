// h264r_device.cuh — device-side building blocks of the reconstruction
// engine: tables, record access, inverse transforms, interpolation, weighted
// prediction, intra predictors, neighbour derivation and deblocking rules.
//
// Every function restates one process of the reference decoder
// (jfu222/h264_video_decoder_demo, paths relative to its
// h264_video_decoder_demo/ directory) bit for bit, including the places
// where the reference departs from the H.264 text ("quirk").
#pragma once

#include <cstdint>
#include "../../include/h264r.h"

#define H264R_CLIP3(lo, hi, v) ((v) < (lo) ? (lo) : ((v) > (hi) ? (hi) : (v)))

namespace h264r {

__device__ __forceinline__ int clip1(int v) { return min(max(v, 0), 255); }

// ---------------------------------------------------------------- tables
// scan index -> raster index (row*4+col / row*8+col), Table 8-12/8-13
// (H264PictureBase.cpp:4542, 4597).  Compile-time tables; the kernels use
// them packed into words (no table loads in the coefficient loops).
constexpr uint8_t kZigzag4x4[16] = {0, 1, 4, 8, 5, 2, 3, 6, 9, 12, 13, 10, 7, 11, 14, 15};
constexpr uint8_t kField4x4[16] = {0, 4, 1, 8, 12, 5, 9, 13, 2, 6, 10, 14, 3, 7, 11, 15};
constexpr uint8_t kZigzag8x8[64] = {
    0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5,
    12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14, 21, 28,
    35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
    58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};
constexpr uint8_t kField8x8[64] = {
    0, 8, 16, 1, 9, 24, 32, 17, 2, 25, 40, 48, 56, 33, 10, 3,
    18, 41, 49, 57, 26, 11, 4, 19, 34, 42, 50, 58, 27, 12, 5, 20,
    35, 43, 51, 59, 28, 13, 6, 21, 36, 44, 52, 60, 29, 14, 22, 37,
    45, 53, 61, 30, 7, 15, 38, 46, 54, 62, 23, 31, 39, 47, 55, 63};
// 4x4: raster of scan index k in bits 4k..4k+3
constexpr uint64_t pack_scan4(const uint8_t (&t)[16])
{
    uint64_t v = 0;
    for (int k = 0; k < 16; k++) v |= (uint64_t)t[k] << (4 * k);
    return v;
}
// 8x8: raster of scan index 8r + i in bits 6i..6i+5 of word r
constexpr uint64_t pack_scan8(const uint8_t (&t)[64], int r)
{
    uint64_t v = 0;
    for (int i = 0; i < 8; i++) v |= (uint64_t)t[8 * r + i] << (6 * i);
    return v;
}
constexpr uint64_t kZigzag4P = pack_scan4(kZigzag4x4), kField4P = pack_scan4(kField4x4);
__constant__ uint64_t kScan8P[2][8] = {
    {pack_scan8(kZigzag8x8, 0), pack_scan8(kZigzag8x8, 1), pack_scan8(kZigzag8x8, 2), pack_scan8(kZigzag8x8, 3),
     pack_scan8(kZigzag8x8, 4), pack_scan8(kZigzag8x8, 5), pack_scan8(kZigzag8x8, 6), pack_scan8(kZigzag8x8, 7)},
    {pack_scan8(kField8x8, 0), pack_scan8(kField8x8, 1), pack_scan8(kField8x8, 2), pack_scan8(kField8x8, 3),
     pack_scan8(kField8x8, 4), pack_scan8(kField8x8, 5), pack_scan8(kField8x8, 6), pack_scan8(kField8x8, 7)}};
// normAdjust (scaling_functions, H264PictureBase.cpp:4900-4951) per qP % 6
// and position class; the kernels read one packed word per qP % 6 (byte c =
// the value of class c)
constexpr uint8_t kV4[6][3] = {{10, 16, 13}, {11, 18, 14}, {13, 20, 16}, {14, 23, 18}, {16, 25, 20}, {18, 29, 23}};
constexpr uint8_t kV8[6][6] = {{20, 18, 32, 19, 25, 24}, {22, 19, 35, 21, 28, 26}, {26, 23, 42, 24, 33, 31},
                               {28, 25, 45, 26, 35, 33}, {32, 28, 51, 30, 40, 38}, {36, 32, 58, 34, 46, 43}};
template <int N> constexpr uint64_t pack_bytes(const uint8_t (&t)[N])
{
    uint64_t v = 0;
    for (int i = 0; i < N; i++) v |= (uint64_t)t[i] << (8 * i);
    return v;
}
__constant__ uint32_t kV4P[6] = {(uint32_t)pack_bytes(kV4[0]), (uint32_t)pack_bytes(kV4[1]), (uint32_t)pack_bytes(kV4[2]),
                                 (uint32_t)pack_bytes(kV4[3]), (uint32_t)pack_bytes(kV4[4]), (uint32_t)pack_bytes(kV4[5])};
__constant__ uint64_t kV8P[6] = {pack_bytes(kV8[0]), pack_bytes(kV8[1]), pack_bytes(kV8[2]),
                                 pack_bytes(kV8[3]), pack_bytes(kV8[4]), pack_bytes(kV8[5])};
// Table 8-15 (H264PictureBase.cpp:4773-4778)
__device__ const uint8_t kQpc[52] = {
    0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25,
    26, 27, 28, 29, 29, 30, 31, 32, 32, 33, 34, 34, 35, 35, 36, 36, 37, 37, 37, 38, 38, 38, 39, 39, 39, 39};
// Tables 8-16 / 8-17 (H264PictureDeblockingFilterProcess.cpp:1330-1409)
__device__ const uint8_t kAlpha[52] = {
    0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 4, 4, 5, 6, 7, 8, 9, 10, 12, 13,
    15, 17, 20, 22, 25, 28, 32, 36, 40, 45, 50, 56, 63, 71, 80, 90, 101, 113, 127, 144, 162, 182, 203, 226, 255, 255};
__device__ const uint8_t kBeta[52] = {
    0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4,
    6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13, 14, 14, 15, 15, 16, 16, 17, 17, 18, 18};
__device__ const uint8_t kTc0[3][52] = {
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1,
     1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 4, 5, 6, 6, 7, 8, 9, 10, 11, 13},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1,
     1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 5, 5, 6, 7, 8, 8, 10, 11, 12, 13, 15, 17},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1,
     1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 4, 5, 6, 6, 7, 8, 9, 10, 11, 13, 14, 16, 18, 20, 23, 25}};

// ---------------------------------------------------------------- picture
// Device view of one picture of a batch (built by the host for every launch).
// A field picture (PAFF) runs as a picture of its field's size: W x H and
// the MB grid are the field's, the destination planes start on the field's
// first line and step two frame lines (ys, cs); its MBs are field MBs for
// scans, reference views, chroma vectors and strengths (fpic).
struct PicDesc {
    int wmb, hmb;            // picture size in MBs (a field picture: its field)
    int W, H, Wc, Hc;        // picture size in samples
    int ys, cs;              // row pitch of the destination luma / chroma planes
    int fH;                  // frame height in luma samples (DPB slot layout)
    int fpic;                // 0 frame, 1 top field, 2 bottom field
    int mbaff, deblock;
    uint32_t num_mbs, num_slices, num_weights, num_pcm;
    uint32_t motion_bytes, coef_bytes;
    const h264r_mb *mbs;
    const h264r_slice *slices;
    const h264r_weight *weights;
    const uint8_t *motion;
    const uint8_t *coef;
    const uint8_t *pcm;
    const uint8_t *scaling;  // 96 bytes ScalingList4x4 then 384 bytes ScalingList8x8
    uint8_t *dst;            // destination luma origin (slot: Y, then Cb, then Cr)
    int coff, cplane;        // Cb origin - dst, Cr origin - Cb origin (bytes)
    const uint8_t *dpb;      // slot 0 of the stream's DPB
    uint64_t slot_bytes;
    int nslots;
    int flat_scaling;        // every scaling list is flat 16
    uint8_t *bs;             // deblocking strengths, kBsBytes per MB
    int16_t *ires;           // intra MBs' residuals, 384 per MB (null: no intra MB)
    int *progress;           // per unit row progress counters (3 * units_h)
    uint32_t mb_base;        // first global MB index of this picture in the batch
    uint32_t row_base;       // first global unit row of this picture in the batch
    uint32_t units_w, units_h;  // wavefront grid: MBs (or MB pairs) per row, rows
    uint32_t db_base, db_units; // MBAFF deblocking: first ticket of this picture in the batch, ticket count
    uint32_t dbf_base, dbf_units; // frame deblocking: first block ticket, block count
    uint32_t deblock_stop;   // first failing bS derivation key (0xFFFFFFFF: none)
};

// Deblocking tickets of a picture.  Frame pictures (k_deblock_frame): one
// block ticket for the luma and one for the chroma of every kDbWarps pairs
// of MB rows, a warp per pair.  MBAFF pictures (k_deblock): one block ticket
// for the luma and one for the chroma of every kMbWarps MB-pair rows, a
// warp per pair row.
constexpr int kDbWarps = 8;   // MB-row pairs (warps) per frame deblocking block
constexpr int kDbXRing = 16;  // MBs of a warp's bottom lines kept for the warp below
constexpr int kMbWarps = 8;   // MB-pair rows (warps) per MBAFF deblocking block
constexpr int kMbXRing = 8;   // MB pairs of a warp's bottom rows kept for the warp below
constexpr int kBsMbsPerBlock = 8;  // k_bs: 4 warps of 2 MBs per block
__host__ __device__ inline uint32_t deblock_units(int mbaff, uint32_t units_h)
{
    return mbaff ? 2u * ((units_h + kMbWarps - 1u) / kMbWarps) : 0u;
}
// warps: MB-row pairs per block of the launch's kernel (k_deblock_frame:
// kDbWarps, k_deblock_frame4: 4)
__host__ __device__ inline uint32_t deblock_frame_units(int mbaff, uint32_t units_h, uint32_t warps = kDbWarps)
{
    const uint32_t pairs = (units_h + 1u) / 2u;
    return mbaff ? 0u : 2u * ((pairs + warps - 1u) / warps);
}

// Engine-wide device state for one launch.
struct LaunchState {
    int *error;              // first error code (0 ok)
    unsigned int *ticket;    // wavefront tickets: [0] k_intra, [1] k_deblock, [2] k_deblock_frame
    unsigned long long spin_limit;
};

// bS table layout per MB (bytes), line-major so that one load gives a line
// its strengths for every edge: luma vertical [16 rows][4 edges], luma
// horizontal [16 cols][4 edges], extra MBAFF top edge [16], chroma vertical
// [8 rows][2 edges], chroma horizontal [8 cols][2 edges], chroma extra top
// edge [8].  A value of 0xFF marks the place where the reference's bS
// derivation fails.  Edges not filtered (disable_deblocking_filter_idc,
// picture borders, 8x8-transform internal edges) hold 0.
// Frame (non-MBAFF) pictures also get the filter thresholds of each edge
// class at kBsParams: [component][left, top, internal] words of
// alpha | beta << 8 | tC0(bS 1..3) << 16, 21, 26 (8.7.2.2).
// MBAFF pictures use the same 64 bytes at kBsParams for the MB's edge
// controls (a word of kDbc* bits) and 5 threshold words per component
// (indexA | alpha << 8 | beta << 16 of the left edge's even and odd lines,
// the top edge, the second top edge and the internal edges).
constexpr int kBsLumaV = 0, kBsLumaH = 64, kBsLumaTop2 = 128, kBsChromaV = 144, kBsChromaH = 160,
              kBsChromaTop2 = 176, kBsParams = 192, kBsBytes = 256;
constexpr uint32_t kDbcLeft = 1, kDbcTop = 2, kDbcInternal = 4, kDbcT8 = 8, kDbcField = 16, kDbcLeftMixed = 32,
                   kDbcTopDouble = 64;
__device__ __forceinline__ constexpr int bs_lv(int e, int k) { return kBsLumaV + 4 * k + e; }
__device__ __forceinline__ constexpr int bs_lh(int e, int k) { return kBsLumaH + 4 * k + e; }
__device__ __forceinline__ constexpr int bs_cv(int e, int k) { return kBsChromaV + 2 * k + e; }
__device__ __forceinline__ constexpr int bs_ch(int e, int k) { return kBsChromaH + 2 * k + e; }

__device__ __forceinline__ uint8_t *plane_y(const PicDesc &p) { return p.dst; }
// from dst and two offsets (no second pointer kept live in the kernels)
__device__ __forceinline__ uint8_t *plane_c(const PicDesc &p, int pl) { return p.dst + p.coff + (size_t)pl * p.cplane; }

// Inverse_macroblock_scanning_process (H264PictureBase.cpp:2503)
__device__ __forceinline__ void mb_origin(const PicDesc &p, int addr, int &x, int &y, int &dy)
{
    if (!p.mbaff) {
        x = (addr % p.wmb) * 16;
        y = (addr / p.wmb) * 16;
        dy = 1;
    } else {
        int pair = addr >> 1;
        x = (pair % p.wmb) * 16;
        int y0 = (pair / p.wmb) * 32;
        if (p.mbs[addr].flags & H264R_MBF_FIELD) {
            y = y0 + (addr & 1);
            dy = 2;
        } else {
            y = y0 + (addr & 1) * 16;
            dy = 1;
        }
    }
}

__device__ __forceinline__ int field_mb(const PicDesc &p, int addr)
{
    return p.mbaff && (p.mbs[addr].flags & H264R_MBF_FIELD);
}

// field scans and field rules: MBAFF field MBs and every MB of a field picture
__device__ __forceinline__ int field_coded(const PicDesc &p, int addr) { return field_mb(p, addr) | (p.fpic != 0); }

__device__ __forceinline__ int chroma_row0(int y) { return (y >> 4) * 8 + (y & 1); }

__device__ __forceinline__ int chroma_qp(int qpy, int offset) { return kQpc[H264R_CLIP3(0, 51, qpy + offset)]; }

__device__ __forceinline__ bool is_intra_type(int t) { return t == H264R_MB_I4x4 || t == H264R_MB_I8x8 || t == H264R_MB_I16x16; }

// ---------------------------------------------------------------- scaling
// LevelScale4x4(m, 0, 0) of scaling list `list` (8.5.9): the DC position is
// scan index 0 in both scans
__device__ __forceinline__ int level_scale_dc(const PicDesc &p, int list, int m)
{
    const int ws = p.flat_scaling ? 16 : p.scaling[list * 16];
    return ws * (int)(kV4P[m] & 255u);
}

// ---------------------------------------------------------------- transforms
// one 8-point pass of 8.5.13.2
__device__ __forceinline__ void idct8_1d(int x0, int x1, int x2, int x3, int x4, int x5, int x6, int x7, int o[8])
{
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
    o[0] = f0 + f7; o[1] = f2 + f5; o[2] = f4 + f3; o[3] = f6 + f1;
    o[4] = f6 - f1; o[5] = f4 - f3; o[6] = f2 - f5; o[7] = f0 - f7;
}

// 8.5.10 Intra16x16 DC (H264PictureBase.cpp:4993-5088): c raster -> dcY raster.
// Out of line: only Intra16x16 MBs take it, and kept out of k_inter's body it
// leaves that kernel's hot code smaller (its warps wait on instruction fetch;
// measured: 22.4 against 22.8 ms of k_inter per step of the 1080p benchmark).
static __device__ __noinline__ void luma_dc(const PicDesc &p, const int32_t c[16], int field, int qp, int32_t dcY[16])
{
    int32_t g[16];
    for (int j = 0; j < 4; j++) {
        g[0 * 4 + j] = c[0 * 4 + j] + c[1 * 4 + j] + c[2 * 4 + j] + c[3 * 4 + j];
        g[1 * 4 + j] = c[0 * 4 + j] + c[1 * 4 + j] - c[2 * 4 + j] - c[3 * 4 + j];
        g[2 * 4 + j] = c[0 * 4 + j] - c[1 * 4 + j] - c[2 * 4 + j] + c[3 * 4 + j];
        g[3 * 4 + j] = c[0 * 4 + j] - c[1 * 4 + j] + c[2 * 4 + j] - c[3 * 4 + j];
    }
    int ls = level_scale_dc(p, 0, qp % 6);
    for (int i = 0; i < 4; i++) {
        int f0 = g[i * 4 + 0] + g[i * 4 + 1] + g[i * 4 + 2] + g[i * 4 + 3];
        int f1 = g[i * 4 + 0] + g[i * 4 + 1] - g[i * 4 + 2] - g[i * 4 + 3];
        int f2 = g[i * 4 + 0] - g[i * 4 + 1] - g[i * 4 + 2] + g[i * 4 + 3];
        int f3 = g[i * 4 + 0] - g[i * 4 + 1] + g[i * 4 + 2] - g[i * 4 + 3];
        int f[4] = {f0, f1, f2, f3};
        for (int j = 0; j < 4; j++) {
            if (qp >= 36) dcY[i * 4 + j] = (f[j] * ls) << (qp / 6 - 6);
            else dcY[i * 4 + j] = (f[j] * ls + (1 << (5 - qp / 6))) >> (6 - qp / 6);
        }
    }
}

// 8.5.11 chroma DC 4:2:0 (H264PictureBase.cpp:3989-4044); quirk: the
// LevelScale4x4 of the MB's luma list (0 intra / 3 inter) is used
__device__ __forceinline__ void chroma_dc(const PicDesc &p, const int32_t lv[4], int field, int qpc, int ls_list, int32_t dcC[4])
{
    int e00 = lv[0] + lv[2], e01 = lv[1] + lv[3], e10 = lv[0] - lv[2], e11 = lv[1] - lv[3];
    int f[4] = {e00 + e01, e00 - e01, e10 + e11, e10 - e11};
    int ls = level_scale_dc(p, ls_list, qpc % 6);
    for (int i = 0; i < 4; i++) dcC[i] = ((f[i] * ls) << (qpc / 6)) >> 5;
}

// ---------------------------------------------------------------- coefficients
// Payload decode: the block list a lane owns.  Returns the number of
// significance words of the block ahead of it.
struct CoefView {
    uint32_t mask;
    const uint16_t *sig;
    const int16_t *lv;
    int t8;
    int max_levels;  // levels that fit in the payload buffer
};

__device__ __forceinline__ bool coef_view(const PicDesc &p, const h264r_mb &m, CoefView &v)
{
    v.mask = 0;
    v.t8 = (m.flags & H264R_MBF_T8x8) != 0;
    if (m.coef == H264R_NONE) return true;
    if ((m.coef & 3) || (uint64_t)m.coef + 4 > p.coef_bytes) return false;
    const uint8_t *base = p.coef + m.coef;
    v.mask = *(const uint32_t *)base;
    if (v.mask >> 27) return false;
    int nw = __popc(v.mask) + (v.t8 ? 3 * __popc(v.mask & 15u) : 0);
    uint64_t voff = (uint64_t)m.coef + ((4 + 2 * nw + 3) & ~3);
    if (voff > p.coef_bytes) return false;
    v.sig = (const uint16_t *)(base + 4);
    v.lv = (const int16_t *)(p.coef + voff);
    v.max_levels = (int)((p.coef_bytes - voff) / 2);
    return true;
}

// ---------------------------------------------------------------- motion
// entry index covering 4x4 block (bx, by) for a motion payload shape
__device__ __forceinline__ int part_of_block(uint32_t shape, int bx, int by)
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

// ---------------------------------------------------------------- MC
struct RefView {
    const uint8_t *y, *cb, *cr;
    int ystride, cstride, xmax, xmaxc;
};

// frame reference, or field of a frame for MBAFF field MBs; quirk: x is
// clamped to the doubled field-view width (H264InterPrediction.cpp:2363).
// Field pictures clamp x to the picture width, as 8.4.2.2 has it (the
// reference decodes no field picture to follow).
__device__ __forceinline__ RefView ref_view(const PicDesc &p, int ref)
{
    RefView r;
    int slot = ref & 31;
    if (slot >= p.nslots) slot = 0;  // out-of-range slots are rejected on the host; stay in bounds regardless
    const uint8_t *base = p.dpb + (uint64_t)slot * p.slot_bytes;
    const uint8_t *cb = base + (size_t)p.W * p.fH, *cr = cb + (size_t)p.Wc * (p.fH / 2);
    if (ref & H264R_REF_FIELD) {
        int bot = (ref & H264R_REF_BOTTOM) ? 1 : 0;
        r.y = base + bot * p.W;
        r.cb = cb + bot * p.Wc;
        r.cr = cr + bot * p.Wc;
        r.ystride = 2 * p.W;
        r.cstride = 2 * p.Wc;
        r.xmax = p.fpic ? p.W - 1 : 2 * p.W - 1;
        r.xmaxc = p.fpic ? p.Wc - 1 : 2 * p.Wc - 1;
    } else {
        r.y = base; r.cb = cb; r.cr = cr;
        r.ystride = p.W; r.cstride = p.Wc;
        r.xmax = p.W - 1; r.xmaxc = p.Wc - 1;
    }
    return r;
}

// ---------------------------------------------------------------- neighbours
__device__ __forceinline__ bool avail_mb(const PicDesc &p, int cur, int n)
{
    return n >= 0 && n <= cur && p.mbs[n].slice == p.mbs[cur].slice;
}

// 6.4.12.1 (getMbAddrN_non_MBAFF_frames, H264PictureBase.cpp:2878)
__device__ __forceinline__ int nb_loc_frame(const PicDesc &p, int cur, int xN, int yN, int maxW, int maxH, int &xW, int &yW)
{
    int W = p.wmb, n;
    if (xN < 0 && yN < 0) n = (cur % W == 0) ? -1 : cur - W - 1;
    else if (xN < 0 && yN < maxH) n = (cur % W == 0) ? -1 : cur - 1;
    else if (xN < maxW && yN < 0) n = cur - W;
    else if (xN < maxW && yN < maxH) n = cur;
    else if (xN >= maxW && yN < 0) n = ((cur + 1) % W == 0) ? -1 : cur - W + 1;
    else return -1;
    if (n != cur && !avail_mb(p, cur, n)) return -1;
    xW = (xN + maxW) % maxW;
    yW = (yN + maxH) % maxH;
    return n;
}

// 6.4.12.2, Table 6-4 (getMbAddrN_MBAFF_frames, H264PictureBase.cpp:2984-3395)
__device__ inline int nb_loc_mbaff(const PicDesc &p, int cur, int xN, int yN, int maxW, int maxH, int &xW, int &yW)
{
    const int W = p.wmb, pair = cur / 2;
    const h264r_mb *mbs = p.mbs;
    int A = 2 * (pair - 1), B = 2 * (pair - W), C = 2 * (pair - W + 1), D = 2 * (pair - W - 1);
    const int sl = mbs[cur].slice;
    if (A < 0 || A > cur || mbs[A].slice != sl || pair % W == 0) A = -2;
    if (B < 0 || B > cur || mbs[B].slice != sl) B = -2;
    if (C < 0 || C > cur || mbs[C].slice != sl || (pair + 1) % W == 0) C = -2;
    if (D < 0 || D > cur || mbs[D].slice != sl || pair % W == 0) D = -2;
#define FRM(a) (!(mbs[a].flags & H264R_MBF_FIELD))
    const bool frame = FRM(cur), top = (cur % 2) == 0;
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
    xW = (xN + maxW) % maxW;
    yW = (yM + maxH) % maxH;
    return n;
}

__device__ __forceinline__ int nb_loc(const PicDesc &p, int cur, int xN, int yN, int maxW, int maxH, int &xW, int &yW)
{
    if (!p.mbaff) return nb_loc_frame(p, cur, xN, yN, maxW, maxH, xW, yW);
    return nb_loc_mbaff(p, cur, xN, yN, maxW, maxH, xW, yW);
}

// Address of neighbouring constructed sample p[xN, yN] of MB cur, or null
// when it is "not available for Intra prediction" (mbAddrN unavailable, or
// an inter MB under constrained_intra_pred_flag).
__device__ __forceinline__ const uint8_t *intra_nb_ptr(const PicDesc &p, int cur, int isChroma, int pl, int xN, int yN)
{
    int maxW = isChroma ? 8 : 16;
    int xW, yW;
    int n = nb_loc(p, cur, xN, yN, maxW, maxW, xW, yW);
    if (n < 0) return nullptr;
    const h264r_mb &mn = p.mbs[n];
    if (n != cur && mn.type == H264R_MB_INTER && (mn.flags & H264R_MBF_CIP)) return nullptr;
    int x, y, dy;
    mb_origin(p, n, x, y, dy);
    if (!isChroma) return plane_y(p) + (size_t)(y + dy * yW) * p.ys + x + xW;
    return plane_c(p, pl) + (size_t)(chroma_row0(y) + dy * yW) * p.cs + x / 2 + xW;
}

// ---------------------------------------------------------------- byte packing
__device__ __forceinline__ void unpack16(uint4 v, int *d)
{
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 16; i++) d[i] = (w[i >> 2] >> (8 * (i & 3))) & 255;
}

__device__ __forceinline__ uint4 pack16(const int *s)
{
    uint32_t w[4] = {0, 0, 0, 0};
#pragma unroll
    for (int i = 0; i < 16; i++) w[i >> 2] |= (uint32_t)(s[i] & 255) << (8 * (i & 3));
    return make_uint4(w[0], w[1], w[2], w[3]);
}

__device__ __forceinline__ void unpack8(uint2 v, int *d)
{
#pragma unroll
    for (int i = 0; i < 8; i++) d[i] = ((i < 4 ? v.x : v.y) >> (8 * (i & 3))) & 255;
}

__device__ __forceinline__ uint2 pack8(const int *s)
{
    uint32_t a = 0, b = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        a |= (uint32_t)(s[i] & 255) << (8 * i);
        b |= (uint32_t)(s[4 + i] & 255) << (8 * i);
    }
    return make_uint2(a, b);
}

}  // namespace h264r
