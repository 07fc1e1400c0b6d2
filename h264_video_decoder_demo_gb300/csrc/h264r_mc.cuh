// h264r_mc.cuh — motion-compensated prediction of one lane's samples:
// 8.4.2.2.1 luma interpolation of a 4-row x 2-column group
// (Luma_sample_interpolation_process, H264InterPrediction.cpp:2344-2480),
// 8.4.2.2.2 chroma interpolation of a 2x2 group (2485-2522) and the
// 8.4.2.3 weighting of a sample pair (2526-2829).  Host and device code, so
// that the same functions are checked on the CPU against a scalar
// restatement of the standard's formulas.
//
// Luma window of a lane: 9 rows of 8 bytes, two 32-bit words per row; byte
// c of row r is the reference sample (xi - 2 + c, yi - 2 + r), so the
// outputs (xi..xi+1, yi..yi+3) sit at bytes 2..3 of rows 2..5.  Four rows
// per lane instead of two need 9 window rows for 4 output rows, and the
// fractional position only selects which of four components are formed:
//   G  full samples (byte 2, or byte 3 for xFrac 3; row r, or r+1 for yFrac 3)
//   B  horizontal half samples b / s      (row r or r+1)
//   V  vertical half samples h / m        (column x or x+1)
//   J  the centre half sample j
// and the output is the rounded byte average of two of them (a component
// averaged with itself when Table 8-12 names one).  Horizontal 6-tap sums
// are two dp4a of the row's words with the taps shifted to the output
// column; vertical sums are dp4a over column words gathered by byte
// permutes (four rows per word) with the taps shifted to the output row.
// All arithmetic is the reference's, in integers, so the result is bit-exact
// whichever order the taps are summed in.
#pragma once

#include <cstdint>

#include "../../include/h264r.h"

namespace h264r {

__host__ __device__ __forceinline__ uint32_t mc_fshr(uint32_t lo, uint32_t hi, int sh)
{
#ifdef __CUDA_ARCH__
    return __funnelshift_r(lo, hi, sh);
#else
    return sh ? (lo >> sh) | (hi << (32 - sh)) : lo;
#endif
}

// sum over k of unsigned byte k of a times signed byte k of b, plus c
__host__ __device__ __forceinline__ int mc_dp4a(uint32_t a, uint32_t b, int c)
{
#ifdef __CUDA_ARCH__
    int d;
    asm("dp4a.u32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
#else
    int s = c;
    for (int k = 0; k < 4; k++) s += (int)((a >> (8 * k)) & 255u) * (int)(int8_t)((b >> (8 * k)) & 255u);
    return s;
#endif
}

// byte n of the result = byte ((s >> 4n) & 7) of the 8 bytes {b, a}
__host__ __device__ __forceinline__ uint32_t mc_prmt(uint32_t a, uint32_t b, uint32_t s)
{
#ifdef __CUDA_ARCH__
    return __byte_perm(a, b, s);
#else
    const uint64_t v = ((uint64_t)b << 32) | a;
    uint32_t r = 0;
    for (int n = 0; n < 4; n++) r |= (uint32_t)((v >> (8 * ((s >> (4 * n)) & 7))) & 255u) << (8 * n);
    return r;
#endif
}

__host__ __device__ __forceinline__ int mc_clip1(int v) { return v < 0 ? 0 : (v > 255 ? 255 : v); }

// c + signed 16-bit half 0 of a times unsigned byte 0 (lo) / 2 (hi) of b +
// signed half 1 of a times byte 1 / 3 of b
__host__ __device__ __forceinline__ int mc_dp2a(uint32_t a, uint32_t b, int c, bool hi)
{
#ifdef __CUDA_ARCH__
    int d;
    if (hi) asm("dp2a.hi.s32.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    else asm("dp2a.lo.s32.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
#else
    const int sh = hi ? 16 : 0;
    return c + (int)(int16_t)(a & 0xFFFFu) * (int)((b >> sh) & 255u) + (int)(int16_t)(a >> 16) * (int)((b >> (sh + 8)) & 255u);
#endif
}

// per byte (a + b + 1) >> 1
__host__ __device__ __forceinline__ uint32_t mc_avg4(uint32_t a, uint32_t b) { return (a | b) - (((a ^ b) >> 1) & 0x7F7F7F7Fu); }

__host__ __device__ __forceinline__ uint32_t mc_pack4(int a, int b, int c, int d)
{
    return (uint32_t)a | ((uint32_t)b << 8) | ((uint32_t)c << 16) | ((uint32_t)d << 24);
}

// 6-tap (1, -5, 20, 20, -5, 1) as signed bytes, shifted to start at byte
// 0 / 1 of the first word (horizontal: output column 0 / 1) and to start at
// byte 0..3 of a column word (vertical: output row 0..3)
constexpr uint32_t kTap0Lo = 0x1414FB01u, kTap0Hi = 0x000001FBu;  // (1,-5,20,20) (-5,1,0,0)
constexpr uint32_t kTap1Lo = 0x14FB0100u, kTap1Hi = 0x0001FB14u;  // (0,1,-5,20) (20,-5,1,0)
constexpr uint32_t kTap2Lo = 0xFB010000u, kTap2Hi = 0x01FB1414u;  // (0,0,1,-5) (20,20,-5,1)
constexpr uint32_t kTap3Lo = 0x01000000u, kTap3Hi = 0xFB1414FBu;  // (0,0,0,1) (-5,20,20,-5), then 1

// horizontal 6-tap sum of output column k (0, 1) of window row (lo, hi), plus c
__host__ __device__ __forceinline__ int mc_hsum(uint32_t lo, uint32_t hi, int k, int c)
{
    return k ? mc_dp4a(lo, kTap1Lo, mc_dp4a(hi, kTap1Hi, c)) : mc_dp4a(lo, kTap0Lo, mc_dp4a(hi, kTap0Hi, c));
}

// V: the vertical half samples of the 4x2 outputs at window byte 2 + dx of
// every row, packed as two words (rows 0-1, rows 2-3; byte 2i + k).
__host__ __device__ __forceinline__ void mc_vhalf(const uint32_t (&w)[18], int dx, uint32_t &v0, uint32_t &v1)
{
    const uint32_t sel = dx ? 0x43u : 0x32u;  // bytes (2, 3) or (3, 4) of the row's 8 bytes
    uint32_t e[9];
#pragma unroll
    for (int r = 0; r < 9; r++) e[r] = mc_prmt(w[2 * r], w[2 * r + 1], sel);
    // column words: byte j = row 4q + j of output column k
    const uint32_t t01 = mc_prmt(e[0], e[1], 0x5140u), t23 = mc_prmt(e[2], e[3], 0x5140u);
    const uint32_t t45 = mc_prmt(e[4], e[5], 0x5140u), t67 = mc_prmt(e[6], e[7], 0x5140u);
    int h[2][4];
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const uint32_t c0 = mc_prmt(t01, t23, k ? 0x7632u : 0x5410u), c1 = mc_prmt(t45, t67, k ? 0x7632u : 0x5410u);
        h[k][0] = mc_dp4a(c0, kTap0Lo, mc_dp4a(c1, kTap0Hi, 16));
        h[k][1] = mc_dp4a(c0, kTap1Lo, mc_dp4a(c1, kTap1Hi, 16));
        h[k][2] = mc_dp4a(c0, kTap2Lo, mc_dp4a(c1, kTap2Hi, 16));
        h[k][3] = mc_dp4a(c0, kTap3Lo, mc_dp4a(c1, kTap3Hi, mc_dp4a(e[8], k ? 0x100u : 0x1u, 16)));
    }
#define MC_H(i, k) mc_clip1(h[k][i] >> 5)
    v0 = mc_pack4(MC_H(0, 0), MC_H(0, 1), MC_H(1, 0), MC_H(1, 1));
    v1 = mc_pack4(MC_H(2, 0), MC_H(2, 1), MC_H(3, 0), MC_H(3, 1));
#undef MC_H
}

// B: the horizontal half samples of window rows 2 + dy .. 5 + dy
__host__ __device__ __forceinline__ void mc_bhalf(const uint32_t (&w)[18], int dy, uint32_t &b0, uint32_t &b1)
{
    int b[4][2];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t lo = dy ? w[2 * (i + 3)] : w[2 * (i + 2)], hi = dy ? w[2 * (i + 3) + 1] : w[2 * (i + 2) + 1];
        b[i][0] = mc_clip1(mc_hsum(lo, hi, 0, 16) >> 5);
        b[i][1] = mc_clip1(mc_hsum(lo, hi, 1, 16) >> 5);
    }
    b0 = mc_pack4(b[0][0], b[0][1], b[1][0], b[1][1]);
    b1 = mc_pack4(b[2][0], b[2][1], b[3][0], b[3][1]);
}

// J: the centre half samples (vertical 6-tap of the unrounded horizontal sums)
__host__ __device__ __forceinline__ void mc_jhalf(const uint32_t (&w)[18], uint32_t &j0, uint32_t &j1)
{
    int jv[4][2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
        int H[9];
#pragma unroll
        for (int r = 0; r < 9; r++) H[r] = mc_hsum(w[2 * r], w[2 * r + 1], k, 0);
#pragma unroll
        for (int i = 0; i < 4; i++)
            jv[i][k] = mc_clip1((H[i] + H[i + 5] - 5 * (H[i + 1] + H[i + 4]) + 20 * (H[i + 2] + H[i + 3]) + 512) >> 10);
    }
    j0 = mc_pack4(jv[0][0], jv[0][1], jv[1][0], jv[1][1]);
    j1 = mc_pack4(jv[2][0], jv[2][1], jv[3][0], jv[3][1]);
}

// G: full samples at window byte 2 + dx of rows 2 + dy .. 5 + dy
__host__ __device__ __forceinline__ void mc_full(const uint32_t (&w)[18], int dx, int dy, uint32_t &g0, uint32_t &g1)
{
    const uint32_t sel = dx ? 0x43u : 0x32u;
    uint32_t e[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t lo = dy ? w[2 * (i + 3)] : w[2 * (i + 2)], hi = dy ? w[2 * (i + 3) + 1] : w[2 * (i + 2) + 1];
        e[i] = mc_prmt(lo, hi, sel);
    }
    g0 = mc_prmt(e[0], e[1], 0x5410u);
    g1 = mc_prmt(e[2], e[3], 0x5410u);
}

// The 4x2 prediction for quarter-sample fractions (xf, yf) (Table 8-12):
// o0 = rows 0-1, o1 = rows 2-3, byte 2i + k = (column k, row i).
//   (0,0) G      (1|3,0) G B    (2,0) B      (0,1|3) G V    (0,2) V
//   (2,2) J      (2,1|3) B J    (1|3,2) V J  (1|3,1|3) B V
__host__ __device__ __forceinline__ void mc_luma_4x2(const uint32_t (&w)[18], int xf, int yf, uint32_t &o0, uint32_t &o1)
{
    const int dx = xf == 3, dy = yf == 3;
    const bool gc = (xf == 0 || yf == 0) && xf != 2 && yf != 2;
    const bool bc = xf != 0 && yf != 2;
    const bool vc = yf != 0 && xf != 2;
    const bool jc = xf != 0 && yf != 0 && (xf == 2 || yf == 2);
    uint32_t g0 = 0, g1 = 0, b0 = 0, b1 = 0, v0 = 0, v1 = 0, j0 = 0, j1 = 0;
    if (gc) mc_full(w, dx, dy, g0, g1);
    if (bc) mc_bhalf(w, dy, b0, b1);
    if (vc) mc_vhalf(w, dx, v0, v1);
    if (jc) mc_jhalf(w, j0, j1);
    const uint32_t p0 = gc ? g0 : (bc ? b0 : (vc ? v0 : j0)), p1 = gc ? g1 : (bc ? b1 : (vc ? v1 : j1));
    const uint32_t q0 = jc ? j0 : (vc ? v0 : (bc ? b0 : g0)), q1 = jc ? j1 : (vc ? v1 : (bc ? b1 : g1));
    o0 = mc_avg4(p0, q0);
    o1 = mc_avg4(p1, q1);
}

// Chroma 2x2 prediction from three window words (row r: bytes 0..2 = the
// samples (xi..xi+2, yi+r)); eighth-sample fractions xf, yf.  Result byte
// 2i + j = (xi + j, yi + i).
__host__ __device__ __forceinline__ uint32_t mc_chroma_2x2(uint32_t r0, uint32_t r1, uint32_t r2, int xf, int yf)
{
    const uint32_t t = (uint32_t)((8 - xf) * (8 - yf)) | ((uint32_t)(xf * (8 - yf)) << 8);  // taps of row i
    const uint32_t u = (uint32_t)((8 - xf) * yf) | ((uint32_t)(xf * yf) << 8);              // taps of row i + 1
    const int a = mc_dp4a(r0, t, mc_dp4a(r1, u, 32)) >> 6, b = mc_dp4a(r0, t << 8, mc_dp4a(r1, u << 8, 32)) >> 6;
    const int c = mc_dp4a(r1, t, mc_dp4a(r2, u, 32)) >> 6, d = mc_dp4a(r1, t << 8, mc_dp4a(r2, u << 8, 32)) >> 6;
    return mc_pack4(a, b, c, d);
}

// 8.4.2.3 as one formula per partition and component:
// Clip1(((p0 * w0 + p1 * w1 + round) >> shift) + offset), covering default
// prediction (H264InterPrediction.cpp:2526-2560), explicit / implicit
// weighting (2560-2829) and the unused-list cases.  Quirk kept: explicit
// weights with only list 1 in use apply w0 / o0 to luma.
struct McWeight {
    int w0, w1, round, shift, offset;
};

// Branch-free, so that the lanes of a MB mixing one- and two-list
// partitions do not diverge: default prediction weighs a used list 1 (two
// lists: round 1, shift 1); explicit weighting takes w / o of the used
// lists, two lists round 2^logWD and shift logWD + 1 with the mean offset,
// one list round 2^(logWD-1) and shift logWD when logWD >= 1.
__host__ __device__ __forceinline__ McWeight mc_weight(const h264r_weight &w, int comp, bool use0, bool use1)
{
    McWeight m;
    const bool wt = w.weighted != 0, bi = use0 && use1, any = use0 || use1;
    const int lw = w.log_wd[comp];
    const int sw1 = comp == 0 ? w.w0[0] : w.w1[comp];  // list 1 alone: luma takes w0 / o0 (quirk)
    const int so1 = comp == 0 ? w.o0[0] : w.o1[comp];
    m.w0 = use0 ? (wt ? (int)w.w0[comp] : 1) : 0;
    m.w1 = use1 ? (wt ? (bi ? (int)w.w1[comp] : sw1) : 1) : 0;
    m.offset = (wt && any) ? (bi ? (w.o0[comp] + w.o1[comp] + 1) >> 1 : (use0 ? (int)w.o0[comp] : so1)) : 0;
    m.shift = any ? (bi ? (wt ? lw + 1 : 1) : ((wt && lw >= 1) ? lw : 0)) : 0;
    m.round = m.shift ? 1 << (m.shift - 1) : 0;
    return m;
}

__host__ __device__ __forceinline__ int mc_weigh(const McWeight &m, int p0, int p1)
{
    return mc_clip1(((p0 * m.w0 + p1 * m.w1 + m.round) >> m.shift) + m.offset);
}

// mc_weigh of two samples at once: a holds list 0's predictions in bytes 0
// and 1, b list 1's; w the weights as 16-bit halves (w0 | w1 << 16), so that
// one byte permute and two dp2a give both weighted sums
__host__ __device__ __forceinline__ uint32_t mc_weight_pair(const McWeight &m)
{
    return ((uint32_t)m.w0 & 0xFFFFu) | ((uint32_t)m.w1 << 16);
}

__host__ __device__ __forceinline__ void mc_weigh2(const McWeight &m, uint32_t w, uint32_t a, uint32_t b, int &v0, int &v1)
{
    const uint32_t src = mc_prmt(a, b, 0x5140u);  // a0 b0 a1 b1
    v0 = mc_clip1((mc_dp2a(w, src, m.round, false) >> m.shift) + m.offset);
    v1 = mc_clip1((mc_dp2a(w, src, m.round, true) >> m.shift) + m.offset);
}

}  // namespace h264r
