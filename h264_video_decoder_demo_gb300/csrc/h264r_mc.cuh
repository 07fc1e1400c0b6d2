// h264r_mc.cuh — 8.4.2.2.1 luma sample interpolation for a 2x4 group of
// samples from a reference window held in registers
// (Luma_sample_interpolation_process, H264InterPrediction.cpp:2344-2480).
//
// The window of a lane is 7 rows of 12 bytes, three 32-bit words per row:
// byte c of row r is the reference sample (xi - 2 + c, yi - 2 + r), so the
// 2x4 outputs (xi..xi+3, yi..yi+1) sit at bytes 2..5 of rows 2 and 3.  A
// horizontal 6-tap sum over bytes j..j+5 of a row is two funnel shifts of
// the row's words (bytes j..j+3 and j+4..j+7) and two four-way byte dot
// products with the taps (1, -5, 20, 20) and (-5, 1, 0, 0); the same shifted
// word gives the full-sample values of columns j and j+1 for the vertical
// taps.  Column loops stay rolled (only shift amounts depend on the column),
// and the outputs are packed by shifts, so no array is indexed at run time.
// The arithmetic is the reference's, in integers, so the result is
// bit-exact whichever order the taps are summed in.
#pragma once

#include <cstdint>

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

__host__ __device__ __forceinline__ int mc_clip1(int v) { return v < 0 ? 0 : (v > 255 ? 255 : v); }

constexpr uint32_t kTapLo = 0x1414FB01u;  // taps 1, -5, 20, 20 as signed bytes
constexpr uint32_t kTapHi = 0x000001FBu;  // taps -5, 1, 0, 0

// 6-tap sum over bytes j..j+5 of a row given its words shifted by 8*j
__host__ __device__ __forceinline__ int mc_htap(uint32_t a, uint32_t b) { return mc_dp4a(a, kTapLo, mc_dp4a(b, kTapHi, 0)); }

__host__ __device__ __forceinline__ int mc_vtap(int a, int b, int c, int d, int e, int f)
{
    return a - 5 * b + 20 * c + 20 * d - 5 * e + f;
}

// w: the window (21 words), xf / yf: quarter-sample fractions.  Returns the
// predicted samples of rows yi and yi+1 as two words (byte j = column xi+j).
__host__ __device__ __forceinline__ void mc_luma_2x4_w(const uint32_t (&w)[21], int xf, int yf, uint32_t &o0, uint32_t &o1)
{
    o0 = o1 = 0;
    if ((xf | yf) == 0) {  // G
        o0 = mc_fshr(w[6], w[7], 16);
        o1 = mc_fshr(w[9], w[10], 16);
        return;
    }
    if (yf == 0) {  // a, b, c: rows 0 and 1
#pragma unroll 1
        for (int j = 0; j < 4; j++) {
            const int sh = 8 * j;
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int R = 3 * (i + 2);
                const uint32_t A = mc_fshr(w[R], w[R + 1], sh), B = mc_fshr(w[R + 1], w[R + 2], sh);
                const int b = mc_clip1((mc_htap(A, B) + 16) >> 5);
                const int g = (int)((A >> (xf == 3 ? 24 : 16)) & 255u);
                const int v = xf == 2 ? b : (g + b + 1) >> 1;
                (i ? o1 : o0) |= (uint32_t)v << sh;
            }
        }
        return;
    }
    if (xf == 0) {  // d, h, n: column j over rows -2..4
#pragma unroll 1
        for (int j = 0; j < 4; j++) {
            const int sh = 8 * j;
            int G[7];
#pragma unroll
            for (int r = 0; r < 7; r++) G[r] = (int)((mc_fshr(w[3 * r], w[3 * r + 1], sh) >> 16) & 255u);
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int h = mc_clip1((mc_vtap(G[i], G[i + 1], G[i + 2], G[i + 3], G[i + 4], G[i + 5]) + 16) >> 5);
                const int v = yf == 2 ? h : ((yf == 1 ? G[i + 2] : G[i + 3]) + h + 1) >> 1;
                (i ? o1 : o0) |= (uint32_t)v << sh;
            }
        }
        return;
    }
    if (xf == 2 || yf == 2) {  // j, f, q, i, k
#pragma unroll 1
        for (int j = 0; j < 4; j++) {
            const int sh = 8 * j;
            int hb[7], gc[7];  // horizontal sums (b1) and full samples of column j (+1 for k)
#pragma unroll
            for (int r = 0; r < 7; r++) {
                const uint32_t A = mc_fshr(w[3 * r], w[3 * r + 1], sh), B = mc_fshr(w[3 * r + 1], w[3 * r + 2], sh);
                hb[r] = mc_htap(A, B);
                gc[r] = (int)((A >> (xf == 3 ? 24 : 16)) & 255u);
            }
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int jv = mc_clip1((mc_vtap(hb[i], hb[i + 1], hb[i + 2], hb[i + 3], hb[i + 4], hb[i + 5]) + 512) >> 10);
                int v;
                if (xf == 2 && yf == 2) {
                    v = jv;
                } else if (xf == 2) {  // f (row i) / q (row i+1)
                    const int b = mc_clip1(((yf == 3 ? hb[i + 3] : hb[i + 2]) + 16) >> 5);
                    v = (b + jv + 1) >> 1;
                } else {  // i (column j) / k (column j+1)
                    const int h = mc_clip1((mc_vtap(gc[i], gc[i + 1], gc[i + 2], gc[i + 3], gc[i + 4], gc[i + 5]) + 16) >> 5);
                    v = (h + jv + 1) >> 1;
                }
                (i ? o1 : o0) |= (uint32_t)v << sh;
            }
        }
        return;
    }
    // e, g, p, r: b at row i (+1) and h at column j (+1)
#pragma unroll 1
    for (int j = 0; j < 4; j++) {
        const int sh = 8 * j;
        int gc[7];
        uint32_t A2 = 0, A3 = 0, A4 = 0;
#pragma unroll
        for (int r = 0; r < 7; r++) {
            const uint32_t A = mc_fshr(w[3 * r], w[3 * r + 1], sh);
            gc[r] = (int)((A >> (xf == 3 ? 24 : 16)) & 255u);
            if (r == 2) A2 = A;
            if (r == 3) A3 = A;
            if (r == 4) A4 = A;
        }
#pragma unroll
        for (int i = 0; i < 2; i++) {
            // b at window row i+2, or i+3 when yf == 3 (selects, not indexing)
            const bool down = yf == 3;
            const uint32_t A = i == 0 ? (down ? A3 : A2) : (down ? A4 : A3);
            const uint32_t B = mc_fshr(down ? w[3 * (i + 3) + 1] : w[3 * (i + 2) + 1], down ? w[3 * (i + 3) + 2] : w[3 * (i + 2) + 2], sh);
            const int b = mc_clip1((mc_htap(A, B) + 16) >> 5);
            const int h = mc_clip1((mc_vtap(gc[i], gc[i + 1], gc[i + 2], gc[i + 3], gc[i + 4], gc[i + 5]) + 16) >> 5);
            (i ? o1 : o0) |= (uint32_t)((b + h + 1) >> 1) << sh;
        }
    }
}

}  // namespace h264r
