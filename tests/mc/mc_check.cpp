// Host check of the motion-compensation helpers of the CUDA kernels
// (h264r_mc.cuh, compiled here as plain C++) against scalar restatements of
// the standard's formulas, as the reference writes them:
//   8.4.2.2.1 luma sample interpolation, Table 8-12
//             (H264InterPrediction.cpp:2344-2480)
//   8.4.2.2.2 chroma sample interpolation (2485-2522)
//   8.4.2.3   weighted sample prediction (2526-2829)
// Every quarter-sample (eighth-sample) position is covered on random and
// extreme windows.  Prints "ok" and exits 0 when every sample matches.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../h264_video_decoder_demo_gb300/csrc/h264r_mc.cuh"

using namespace h264r;

static uint64_t g_state = 0x9E3779B97F4A7C15ull;
static uint32_t rnd()
{
    g_state ^= g_state << 13;
    g_state ^= g_state >> 7;
    g_state ^= g_state << 17;
    return (uint32_t)(g_state >> 11);
}

static int clip1(int v) { return v < 0 ? 0 : (v > 255 ? 255 : v); }
static int tap(int a, int b, int c, int d, int e, int f) { return a - 5 * b + 20 * c + 20 * d - 5 * e + f; }

// window samples: S(x, y) for x = -2..4, y = -2..6 relative to the lane's
// first output sample
struct Win {
    uint8_t s[9][8];
    int S(int x, int y) const { return s[y + 2][x + 2]; }
};

// the luma prediction sample at (x, y) of the lane (x = 0..1, y = 0..3)
static int luma_ref(const Win &w, int x, int y, int xf, int yf)
{
    auto b1 = [&](int yy) { return tap(w.S(x - 2, yy), w.S(x - 1, yy), w.S(x, yy), w.S(x + 1, yy), w.S(x + 2, yy), w.S(x + 3, yy)); };
    auto h1 = [&](int xx) { return tap(w.S(xx, y - 2), w.S(xx, y - 1), w.S(xx, y), w.S(xx, y + 1), w.S(xx, y + 2), w.S(xx, y + 3)); };
    const int G = w.S(x, y);
    const int b = clip1((b1(y) + 16) >> 5), h = clip1((h1(x) + 16) >> 5);
    const int s = clip1((b1(y + 1) + 16) >> 5), m = clip1((h1(x + 1) + 16) >> 5);
    int j1;
    {
        int hb[6];
        for (int k = 0; k < 6; k++) hb[k] = b1(y - 2 + k);
        j1 = tap(hb[0], hb[1], hb[2], hb[3], hb[4], hb[5]);
    }
    const int j = clip1((j1 + 512) >> 10);
    switch (yf * 4 + xf) {
    case 0: return G;                                  // G
    case 1: return (G + b + 1) >> 1;                   // a
    case 2: return b;                                  // b
    case 3: return (b + w.S(x + 1, y) + 1) >> 1;       // c
    case 4: return (G + h + 1) >> 1;                   // d
    case 5: return (b + h + 1) >> 1;                   // e
    case 6: return (b + j + 1) >> 1;                   // f
    case 7: return (b + m + 1) >> 1;                   // g
    case 8: return h;                                  // h
    case 9: return (h + j + 1) >> 1;                   // i
    case 10: return j;                                 // j
    case 11: return (j + m + 1) >> 1;                  // k
    case 12: return (h + w.S(x, y + 1) + 1) >> 1;      // n
    case 13: return (h + s + 1) >> 1;                  // p
    case 14: return (j + s + 1) >> 1;                  // q
    default: return (m + s + 1) >> 1;                  // r
    }
}

static int check_luma(const Win &w)
{
    uint32_t words[18];
    for (int r = 0; r < 9; r++) {
        uint32_t lo = 0, hi = 0;
        for (int c = 0; c < 4; c++) {
            lo |= (uint32_t)w.s[r][c] << (8 * c);
            hi |= (uint32_t)w.s[r][c + 4] << (8 * c);
        }
        words[2 * r] = lo;
        words[2 * r + 1] = hi;
    }
    int bad = 0;
    for (int yf = 0; yf < 4; yf++)
        for (int xf = 0; xf < 4; xf++) {
            uint32_t o0, o1;
            mc_luma_4x2(words, xf, yf, o0, o1);
            for (int i = 0; i < 4; i++)
                for (int k = 0; k < 2; k++) {
                    const int got = (int)(((i < 2 ? o0 : o1) >> (8 * (2 * (i & 1) + k))) & 255u);
                    const int want = luma_ref(w, k, i, xf, yf);
                    if (got != want && bad++ < 5)
                        fprintf(stderr, "luma xf %d yf %d sample (%d, %d): %d != %d\n", xf, yf, k, i, got, want);
                }
        }
    return bad;
}

static int check_chroma(const uint8_t s[3][4])
{
    uint32_t rw[3];
    for (int r = 0; r < 3; r++) rw[r] = s[r][0] | (s[r][1] << 8) | (s[r][2] << 16) | ((uint32_t)s[r][3] << 24);
    int bad = 0;
    for (int yf = 0; yf < 8; yf++)
        for (int xf = 0; xf < 8; xf++) {
            const uint32_t o = mc_chroma_2x2(rw[0], rw[1], rw[2], xf, yf);
            for (int i = 0; i < 2; i++)
                for (int j = 0; j < 2; j++) {
                    const int A = s[i][j], B = s[i][j + 1], C = s[i + 1][j], D = s[i + 1][j + 1];
                    const int want = ((8 - xf) * (8 - yf) * A + xf * (8 - yf) * B + (8 - xf) * yf * C + xf * yf * D + 32) >> 6;
                    const int got = (int)((o >> (8 * (2 * i + j))) & 255u);
                    if (got != want && bad++ < 5) fprintf(stderr, "chroma xf %d yf %d (%d, %d): %d != %d\n", xf, yf, j, i, got, want);
                }
        }
    return bad;
}

// 8.4.2.3.1 / 8.4.2.3.2 as the reference branches (explicit weights with
// only list 1 in use apply w0 / o0 to luma)
static int weigh_ref(const h264r_weight &w, int comp, bool use0, bool use1, int p0, int p1)
{
    if (!use0 && !use1) return 0;
    if (!w.weighted) {
        if (use0 && use1) return (p0 + p1 + 1) >> 1;
        return use0 ? p0 : p1;
    }
    const int lw = w.log_wd[comp];
    if (use0 && use1)
        return clip1(((p0 * w.w0[comp] + p1 * w.w1[comp] + (1 << lw)) >> (lw + 1)) + ((w.o0[comp] + w.o1[comp] + 1) >> 1));
    const int pv = use0 ? p0 : p1;
    const bool first = use0 || comp == 0;
    const int ww = first ? w.w0[comp] : w.w1[comp], oo = first ? w.o0[comp] : w.o1[comp];
    if (lw >= 1) return clip1(((pv * ww + (1 << (lw - 1))) >> lw) + oo);
    return clip1(pv * ww + oo);
}

int main()
{
    int bad = 0;
    // luma: extreme windows, then random ones
    Win w;
    for (int pat = 0; pat < 6; pat++) {
        for (int r = 0; r < 9; r++)
            for (int c = 0; c < 8; c++) {
                int v = 0;
                switch (pat) {
                case 0: v = 0; break;
                case 1: v = 255; break;
                case 2: v = ((r + c) & 1) ? 255 : 0; break;
                case 3: v = (c & 1) ? 255 : 0; break;
                case 4: v = (r & 1) ? 255 : 0; break;
                default: v = ((r * 3 + c * 5) % 7 < 3) ? 255 : 0; break;
                }
                w.s[r][c] = (uint8_t)v;
            }
        bad += check_luma(w);
    }
    for (int t = 0; t < 40000 && bad == 0; t++) {
        const int mode = t % 3;  // full range, near-black / near-white, few levels
        for (int r = 0; r < 9; r++)
            for (int c = 0; c < 8; c++) {
                uint32_t v = rnd() & 255u;
                if (mode == 1) v = (rnd() & 1) ? (v & 7u) : 248u + (v & 7u);
                if (mode == 2) v = (rnd() & 1) ? 0u : 255u;
                w.s[r][c] = (uint8_t)v;
            }
        bad += check_luma(w);
    }
    // chroma
    uint8_t cs[3][4];
    for (int t = 0; t < 20000 && bad == 0; t++) {
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 4; c++) cs[r][c] = (uint8_t)(t < 2 ? 255 * t : rnd() & 255u);
        bad += check_chroma(cs);
    }
    // weighting
    for (int t = 0; t < 400000 && bad == 0; t++) {
        h264r_weight hw;
        memset(&hw, 0, sizeof(hw));
        hw.weighted = (int8_t)(rnd() & 1);
        for (int c = 0; c < 3; c++) {
            hw.log_wd[c] = (int8_t)(rnd() % 8);
            hw.w0[c] = (int16_t)((int)(rnd() % 256) - 128);
            hw.w1[c] = (int16_t)((int)(rnd() % 256) - 128);
            hw.o0[c] = (int16_t)((int)(rnd() % 256) - 128);
            hw.o1[c] = (int16_t)((int)(rnd() % 256) - 128);
        }
        const int comp = (int)(rnd() % 3);
        const bool use0 = rnd() & 1, use1 = rnd() & 1;
        const int p0 = (int)(rnd() & 255u), p1 = (int)(rnd() & 255u);
        const int want = weigh_ref(hw, comp, use0, use1, p0, p1);
        const int got = mc_weigh(mc_weight(hw, comp, use0, use1), p0, p1);
        if (got != want && bad++ < 5)
            fprintf(stderr, "weight comp %d use %d%d p %d %d: %d != %d\n", comp, use0, use1, p0, p1, got, want);
        // two samples at once (dp2a form): the second pair of samples differs
        const int q0 = (int)(rnd() & 255u), q1 = (int)(rnd() & 255u);
        const McWeight mw = mc_weight(hw, comp, use0, use1);
        int g0, g1;
        mc_weigh2(mw, mc_weight_pair(mw), (uint32_t)p0 | ((uint32_t)q0 << 8) | 0xA5000000u,
                  (uint32_t)p1 | ((uint32_t)q1 << 8) | 0x5A0000u, g0, g1);
        const int want1 = weigh_ref(hw, comp, use0, use1, q0, q1);
        if ((g0 != want || g1 != want1) && bad++ < 5)
            fprintf(stderr, "weight pair comp %d use %d%d: %d %d != %d %d\n", comp, use0, use1, g0, g1, want, want1);
    }
    if (bad) {
        printf("%d mismatches\n", bad);
        return 1;
    }
    printf("ok\n");
    return 0;
}
