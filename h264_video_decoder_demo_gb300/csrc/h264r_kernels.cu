// h264r_kernels.cu — the reconstruction kernels (sm_103a).
//
//  k_inter     inter MBs (8.4 MC + 8.4.2.3 weighting + 8.5 residual), I_PCM
//              and undecoded MBs; fully parallel over the MBs of a batch.
//  k_intra     intra MBs (8.3 + 8.5) as an anti-diagonal wavefront: one warp
//              per MB row (MB-pair row for MBAFF), each row trailing the row
//              above by two units (the top-right neighbour).
//  k_bs        8.7.2.1 boundary strengths of every edge sample row, fully
//              parallel (bS depends on records only, not on samples).
//  k_deblock   8.7 filtering in the reference's raster order as a wavefront
//              (each MB's top edge filter needs the MB above-right done).
//
// Cross-row waits spin on per-row progress counters with an iteration
// limit; on expiry the kernel records H264R_ERR_DEVICE_TIMEOUT and returns.
#include "h264r_device.cuh"
#include "h264r_mc.cuh"

namespace h264r {

// ------------------------------------------------------------ batch lookup
__device__ __forceinline__ int find_pic_by_mb(const PicDesc *pics, int npics, uint32_t g)
{
    int lo = 0, hi = npics - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pics[mid].mb_base <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int find_pic_by_row(const PicDesc *pics, int npics, uint32_t g)
{
    int lo = 0, hi = npics - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pics[mid].row_base <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int find_pic_by_db(const PicDesc *pics, int npics, uint32_t g)
{
    int lo = 0, hi = npics - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pics[mid].db_base <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// last picture whose first frame-deblocking block is <= g (pictures without
// frame blocks share the next picture's base and are skipped by "last")
__device__ __forceinline__ int find_pic_by_dbf(const PicDesc *pics, int npics, uint32_t g)
{
    int lo = 0, hi = npics - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pics[mid].dbf_base <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void set_error(const LaunchState &st, int code) { atomicCAS(st.error, 0, code); }

__device__ __forceinline__ uint32_t pack4(int a, int b, int c, int d)
{
    return (uint32_t)(a & 255) | ((uint32_t)(b & 255) << 8) | ((uint32_t)(c & 255) << 16) | ((uint32_t)(d & 255) << 24);
}

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int *p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Wait (whole warp) until the global counter *flag >= target, with the last
// value seen cached by the caller (no load when it already satisfies the
// target).  Returns false on timeout or when another block reported an error.
__device__ __forceinline__ bool db_wait(const LaunchState &st, const int *flag, int target, int &seen)
{
    int ok = 1;
    if ((threadIdx.x & 31) == 0 && seen < target) {
        unsigned long long n = 0;
        while ((seen = ld_acquire(flag)) < target) {
            if (++n > st.spin_limit) {
                set_error(st, H264R_ERR_DEVICE_TIMEOUT);
                ok = 0;
                break;
            }
            if (n > 64) {
                if (*(volatile int *)st.error != 0) { ok = 0; break; }
                __nanosleep(32);
            }
        }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    __syncwarp();
    return ok != 0;
}

// Wait (whole warp) until the shared-memory counter *flag >= target, with
// the last value seen cached; bounded like the global waits.
__device__ __forceinline__ bool cta_wait(const LaunchState &st, const int *flag, int target, int &seen)
{
    int ok = 1;
    if ((threadIdx.x & 31) == 0 && seen < target) {
        unsigned long long n = 0;
        while ((seen = *(const volatile int *)flag) < target) {
            if (++n > st.spin_limit) {
                set_error(st, H264R_ERR_DEVICE_TIMEOUT);
                ok = 0;
                break;
            }
            if ((n & 255) == 0 && *(volatile int *)st.error != 0) {
                ok = 0;
                break;
            }
        }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    __syncwarp();
    __threadfence_block();
    return ok != 0;
}

// ======================================================================
// Residual of one macroblock (8.5), whole warp
// ======================================================================
// The significance words of the payload are spread over the lanes and a
// warp prefix sum gives the level index each word starts at; every block
// then scatters its levels, already scaled (8.5.12.1 / 8.5.13.1), into the
// residual tile, and the inverse transforms run in place.  No per-lane
// arrays are indexed at run time.

// 8.5.12.2 on a 4x4 block of the tile (row stride `st`), including the
// final (x + 32) >> 6 (H264PictureBase.cpp:4229-4260)
__device__ __forceinline__ void itrans4_tile(int32_t *b, int st)
{
    int32_t f[16];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int d0 = b[i * st], d1 = b[i * st + 1], d2 = b[i * st + 2], d3 = b[i * st + 3];
        const int e0 = d0 + d2, e1 = d0 - d2, e2 = (d1 >> 1) - d3, e3 = d1 + (d3 >> 1);
        f[i * 4 + 0] = e0 + e3; f[i * 4 + 1] = e1 + e2; f[i * 4 + 2] = e1 - e2; f[i * 4 + 3] = e0 - e3;
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int g0 = f[j] + f[8 + j], g1 = f[j] - f[8 + j];
        const int g2 = (f[4 + j] >> 1) - f[12 + j], g3 = f[4 + j] + (f[12 + j] >> 1);
        b[0 * st + j] = (g0 + g3 + 32) >> 6;
        b[1 * st + j] = (g1 + g2 + 32) >> 6;
        b[2 * st + j] = (g1 - g2 + 32) >> 6;
        b[3 * st + j] = (g0 - g3 + 32) >> 6;
    }
}

// Dequantisation of the levels of one block list (8.5.12.1 / 8.5.13.1),
// prepared once per lane: the normAdjust values of qP % 6 by position class
// and the shifts of qP / 6, so that a level costs a multiply and two shifts.
struct Dequant {
    uint64_t v;  // byte c: normAdjust of position class c
    int lsh, rnd, rsh;
};

// 4x4: qP >= 24 shifts left by qP/6 - 4, else rounds and shifts right by 4 - qP/6
__device__ __forceinline__ Dequant dequant4(int qp)
{
    const int q6 = qp / 6;
    Dequant d;
    d.v = kV4P[qp % 6];
    d.lsh = q6 >= 4 ? q6 - 4 : 0;
    d.rnd = q6 >= 4 ? 0 : 1 << (3 - q6);
    d.rsh = q6 >= 4 ? 0 : 4 - q6;
    return d;
}

// 8x8: qP >= 36 shifts left by qP/6 - 6, else rounds and shifts right by 6 - qP/6
__device__ __forceinline__ Dequant dequant8(int qp)
{
    const int q6 = qp / 6;
    Dequant d;
    d.v = kV8P[qp % 6];
    d.lsh = q6 >= 6 ? q6 - 6 : 0;
    d.rnd = q6 >= 6 ? 0 : 1 << (5 - q6);
    d.rsh = q6 >= 6 ? 0 : 6 - q6;
    return d;
}

__device__ __forceinline__ int dequant(const Dequant &d, int cls, int ws, int level)
{
    const int ls = ws * (int)((d.v >> (8 * cls)) & 255u);
    return (((level * ls) << d.lsh) + d.rnd) >> d.rsh;
}

// position class of raster index rp of a 4x4 block: 0 even row and column,
// 1 odd row and column, 2 otherwise
__device__ __forceinline__ int class4(int rp)
{
    const int t = rp & 5;
    return t == 0 ? 0 : (t == 5 ? 1 : 2);
}

// position class of (i, j) in an 8x8 block (the six normAdjust8x8 cases)
constexpr int norm8_class_of(int i, int j)
{
    return (i % 4 == 0 && j % 4 == 0) ? 0
         : (i % 2 == 1 && j % 2 == 1) ? 1
         : (i % 4 == 2 && j % 4 == 2) ? 2
         : ((i % 4 == 0 && j % 2 == 1) || (i % 2 == 1 && j % 4 == 0)) ? 3
         : ((i % 4 == 0 && j % 4 == 2) || (i % 4 == 2 && j % 4 == 0)) ? 4 : 5;
}
// the class depends on (i & 3, j & 3) only: 3 bits at 3 * (4 (i & 3) + (j & 3))
constexpr uint64_t pack_class8()
{
    uint64_t v = 0;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) v |= (uint64_t)norm8_class_of(i, j) << (3 * (4 * i + j));
    return v;
}
constexpr uint64_t kClass8 = pack_class8();

__device__ __forceinline__ int class8(int rp) { return (int)((kClass8 >> (3 * (((rp >> 1) & 12) | (rp & 3)))) & 7u); }

// res: 384 ints (luma 16x16 raster, Cb 8x8, Cr 8x8); dcs: 32 ints of
// scratch; lev: 512 int16 of scratch (the MB's levels, copied in once).
// ls4 / ls8: LevelScale lists of the luma blocks (intra 0 / 0, inter 3 /
// 1); the chroma blocks use ls4 as well (quirk: the reference scales chroma
// with the LevelScale4x4 it computed last, the luma one,
// H264PictureBase.cpp:3752-3940).  Luma 4x4 blocks (lanes 0-15) and chroma
// AC blocks (lanes 16-23) are scattered and transformed in one pass.
// Returns false for a malformed payload (the residual is then zero).
__device__ bool mb_residual(const PicDesc &p, const h264r_mb &m, int field, int ls4, int ls8, int32_t *res, int32_t *dcs,
                            int16_t *lev)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int4 *res4 = reinterpret_cast<int4 *>(res);
#pragma unroll
    for (int i = 0; i < 3; i++) res4[lane + 32 * i] = make_int4(0, 0, 0, 0);
    CoefView cv;
    const bool ok = coef_view(p, m, cv);
    const uint32_t mask = ok ? cv.mask : 0u;
    if (mask == 0) {
        __syncwarp();
        return ok;
    }
    const int t8 = cv.t8;
    const int nw = __popc(mask) + (t8 ? 3 * __popc(mask & 15u) : 0);
    const uint32_t sw = lane < nw ? (uint32_t)cv.sig[lane] : 0u;
    const int cnt = __popc(sw);
    int inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += t;
    }
    const int off = inc - cnt;
    const int total = __shfl_sync(FULL, inc, 31);  // at most 32 words of 16 bits
    if (total > cv.max_levels) {
        __syncwarp();
        return false;
    }
    for (int i = lane; i < total; i += 32) lev[i] = cv.lv[i];
    __syncwarp();
    auto word_of = [&](int bit) -> int {
        const uint32_t before = mask & ((1u << bit) - 1u);
        return __popc(before) + (t8 ? 3 * __popc(before & 15u) : 0);
    };
    const int qp = m.qpy;
    const bool i16 = m.type == H264R_MB_I16x16;
    const uint64_t scan4 = field ? kField4P : kZigzag4P;
    // ---- Intra16x16 DC (8.5.10)
    if (i16) {
        const int w = word_of(16) & 31;
        const uint32_t sg = (mask & H264R_CM_LUMA_DC) ? __shfl_sync(FULL, sw, w) : 0u;
        const int o = __shfl_sync(FULL, off, w);
        if (lane < 16) {
            const int k = lane;
            dcs[(scan4 >> (4 * k)) & 15u] = ((sg >> k) & 1) ? lev[o + __popc(sg & ((1u << k) - 1u))] : 0;
        }
        __syncwarp();
        if (lane == 0) luma_dc(p, dcs, field, qp, dcs + 16);
        __syncwarp();
    }
    // ---- luma 8x8 levels: lane (b, r) owns scan indices 8r..8r+7 of block b
    if (t8) {
        const int b = lane >> 3, r = lane & 7;
        const int w = (word_of(b) + (r >> 1)) & 31;
        const uint32_t sg = __shfl_sync(FULL, sw, w);
        const int o = __shfl_sync(FULL, off, w);
        if (mask & (1u << b)) {
            const int half = (r & 1) * 8;
            int l = o + __popc(sg & ((1u << half) - 1u));
            uint32_t bits = (sg >> half) & 255u;
            const uint64_t sc = kScan8P[field][r];
            const Dequant dq = dequant8(qp);
            int32_t *blk = res + (b >> 1) * 128 + (b & 1) * 8;
            while (bits) {
                const int t = __ffs(bits) - 1;
                bits &= bits - 1;
                const int rp = (int)((sc >> (6 * t)) & 63u);
                const int ws = p.flat_scaling ? 16 : p.scaling[96 + ls8 * 64 + 8 * r + t];
                blk[(rp >> 3) * 16 + (rp & 7)] = dequant(dq, class8(rp), ws, lev[l++]);
            }
        }
    }
    // ---- 4x4 levels: lanes 0-15 luma block `lane` (unless 8x8), lanes
    // 16-23 chroma AC block (plane (lane-16)>>2, block (lane-16)&3)
    const int pl = ((lane - 16) >> 2) & 1, cb = (lane - 16) & 3;
    const bool chroma_lane = lane >= 16 && lane < 24;
    const bool any_chroma = (mask >> 17) != 0;
    const int bx = (((lane >> 2) & 1) << 1) | (lane & 1), by = (((lane >> 3) & 1) << 1) | ((lane >> 1) & 1);
    const int my_bit = lane < 16 ? lane : (H264R_CM_CB_AC0 + 4 * pl + cb);
    const int wq = word_of(my_bit) & 31, wdc = word_of(17 + pl) & 31;
    const uint32_t sq = __shfl_sync(FULL, sw, wq), sdc = __shfl_sync(FULL, sw, wdc);
    const int oq = __shfl_sync(FULL, off, wq), odc = __shfl_sync(FULL, off, wdc);
    int qpc = qp;
    if (chroma_lane) qpc = chroma_qp(qp, p.slices[min((uint32_t)m.slice, p.num_slices - 1)].chroma_qp_offset[pl]);
    int32_t *blk = lane < 16 ? res + by * 64 + bx * 4 : res + 256 + pl * 64 + (cb >> 1) * 32 + (cb & 1) * 4;
    const int stride = lane < 16 ? 16 : 8;
    {
        uint32_t bits = 0;
        if (lane < 16 ? (!t8 && ((mask >> lane) & 1)) : (chroma_lane && ((mask >> my_bit) & 1))) bits = sq & 0xFFFFu;
        const Dequant dq = dequant4(lane < 16 ? qp : qpc);
        int l = oq;
        // chroma: AC list (a level at position 0 is replaced by the DC below)
        while (bits) {
            const int k = __ffs(bits) - 1;
            bits &= bits - 1;
            const int rp = (int)((scan4 >> (4 * k)) & 15u);
            const int ws = p.flat_scaling ? 16 : p.scaling[ls4 * 16 + k];
            blk[(rp >> 2) * stride + (rp & 3)] = dequant(dq, class4(rp), ws, lev[l++]);
        }
    }
    if (lane < 16 && i16 && !t8) blk[0] = dcs[16 + by * 4 + bx];
    if (chroma_lane && any_chroma) {
        int32_t dc4[4] = {0, 0, 0, 0}, dcC[4];
        if (mask & (1u << (17 + pl))) {
#pragma unroll
            for (int k = 0; k < 4; k++) dc4[k] = ((sdc >> k) & 1) ? lev[odc + __popc(sdc & ((1u << k) - 1u))] : 0;
        }
        chroma_dc(p, dc4, field, qpc, ls4, dcC);
        blk[0] = cb == 0 ? dcC[0] : cb == 1 ? dcC[1] : cb == 2 ? dcC[2] : dcC[3];
    }
    __syncwarp();
    // ---- inverse transforms in place
    if (t8) {
        const int b = lane >> 3, r = lane & 7;
        const int x8 = (b & 1) * 8, y8 = (b >> 1) * 8;
        const bool on = (mask >> b) & 1;
        int o8[8];
        if (on) {
            int32_t *row = res + (y8 + r) * 16 + x8;
            idct8_1d(row[0], row[1], row[2], row[3], row[4], row[5], row[6], row[7], o8);
#pragma unroll
            for (int j = 0; j < 8; j++) row[j] = o8[j];
        }
        __syncwarp();
        if (on) {
            int32_t *col = res + y8 * 16 + x8 + r;
            idct8_1d(col[0], col[16], col[32], col[48], col[64], col[80], col[96], col[112], o8);
#pragma unroll
            for (int i = 0; i < 8; i++) col[i * 16] = (o8[i] + 32) >> 6;
        }
    }
    const bool on4 = lane < 16 ? (!t8 && (((mask >> lane) & 1) || (i16 && dcs[16 + by * 4 + bx] != 0))) : (chroma_lane && any_chroma);
    if (on4) itrans4_tile(blk, stride);
    __syncwarp();
    return ok;
}

// ======================================================================
// K1: inter macroblocks, I_PCM, undecoded macroblocks
// ======================================================================
// One warp per MB, 4 MBs per block.  Lane l predicts the 4x2 luma samples
// in columns 2*(l&1), +1 of 4x4 block l>>1 (raster order within the MB)
// from a 9x8 window of the reference held in registers, and the 2x2 chroma
// samples of the same block in plane l&1, so that the partition, its
// references and its weights are looked up once per lane; residuals come
// from lanes owning whole blocks.
constexpr int kInterWarps = 4;  // 6 blocks (24 warps) per SM: registers capped at 80

struct InterWarpSmem {
    int32_t res[384];      // residual: luma raster 16x16, Cb 8x8, Cr 8x8
    int32_t dcs[32];       // Intra16x16 DC work area
    __align__(16) uint8_t out[384];
    int16_t lev[512];      // the MB's coefficient levels
};


// Reference window of one lane: rows yi-2..yi+6, columns xi-2..xi+5 of a
// luma plane, clamped at the picture edges like 8.4.2.2.1
// (H264InterPrediction.cpp:2344-2363), as 9 rows of 8 bytes (byte c of row
// r holds sample (xi-2+c, yi-2+r); byte 7 is not used).  Away from the edges
// each row is three aligned 32-bit loads and two funnel shifts; the loads
// may read up to five bytes past the window, which stay inside the picture
// slot (the chroma planes and the slot padding follow every luma row).
__device__ __forceinline__ void load_luma_window(const RefView &rv, int ymax, int xi, int yi, uint32_t (&win)[18])
{
    const int x0 = xi - 2, y0 = yi - 2;
    if (x0 >= 0 && xi + 4 <= rv.xmax && y0 >= 0 && yi + 6 <= ymax) {
        const int sh = (x0 & 3) * 8;
        const uint8_t *row = rv.y + (size_t)y0 * rv.ystride + (x0 & ~3);
#pragma unroll
        for (int r = 0; r < 9; r++) {
            const uint32_t *q = (const uint32_t *)(row + (size_t)r * rv.ystride);
            const uint32_t a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
            win[2 * r] = __funnelshift_r(a, b, sh);
            win[2 * r + 1] = __funnelshift_r(b, c, sh);
        }
        return;
    }
#pragma unroll
    for (int r = 0; r < 9; r++) {
        const uint8_t *row = rv.y + (size_t)H264R_CLIP3(0, ymax, y0 + r) * rv.ystride;
        uint32_t w0 = 0, w1 = 0;
#pragma unroll
        for (int c = 0; c < 7; c++) {
            const uint32_t v = __ldg(row + H264R_CLIP3(0, rv.xmax, x0 + c));
            if (c < 4) w0 |= v << (8 * c);
            else w1 |= v << (8 * (c - 4));
        }
        win[2 * r] = w0;
        win[2 * r + 1] = w1;
    }
}

// The 3x3 chroma neighbourhood of the 2x2 samples at (xi, yi) .. (xi+1,
// yi+1) for 8.4.2.2.2 (Chroma_sample_interpolation_process,
// H264InterPrediction.cpp:2485-2522), clamped at the picture edges, in three
// registers (row r: bytes 0..2).
__device__ __forceinline__ void load_chroma_window(const uint8_t *pl, int stride, int xmax, int ymax, int xi, int yi,
                                                   uint32_t (&rw)[3])
{
    if (xi >= 0 && xi + 2 <= xmax && yi >= 0 && yi + 2 <= ymax) {
        const int sh = (xi & 3) * 8;
        const uint8_t *row = pl + (size_t)yi * stride + (xi & ~3);
#pragma unroll
        for (int r = 0; r < 3; r++) {
            const uint32_t *q = (const uint32_t *)(row + (size_t)r * stride);
            rw[r] = __funnelshift_r(__ldg(q), __ldg(q + 1), sh);
        }
    } else {
#pragma unroll
        for (int r = 0; r < 3; r++) {
            const uint8_t *row = pl + (size_t)H264R_CLIP3(0, ymax, yi + r) * stride;
            uint32_t w = 0;
#pragma unroll
            for (int c = 0; c < 3; c++) w |= (uint32_t)__ldg(row + H264R_CLIP3(0, xmax, xi + c)) << (8 * c);
            rw[r] = w;
        }
    }
}


// The MB work of k_inter for blocks of W MBs (one warp each).  The launch
// shape is a tuning choice: k_inter (4 MBs per block) is the default, and
// k_inter2 / k_inter8 are the shapes the autotuner also tries.  Every shape
// keeps 24 warps per SM (registers capped at 80).
template <int W>
__device__ __forceinline__ void inter_body(InterWarpSmem (&smem)[W], const PicDesc *__restrict__ pics, int npics,
                                           uint32_t total_mbs, const LaunchState &st)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t g = blockIdx.x * W + wid;
    if (g >= total_mbs) return;
    InterWarpSmem &s = smem[wid];
    const PicDesc &p = pics[find_pic_by_mb(pics, npics, g)];
    const int addr = (int)(g - p.mb_base);
    const h264r_mb m = p.mbs[addr];
    const int field = field_mb(p, addr);  // geometry: a field MB of an MBAFF frame
    const bool intra = is_intra_type(m.type);
    if (intra && !p.ires) return;
    // ---- residual (8.5) into s.res: one call site for intra and inter MBs
    // (the code of this kernel is kept compact: instruction fetch, not
    // arithmetic or memory, is what its warps wait on)
    if (intra || m.type == H264R_MB_INTER) {
        if (!mb_residual(p, m, field | (p.fpic != 0), intra ? 0 : 3, intra ? 0 : 1, s.res, s.dcs, s.lev) && lane == 0) set_error(st, H264R_ERR_BAD_RECORD);
    }
    if (intra) {
        // intra MB: only its residual, for the intra wavefront (k_intra).
        // Stored clamped to [-255, 255]: Clip1(pred + r) is the same for
        // every r beyond that range.
        uint32_t *dst = (uint32_t *)(p.ires + (size_t)addr * 384);
#pragma unroll
        for (int t = 0; t < 6; t++) {
            const int i = lane + 32 * t;
            const int a = H264R_CLIP3(-255, 255, s.res[2 * i]), b = H264R_CLIP3(-255, 255, s.res[2 * i + 1]);
            dst[i] = ((uint32_t)a & 0xFFFFu) | ((uint32_t)b << 16);
        }
        return;
    }
    int x, y, dy;
    mb_origin(p, addr, x, y, dy);

    if (m.type == H264R_MB_NONE) {
        for (int i = lane; i < 96; i += 32) ((uint32_t *)s.out)[i] = 0;
    } else if (m.type == H264R_MB_IPCM) {
        if (m.aux >= p.num_pcm) { if (lane == 0) set_error(st, H264R_ERR_BAD_RECORD); return; }
        const uint32_t *src = (const uint32_t *)(p.pcm + (size_t)m.aux * 384);
        for (int i = lane; i < 96; i += 32) ((uint32_t *)s.out)[i] = __ldg(src + i);
    } else {
        bool bad = (m.aux & 3) || (uint64_t)m.aux + 4 > p.motion_bytes;
        const uint32_t hdr = bad ? 0 : __ldg((const uint32_t *)(p.motion + m.aux));
        const uint32_t shape = hdr & 0xFFFF, count = hdr >> 16;
        if (bad || count == 0 || (uint64_t)m.aux + 4 + 16ull * count > p.motion_bytes) {
            if (lane == 0) set_error(st, H264R_ERR_BAD_RECORD);
            return;
        }
        const h264r_part *parts = (const h264r_part *)(p.motion + m.aux + 4);
        // Table 8-10 (H264InterPrediction.cpp:2006-2047): a field MB (MBAFF
        // field MB or field picture) moves the chroma vector of a reference
        // field of the other parity by +2 (bottom MB, top field) or -2 (top
        // MB, bottom field)
        const int cadj = (field || p.fpic) ? ((p.mbaff ? (addr & 1) : (p.fpic == 2)) ? 2 : -2) : 0;
        const int yAL0 = field ? (y - (y & 1)) / 2 : y;
        const int ymax = field ? p.H / 2 - 1 : p.H - 1;
        const int ymaxc = field ? p.Hc / 2 - 1 : p.Hc - 1;
        const int blk = lane >> 1, half = lane & 1, bx = blk & 3, by = blk >> 2;
        int e = part_of_block(shape, bx, by);
        if (e >= (int)count) e = 0;
        const h264r_part pp = parts[e];
        const bool use0 = pp.ref[0] >= 0, use1 = pp.ref[1] >= 0;
        // predictions of list 0 / 1: luma rows 0-1 and 2-3 (byte 2i + k),
        // chroma 2x2 of plane `half` (byte 2i + j)
        uint32_t ya0 = 0, ya1 = 0, yb0 = 0, yb1 = 0, ca = 0, cb = 0;
#pragma unroll 1
        for (int l = 0; l < 2; l++) {
            if (!(l ? use1 : use0)) continue;
            const int ref = l ? pp.ref[1] : pp.ref[0];
            const int mvx = l ? pp.mv[1][0] : pp.mv[0][0], mvy = l ? pp.mv[1][1] : pp.mv[0][1];
            const RefView rv = ref_view(p, ref);
            uint32_t win[18];
            load_luma_window(rv, ymax, x + bx * 4 + 2 * half + (mvx >> 2), yAL0 + by * 4 + (mvy >> 2), win);
            int cmvy = mvy;
            if ((cadj > 0) != ((ref & H264R_REF_BOTTOM) != 0) && cadj != 0) cmvy += cadj;
            // the chroma loads are issued before the luma arithmetic, which
            // hides their latency
            uint32_t cw[3];
            load_chroma_window(half ? rv.cr : rv.cb, rv.cstride, rv.xmaxc, ymaxc, x / 2 + bx * 2 + (mvx >> 3),
                               yAL0 / 2 + by * 2 + (cmvy >> 3), cw);
            uint32_t o0, o1;
            mc_luma_4x2(win, mvx & 3, mvy & 3, o0, o1);
            const uint32_t c = mc_chroma_2x2(cw[0], cw[1], cw[2], mvx & 7, cmvy & 7);
            if (l) { yb0 = o0; yb1 = o1; cb = c; } else { ya0 = o0; ya1 = o1; ca = c; }
        }
        // ---- weighting (8.4.2.3) and residual, two samples per row
        const h264r_weight wt = p.weights[pp.wt < p.num_weights ? pp.wt : 0];
        {
            const McWeight mw = mc_weight(wt, 0, use0, use1);
            const uint32_t wp = mc_weight_pair(mw);
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const uint32_t a = (i < 2 ? ya0 : ya1) >> (16 * (i & 1)), b = (i < 2 ? yb0 : yb1) >> (16 * (i & 1));
                const int o = (by * 4 + i) * 16 + bx * 4 + 2 * half;
                const int2 r = *(const int2 *)&s.res[o];
                int v0, v1;
                mc_weigh2(mw, wp, a, b, v0, v1);
                *(uint16_t *)&s.out[o] = (uint16_t)(clip1(v0 + r.x) | (clip1(v1 + r.y) << 8));
            }
        }
        {
            const McWeight mw = mc_weight(wt, 1 + half, use0, use1);
            const uint32_t wp = mc_weight_pair(mw);
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const uint32_t a = ca >> (16 * i), b = cb >> (16 * i);
                const int o = 256 + half * 64 + (by * 2 + i) * 8 + bx * 2;
                const int2 r = *(const int2 *)&s.res[o];
                int v0, v1;
                mc_weigh2(mw, wp, a, b, v0, v1);
                *(uint16_t *)&s.out[o] = (uint16_t)(clip1(v0 + r.x) | (clip1(v1 + r.y) << 8));
            }
        }
    }
    __syncwarp();
    // ---- store: 16 luma rows of 16 bytes, 2 x 8 chroma rows of 8 bytes
    if (lane < 16) {
        *(uint4 *)(plane_y(p) + (size_t)(y + lane * dy) * p.ys + x) = *(const uint4 *)(s.out + lane * 16);
    } else {
        const int pl = (lane - 16) >> 3, r = (lane - 16) & 7;
        *(uint2 *)(plane_c(p, pl) + (size_t)(chroma_row0(y) + r * dy) * p.cs + x / 2) = *(const uint2 *)(s.out + 256 + pl * 64 + r * 8);
    }
}

__global__ void __launch_bounds__(32 * kInterWarps, 24 / kInterWarps) k_inter(const PicDesc *__restrict__ pics, int npics,
                                                                             uint32_t total_mbs, LaunchState st)
{
    __shared__ InterWarpSmem smem[kInterWarps];
    inter_body<kInterWarps>(smem, pics, npics, total_mbs, st);
}

__global__ void __launch_bounds__(64, 12) k_inter2(const PicDesc *__restrict__ pics, int npics, uint32_t total_mbs, LaunchState st)
{
    __shared__ InterWarpSmem smem[2];
    inter_body<2>(smem, pics, npics, total_mbs, st);
}

__global__ void __launch_bounds__(256, 3) k_inter8(const PicDesc *__restrict__ pics, int npics, uint32_t total_mbs, LaunchState st)
{
    __shared__ InterWarpSmem smem[8];
    inter_body<8>(smem, pics, npics, total_mbs, st);
}

// ======================================================================
// K2: intra macroblocks, wavefront
// ======================================================================
// Intra_4x4 prediction (8.3.1.2.1 - 8.3.1.2.9, H264PictureBase.cpp:1062-1419)
// as one formula: every sample of every mode but DC is
// (w0*E[i0] + w1*E[i1] + w2*E[i2] + 2) >> 2 over E = {p[-1,-1], p[-1,0..3],
// p[0..7,-1]} (a single sample is w = 4,0,0; a two-tap average 2,2,0; the
// three-tap filter 1,2,1; the two corner cases 1,3,0).  Entry [mode][4y+x]:
// i0 | i1 << 4 | i2 << 8 | w0 << 12 | w1 << 15 | w2 << 18, derived from the
// mode formulas and checked against them sample by sample.
__constant__ uint32_t kPred4[9][16] = {
    {0x04005, 0x04006, 0x04007, 0x04008, 0x04005, 0x04006, 0x04007, 0x04008, 0x04005, 0x04006, 0x04007, 0x04008, 0x04005, 0x04006, 0x04007, 0x04008},
    {0x04001, 0x04001, 0x04001, 0x04001, 0x04002, 0x04002, 0x04002, 0x04002, 0x04003, 0x04003, 0x04003, 0x04003, 0x04004, 0x04004, 0x04004, 0x04004},
    {0x00000, 0x00000, 0x00000, 0x00000, 0x00000, 0x00000, 0x00000, 0x00000, 0x00000, 0x00000, 0x00000, 0x00000, 0x00000, 0x00000, 0x00000, 0x00000},
    {0x51765, 0x51876, 0x51987, 0x51a98, 0x51876, 0x51987, 0x51a98, 0x51ba9, 0x51987, 0x51a98, 0x51ba9, 0x51cba, 0x51a98, 0x51ba9, 0x51cba, 0x190cb},
    {0x51105, 0x51650, 0x51765, 0x51876, 0x51210, 0x51105, 0x51650, 0x51765, 0x51321, 0x51210, 0x51105, 0x51650, 0x51432, 0x51321, 0x51210, 0x51105},
    {0x12050, 0x12065, 0x12076, 0x12087, 0x51501, 0x51650, 0x51765, 0x51876, 0x51012, 0x12050, 0x12065, 0x12076, 0x51123, 0x51501, 0x51650, 0x51765},
    {0x12010, 0x51501, 0x51056, 0x51567, 0x12021, 0x51210, 0x12010, 0x51501, 0x12032, 0x51321, 0x12021, 0x51210, 0x12043, 0x51432, 0x12032, 0x51321},
    {0x12065, 0x12076, 0x12087, 0x12098, 0x51765, 0x51876, 0x51987, 0x51a98, 0x12076, 0x12087, 0x12098, 0x120a9, 0x51876, 0x51987, 0x51a98, 0x51ba9},
    {0x12021, 0x51321, 0x12032, 0x51432, 0x12032, 0x51432, 0x12043, 0x19043, 0x12043, 0x19043, 0x04004, 0x04004, 0x04004, 0x04004, 0x04004, 0x04004},
};

// Intra_8x8 prediction (8.3.2.2.2 - 8.3.2.2.10, H264PictureBase.cpp:1600-1846)
// in the same form over the filtered E = {p'[-1,-1], p'[-1,0..7],
// p'[0..15,-1]}: entry [mode][8y+x] = i0 | i1 << 5 | i2 << 10 | w0 << 15 |
// w1 << 18 | w2 << 21.  Global memory: the 32 lanes of a warp read 32
// consecutive entries.
__device__ const uint32_t kPred8[9][64] = {
    {0x020009, 0x02000a, 0x02000b, 0x02000c, 0x02000d, 0x02000e, 0x02000f, 0x020010, 0x020009, 0x02000a, 0x02000b, 0x02000c, 0x02000d, 0x02000e, 0x02000f, 0x020010, 0x020009, 0x02000a, 0x02000b, 0x02000c, 0x02000d, 0x02000e, 0x02000f, 0x020010, 0x020009, 0x02000a, 0x02000b, 0x02000c, 0x02000d, 0x02000e, 0x02000f, 0x020010, 0x020009, 0x02000a, 0x02000b, 0x02000c, 0x02000d, 0x02000e, 0x02000f, 0x020010, 0x020009, 0x02000a, 0x02000b, 0x02000c, 0x02000d, 0x02000e, 0x02000f, 0x020010, 0x020009, 0x02000a, 0x02000b, 0x02000c, 0x02000d, 0x02000e, 0x02000f, 0x020010, 0x020009, 0x02000a, 0x02000b, 0x02000c, 0x02000d, 0x02000e, 0x02000f, 0x020010},
    {0x020001, 0x020001, 0x020001, 0x020001, 0x020001, 0x020001, 0x020001, 0x020001, 0x020002, 0x020002, 0x020002, 0x020002, 0x020002, 0x020002, 0x020002, 0x020002, 0x020003, 0x020003, 0x020003, 0x020003, 0x020003, 0x020003, 0x020003, 0x020003, 0x020004, 0x020004, 0x020004, 0x020004, 0x020004, 0x020004, 0x020004, 0x020004, 0x020005, 0x020005, 0x020005, 0x020005, 0x020005, 0x020005, 0x020005, 0x020005, 0x020006, 0x020006, 0x020006, 0x020006, 0x020006, 0x020006, 0x020006, 0x020006, 0x020007, 0x020007, 0x020007, 0x020007, 0x020007, 0x020007, 0x020007, 0x020007, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008},
    {0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000, 0x000000},
    {0x28ad49, 0x28b16a, 0x28b58b, 0x28b9ac, 0x28bdcd, 0x28c1ee, 0x28c60f, 0x28ca30, 0x28b16a, 0x28b58b, 0x28b9ac, 0x28bdcd, 0x28c1ee, 0x28c60f, 0x28ca30, 0x28ce51, 0x28b58b, 0x28b9ac, 0x28bdcd, 0x28c1ee, 0x28c60f, 0x28ca30, 0x28ce51, 0x28d272, 0x28b9ac, 0x28bdcd, 0x28c1ee, 0x28c60f, 0x28ca30, 0x28ce51, 0x28d272, 0x28d693, 0x28bdcd, 0x28c1ee, 0x28c60f, 0x28ca30, 0x28ce51, 0x28d272, 0x28d693, 0x28dab4, 0x28c1ee, 0x28c60f, 0x28ca30, 0x28ce51, 0x28d272, 0x28d693, 0x28dab4, 0x28ded5, 0x28c60f, 0x28ca30, 0x28ce51, 0x28d272, 0x28d693, 0x28dab4, 0x28ded5, 0x28e2f6, 0x28ca30, 0x28ce51, 0x28d272, 0x28d693, 0x28dab4, 0x28ded5, 0x28e2f6, 0x0c8317},
    {0x288409, 0x28a920, 0x28ad49, 0x28b16a, 0x28b58b, 0x28b9ac, 0x28bdcd, 0x28c1ee, 0x288820, 0x288409, 0x28a920, 0x28ad49, 0x28b16a, 0x28b58b, 0x28b9ac, 0x28bdcd, 0x288c41, 0x288820, 0x288409, 0x28a920, 0x28ad49, 0x28b16a, 0x28b58b, 0x28b9ac, 0x289062, 0x288c41, 0x288820, 0x288409, 0x28a920, 0x28ad49, 0x28b16a, 0x28b58b, 0x289483, 0x289062, 0x288c41, 0x288820, 0x288409, 0x28a920, 0x28ad49, 0x28b16a, 0x2898a4, 0x289483, 0x289062, 0x288c41, 0x288820, 0x288409, 0x28a920, 0x28ad49, 0x289cc5, 0x2898a4, 0x289483, 0x289062, 0x288c41, 0x288820, 0x288409, 0x28a920, 0x28a0e6, 0x289cc5, 0x2898a4, 0x289483, 0x289062, 0x288c41, 0x288820, 0x288409},
    {0x090120, 0x090149, 0x09016a, 0x09018b, 0x0901ac, 0x0901cd, 0x0901ee, 0x09020f, 0x28a401, 0x28a920, 0x28ad49, 0x28b16a, 0x28b58b, 0x28b9ac, 0x28bdcd, 0x28c1ee, 0x288022, 0x090120, 0x090149, 0x09016a, 0x09018b, 0x0901ac, 0x0901cd, 0x0901ee, 0x288443, 0x28a401, 0x28a920, 0x28ad49, 0x28b16a, 0x28b58b, 0x28b9ac, 0x28bdcd, 0x288864, 0x288022, 0x090120, 0x090149, 0x09016a, 0x09018b, 0x0901ac, 0x0901cd, 0x288c85, 0x288443, 0x28a401, 0x28a920, 0x28ad49, 0x28b16a, 0x28b58b, 0x28b9ac, 0x2890a6, 0x288864, 0x288022, 0x090120, 0x090149, 0x09016a, 0x09018b, 0x0901ac, 0x2894c7, 0x288c85, 0x288443, 0x28a401, 0x28a920, 0x28ad49, 0x28b16a, 0x28b58b},
    {0x090020, 0x28a401, 0x28812a, 0x28a54b, 0x28a96c, 0x28ad8d, 0x28b1ae, 0x28b5cf, 0x090041, 0x288820, 0x090020, 0x28a401, 0x28812a, 0x28a54b, 0x28a96c, 0x28ad8d, 0x090062, 0x288c41, 0x090041, 0x288820, 0x090020, 0x28a401, 0x28812a, 0x28a54b, 0x090083, 0x289062, 0x090062, 0x288c41, 0x090041, 0x288820, 0x090020, 0x28a401, 0x0900a4, 0x289483, 0x090083, 0x289062, 0x090062, 0x288c41, 0x090041, 0x288820, 0x0900c5, 0x2898a4, 0x0900a4, 0x289483, 0x090083, 0x289062, 0x090062, 0x288c41, 0x0900e6, 0x289cc5, 0x0900c5, 0x2898a4, 0x0900a4, 0x289483, 0x090083, 0x289062, 0x090107, 0x28a0e6, 0x0900e6, 0x289cc5, 0x0900c5, 0x2898a4, 0x0900a4, 0x289483},
    {0x090149, 0x09016a, 0x09018b, 0x0901ac, 0x0901cd, 0x0901ee, 0x09020f, 0x090230, 0x28ad49, 0x28b16a, 0x28b58b, 0x28b9ac, 0x28bdcd, 0x28c1ee, 0x28c60f, 0x28ca30, 0x09016a, 0x09018b, 0x0901ac, 0x0901cd, 0x0901ee, 0x09020f, 0x090230, 0x090251, 0x28b16a, 0x28b58b, 0x28b9ac, 0x28bdcd, 0x28c1ee, 0x28c60f, 0x28ca30, 0x28ce51, 0x09018b, 0x0901ac, 0x0901cd, 0x0901ee, 0x09020f, 0x090230, 0x090251, 0x090272, 0x28b58b, 0x28b9ac, 0x28bdcd, 0x28c1ee, 0x28c60f, 0x28ca30, 0x28ce51, 0x28d272, 0x0901ac, 0x0901cd, 0x0901ee, 0x09020f, 0x090230, 0x090251, 0x090272, 0x090293, 0x28b9ac, 0x28bdcd, 0x28c1ee, 0x28c60f, 0x28ca30, 0x28ce51, 0x28d272, 0x28d693},
    {0x090041, 0x288c41, 0x090062, 0x289062, 0x090083, 0x289483, 0x0900a4, 0x2898a4, 0x090062, 0x289062, 0x090083, 0x289483, 0x0900a4, 0x2898a4, 0x0900c5, 0x289cc5, 0x090083, 0x289483, 0x0900a4, 0x2898a4, 0x0900c5, 0x289cc5, 0x0900e6, 0x28a0e6, 0x0900a4, 0x2898a4, 0x0900c5, 0x289cc5, 0x0900e6, 0x28a0e6, 0x090107, 0x0c8107, 0x0900c5, 0x289cc5, 0x0900e6, 0x28a0e6, 0x090107, 0x0c8107, 0x020008, 0x020008, 0x0900e6, 0x28a0e6, 0x090107, 0x0c8107, 0x020008, 0x020008, 0x020008, 0x020008, 0x090107, 0x0c8107, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008, 0x020008},
};

struct IntraSmem {
    int nb[40];           // neighbouring samples (-1: not available)
    int nbf[40];          // filtered (8x8) neighbours
    uint32_t d4[10][32];  // Intra_4x4: what each lane computes in each wave
    // record and residual (int16 pairs, as k_inter stored them) of an intra
    // MB, copied in ahead of its turn; two buffers so that the next MB's copy
    // overlaps the current MB's work
    __align__(16) uint32_t raw[2][192];
    __align__(16) h264r_mb rec[2];
    uint32_t pred4[9][16];  // kPred4, for lane-varying reads
    uint32_t pred8[9][64];  // kPred8
    int cpar[8];            // chroma: DC per plane and quadrant, or plane a, b, c per plane
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}

// start copying MB addr's record and residual into buffer buf (one commit group)
__device__ __forceinline__ void intra_prefetch(const PicDesc &p, int addr, IntraSmem &s, int buf)
{
    const int lane = threadIdx.x & 31;
    const uint8_t *src = (const uint8_t *)(p.ires + (size_t)addr * 384);
    for (int i = lane; i < 48; i += 32) cp_async16(&s.raw[buf][4 * i], src + 16 * i);
    // the residual buffer is the engine's (768 bytes per MB); the record array
    // may be a caller's with 4-byte alignment only: plain copy then
    const uint8_t *rec = (const uint8_t *)(p.mbs + addr);
    if (((uintptr_t)rec & 15u) == 0) {
        if (lane < 2) cp_async16((uint8_t *)&s.rec[buf] + 16 * lane, rec + 16 * lane);
    } else if (lane < 8) {
        ((uint32_t *)&s.rec[buf])[lane] = ((const uint32_t *)rec)[lane];
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// ---------------------------------------------------------------- tiled intra MB
// Intra MB with its neighbourhood staged in shared memory: the left column,
// top row (with the top-right MB's samples) and corner are loaded once; the
// 4x4 / 8x8 blocks predict from and write into the tile; the MB is stored
// once.  Neighbour availability follows getMbAddrN_non_MBAFF_frames or
// getMbAddrN_MBAFF_frames for the MB's border and the Intra_4x4/8x8 block
// rules inside it.
struct IntraTile {
    int16_t l[17][25];     // luma rows -1..15 (index +1), cols -1..23 (index +1)
    int16_t c[2][9][9];    // chroma rows -1..7, cols -1..7
};

// luma neighbour p[xN, yN] (relative to the MB) of a block, -1 when not
// available; tr_ok: block rule for samples inside the MB to the top right
__device__ __forceinline__ int tile_nb(const IntraTile &t, int xN, int yN, bool inside_tr_ok)
{
    if (yN >= 0 && xN >= 16) return -1;
    if (yN >= 0 && xN >= 0 && !inside_tr_ok) return -1;
    return t.l[yN + 1][xN + 1];
}

// buf: the IntraSmem buffer holding the MB's record and residual
__device__ void intra_mb_tiled(const PicDesc &p, int addr, IntraSmem &s, IntraTile &t, int buf, const LaunchState &st)
{
    const int lane = threadIdx.x & 31;
    const h264r_mb m = s.rec[buf];
    const int W = p.ys, Wc = p.cs, wmb = p.wmb;  // row pitches
    int x, y, dy;  // first luma sample and row step (2 for a field MB of an MBAFF picture)
    uint8_t *Y = plane_y(p);
    // residual (computed by k_inter, luma raster 16x16, Cb 8x8, Cr 8x8) in
    // the prefetch buffer; the reconstructed chroma replaces it in place
    int16_t *res = reinterpret_cast<int16_t *>(s.raw[buf]);
    // ---- stage the neighbourhood (luma: corner, 16 left, 24 top; chroma:
    //      corner, 8 left, 8 top), -1 where not available for intra
    //      prediction.  Item i (lane + 32 * it): 0 luma corner, 1..16 left,
    //      17..40 top; 41..74 chroma (17 per plane: corner, 8 left, 8 top).
    uint32_t avail[3];
    if (p.mbaff) {
        // every sample through the MBAFF neighbour derivation (6.4.12.2):
        // the left column of a frame MB beside a field pair alternates
        // between the pair's MBs, and under constrained intra prediction
        // parts of it can be missing
        mb_origin(p, addr, x, y, dy);
#pragma unroll
        for (int it = 0; it < 3; it++) {
            const int i = lane + 32 * it;
            int v = -1;
            if (i < 41) {
                const int xN = i == 0 ? -1 : (i < 17 ? -1 : i - 17), yN = i == 0 ? -1 : (i < 17 ? i - 1 : -1);
                const uint8_t *ptr = intra_nb_ptr(p, addr, 0, 0, xN, yN);
                if (ptr) v = __ldcg(ptr);
                t.l[yN + 1][xN + 1] = v;
            } else if (i < 75) {
                const int j = i - 41, pl = j / 17, q = j % 17;
                const int xN = q < 9 ? -1 : q - 9, yN = q < 9 ? q - 1 : -1;
                const uint8_t *ptr = intra_nb_ptr(p, addr, 1, pl, xN, yN);
                if (ptr) v = __ldcg(ptr);
                t.c[pl][yN + 1][xN + 1] = v;
            }
            avail[it] = __ballot_sync(0xffffffffu, v >= 0);
        }
    } else {
        // Neighbour MBs A (left), B (above), C (above right), D (above left)
        // (6.4.9, getMbAddrN_non_MBAFF_frames) and every neighbouring sample
        // are loaded together; availability for intra prediction (same slice,
        // constrained intra prediction) is applied to the samples afterwards.
        const int mx = addr % wmb, my = addr / wmb;
        x = mx * 16;
        y = my * 16;
        dy = 1;
        const bool inA = mx > 0, inB = my > 0, inC = my > 0 && mx + 1 < wmb, inD = mx > 0 && my > 0;
        uint32_t r0 = 0, r2 = 0;  // record words 0 (type, flags) and 2 (slice) of neighbour `lane`
        const bool nb_in = lane < 4 && (lane == 0 ? inA : lane == 1 ? inB : lane == 2 ? inC : inD);
        if (nb_in) {
            const int n = lane == 0 ? addr - 1 : lane == 1 ? addr - wmb : lane == 2 ? addr - wmb + 1 : addr - wmb - 1;
            const uint32_t *q = (const uint32_t *)(p.mbs + n);
            r0 = __ldg(q);
            r2 = __ldg(q + 2);
        }
        int v[3], owner[3];  // owner: the neighbour MB (0 A, 1 B, 2 C, 3 D) of the item, -1 none
#pragma unroll
        for (int it = 0; it < 3; it++) {
            const int i = lane + 32 * it;
            v[it] = -1;
            owner[it] = -1;
            if (i < 41) {
                const int xN = i == 0 ? -1 : (i < 17 ? -1 : i - 17), yN = i == 0 ? -1 : (i < 17 ? i - 1 : -1);
                const int o = i == 0 ? 3 : (i < 17 ? 0 : (xN < 16 ? 1 : 2));
                if (o == 0 ? inA : o == 1 ? inB : o == 2 ? inC : inD) {
                    owner[it] = o;
                    v[it] = __ldcg(Y + (size_t)(y + yN) * W + x + xN);
                }
            } else if (i < 75) {
                const int j = i - 41, pl = j / 17, q = j % 17;
                const int xN = q < 9 ? -1 : q - 9, yN = q < 9 ? q - 1 : -1;
                const int o = q == 0 ? 3 : (q < 9 ? 0 : 1);
                if (o == 0 ? inA : o == 1 ? inB : inD) {
                    owner[it] = o;
                    v[it] = __ldcg(plane_c(p, pl) + (size_t)(y / 2 + yN) * Wc + x / 2 + xN);
                }
            }
        }
        // same slice, and not an inter MB under constrained intra prediction
        const bool usable = nb_in && (r2 & 0xFFFFu) == m.slice && !((r0 & 255u) == H264R_MB_INTER && ((r0 >> 8) & H264R_MBF_CIP));
        const uint32_t um = __ballot_sync(0xffffffffu, usable);
#pragma unroll
        for (int it = 0; it < 3; it++) {
            const int i = lane + 32 * it;
            const int val = (owner[it] >= 0 && ((um >> owner[it]) & 1u)) ? v[it] : -1;
            if (i < 41) {
                const int xN = i == 0 ? -1 : (i < 17 ? -1 : i - 17), yN = i == 0 ? -1 : (i < 17 ? i - 1 : -1);
                t.l[yN + 1][xN + 1] = val;
            } else if (i < 75) {
                const int j = i - 41, pl = j / 17, q = j % 17;
                const int xN = q < 9 ? -1 : q - 9, yN = q < 9 ? q - 1 : -1;
                t.c[pl][yN + 1][xN + 1] = val;
            }
            avail[it] = __ballot_sync(0xffffffffu, val >= 0);
        }
    }
    // whole-edge availability from the staged samples (item i is bit i % 32
    // of avail[i / 32]): luma left 1..16, top 17..32; Cb corner 41, left
    // 42..49, top 50..57 (Cr is the same)
    const bool la = ((avail[0] >> 1) & 0xFFFFu) == 0xFFFFu;
    const bool ta = (avail[0] >> 17) == 0x7FFFu && (avail[1] & 1u);
    const bool cA = ((avail[1] >> 10) & 0xFFu) == 0xFFu, cB = ((avail[1] >> 18) & 0xFFu) == 0xFFu;
    const bool cD = (avail[1] >> 9) & 1u;
    __syncwarp();
    // ---- luma
    // MB-edge availability of the luma neighbours (item bitmaps above)
    const uint32_t leftm = (avail[0] >> 1) & 0xFFFFu;                     // p[-1, 0..15]
    const uint32_t topm = (avail[0] >> 17) | ((avail[1] & 0x1FFu) << 15);  // p[0..23, -1]
    const bool cornerm = avail[0] & 1u;
    if (m.type == H264R_MB_I4x4) {
        // The 4x4 blocks on one anti-diagonal of the block grid (bx + 2*by
        // constant) depend on none of each other (left, top, top-left and
        // top-right all lie on earlier diagonals): 10 waves of at most two
        // blocks, one per half-warp, in place of 16 steps.  What a lane
        // computes in each wave depends only on the modes and on
        // availability, so it is worked out for all waves first (independent
        // iterations) and the waves themselves only read three samples (or
        // the DC sums) from the tile.  Availability comes from the MB-edge
        // bitmaps and the block position: inside the MB every earlier block
        // is reconstructed, and the top-right block is not yet for blocks
        // 3, 7, 11, 13 and 15 (8.3.1.2).  Wave word: bits 0-1 kind (0 none,
        // 1 three taps, 2 DC), 2-3 bx, 4-5 by; three taps: 6-17 the three
        // neighbour indices of {p[-1,-1], p[-1,0..3], p[0..7,-1]} after the
        // p[3,-1] substitution, 18-26 the weights; DC: bit 6 top, 7 left.
        const int half = lane >> 4, hl = lane & 15, i = hl >> 2, j = hl & 3;
#pragma unroll 2
        for (int wv = 0; wv < 10; wv++) {
            const int by = min(3, wv >> 1) - half, bx = wv - 2 * by;
            uint32_t d = 0;
            if (by >= 0 && bx >= 0 && bx <= 3) {
                const int b = 8 * (by >> 1) + 4 * (bx >> 1) + 2 * (by & 1) + (bx & 1);
                const int xO = bx * 4, yO = by * 4;
                const bool left = bx > 0 || ((leftm >> yO) & 15u) == 15u;
                const bool top = by > 0 || ((topm >> xO) & 15u) == 15u;
                const bool corner = bx > 0 ? (by > 0 || ((topm >> (xO - 1)) & 1u)) : (by > 0 ? ((leftm >> (yO - 1)) & 1u) : cornerm);
                // p[4..7, -1]: bit k available (else p[3, -1] stands in)
                const uint32_t trm = by > 0 ? ((bx < 3 && b != 3 && b != 11) ? 15u : 0u) : ((topm >> (xO + 4)) & 15u);
                const int mode = (((b >> 3) ? m.ipred[1] : m.ipred[0]) >> (4 * (b & 7))) & 15;
                const uint32_t pos = ((uint32_t)bx << 2) | ((uint32_t)by << 4);
                if (mode == 2) {
                    d = 2u | pos | ((uint32_t)top << 6) | ((uint32_t)left << 7);
                } else {
                    const bool ok = mode == 0 ? top : (mode == 1 || mode == 8) ? left : (mode == 3 || mode == 7) ? top
                                                                                                      : (top && left && corner);
                    // a mode without its samples predicts 0 (the cleared buffer): all weights 0
                    const uint32_t e = (ok && mode <= 8) ? s.pred4[mode][hl] : 0u;
                    uint32_t k3 = 0;
#pragma unroll
                    for (int q = 0; q < 3; q++) {
                        uint32_t k = (e >> (4 * q)) & 15u;
                        if (k >= 9 && !((trm >> (k - 9)) & 1u)) k = 8;
                        k3 |= k << (4 * q);
                    }
                    d = 1u | pos | (k3 << 6) | (((e >> 12) & 0x1FFu) << 18);
                }
            }
            s.d4[wv][lane] = d;
        }
        // tile offset of neighbour index k relative to p[-1,-1] of the block
        auto at = [](uint32_t k) -> int { return k == 0 ? 0 : (k <= 4 ? 25 * (int)k : (int)k - 4); };
        for (int wv = 0; wv < 10; wv++) {
            const uint32_t d = s.d4[wv][lane];
            if (d & 3u) {
                const int xO = ((d >> 2) & 3u) * 4, yO = ((d >> 4) & 3u) * 4;
                const int16_t *T = &t.l[yO][xO];  // T[r * 25 + c] = p[xO + c - 1, yO + r - 1]
                int pv;
                if (d & 2u) {
                    const bool top = (d >> 6) & 1u, left = (d >> 7) & 1u;
                    const int st4 = top ? T[1] + T[2] + T[3] + T[4] : 0, sl4 = left ? T[25] + T[50] + T[75] + T[100] : 0;
                    pv = (top && left) ? (st4 + sl4 + 4) >> 3 : left ? (sl4 + 2) >> 2 : top ? (st4 + 2) >> 2 : 128;
                } else {
                    pv = ((int)((d >> 18) & 7u) * T[at((d >> 6) & 15u)] + (int)((d >> 21) & 7u) * T[at((d >> 10) & 15u)] +
                          (int)((d >> 24) & 7u) * T[at((d >> 14) & 15u)] + 2) >> 2;
                }
                t.l[yO + i + 1][xO + j + 1] = clip1(pv + res[(yO + i) * 16 + xO + j]);
            }
            __syncwarp();
        }
    } else if (m.type == H264R_MB_I8x8) {
        // availability of q = {p[-1,-1], p[-1,0..7], p[0..15,-1]} per 8x8
        // block from the MB-edge bitmaps: inside the MB every earlier block is
        // reconstructed; the top-right octet of block 3 is right of the MB
        for (int b = 0; b < 4; b++) {
            const int xO = (b & 1) * 8, yO = (b >> 1) * 8;
            const bool cor = b == 3 || (b == 0 ? cornerm : (b == 1 ? ((topm >> 7) & 1u) : ((leftm >> 7) & 1u)));
            const bool left8 = (b & 1) || ((leftm >> yO) & 0xFFu) == 0xFFu;
            const bool top8 = (b & 2) || ((topm >> xO) & 0xFFu) == 0xFFu;
            // p[8..15, -1] of the block: bit k available (else p[7, -1] stands in)
            const uint32_t trm = b == 0 ? ((topm >> 8) & 0xFFu) : (b == 1 ? ((topm >> 16) & 0xFFu) : (b == 2 ? 0xFFu : 0u));
            // an unavailable top-right octet takes p[7,-1], so the 16 top
            // samples are available exactly when the first 8 are
            const bool top16 = top8;
            // the staged samples themselves (-1 where not available: the
            // filter looks at single samples of a partly available edge)
            if (lane < 25) {
                int v;
                if (lane == 0) {
                    v = t.l[yO][xO];
                } else if (lane < 9) {
                    v = t.l[yO + lane][xO];
                } else {
                    const int i = lane - 9;
                    v = t.l[yO][xO + 1 + ((i > 7 && !((trm >> (i - 8)) & 1u)) ? 7 : i)];
                }
                s.nb[lane] = v;
            }
            __syncwarp();
            // 8.3.2.2.1 reference sample filtering, one sample per lane
            // (H264PictureBase.cpp:1540-1600)
            int f = -1;
            if (lane < 25) {
                const int *q = s.nb;
                if (lane == 0) {
                    if (q[0] >= 0) {
                        if (q[9] < 0 || q[1] < 0)
                            f = q[9] >= 0 ? (3 * q[0] + q[9] + 2) >> 2 : q[1] >= 0 ? (3 * q[0] + q[1] + 2) >> 2 : q[0];
                        else
                            f = (q[9] + 2 * q[0] + q[1] + 2) >> 2;
                    }
                } else if (lane < 9) {
                    if (left8) {
                        if (lane == 1) f = q[0] >= 0 ? (q[0] + 2 * q[1] + q[2] + 2) >> 2 : (3 * q[1] + q[2] + 2) >> 2;
                        else if (lane < 8) f = (q[lane - 1] + 2 * q[lane] + q[lane + 1] + 2) >> 2;
                        else f = (q[7] + 3 * q[8] + 2) >> 2;
                    }
                } else if (top16) {
                    if (lane == 9) f = q[0] >= 0 ? (q[0] + 2 * q[9] + q[10] + 2) >> 2 : (3 * q[9] + q[10] + 2) >> 2;
                    else if (lane < 24) f = (q[lane - 1] + 2 * q[lane] + q[lane + 1] + 2) >> 2;
                    else f = (q[23] + 3 * q[24] + 2) >> 2;
                }
                s.nbf[lane] = f;
            }
            const int mode = (m.ipred[0] >> (4 * b)) & 15;
            // availability of the filtered samples: corner, left 8, top 8, top 16
            const bool corner = cor, left = left8, top = top16, topr = top16;
            const bool ok = mode == 0 ? top : (mode == 1 || mode == 8) ? left : (mode == 3 || mode == 7) ? topr
                                                                                              : (top && left && corner);
            int dcv = 128;
            if (mode == 2) {
                const int st8 = __reduce_add_sync(0xffffffffu, (top && lane >= 9 && lane < 17) ? f : 0);
                const int sl8 = __reduce_add_sync(0xffffffffu, (left && lane >= 1 && lane < 9) ? f : 0);
                dcv = (top && left) ? (st8 + sl8 + 8) >> 4 : left ? (sl8 + 4) >> 3 : top ? (st8 + 4) >> 3 : 128;
            }
            __syncwarp();
            for (int kk = lane; kk < 64; kk += 32) {
                const int i = kk >> 3, j = kk & 7;
                int pv = 0;  // a mode without its samples writes no prediction: the cleared buffer
                if (mode == 2) {
                    pv = dcv;
                } else if (mode <= 8 && ok) {
                    const uint32_t e = s.pred8[mode][kk];
                    pv = ((int)((e >> 15) & 7u) * s.nbf[e & 31u] + (int)((e >> 18) & 7u) * s.nbf[(e >> 5) & 31u] +
                          (int)((e >> 21) & 7u) * s.nbf[(e >> 10) & 31u] + 2) >> 2;
                }
                t.l[yO + i + 1][xO + j + 1] = clip1(pv + res[(yO + i) * 16 + xO + j]);
            }
            __syncwarp();
        }
    } else {
        // Intra_16x16 (H264PictureBase.cpp:1847-2059)
        const int16_t *top = &t.l[0][1];
        const int mode = m.i16_mode;
        int a = 0, bb = 0, cc = 0, dcv = 128;
        if (mode == 2) {
            int stp = 0, slf = 0;
            for (int i = 0; i < 16; i++) { stp += top[i]; slf += t.l[1 + i][0]; }
            if (ta && la) dcv = (stp + slf + 16) >> 5;
            else if (la) dcv = (slf + 8) >> 4;
            else if (ta) dcv = (stp + 8) >> 4;
        } else if (mode == 3) {
            // quirk: p[-1,-1] is not required; when unavailable -1 enters H, V
            int H = 0, V = 0;
            for (int i = 0; i <= 7; i++) {
                H += (i + 1) * (top[8 + i] - (6 - i >= 0 ? top[6 - i] : t.l[0][0]));
                V += (i + 1) * (t.l[1 + 8 + i][0] - (6 - i >= 0 ? t.l[1 + 6 - i][0] : t.l[0][0]));
            }
            a = 16 * (t.l[16][0] + top[15]);
            bb = (5 * H + 32) >> 6;
            cc = (5 * V + 32) >> 6;
        }
        for (int kk = lane; kk < 256; kk += 32) {
            int i = kk >> 4, j = kk & 15, pv;
            if (mode == 0) pv = ta ? top[j] : 0;
            else if (mode == 1) pv = la ? t.l[1 + i][0] : 0;
            else if (mode == 2) pv = dcv;
            else if (mode == 3) pv = (ta && la) ? clip1((a + bb * (j - 7) + cc * (i - 7) + 16) >> 5) : 0;
            else pv = 0;
            t.l[1 + i][1 + j] = clip1(pv + res[kk]);
        }
        __syncwarp();
    }
    // ---- chroma (Intra_chroma_sample_prediction, H264PictureBase.cpp:2076-2385):
    //      the per-MB values first (DC of each 4x4 quadrant, or the plane
    //      parameters), one per lane; quirk: DC treats a neighbouring value
    //      0 as unavailable
    const int cmode = m.chroma_mode;
    if (cmode == 0 && lane < 8) {
        const int pl = lane >> 2, xO = (lane & 1) * 4, yO = (lane & 2) * 2;
        const int16_t(*c)[9] = t.c[pl];  // c[0][0] corner, c[1+u][0] left, c[0][1+u] top
        const bool t4 = c[0][1 + xO] > 0 && c[0][2 + xO] > 0 && c[0][3 + xO] > 0 && c[0][4 + xO] > 0;
        const bool l4 = c[1 + yO][0] > 0 && c[2 + yO][0] > 0 && c[3 + yO][0] > 0 && c[4 + yO][0] > 0;
        const int stp = t4 ? c[0][1 + xO] + c[0][2 + xO] + c[0][3 + xO] + c[0][4 + xO] : 0;
        const int slf = l4 ? c[1 + yO][0] + c[2 + yO][0] + c[3 + yO][0] + c[4 + yO][0] : 0;
        int pv;
        if ((xO == 0 && yO == 0) || (xO > 0 && yO > 0)) pv = (t4 && l4) ? (stp + slf + 4) >> 3 : l4 ? (slf + 2) >> 2 : t4 ? (stp + 2) >> 2 : 128;
        else if (xO > 0) pv = t4 ? (stp + 2) >> 2 : l4 ? (slf + 2) >> 2 : 128;
        else pv = l4 ? (slf + 2) >> 2 : t4 ? (stp + 2) >> 2 : 128;
        s.cpar[lane] = pv;
    } else if (cmode == 3 && lane < 2 && cA && cB && cD) {
        const int16_t(*c)[9] = t.c[lane];
        int H = 0, V = 0;
        for (int u = 0; u <= 3; u++) {
            H += (u + 1) * (c[0][5 + u] - (2 - u >= 0 ? c[0][3 - u] : c[0][0]));
            V += (u + 1) * (c[5 + u][0] - (2 - u >= 0 ? c[3 - u][0] : c[0][0]));
        }
        s.cpar[3 * lane] = 16 * (c[8][0] + c[0][8]);
        s.cpar[3 * lane + 1] = (34 * H + 32) >> 6;
        s.cpar[3 * lane + 2] = (34 * V + 32) >> 6;
    }
    __syncwarp();
    for (int kk = lane; kk < 128; kk += 32) {
        const int pl = kk >> 6, i = (kk & 63) >> 3, j = kk & 7;
        const int16_t(*c)[9] = t.c[pl];
        int pv = 0;
        if (cmode == 0) pv = s.cpar[4 * pl + (i >> 2) * 2 + (j >> 2)];
        else if (cmode == 1) pv = cA ? c[1 + i][0] : 0;
        else if (cmode == 2) pv = cB ? c[0][1 + j] : 0;
        else if (cmode == 3 && cA && cB && cD)
            pv = clip1((s.cpar[3 * pl] + s.cpar[3 * pl + 1] * (j - 3) + s.cpar[3 * pl + 2] * (i - 3) + 16) >> 5);
        res[256 + kk] = (int16_t)clip1(pv + res[256 + kk]);  // reconstructed chroma, in place
    }
    __syncwarp();
    // ---- store the MB: 16 luma rows of 16 bytes, 2 x 8 chroma rows of 8 bytes
    if (lane < 16) {
        const int16_t *q = &t.l[1 + lane][1];
        uint32_t w[4] = {0, 0, 0, 0};
#pragma unroll
        for (int k = 0; k < 16; k++) w[k >> 2] |= (uint32_t)(q[k] & 255) << (8 * (k & 3));
        *(uint4 *)(Y + (size_t)(y + lane * dy) * W + x) = make_uint4(w[0], w[1], w[2], w[3]);
    } else {
        const int pl = (lane - 16) >> 3, r = (lane - 16) & 7;
        const uint4 q = *reinterpret_cast<const uint4 *>(res + 256 + pl * 64 + r * 8);  // 8 samples as int16
        *(uint2 *)(plane_c(p, pl) + (size_t)(chroma_row0(y) + r * dy) * Wc + x / 2) =
            make_uint2(__byte_perm(q.x, q.y, 0x6420), __byte_perm(q.z, q.w, 0x6420));
    }
    __threadfence_block();
    __syncwarp();
}

// 21 resident row warps per SM (registers capped at 80): a batch of many
// pictures keeps more rows of its wavefronts in flight
__global__ void __launch_bounds__(32, 21) k_intra(const PicDesc *__restrict__ pics, int npics, uint32_t total_rows, LaunchState st)
{
    __shared__ IntraSmem s;
    __shared__ IntraTile tile;
    __shared__ uint32_t s_row;
    const int lane = threadIdx.x;
    if (lane == 0) s_row = atomicAdd(&st.ticket[0], 1u);
    for (int i = lane; i < 9 * 16; i += 32) (&s.pred4[0][0])[i] = (&kPred4[0][0])[i];
    for (int i = lane; i < 9 * 64; i += 32) (&s.pred8[0][0])[i] = __ldg(&kPred8[0][0] + i);
    __syncwarp();
    const uint32_t g = s_row;
    if (g >= total_rows) return;
    const int pi = find_pic_by_row(pics, npics, g);
    const PicDesc p = pics[pi];
    const int row = (int)(g - p.row_base);
    const int uw = (int)p.units_w;
    const int per = p.mbaff ? 2 : 1;
    int *prog = p.progress;
    // Units without intra MBs were completed by k_inter: progress is only
    // published before this row waits and after each intra unit.
    int posted = 0, seen = 0;
    int buf = 0, ahead = -1;  // ahead: MB whose copy into buffer buf is in flight
    for (int u0 = 0; u0 < uw; u0 += 32) {
        // which of the next 32 units hold intra MBs: one record load per lane
        bool mine = false;
        if (u0 + lane < uw) {
            for (int k = 0; k < per; k++) {
                const int addr = p.mbaff ? 2 * (row * uw + u0 + lane) + k : row * uw + u0 + lane;
                mine = mine || is_intra_type(p.mbs[addr].type);
            }
        }
        uint32_t todo = __ballot_sync(0xffffffffu, mine);
        // Frame pictures: an intra MB whose neighbours above (top-left, top,
        // top-right) are all inter MBs, final since k_inter, need not wait for
        // the row above; only intra neighbours are still being written.  Bit
        // c - (u0 - 1) of `up`: MB (row - 1, c) is intra.
        uint64_t up = ~0ull;
        if (!p.mbaff && row > 0 && todo) {
            const int c0 = u0 - 1 + lane, c1 = u0 + 31 + lane;
            const bool a0 = c0 >= 0 && c0 < uw && is_intra_type(p.mbs[(row - 1) * uw + c0].type);
            const bool a1 = lane < 2 && c1 < uw && is_intra_type(p.mbs[(row - 1) * uw + c1].type);
            up = (uint64_t)__ballot_sync(0xffffffffu, a0) | ((uint64_t)(__ballot_sync(0xffffffffu, a1) & 3u) << 32);
        }
        while (todo) {
            const int u = u0 + __ffs(todo) - 1;
            todo &= todo - 1;
            if (lane == 0 && posted < u) st_release(prog + row, u);
            posted = u;
            if (row > 0 && ((up >> (u - u0)) & 7u) && !db_wait(st, prog + row - 1, min(u + 2, uw), seen)) return;
            if (p.mbaff) {
                // the pair's intra MBs; the copy of the next intra MB (the
                // pair's second, else the next pair's first of this group)
                // overlaps the current one
                const int pa = 2 * (row * uw + u);
                const bool in0 = is_intra_type(p.mbs[pa].type), in1 = is_intra_type(p.mbs[pa + 1].type);
                int nxt = -1;  // first intra MB of the next pair with intra MBs in this group
                if (todo) {
                    const int pn = 2 * (row * uw + u0 + __ffs(todo) - 1);
                    nxt = is_intra_type(p.mbs[pn].type) ? pn : pn + 1;
                }
                for (int k = 0; k < 2; k++) {
                    if (!(k ? in1 : in0)) continue;
                    const int addr = pa + k;
                    if (ahead != addr) intra_prefetch(p, addr, s, buf);
                    ahead = (k == 0 && in1) ? pa + 1 : nxt;
                    if (ahead >= 0) {
                        intra_prefetch(p, ahead, s, buf ^ 1);
                        asm volatile("cp.async.wait_group 1;" ::: "memory");
                    } else {
                        asm volatile("cp.async.wait_group 0;" ::: "memory");
                    }
                    __syncwarp();
                    intra_mb_tiled(p, addr, s, tile, buf, st);
                    buf ^= 1;
                }
            } else {
                // the next intra MB of this group of 32 is copied in while this one runs
                const int addr = row * uw + u;
                if (ahead != addr) intra_prefetch(p, addr, s, buf);
                const bool more = todo != 0;
                if (more) {
                    ahead = row * uw + u0 + __ffs(todo) - 1;
                    intra_prefetch(p, ahead, s, buf ^ 1);
                    asm volatile("cp.async.wait_group 1;" ::: "memory");
                } else {
                    ahead = -1;
                    asm volatile("cp.async.wait_group 0;" ::: "memory");
                }
                __syncwarp();
                intra_mb_tiled(p, addr, s, tile, buf, st);
                buf ^= 1;
            }
            __syncwarp();
            if (lane == 0) st_release(prog + row, u + 1);
            posted = u + 1;
        }
    }
    if (lane == 0 && posted < uw) st_release(prog + row, uw);
}

// ======================================================================
// K3a: boundary strengths
// ======================================================================
struct BlkMotion {
    int mv[2][2];
    int pf[2];
    int id[2];
};

// motion of 4x4 block (bx, by) of a macroblock of type `type` whose motion
// payload is at `aux`
__device__ __forceinline__ void block_motion(const PicDesc &p, int type, uint32_t aux, int bx, int by, BlkMotion &o)
{
    o.mv[0][0] = o.mv[0][1] = o.mv[1][0] = o.mv[1][1] = 0;
    o.pf[0] = o.pf[1] = 0;
    o.id[0] = o.id[1] = -1;
    if (type != H264R_MB_INTER || aux == H264R_NONE || (aux & 3) || (uint64_t)aux + 4 > p.motion_bytes) return;
    uint32_t hdr = *(const uint32_t *)(p.motion + aux);
    int e = part_of_block(hdr & 0xFFFF, bx, by);
    if (e >= (int)(hdr >> 16) || (uint64_t)aux + 4 + 16ull * (e + 1) > p.motion_bytes) return;
    const h264r_part pp = ((const h264r_part *)(p.motion + aux + 4))[e];
    for (int l = 0; l < 2; l++) {
        o.mv[l][0] = pp.mv[l][0];
        o.mv[l][1] = pp.mv[l][1];
        o.pf[l] = pp.ref[l] >= 0;
        o.id[l] = pp.dref[l];
    }
}

// The motion rules of 8.7.2.1 for two blocks of inter MBs: 1 when the
// references or the motion vectors differ (vertical limit lim), else 0
// (H264PictureDeblockingFilterProcess.cpp:1230-1310)
__device__ __forceinline__ int bs_motion(const BlkMotion &a, const BlkMotion &b, int lim)
{
#define DIFF(u, v) (abs((u)[0] - (v)[0]) >= 4 || abs((u)[1] - (v)[1]) >= lim)
    int r0p = a.id[0], r1p = a.id[1], r0q = b.id[0], r1q = b.id[1];
    int np = a.pf[0] + a.pf[1], nq = b.pf[0] + b.pf[1];
    if (!(((r0p == r0q && r1p == r1q) || (r0p == r1q && r1p == r0q)) && np == nq)) return 1;
    if (a.pf[0] && !a.pf[1] && b.pf[0] && !b.pf[1] && DIFF(a.mv[0], b.mv[0])) return 1;
    if (a.pf[0] && !a.pf[1] && !b.pf[0] && b.pf[1] && DIFF(a.mv[0], b.mv[1])) return 1;
    if (!a.pf[0] && a.pf[1] && b.pf[0] && !b.pf[1] && DIFF(a.mv[1], b.mv[0])) return 1;
    if (!a.pf[0] && a.pf[1] && !b.pf[0] && b.pf[1] && DIFF(a.mv[1], b.mv[1])) return 1;
    if (a.pf[0] && a.pf[1] && r0p != r1p && b.pf[0] && b.pf[1] && ((r0q == r0p && r1q == r1p) || (r0q == r1p && r1q == r0p))) {
        if (r0q == r0p && (DIFF(a.mv[0], b.mv[0]) || DIFF(a.mv[1], b.mv[1]))) return 1;
        else if (r0q == r1p && (DIFF(a.mv[1], b.mv[0]) || DIFF(a.mv[0], b.mv[1]))) return 1;
    }
    // quirk: parsed as (A || B) && C || D (1289-1298)
    if (a.pf[0] && a.pf[1] && r0p == r1p && b.pf[0] && b.pf[1] && r0q == r1q && r0q == r0p) {
        if (((DIFF(a.mv[0], b.mv[0]) || DIFF(a.mv[1], b.mv[1])) && DIFF(a.mv[0], b.mv[1])) || DIFF(a.mv[1], b.mv[0])) return 1;
    }
#undef DIFF
    return 0;
}

// 8.7.2.1 (Derivation_process_for_the_luma_content_dependent_boundary_
// filtering_strength, H264PictureDeblockingFilterProcess.cpp:994-1310).
// Returns 0xFF where the reference's derivation fails (it reaches the
// partition lookup of a macroblock that was never decoded).
__device__ int derive_bs(const PicDesc &p, int mbP, int mbQ, int xp, int yp, int xq, int yq, int vertical)
{
    const h264r_mb P = p.mbs[mbP], Q = p.mbs[mbQ];
    const int mbaff = p.mbaff, fpic = p.fpic != 0;
    // every MB of a field picture is a field MB
    int fP = ((P.flags & H264R_MBF_FIELD) && mbaff) || fpic, fQ = ((Q.flags & H264R_MBF_FIELD) && mbaff) || fpic;
    int mixed = mbaff && mbP != mbQ && fP != fQ;
    bool intraP = is_intra_type(P.type), intraQ = is_intra_type(Q.type);
    int stP = p.slices[min((uint32_t)P.slice, p.num_slices - 1)].slice_type;
    int stQ = p.slices[min((uint32_t)Q.slice, p.num_slices - 1)].slice_type;
    bool spP = stP == 3 || stP == 4, spQ = stQ == 3 || stQ == 4;
    if (mbP != mbQ) {
        if ((!fP && !fQ && (intraP || intraQ)) || (!fP && !fQ && (spP || spQ)) || ((mbaff || fpic) && vertical && (intraP || intraQ)) ||
            ((mbaff || fpic) && vertical && (spP || spQ)))
            return 4;
    }
    if ((!mixed && (intraP || intraQ)) || (!mixed && (spP || spQ)) || (mixed && !vertical && (intraP || intraQ)) ||
        (mixed && !vertical && (spP || spQ)))
        return 3;
    int bp4 = 8 * (yp / 8) + 4 * (xp / 8) + 2 * ((yp % 8) / 4) + ((xp % 8) / 4);
    int bq4 = 8 * (yq / 8) + 4 * (xq / 8) + 2 * ((yq % 8) / 4) + ((xq % 8) / 4);
    int bp8 = 2 * (yp / 8) + (xp / 8), bq8 = 2 * (yq / 8) + (xq / 8);
    int nzP = (P.flags & H264R_MBF_T8x8) ? ((P.nz8x8 >> bp8) & 1) : ((P.nz4x4 >> bp4) & 1);
    int nzQ = (Q.flags & H264R_MBF_T8x8) ? ((Q.nz8x8 >> bq8) & 1) : ((Q.nz4x4 >> bq4) & 1);
    if (nzP || nzQ) return 2;
    if (P.type == H264R_MB_NONE || Q.type == H264R_MB_NONE) return 0xFF;
    if (mixed) return 1;
    const int lim = fQ ? 2 : 4;
    BlkMotion a, b;
    block_motion(p, P.type, P.aux, xp >> 2, yp >> 2, a);
    block_motion(p, Q.type, Q.aux, xq >> 2, yq >> 2, b);
    return bs_motion(a, b, lim);
}

// Per-MB filter controls of Deblocking_filter_process (76-160)
struct EdgeCtl {
    int mbA, mbB, field, left, top, internal, t8, leftMixed, topDouble;
};

__device__ __forceinline__ EdgeCtl edge_ctl(const PicDesc &p, int cur)
{
    EdgeCtl e;
    const h264r_mb m = p.mbs[cur];
    int xW, yW;
    e.mbA = nb_loc(p, cur, -1, 0, 16, 16, xW, yW);
    e.mbB = nb_loc(p, cur, 0, -1, 16, 16, xW, yW);
    const int W = p.wmb, mbaff = p.mbaff;
    e.field = mbaff && (m.flags & H264R_MBF_FIELD);
    int idc = p.slices[min((uint32_t)m.slice, p.num_slices - 1)].disable_deblocking_filter_idc;
    e.internal = idc != 1;
    e.left = !((!mbaff && cur % W == 0) || (mbaff && (cur >> 1) % W == 0) || idc == 1 || (idc == 2 && e.mbA < 0));
    e.top = !((!mbaff && cur < W) || (mbaff && (cur >> 1) < W && e.field) || (mbaff && (cur >> 1) < W && !e.field && (cur % 2) == 0) ||
              idc == 1 || (idc == 2 && e.mbB < 0));
    e.t8 = (m.flags & H264R_MBF_T8x8) != 0;
    e.leftMixed = mbaff && cur >= 2 && !e.field && (p.mbs[cur - 2].flags & H264R_MBF_FIELD);
    e.topDouble = mbaff && (cur % 2) == 0 && cur >= 2 * W && !e.field && (p.mbs[cur - 2 * W + 1].flags & H264R_MBF_FIELD);
    return e;
}

// bS of row/col k of one edge (8.7.1 p-side rules, 639-805); e = edge
// offset in samples of the component; mbN: neighbour handed to the filter
__device__ __forceinline__ int edge_bs(const PicDesc &p, int cur, int chroma, int vertical, int e, int mbN, int leftMbEdge, int k)
{
    int xE = vertical ? e : k, yE = vertical ? k : e;
    int mbP = cur, xp0, yp0, xq0, yq0;
    if (vertical) {
        xp0 = xE - 1;
        if (xp0 < 0) {
            if (mbN >= 0) mbP = leftMbEdge ? mbN + (yE % 2) : mbN;
            xp0 += chroma ? 8 : 16;
        }
        yp0 = yE; xq0 = xE; yq0 = yE;
    } else {
        xp0 = xE;
        yp0 = (yE - 1) - (yE % 2);
        if (yp0 < 0) {
            if (mbN >= 0) mbP = mbN;
            yp0 += chroma ? 8 : 16;
        }
        xq0 = xE; yq0 = yE - (yE % 2);
    }
    int sx = chroma ? 2 : 1;
    return derive_bs(p, mbP, cur, xp0 * sx, yp0 * sx, xq0 * sx, yq0 * sx, vertical);
}

// edge sequence numbers in the reference's per-MB filtering order
enum { SEQ_LV0 = 0, SEQ_LV4, SEQ_LV8, SEQ_LV12, SEQ_LH0, SEQ_LH0B, SEQ_LH4, SEQ_LH8, SEQ_LH12,
       SEQ_CBV0, SEQ_CRV0, SEQ_CBV4, SEQ_CRV4, SEQ_CBH0, SEQ_CRH0, SEQ_CBH0B, SEQ_CRH0B, SEQ_CBH4, SEQ_CRH4 };

__device__ __forceinline__ uint32_t stop_key(int mb, int seq, int k) { return ((uint32_t)mb << 10) | ((uint32_t)seq << 4) | (uint32_t)k; }

// indexA / alpha / beta of an edge between MBs mbP and cur (8.7.2.2,
// H264PictureDeblockingFilterProcess.cpp:1314-1369)
__device__ __forceinline__ void edge_params(const PicDesc &p, int mbP, int cur, int comp, int &indexA, int &alpha, int &beta)
{
    const h264r_mb P = p.mbs[mbP], Q = p.mbs[cur];
    const h264r_slice sq = p.slices[min((uint32_t)Q.slice, p.num_slices - 1)];
    int qPp, qPq;
    if (comp == 0) {
        qPp = P.type == H264R_MB_IPCM ? 0 : P.qpy;
        qPq = Q.type == H264R_MB_IPCM ? 0 : Q.qpy;
    } else {
        int off = sq.chroma_qp_offset[comp - 1];
        qPp = chroma_qp(P.type == H264R_MB_IPCM ? 0 : P.qpy, off);
        qPq = chroma_qp(Q.type == H264R_MB_IPCM ? 0 : Q.qpy, off);
    }
    int qPav = (qPp + qPq + 1) >> 1;
    indexA = H264R_CLIP3(0, 51, qPav + sq.filter_offset_a);
    int indexB = H264R_CLIP3(0, 51, qPav + sq.filter_offset_b);
    alpha = kAlpha[indexA];
    beta = kBeta[indexB];
}

// Motion of a 4x4 block for the frame-picture strength rules, with the
// block's MB-level facts: mv0 / mv1 the list 0 / 1 vectors (x | y << 16);
// rf: dref[0] | dref[1] << 8 (0xFF: none), bit 16 / 17 list 0 / 1 used,
// bit 18 the block has non-zero levels, bit 19 its MB is intra (I4x4, I8x8,
// I16x16), bit 20 its MB was never decoded.  The motion is block_motion's.
struct BsBlock {
    uint32_t mv0, mv1, rf;
};

__device__ __forceinline__ BsBlock bs_block(const PicDesc &p, int type, int flags, int nz4, int nz8, uint32_t aux, int bx, int by)
{
    const int nz = (flags & H264R_MBF_T8x8) ? (nz8 >> (2 * (by >> 1) + (bx >> 1))) & 1
                                            : (nz4 >> (8 * (by >> 1) + 4 * (bx >> 1) + 2 * (by & 1) + (bx & 1))) & 1;
    BsBlock o;
    o.mv0 = o.mv1 = 0;
    o.rf = 0xFFFFu | ((uint32_t)nz << 18) | ((uint32_t)is_intra_type(type) << 19) | ((uint32_t)(type == H264R_MB_NONE) << 20);
    if (type != H264R_MB_INTER || aux == H264R_NONE || (aux & 3) || (uint64_t)aux + 4 > p.motion_bytes) return o;
    const uint32_t hdr = *(const uint32_t *)(p.motion + aux);
    const int e = part_of_block(hdr & 0xFFFF, bx, by);
    if (e >= (int)(hdr >> 16) || (uint64_t)aux + 4 + 16ull * (e + 1) > p.motion_bytes) return o;
    // h264r_part: mv[2][2] (8 bytes), ref[2], dref[2]
    const uint32_t *q = (const uint32_t *)(p.motion + aux + 4 + 16 * e);
    const uint32_t w = q[2];
    o.mv0 = q[0];
    o.mv1 = q[1];
    o.rf = (o.rf & 0x1C0000u) | (w >> 16) | ((w & 0x80u) ? 0u : 0x10000u) | ((w & 0x8000u) ? 0u : 0x20000u);
    return o;
}

// bs_motion on packed blocks: a the p side, b the q side.  Once the two
// blocks use the same reference pictures in the same number of lists, one
// list each compares the vectors used; two lists compare the vectors of the
// same reference picture, or (both lists on one picture) the reference's
// (A || B) && C || D (H264PictureDeblockingFilterProcess.cpp:1230-1310).
__device__ __forceinline__ int bs_motion_packed(const BsBlock &a, const BsBlock &b, int lim)
{
    const uint32_t ra = a.rf, rb = b.rf;
    const uint32_t r0p = ra & 255u, r1p = (ra >> 8) & 255u, r0q = rb & 255u, r1q = (rb >> 8) & 255u;
    const int np = (int)((ra >> 16) & 1u) + (int)((ra >> 17) & 1u), nq = (int)((rb >> 16) & 1u) + (int)((rb >> 17) & 1u);
    if (!(((r0p == r0q && r1p == r1q) || (r0p == r1q && r1p == r0q)) && np == nq)) return 1;
    auto diff = [lim](uint32_t u, uint32_t v) {
        const int dx = abs(((int)(u << 16) >> 16) - ((int)(v << 16) >> 16));
        const int dy = abs(((int)u >> 16) - ((int)v >> 16));
        return dx >= 4 || dy >= lim;
    };
    if (np == 1) return diff((ra & 0x10000u) ? a.mv0 : a.mv1, (rb & 0x10000u) ? b.mv0 : b.mv1);
    if (np == 2) {
        const bool d00 = diff(a.mv0, b.mv0), d11 = diff(a.mv1, b.mv1), d01 = diff(a.mv0, b.mv1), d10 = diff(a.mv1, b.mv0);
        if (r0p != r1p) return r0q == r0p ? (d00 || d11) : (d10 || d01);
        return ((d00 || d11) && d01) || d10;
    }
    return 0;
}

// Strengths and thresholds of a frame or field picture's MB (no MBAFF), two
// MBs per warp: half h of the warp takes MB g, lane j of the half its 4x4
// block (j & 3, j >> 2), whose left edge (vertical edge j & 3, lines
// 4(j >> 2)..+3) and top edge (horizontal edge j >> 2, columns 4(j & 3)..+3)
// it derives.  In a frame picture a strength depends only on the pair of
// blocks the edge joins (no field or mixed edges); the 4:2:0 chroma
// strengths are the luma ones of the same edge at line 2k (the reference
// derives them from the luma positions, 994-1310).  Each lane reads the
// motion of its block; the lanes of column 3 also read the block left of
// their row (column 3 of the left MB) and those of row 3 the block above
// their column (row 3 of the MB above), so that every edge takes its p side
// in one shuffle.  A neighbour MB is available only in the MB's own slice,
// so the SP / SI rule reads the MB's slice alone.  The rules are derive_bs's
// for a frame picture (no field MBs) or a field picture (all field MBs: bS 3
// on horizontal MB edges of intra MBs, vertical MV limit 2).  All lanes run
// this; `on` false: the half's MB is not a deblocked frame-picture MB, and
// nothing is written for it.
__device__ __forceinline__ void bs_frame_half(const PicDesc *__restrict__ pics, int pi, uint32_t g, bool on)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, j = lane & 15, hb = lane & 16, bx = j & 3, by = j >> 2;
    const PicDesc &p = pics[pi];
    const int cur = on ? (int)(g - p.mb_base) : 0;
    const int W = p.wmb, col = cur % W;
    const h264r_mb Q = p.mbs[cur];
    const h264r_mb A0 = p.mbs[col != 0 ? cur - 1 : cur], B0 = p.mbs[cur >= W ? cur - W : cur];
    const bool hasA = col != 0 && A0.slice == Q.slice, hasB = cur >= W && B0.slice == Q.slice;
    const h264r_slice sl = p.slices[min((uint32_t)Q.slice, p.num_slices - 1)];
    const int idc = sl.disable_deblocking_filter_idc;
    const bool sp = sl.slice_type == 3 || sl.slice_type == 4;
    const bool t8 = (Q.flags & H264R_MBF_T8x8) != 0;
    const bool onL = bx == 0 ? !(col == 0 || idc == 1 || (idc == 2 && !hasA)) : (idc != 1 && (bx == 2 || !t8));
    const bool onT = by == 0 ? !(cur < W || idc == 1 || (idc == 2 && !hasB)) : (idc != 1 && (by == 2 || !t8));
    // an MB edge whose neighbour is not available (another slice under
    // disable_deblocking_filter_idc 0) takes the MB itself as its p side
    const BsBlock own = bs_block(p, Q.type, Q.flags, Q.nz4x4, Q.nz8x8, Q.aux, bx, by);
    BsBlock sendL = own, sendT = own;
    if (bx == 3) {
        sendL = hasA ? bs_block(p, A0.type, A0.flags, A0.nz4x4, A0.nz8x8, A0.aux, 3, by)
                     : bs_block(p, Q.type, Q.flags, Q.nz4x4, Q.nz8x8, Q.aux, 3, by);
    }
    if (by == 3) {
        sendT = hasB ? bs_block(p, B0.type, B0.flags, B0.nz4x4, B0.nz8x8, B0.aux, bx, 3)
                     : bs_block(p, Q.type, Q.flags, Q.nz4x4, Q.nz8x8, Q.aux, bx, 3);
    }
    const int srcL = hb + (bx > 0 ? j - 1 : 4 * by + 3), srcT = hb + (by > 0 ? j - 4 : 12 + bx);
    BsBlock pl, pt;
    pl.mv0 = __shfl_sync(FULL, sendL.mv0, srcL);
    pl.mv1 = __shfl_sync(FULL, sendL.mv1, srcL);
    pl.rf = __shfl_sync(FULL, sendL.rf, srcL);
    pt.mv0 = __shfl_sync(FULL, sendT.mv0, srcT);
    pt.mv1 = __shfl_sync(FULL, sendT.mv1, srcT);
    pt.rf = __shfl_sync(FULL, sendT.rf, srcT);
    const int lim = p.fpic ? 2 : 4;
    auto strength = [&](const BsBlock &pb, bool edge_on, bool mbedge, bool vertical) -> int {
        if (!edge_on) return 0;
        const uint32_t f = pb.rf | own.rf;
        if ((f & (1u << 19)) || sp) return mbedge && (vertical || !p.fpic) ? 4 : 3;
        if (f & (1u << 18)) return 2;
        if (f & (1u << 20)) return 0xFF;
        return bs_motion_packed(pb, own, lim);
    };
    const int bsL = strength(pl, onL, bx == 0 && hasA, true);
    const int bsT = strength(pt, onT, by == 0 && hasB, false);
    uint32_t mystop = 0xFFFFFFFFu;
    if (bsL == 0xFF) mystop = stop_key(cur, SEQ_LV0 + bx, 4 * by);
    if (bsT == 0xFF) mystop = min(mystop, stop_key(cur, by == 0 ? SEQ_LH0 : SEQ_LH4 + by - 1, 4 * bx));
    if (__any_sync(FULL, on && mystop != 0xFFFFFFFFu)) {
        for (int o = 8; o > 0; o >>= 1) mystop = min(mystop, __shfl_xor_sync(FULL, mystop, o));
        if (on && j == 0 && mystop != 0xFFFFFFFFu) atomicMin(&const_cast<PicDesc *>(&p)->deblock_stop, mystop);
    }
    // line / column j (block row / column j >> 2): byte e the strength of
    // edge e there
    const int jq = j >> 2;
    uint32_t vrow = 0, hrow = 0;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        vrow |= (uint32_t)(__shfl_sync(FULL, bsL, hb + 4 * jq + e) & 255) << (8 * e);
        hrow |= (uint32_t)(__shfl_sync(FULL, bsT, hb + 4 * e + jq) & 255) << (8 * e);
    }
    uint8_t *out = p.bs + (size_t)cur * kBsBytes;
    if (on) {
        *(uint32_t *)(out + bs_lv(0, j)) = vrow;
        *(uint32_t *)(out + bs_lh(0, j)) = hrow;
    }
    // chroma line / column ck: edges 0 and 4 are luma edges 0 and 8 at luma
    // line / column 2ck
    const uint32_t cv = __shfl_sync(FULL, (vrow & 255u) | ((vrow >> 8) & 0xFF00u), hb + 2 * (j & 7));
    const uint32_t ch = __shfl_sync(FULL, (hrow & 255u) | ((hrow >> 8) & 0xFF00u), hb + 2 * (j & 7));
    if (on) {
        if (j < 8) *(uint16_t *)(out + bs_cv(0, j)) = (uint16_t)cv;
        else *(uint16_t *)(out + bs_ch(0, j - 8)) = (uint16_t)ch;
    }
    // thresholds of each edge class for k_deblock_frame: lane j < 9 the
    // component j / 3 and the class j % 3 (left, top, internal) of edge_params
    if (on && j < 9) {
        const int comp = j / 3, kind = j % 3;
        const bool useA = kind == 0 && hasA, useB = kind == 1 && hasB;
        const int ptype = useA ? A0.type : (useB ? B0.type : Q.type);
        const int pqp = useA ? A0.qpy : (useB ? B0.qpy : Q.qpy);
        int qPp = ptype == H264R_MB_IPCM ? 0 : pqp, qPq = Q.type == H264R_MB_IPCM ? 0 : Q.qpy;
        if (comp > 0) {
            const int off = sl.chroma_qp_offset[comp - 1];
            qPp = chroma_qp(qPp, off);
            qPq = chroma_qp(qPq, off);
        }
        const int qPav = (qPp + qPq + 1) >> 1;
        const int iA = H264R_CLIP3(0, 51, qPav + sl.filter_offset_a), iB = H264R_CLIP3(0, 51, qPav + sl.filter_offset_b);
        const uint32_t w = (uint32_t)kAlpha[iA] | ((uint32_t)kBeta[iB] << 8) | ((uint32_t)kTc0[0][iA] << 16) |
                           ((uint32_t)kTc0[1][iA] << 21) | ((uint32_t)kTc0[2][iA] << 26);
        *(uint32_t *)(out + kBsParams + 16 * comp + 4 * kind) = w;
    }
}

// MBAFF pictures: the strengths, edge controls and thresholds of MB cur with
// the whole warp.
__device__ __noinline__ void bs_mbaff_mb(const PicDesc &p, PicDesc *pp, int cur)
{
    const int lane = threadIdx.x & 31;
    EdgeCtl c = edge_ctl(p, cur);
    uint8_t *out = p.bs + (size_t)cur * kBsBytes;
    uint32_t mystop = 0xFFFFFFFFu;
    // Internal edges join two 4x4 blocks of the same MB (never a
    // mixed edge), so their strength is uniform over the 4 lines of a
    // block pair as in frame pictures: lanes 0..23 derive them
    // (dir, edge 1..3, block), and 4:2:0 chroma takes the luma value of
    // edge 8 at luma line 2k.  The MB edges (left, top, second top of a
    // frame MB under a field pair) are derived per line.
    uint32_t ivrow = 0, ihrow = 0;  // lane k < 16: internal strengths of line / column k, byte e
    {
        int bs = 0, dir = 0, ei = 1, b = 0;
        if (lane < 24) {
            dir = lane / 12;
            ei = 1 + (lane % 12) / 4;
            b = lane & 3;
            if (c.internal && (ei == 2 || !c.t8))
                bs = dir == 0 ? edge_bs(p, cur, 0, 1, 4 * ei, c.mbA, 0, 4 * b) : edge_bs(p, cur, 0, 0, 4 * ei, c.mbB, 0, 4 * b);
            if (bs == 0xFF) mystop = min(mystop, stop_key(cur, dir == 0 ? SEQ_LV0 + ei : SEQ_LH4 + ei - 1, 4 * b));
        }
        const int k = lane & 15;
#pragma unroll
        for (int e2 = 1; e2 < 4; e2++) {
            ivrow |= (uint32_t)(__shfl_sync(0xffffffffu, bs, (e2 - 1) * 4 + (k >> 2)) & 255) << (8 * e2);
            ihrow |= (uint32_t)(__shfl_sync(0xffffffffu, bs, 12 + (e2 - 1) * 4 + (k >> 2)) & 255) << (8 * e2);
        }
    }
    // MB edges per line: left (0..15), top (16..31), second top (32..47) luma;
    // chroma left (48..55), top (56..63), second top (64..71)
    uint32_t lv0 = 0, lh0 = 0;  // lane k < 16: luma left / top strength of line / column k
    for (int it = lane; it < 72; it += 32) {
        int bs = 0, seq = 0, k = 0;
        if (it < 16) {
            k = it;
            if (c.left) bs = edge_bs(p, cur, 0, 1, 0, c.mbA, c.leftMixed, k);
            seq = SEQ_LV0;
            lv0 = (uint32_t)bs;
        } else if (it < 32) {
            k = it - 16;
            if (c.top) bs = c.topDouble ? edge_bs(p, cur, 0, 0, 0, c.mbB - 1, 0, k) : edge_bs(p, cur, 0, 0, 0, c.mbB, 0, k);
            seq = SEQ_LH0;
        } else if (it < 48) {
            k = it - 32;
            if (c.top && c.topDouble) bs = edge_bs(p, cur, 0, 0, 1, c.mbB, 0, k);
            seq = SEQ_LH0B;
            out[kBsLumaTop2 + k] = (uint8_t)bs;
        } else if (it < 56) {
            k = it - 48;
            if (c.left) bs = edge_bs(p, cur, 1, 1, 0, c.mbA, c.leftMixed, k);
            seq = SEQ_CBV0;
            out[bs_cv(0, k)] = (uint8_t)bs;
        } else if (it < 64) {
            k = it - 56;
            if (c.top) bs = edge_bs(p, cur, 1, 0, 0, c.mbB, 0, k);
            seq = SEQ_CBH0;
            out[bs_ch(0, k)] = (uint8_t)bs;
        } else {
            k = it - 64;
            if (c.top && c.topDouble) bs = edge_bs(p, cur, 1, 0, 1, c.mbB, 0, k);
            seq = SEQ_CBH0B;
            out[kBsChromaTop2 + k] = (uint8_t)bs;
        }
        if (it >= 16 && it < 32) lh0 = (uint32_t)bs;
        if (bs == 0xFF) mystop = min(mystop, stop_key(cur, seq, k));
    }
    // lanes 16..31 derived the top edge of column lane-16 in their first item
    lh0 = __shfl_sync(0xffffffffu, lh0, (lane & 15) + 16);
    if (lane < 16) {
        *(uint32_t *)(out + bs_lv(0, lane)) = ivrow | (lv0 & 255);
        *(uint32_t *)(out + bs_lh(0, lane)) = ihrow | (lh0 & 255);
    }
    // chroma internal edge (4): luma edge 8 at luma line / column 2k
    const int ck = lane & 7;
    const uint32_t civ = __shfl_sync(0xffffffffu, (ivrow >> 16) & 255, 2 * ck);
    const uint32_t cih = __shfl_sync(0xffffffffu, (ihrow >> 16) & 255, 2 * ck);
    if (lane < 8) out[bs_cv(1, ck)] = (uint8_t)civ;
    else if (lane < 16) out[bs_ch(1, ck)] = (uint8_t)cih;
    // the edge controls of the MB and the thresholds of its edges, so that
    // the deblocking wavefront reads no records
    if (lane < 16) {
        uint32_t w;
        if (lane == 15) {
            w = (c.left ? kDbcLeft : 0u) | (c.top ? kDbcTop : 0u) | (c.internal ? kDbcInternal : 0u) | (c.t8 ? kDbcT8 : 0u) |
                (c.field ? kDbcField : 0u) | (c.leftMixed ? kDbcLeftMixed : 0u) | (c.topDouble ? kDbcTopDouble : 0u);
        } else {
            // 5 words per component: left (even lines), left (odd lines), top,
            // second top, internal; the p-side MB as deblock_mb's rules
            const int comp = lane / 5, kind = lane % 5;
            int mbP = cur;
            if (kind <= 1 && c.mbA >= 0) mbP = c.leftMixed ? c.mbA + kind : c.mbA;
            if (kind == 2) {
                const int mT = (c.topDouble && comp == 0) ? c.mbB - 1 : c.mbB;
                if (mT >= 0) mbP = mT;
            }
            if (kind == 3 && c.topDouble && c.mbB >= 0) mbP = c.mbB;
            int iA, al, be;
            edge_params(p, mbP, cur, comp, iA, al, be);
            w = (uint32_t)iA | ((uint32_t)al << 8) | ((uint32_t)be << 16);
        }
        *(uint32_t *)(out + kBsParams + 4 * (lane == 15 ? 0 : 1 + lane)) = w;
    }
    for (int o = 16; o > 0; o >>= 1) mystop = min(mystop, __shfl_xor_sync(0xffffffffu, mystop, o));
    if (lane == 0 && mystop != 0xFFFFFFFFu) atomicMin(&pp->deblock_stop, mystop);
}

// Boundary strengths of a batch: warp w takes MBs 2w and 2w + 1 (4 warps,
// 8 MBs per block); frame and field pictures a half-warp per MB, MBAFF
// pictures the whole warp per MB, one after the other.
__global__ void __launch_bounds__(128) k_bs(const PicDesc *__restrict__ pics, int npics, uint32_t total_mbs, LaunchState st)
{
    const uint32_t w = blockIdx.x * 4 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (2 * w >= total_mbs) return;
    const uint32_t g = 2 * w + (lane >> 4);
    const bool in = g < total_mbs;
    const int pi = find_pic_by_mb(pics, npics, in ? g : 2 * w);
    const bool frame = in && !pics[pi].mbaff && pics[pi].deblock;
    if (__any_sync(0xffffffffu, frame)) bs_frame_half(pics, pi, g, frame);
    for (int h = 0; h < 2; h++) {
        const int ph = __shfl_sync(0xffffffffu, pi, 16 * h);
        const bool inh = __shfl_sync(0xffffffffu, in, 16 * h);
        if (inh && pics[ph].mbaff && pics[ph].deblock)
            bs_mbaff_mb(pics[ph], const_cast<PicDesc *>(&pics[ph]), (int)(2 * w + h - pics[ph].mb_base));
    }
}

// ======================================================================
// K3b: deblocking wavefront
// ======================================================================
// filter one line (8.7.2.3 / 8.7.2.4, H264PictureDeblockingFilterProcess.cpp:1373-1522)
__device__ __forceinline__ void filter_line(int *pv, int *qv, int bS, bool chroma, int indexA, int alpha, int beta)
{
    if (!(bS != 0 && abs(pv[0] - qv[0]) < alpha && abs(pv[1] - pv[0]) < beta && abs(qv[1] - qv[0]) < beta)) return;
    int ap = abs(pv[2] - pv[0]), aq = abs(qv[2] - qv[0]);
    int np0 = pv[0], np1 = pv[1], np2 = pv[2], nq0 = qv[0], nq1 = qv[1], nq2 = qv[2];
    if (bS < 4) {
        int tc0 = kTc0[bS - 1][indexA];
        int tc = chroma ? tc0 + 1 : tc0 + (ap < beta) + (aq < beta);
        int delta = H264R_CLIP3(-tc, tc, ((((qv[0] - pv[0]) << 2) + (pv[1] - qv[1]) + 4) >> 3));
        np0 = clip1(pv[0] + delta);
        nq0 = clip1(qv[0] - delta);
        if (!chroma && ap < beta) np1 = (uint8_t)(pv[1] + H264R_CLIP3(-tc0, tc0, (pv[2] + ((pv[0] + qv[0] + 1) >> 1) - (pv[1] << 1)) >> 1));
        if (!chroma && aq < beta) nq1 = (uint8_t)(qv[1] + H264R_CLIP3(-tc0, tc0, (qv[2] + ((pv[0] + qv[0] + 1) >> 1) - (qv[1] << 1)) >> 1));
    } else {
        bool sm = abs(pv[0] - qv[0]) < ((alpha >> 2) + 2);
        if (!chroma && ap < beta && sm) {
            np0 = (pv[2] + 2 * pv[1] + 2 * pv[0] + 2 * qv[0] + qv[1] + 4) >> 3;
            np1 = (pv[2] + pv[1] + pv[0] + qv[0] + 2) >> 2;
            np2 = (2 * pv[3] + 3 * pv[2] + pv[1] + pv[0] + qv[0] + 4) >> 3;
        } else {
            np0 = (2 * pv[1] + pv[0] + qv[1] + 2) >> 2;
        }
        if (!chroma && aq < beta && sm) {
            nq0 = (pv[1] + 2 * pv[0] + 2 * qv[0] + 2 * qv[1] + qv[2] + 4) >> 3;
            nq1 = (pv[0] + qv[0] + qv[1] + qv[2] + 2) >> 2;
            nq2 = (2 * qv[3] + 3 * qv[2] + qv[1] + qv[0] + pv[0] + 4) >> 3;
        } else {
            nq0 = (2 * qv[1] + qv[0] + pv[1] + 2) >> 2;
        }
    }
    pv[0] = np0; pv[1] = np1; pv[2] = np2;
    qv[0] = nq0; qv[1] = nq1; qv[2] = nq2;
}

// Samples of one component around the MB pair being filtered, staged in
// shared memory: sample (x, y) of the plane is base[(y - y0) * stride + (x - x0)].
struct DbWin {
    uint8_t *base;
    int x0, y0, stride, size;  // size: bytes of the window
};

// Thresholds of one edge between MBs P and Q (8.7.2.2, 1314-1369).
struct EdgeQ {
    int iA, al, be;
};

__device__ __forceinline__ EdgeQ edge_q(const h264r_mb &P, const h264r_mb &Q, const h264r_slice &sq, int comp)
{
    int qPp = P.type == H264R_MB_IPCM ? 0 : P.qpy, qPq = Q.type == H264R_MB_IPCM ? 0 : Q.qpy;
    if (comp) {
        const int off = sq.chroma_qp_offset[comp - 1];
        qPp = chroma_qp(qPp, off);
        qPq = chroma_qp(qPq, off);
    }
    const int qPav = (qPp + qPq + 1) >> 1;
    EdgeQ q;
    q.iA = H264R_CLIP3(0, 51, qPav + sq.filter_offset_a);
    q.al = kAlpha[q.iA];
    q.be = kBeta[H264R_CLIP3(0, 51, qPav + sq.filter_offset_b)];
    return q;
}

// One edge step, one line per active lane (8.7.1, 639-840).  comp: 0 luma,
// 1 Cb, 2 Cr; (xP, yP): the MB's first sample of this component; k: line
// index of this lane; bs: its strength; q: the edge's thresholds.
__device__ __forceinline__ void edge_line(int xP, int yP, int comp, int vertical, int e, int fieldMode, int k, int bs,
                                          const EdgeQ &q, const DbWin &w)
{
    if (bs == 0) return;
    const int ddy = 1 + fieldMode;
    const int xE = vertical ? e : k, yE = vertical ? k : e;
    int qi[4], pi[4];
    for (int i = 0; i < 4; i++) {
        int qy, qx, py, px;
        if (vertical) {
            qy = py = yP + ddy * yE;
            qx = xP + xE + i;
            px = xP + xE - i - 1;
        } else {
            qy = yP + ddy * (yE + i) - (yE % 2);
            py = yP + ddy * (yE - i - 1) - (yE % 2);
            qx = px = xP + xE;
        }
        qi[i] = (qy - w.y0) * w.stride + (qx - w.x0);
        pi[i] = (py - w.y0) * w.stride + (px - w.x0);
        // the window covers every sample an MBAFF edge can reach; a line that
        // would leave it is not filtered (and shows as a parity difference)
        if ((unsigned)qi[i] >= (unsigned)w.size || (unsigned)pi[i] >= (unsigned)w.size) return;
    }
    int pv[4], qv[4];
    for (int i = 0; i < 4; i++) {
        pv[i] = w.base[pi[i]];
        qv[i] = w.base[qi[i]];
    }
    filter_line(pv, qv, bs, comp != 0, q.iA, q.al, q.be);
    for (int i = 0; i < 3; i++) {
        w.base[qi[i]] = (uint8_t)qv[i];
        w.base[pi[i]] = (uint8_t)pv[i];
    }
}

// ---------------------------------------------------------------- MBAFF pictures
// One warp per MB-pair row and plane group: luma (even ticket), or Cb and Cr
// together (odd ticket); progress of pair row r is published per plane,
// luma at index 2r + 1, chroma at 2r.  Lanes 0..15 (or 0..7 / 8..15 per
// chroma plane) take the lines of the pair's top MB, lanes 16..31 those of
// the bottom MB.  The reference filters a pair as top MB (vertical, then
// horizontal edges), then bottom MB; the bottom MB's vertical edges touch
// only its own lines (rows 16..31 of a frame pair, the odd rows of a field
// pair) and the top MB's horizontal edges never do, so the vertical edges of
// both MBs run together, before the wait for the row above (they reach no
// row above the pair).  The horizontal edges of a field pair's two MBs touch
// opposite parities and run together too; a frame pair's bottom MB follows
// its top MB on the same lanes.  Within one MB a lane owns a line (vertical
// edges) or a column (horizontal edges), so the edge steps of a direction
// need no barrier.  Samples are filtered on a window in shared memory
// (DbWin): luma columns x0-4..x0+15 and rows y0-8..y0+31, chroma x0/2-4..
// x0/2+7 and y0/2-8..y0/2+15 per plane.  The window slides right one pair
// at a time: its first four columns are the previous window's last four
// (final once the previous pair is done), the pair's own rows are fetched
// one pair ahead (nothing in this kernel writes them before the pair), and
// only the eight rows above are loaded after the wait.

// Edge controls, thresholds and strengths of one MB for one lane, from k_bs.
struct MbaffEdges {
    uint32_t ctl;                     // kDbc* bits
    uint32_t qL0, qL1, qT, qT2, qI;   // thresholds of the lane's component (iA | alpha << 8 | beta << 16)
    uint32_t bv, bh, b2;              // the lane's strengths: vertical edge e (byte e), horizontal edge e, second top edge
};

__device__ __forceinline__ EdgeQ unq(uint32_t v)
{
    EdgeQ q;
    q.iA = v & 255;
    q.al = (v >> 8) & 255;
    q.be = (v >> 16) & 255;
    return q;
}

// comp: 0 luma, 1 Cb, 2 Cr; k: line (or column) of the lane within the MB
__device__ __forceinline__ void mbaff_fetch(const PicDesc &p, int cur, int comp, int k, MbaffEdges &m)
{
    const uint8_t *bs = p.bs + (size_t)cur * kBsBytes;
    const uint32_t *prm = (const uint32_t *)(bs + kBsParams);
    const uint32_t *pc = prm + 1 + 5 * comp;
    m.ctl = __ldcg(prm);
    m.qL0 = __ldcg(pc);
    m.qL1 = __ldcg(pc + 1);
    m.qT = __ldcg(pc + 2);
    m.qT2 = __ldcg(pc + 3);
    m.qI = __ldcg(pc + 4);
    if (comp == 0) {
        m.bv = __ldcg((const uint32_t *)(bs + bs_lv(0, k)));
        m.bh = __ldcg((const uint32_t *)(bs + bs_lh(0, k)));
        m.b2 = __ldcg(bs + kBsLumaTop2 + k);
    } else {
        m.bv = __ldcg((const uint16_t *)(bs + bs_cv(0, k)));
        m.bh = __ldcg((const uint16_t *)(bs + bs_ch(0, k)));
        m.b2 = __ldcg(bs + kBsChromaTop2 + k);
    }
    // a step at or after the reference's early return (a failed bS
    // derivation) is not filtered
    const uint32_t stop = p.deblock_stop;
    if ((uint32_t)cur >= (stop >> 10)) {
        const int cseq = comp == 2 ? 1 : 0;
        for (int e = 0; e < 4; e++) {
            const int sv = comp ? (e == 0 ? SEQ_CBV0 : SEQ_CBV4) + cseq : SEQ_LV0 + e;
            const int sh = comp ? (e == 0 ? SEQ_CBH0 : SEQ_CBH4) + cseq : (e == 0 ? SEQ_LH0 : SEQ_LH4 + e - 1);
            if (stop_key(cur, sv, k) >= stop) m.bv &= ~(0xFFu << (8 * e));
            if (stop_key(cur, sh, k) >= stop) m.bh &= ~(0xFFu << (8 * e));
        }
        if (stop_key(cur, comp ? SEQ_CBH0B + cseq : SEQ_LH0B, k) >= stop) m.b2 = 0;
    }
}

__device__ __forceinline__ MbaffEdges mbaff_shfl(const MbaffEdges &m, int src)
{
    MbaffEdges r;
    r.ctl = __shfl_sync(0xffffffffu, m.ctl, src);
    r.qL0 = __shfl_sync(0xffffffffu, m.qL0, src);
    r.qL1 = __shfl_sync(0xffffffffu, m.qL1, src);
    r.qT = __shfl_sync(0xffffffffu, m.qT, src);
    r.qT2 = __shfl_sync(0xffffffffu, m.qT2, src);
    r.qI = __shfl_sync(0xffffffffu, m.qI, src);
    r.bv = __shfl_sync(0xffffffffu, m.bv, src);
    r.bh = __shfl_sync(0xffffffffu, m.bh, src);
    r.b2 = __shfl_sync(0xffffffffu, m.b2, src);
    return r;
}

// Edges of one direction of one MB on the lane's line (vertical) or column
// (horizontal).  (xP, yP): the MB's first sample of the component.  The
// p-side MB of each edge is the one k_bs chose: alternate lines of a mixed
// left edge take the two MBs of the left field pair; a frame MB under a
// field pair filters its top edge twice, as a top-field and a bottom-field
// edge (Deblocking_filter_process, H264PictureDeblockingFilterProcess.cpp:
// 76-160, 246-278).
template <bool CHROMA>
__device__ __forceinline__ void mbaff_edges_v(int xP, int yP, int k, const MbaffEdges &m, const DbWin &w)
{
    const int comp = CHROMA ? 1 : 0;  // only the filter kind matters to edge_line
    const int field = (m.ctl & kDbcField) != 0;
    if (m.ctl & kDbcLeft)
        edge_line(xP, yP, comp, 1, 0, field, k, m.bv & 255, unq((m.ctl & kDbcLeftMixed) && (k & 1) ? m.qL1 : m.qL0), w);
    if (m.ctl & kDbcInternal) {
        const EdgeQ qI = unq(m.qI);
#pragma unroll 1
        for (int e = 1; e < (CHROMA ? 2 : 4); e++)
            if (CHROMA || e == 2 || !(m.ctl & kDbcT8)) edge_line(xP, yP, comp, 1, 4 * e, field, k, (m.bv >> (8 * e)) & 255, qI, w);
    }
}

template <bool CHROMA>
__device__ __forceinline__ void mbaff_edges_h(int xP, int yP, int k, const MbaffEdges &m, const DbWin &w)
{
    const int comp = CHROMA ? 1 : 0;
    const int field = (m.ctl & kDbcField) != 0;
    if (m.ctl & kDbcTop) {
        if (m.ctl & kDbcTopDouble) {
            edge_line(xP, yP, comp, 0, 0, 1, k, m.bh & 255, unq(m.qT), w);
            edge_line(xP, yP, comp, 0, 1, 1, k, m.b2, unq(m.qT2), w);
        } else {
            edge_line(xP, yP, comp, 0, 0, field, k, m.bh & 255, unq(m.qT), w);
        }
    }
    if (m.ctl & kDbcInternal) {
        const EdgeQ qI = unq(m.qI);
#pragma unroll 1
        for (int e = 1; e < (CHROMA ? 2 : 4); e++)
            if (CHROMA || e == 2 || !(m.ctl & kDbcT8)) edge_line(xP, yP, comp, 0, 4 * e, field, k, (m.bh >> (8 * e)) & 255, qI, w);
    }
}

// An MBAFF deblocking block: kMbWarps warps on consecutive MB-pair rows of
// one plane.  As in frame pictures, a warp takes the rows above from the
// warp before it through shared memory (x: that warp's bottom eight rows of
// each pair, own columns; the last word is filled in once the next pair's
// left edge is done) and waits on its shared-memory progress; the block's
// first warp reads and waits on global memory, its last warp publishes.
struct DbMbaffShared {
    union {
        uint32_t l[kMbWarps][200];  // luma windows: 40 rows of 5 words
        uint32_t c[kMbWarps][144];  // chroma windows: 2 planes x 24 rows of 3 words
    } win;
    union {
        uint32_t l[kMbWarps - 1][kMbXRing][8][4];     // luma rows 24..31 of the pair
        uint32_t c[kMbWarps - 1][kMbXRing][2][8][2];  // chroma rows 8..15 per plane
    } x;
    int done[kMbWarps];  // pairs completed
    int used[kMbWarps];  // pairs whose rows above were taken
};

// Luma of MB-pair row `row`, warp wi of nw in its block.
__device__ void mbaff_luma_row(const PicDesc &p, int row, int wi, int nw, DbMbaffShared &S, const LaunchState &st)
{
    uint32_t *win = S.win.l[wi];
    const bool from_cta = wi > 0, to_cta = wi + 1 < nw;
    int seen_used = 0;
    const int lane = threadIdx.x & 31, h = lane >> 4, k = lane & 15;
    const int uw = (int)p.units_w, W = p.ys, y0 = row * 32;
    int *prog = p.progress + p.units_h;
    uint8_t *Y = plane_y(p);
    const DbWin w0 = {(uint8_t *)win, 0, y0 - 8, 20, 40 * 20};
    int seen = 0;
    uint4 nown;  // row y0 + lane of the next pair
    MbaffEdges nm;
    auto fetch = [&](int u) {
        nown = __ldcg((const uint4 *)(Y + (size_t)(y0 + lane) * W + u * 16));
        mbaff_fetch(p, 2 * (row * uw + u) + h, 0, k, nm);
    };
    fetch(0);
    for (int u = 0; u < uw; u++) {
        // the warp below must have taken the rows this pair's end overwrites
        if (to_cta && !cta_wait(st, &S.used[wi + 1], u + 1 - kMbXRing, seen_used)) return;
        const int x0 = u * 16;
        const MbaffEdges m = nm;
        uint32_t *wr = win + (8 + lane) * 5;  // the lane's own row
        if (u > 0) {
            wr[0] = wr[4];
            if (lane < 8) win[lane * 5] = win[lane * 5 + 4];
        }
        wr[1] = nown.x;
        wr[2] = nown.y;
        wr[3] = nown.z;
        wr[4] = nown.w;
        __syncwarp();
        if (u + 1 < uw) fetch(u + 1);
        DbWin w = w0;
        w.x0 = x0 - 4;
        const int field = (m.ctl & kDbcField) != 0;
        mbaff_edges_v<false>(x0, field ? y0 + h : y0 + 16 * h, k, m, w);
        // the row above is final once its warp is two pairs ahead
        if (row > 0) {
            const bool ok = from_cta ? cta_wait(st, &S.done[wi - 1], min(u + 2, uw), seen)
                                     : db_wait(st, prog + 2 * row - 1, min(u + 2, uw), seen);
            if (!ok) return;
        }
        if (row > 0 && lane < 8) {
            uint32_t *wt = win + lane * 5;
            if (from_cta) {
                const uint32_t *e = S.x.l[wi - 1][u % kMbXRing][lane];
                wt[1] = e[0];
                wt[2] = e[1];
                wt[3] = e[2];
                wt[4] = e[3];
            } else {
                const uint4 t = __ldcg((const uint4 *)(Y + (size_t)(y0 - 8 + lane) * W + x0));
                wt[1] = t.x;
                wt[2] = t.y;
                wt[3] = t.z;
                wt[4] = t.w;
            }
        }
        const MbaffEdges mb = mbaff_shfl(m, lane | 16);  // the bottom MB's, for a frame pair
        __syncwarp();
        if (field) mbaff_edges_h<false>(x0, y0 + h, k, m, w);
        else if (h == 0) {
            mbaff_edges_h<false>(x0, y0, k, m, w);
            mbaff_edges_h<false>(x0, y0 + 16, k, mb, w);
        }
        __syncwarp();
        // rows y0-6..y0+31 (the top edges change at most three field rows up)
        for (int r = lane + 2; r < 40; r += 32) {
            const int y = y0 - 8 + r;
            if (y < 0) continue;
            const uint32_t *s = win + r * 5;
            uint8_t *d = Y + (size_t)y * W + x0;
            *(uint4 *)d = make_uint4(s[1], s[2], s[3], s[4]);
            if (x0 > 0) *(uint32_t *)(d - 4) = s[0];
        }
        // the bottom rows for the warp below; this pair's left edge finished
        // the previous pair's last columns
        if (to_cta && lane < 8) {
            const uint32_t *s = win + (32 + lane) * 5;
            uint32_t *e = S.x.l[wi][u % kMbXRing][lane];
            e[0] = s[1];
            e[1] = s[2];
            e[2] = s[3];
            e[3] = s[4];
            if (u > 0) S.x.l[wi][(u - 1) % kMbXRing][lane][3] = s[0];
        }
        __syncwarp();
        if (to_cta) {
            __threadfence_block();
            if (lane == 0) *(volatile int *)&S.done[wi] = u + 1;
        } else if (lane == 0) {
            st_release(prog + 2 * row + 1, u + 1);
        }
        if (from_cta && row > 0) {
            __threadfence_block();
            if (lane == 0) *(volatile int *)&S.used[wi] = u + 1;
        }
    }
}

// Cb and Cr of MB-pair row `row`, warp wi of nw in its block.
__device__ void mbaff_chroma_row(const PicDesc &p, int row, int wi, int nw, DbMbaffShared &S, const LaunchState &st)
{
    uint32_t *win = S.win.c[wi];
    const bool from_cta = wi > 0, to_cta = wi + 1 < nw;
    int seen_used = 0;
    const int lane = threadIdx.x & 31, h = lane >> 4, pl = (lane >> 3) & 1, k = lane & 7;
    const int uw = (int)p.units_w, Wc = p.cs, yc0 = row * 16;
    int *prog = p.progress + p.units_h;
    // staging lanes: plane sp, row 8 + sr of the window (and sr when sr < 8)
    const int sp = lane >> 4, sr = lane & 15;
    uint8_t *Cs = plane_c(p, sp);
    const DbWin w0 = {(uint8_t *)(win + 72 * pl), 0, yc0 - 8, 12, 24 * 12};
    int seen = 0;
    uint2 nown;
    MbaffEdges nm;
    auto fetch = [&](int u) {
        nown = __ldcg((const uint2 *)(Cs + (size_t)(yc0 + sr) * Wc + u * 8));
        mbaff_fetch(p, 2 * (row * uw + u) + h, 1 + pl, k, nm);
    };
    fetch(0);
    for (int u = 0; u < uw; u++) {
        if (to_cta && !cta_wait(st, &S.used[wi + 1], u + 1 - kMbXRing, seen_used)) return;
        const int xc0 = u * 8;
        const MbaffEdges m = nm;
        uint32_t *ws = win + 72 * sp;
        uint32_t *wr = ws + (8 + sr) * 3;
        if (u > 0) {
            wr[0] = wr[2];
            if (sr < 8) ws[sr * 3] = ws[sr * 3 + 2];
        }
        wr[1] = nown.x;
        wr[2] = nown.y;
        __syncwarp();
        if (u + 1 < uw) fetch(u + 1);
        DbWin w = w0;
        w.x0 = xc0 - 4;
        const int field = (m.ctl & kDbcField) != 0;
        // (yI + 1) / 2 of the MB's first luma row yI
        mbaff_edges_v<true>(xc0, field ? yc0 + h : yc0 + 8 * h, k, m, w);
        if (row > 0) {
            const bool ok = from_cta ? cta_wait(st, &S.done[wi - 1], min(u + 2, uw), seen)
                                     : db_wait(st, prog + 2 * row - 2, min(u + 2, uw), seen);
            if (!ok) return;
        }
        if (row > 0 && sr < 8) {
            if (from_cta) {
                const uint32_t *e = S.x.c[wi - 1][u % kMbXRing][sp][sr];
                ws[sr * 3 + 1] = e[0];
                ws[sr * 3 + 2] = e[1];
            } else {
                const uint2 t = __ldcg((const uint2 *)(Cs + (size_t)(yc0 - 8 + sr) * Wc + xc0));
                ws[sr * 3 + 1] = t.x;
                ws[sr * 3 + 2] = t.y;
            }
        }
        const MbaffEdges mb = mbaff_shfl(m, lane | 16);
        __syncwarp();
        if (field) mbaff_edges_h<true>(xc0, yc0 + h, k, m, w);
        else if (h == 0) {
            mbaff_edges_h<true>(xc0, yc0, k, m, w);
            mbaff_edges_h<true>(xc0, yc0 + 8, k, mb, w);
        }
        __syncwarp();
        // rows yc0-4..yc0+15 of both planes (chroma edges change one row on each side)
        for (int i = lane; i < 40; i += 32) {
            const int q = i / 20, r = 4 + i % 20, y = yc0 - 8 + r;
            if (y < 0) continue;
            const uint32_t *s = win + 72 * q + r * 3;
            uint8_t *d = plane_c(p, q) + (size_t)y * Wc + xc0;
            *(uint2 *)d = make_uint2(s[1], s[2]);
            if (xc0 > 0) *(uint32_t *)(d - 4) = s[0];
        }
        if (to_cta && sr < 8) {
            const uint32_t *s = ws + (16 + sr) * 3;
            uint32_t *e = S.x.c[wi][u % kMbXRing][sp][sr];
            e[0] = s[1];
            e[1] = s[2];
            if (u > 0) S.x.c[wi][(u - 1) % kMbXRing][sp][sr][1] = s[0];
        }
        __syncwarp();
        if (to_cta) {
            __threadfence_block();
            if (lane == 0) *(volatile int *)&S.done[wi] = u + 1;
        } else if (lane == 0) {
            st_release(prog + 2 * row, u + 1);
        }
        if (from_cta && row > 0) {
            __threadfence_block();
            if (lane == 0) *(volatile int *)&S.used[wi] = u + 1;
        }
    }
}

// ---------------------------------------------------------------- frame fast path
// Non-MBAFF pictures.  Luma and chroma are filtered by separate warps (the
// planes never interact), each warp taking a pair of MB rows: lanes 0..15
// work on the first row, 16..31 on the second, which trails the first by
// one MB: in the reference's raster order a MB's top edge comes after the
// left edge of the MB above-right, and every step runs both rows' vertical
// edges before either row's horizontal edges.  A luma lane owns one line of the MB;
// a chroma lane one line of Cb (lanes 0..7 of the half) or Cr (8..15).  A
// line is filtered in registers across all edges of one direction, and the
// MB passes through a byte tile in shared memory once, between its vertical
// and horizontal edges.  The vertical edges of a MB touch only its own MB
// row, so they run before the wait for the row above.  The second row takes
// the first row's bottom lines from a ring in shared memory.  Strengths and
// thresholds come from k_bs.  Progress of a pair's second row is published
// per plane: luma at the odd row index, chroma at the even one.
struct DbLumaSmem {
    __align__(16) uint8_t t[2][20][16];  // per half: rows -4..15 of the MB
    uint4 ring[3][4];                    // first row: rows 12..15 of the MB in column % 3
};

struct DbChromaSmem {
    __align__(16) uint8_t t[2][2][12][8];  // per half and plane: rows -4..7 of the MB
    uint2 ring[3][2][4];                   // first row: rows 4..7, per plane
};

// A frame deblocking block: kDbWarps warps on consecutive MB-row pairs of one
// plane.  A warp's first row takes the rows above from the warp before it
// through shared memory (x: that warp's second row's bottom lines, kDbXRing
// MBs deep) and waits on its shared-memory progress (done); only the block's
// first warp waits on, and reads, global memory, and only its last warp
// publishes global progress.  used is the consumer's progress, which keeps a
// producer from overwriting lines not yet taken.
// W row-pair warps per block: k_deblock_frame uses kDbWarps, k_deblock_frame4
// four (the other shape the autotuner tries).
template <int W>
struct DbFrameShared {
    union {
        DbLumaSmem l[W];
        DbChromaSmem c[W];
    } w;
    union {
        uint4 l[W - 1][kDbXRing][4];     // luma rows 12..15
        uint2 c[W - 1][kDbXRing][2][4];  // chroma rows 4..7 per plane
    } x;
    int done[W];  // second row: MBs up to done-2 completed and the vertical edges of MB done-1 (uw+1: all)
    int used[W];  // first row: MBs whose rows above were taken
};


__device__ __forceinline__ int db_tc0(uint32_t prm, int bS) { return (prm >> (11 + 5 * bS)) & 31; }

// 8.7.2.3 / 8.7.2.4 on the luma line v with q0 at index Q
// (Filtering_process_for_edges_with_bS_less_than_4 / _equal_to_4,
// H264PictureDeblockingFilterProcess.cpp:1373-1522).  bS 4 occurs on MB
// edges only.
template <int Q, bool MBEDGE, int N>
__device__ __forceinline__ void db_luma(int (&v)[N], int bS, uint32_t prm)
{
    const int alpha = prm & 255, beta = (prm >> 8) & 255;
    const int p0 = v[Q - 1], p1 = v[Q - 2], p2 = v[Q - 3], q0 = v[Q], q1 = v[Q + 1], q2 = v[Q + 2];
    if (bS == 0 || abs(p0 - q0) >= alpha || abs(p1 - p0) >= beta || abs(q1 - q0) >= beta) return;
    const bool ap = abs(p2 - p0) < beta, aq = abs(q2 - q0) < beta;
    if (MBEDGE && bS == 4) {
        const int p3 = v[Q - 4], q3 = v[Q + 3];
        const bool sm = abs(p0 - q0) < ((alpha >> 2) + 2);
        if (ap && sm) {
            v[Q - 1] = (p2 + 2 * p1 + 2 * p0 + 2 * q0 + q1 + 4) >> 3;
            v[Q - 2] = (p2 + p1 + p0 + q0 + 2) >> 2;
            v[Q - 3] = (2 * p3 + 3 * p2 + p1 + p0 + q0 + 4) >> 3;
        } else {
            v[Q - 1] = (2 * p1 + p0 + q1 + 2) >> 2;
        }
        if (aq && sm) {
            v[Q] = (p1 + 2 * p0 + 2 * q0 + 2 * q1 + q2 + 4) >> 3;
            v[Q + 1] = (p0 + q0 + q1 + q2 + 2) >> 2;
            v[Q + 2] = (2 * q3 + 3 * q2 + q1 + q0 + p0 + 4) >> 3;
        } else {
            v[Q] = (2 * q1 + q0 + p1 + 2) >> 2;
        }
        return;
    }
    const int tc0 = db_tc0(prm, bS);
    const int tc = tc0 + ap + aq;
    const int delta = H264R_CLIP3(-tc, tc, (((q0 - p0) << 2) + (p1 - q1) + 4) >> 3);
    v[Q - 1] = clip1(p0 + delta);
    v[Q] = clip1(q0 - delta);
    if (ap) v[Q - 2] = (p1 + H264R_CLIP3(-tc0, tc0, (p2 + ((p0 + q0 + 1) >> 1) - (p1 << 1)) >> 1)) & 255;
    if (aq) v[Q + 1] = (q1 + H264R_CLIP3(-tc0, tc0, (q2 + ((p0 + q0 + 1) >> 1) - (q1 << 1)) >> 1)) & 255;
}

// chroma line (chromaStyleFilteringFlag = 1): only p0 and q0 change
template <int Q, bool MBEDGE, int N>
__device__ __forceinline__ void db_chroma(int (&v)[N], int bS, uint32_t prm)
{
    const int alpha = prm & 255, beta = (prm >> 8) & 255;
    const int p0 = v[Q - 1], p1 = v[Q - 2], q0 = v[Q], q1 = v[Q + 1];
    if (bS == 0 || abs(p0 - q0) >= alpha || abs(p1 - p0) >= beta || abs(q1 - q0) >= beta) return;
    if (MBEDGE && bS == 4) {
        v[Q - 1] = (2 * p1 + p0 + q1 + 2) >> 2;
        v[Q] = (2 * q1 + q0 + p1 + 2) >> 2;
        return;
    }
    const int tc = db_tc0(prm, bS) + 1;
    const int delta = H264R_CLIP3(-tc, tc, (((q0 - p0) << 2) + (p1 - q1) + 4) >> 3);
    v[Q - 1] = clip1(p0 + delta);
    v[Q] = clip1(q0 - delta);
}

template <int NW>
__device__ void deblock_pair_luma(const PicDesc &p, int pair, int wi, int nw, DbLumaSmem &s, DbFrameShared<NW> &S,
                                  const LaunchState &st)
{
    const int lane = threadIdx.x & 31;
    const int h = lane >> 4, k = lane & 15;
    const int uw = (int)p.units_w, rows = (int)p.units_h, W = p.ys;
    const int row = 2 * pair + h;
    const bool row_ok = row < rows;
    const bool has_second = 2 * pair + 1 < rows;
    const int steps = has_second ? uw + 1 : uw;
    const bool from_cta = wi > 0;                  // rows above from the warp before, in shared memory
    const bool to_cta = wi + 1 < nw && has_second;  // bottom lines to the warp after
    int *prog = p.progress + p.units_h;
    uint8_t *Y = plane_y(p);
    uint8_t(*t)[16] = s.t[h];
    const uint32_t stop = p.deblock_stop;
    int left[4] = {0, 0, 0, 0};
    int seen = 0, seen_used = 0;
    // prefetched per MB: the lane's line, its strengths (byte e: edge e), the thresholds
    uint4 nl = make_uint4(0, 0, 0, 0), npl = nl;
    uint32_t nlv = 0, nlh = 0;
    auto fetch = [&](int u) {
        const int cur = row * uw + u;
        const uint8_t *bs = p.bs + (size_t)cur * kBsBytes;
        nl = __ldcg((const uint4 *)(Y + (size_t)(row * 16 + k) * W + u * 16));
        nlv = __ldcg((const uint32_t *)(bs + bs_lv(0, k)));
        nlh = __ldcg((const uint32_t *)(bs + bs_lh(0, k)));
        npl = __ldcg((const uint4 *)(bs + kBsParams));
    };
    if (row_ok && h == 0) fetch(0);
    for (int step = 0; step < steps; step++) {
        const int u = step - h;
        const bool act = row_ok && u >= 0 && u < uw;
        const uint4 line = nl, prm = npl;
        uint32_t lv = nlv, lh = nlh;
        if (row_ok && u + 1 >= 0 && u + 1 < uw) fetch(u + 1);
        // the warp after must have taken the lines this step overwrites
        if (to_cta && step >= 1 && !cta_wait(st, &S.used[wi + 1], min(step - kDbXRing, uw), seen_used)) return;
        const int x0 = u * 16, y0 = row * 16;
        if (act) {
            const int cur = row * uw + u;
            if ((uint32_t)cur >= (stop >> 10)) {  // the reference's bS derivation fails at or before this MB
                if ((uint32_t)cur > (stop >> 10)) lv = lh = 0;
                else {
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        if (stop_key(cur, SEQ_LV0 + e, k) >= stop) lv &= ~(0xFFu << (8 * e));
                        if (stop_key(cur, e == 0 ? SEQ_LH0 : SEQ_LH4 + e - 1, k) >= stop) lh &= ~(0xFFu << (8 * e));
                    }
                }
            }
            int v[20];
#pragma unroll
            for (int i = 0; i < 4; i++) v[i] = left[i];
            unpack16(line, &v[4]);
            db_luma<4, true>(v, lv & 255, prm.x);
            db_luma<8, false>(v, (lv >> 8) & 255, prm.z);
            db_luma<12, false>(v, (lv >> 16) & 255, prm.z);
            db_luma<16, false>(v, lv >> 24, prm.z);
            if (u > 0) {
                // the left MB's last columns are final now
                const uint32_t lw = pack4(v[0], v[1], v[2], v[3]);
                *(uint32_t *)(Y + (size_t)(y0 + k) * W + x0 - 4) = lw;
                if (h == 0 && k >= 12) s.ring[(u - 1) % 3][k - 12].w = lw;
                if (h == 1 && to_cta && k >= 12) S.x.l[wi][(u - 1) % kDbXRing][k - 12].w = lw;
            }
            *(uint4 *)&t[k + 4][0] = pack16(&v[4]);
        }
        // the warp below needs MB u of this warp's second row and the vertical
        // edges of MB u+1: both are done once this step's vertical edges are
        if (to_cta && step >= 1) {
            __syncwarp();
            __threadfence_block();
            if (lane == 0) *(volatile int *)&S.done[wi] = step;
        }
        // ---- the row above: final once its warp is two MBs ahead
        if (2 * pair > 0 && step < uw) {
            // in the block: MB step and the vertical edges of MB step+1 of the
            // row above (its last MB: the end of that warp's last step, uw+1);
            // across blocks: MBs 0..step+1 completed
            const bool ok = from_cta ? cta_wait(st, &S.done[wi - 1], step + 2, seen)
                                     : db_wait(st, prog + 2 * pair - 1, min(step + 2, uw), seen);
            if (!ok) return;
        }
        __syncwarp();  // the first row's vertical edges of this step updated the ring
        if (act && row > 0 && k < 4)
            *(uint4 *)&t[k][0] = h == 1 ? s.ring[u % 3][k]
                                        : (from_cta ? S.x.l[wi - 1][u % kDbXRing][k]
                                                    : __ldcg((const uint4 *)(Y + (size_t)(y0 - 4 + k) * W + x0)));
        __syncwarp();
        // ---- horizontal edges: the lane owns a column
        if (act) {
            int v[20];
#pragma unroll
            for (int i = 0; i < 20; i++) v[i] = t[i][k];
            db_luma<4, true>(v, lh & 255, prm.y);
            db_luma<8, false>(v, (lh >> 8) & 255, prm.z);
            db_luma<12, false>(v, (lh >> 16) & 255, prm.z);
            db_luma<16, false>(v, lh >> 24, prm.z);
#pragma unroll
            for (int i = 1; i < 19; i++) t[i][k] = (uint8_t)v[i];
        }
        __syncwarp();
        // ---- store the MB and the three rows above it
        if (act) {
            const uint4 lr = *(const uint4 *)&t[k + 4][0];
            *(uint4 *)(Y + (size_t)(y0 + k) * W + x0) = lr;
#pragma unroll
            for (int i = 0; i < 4; i++) left[i] = (lr.w >> (8 * i)) & 255;
            if (h == 0 && k >= 12) s.ring[u % 3][k - 12] = lr;
            if (h == 1 && to_cta && k >= 12) S.x.l[wi][u % kDbXRing][k - 12] = lr;
            if (row > 0 && k < 3) *(uint4 *)(Y + (size_t)(y0 - 3 + k) * W + x0) = *(const uint4 *)&t[1 + k][0];
        }
        __syncwarp();
        if (has_second && step >= 1 && !to_cta && lane == 0)  // the second row has MBs 0..step-1 done
            st_release(prog + 2 * pair + 1, step);
        if (to_cta && step == uw) {  // the second row's last MB is complete
            __syncwarp();
            __threadfence_block();
            if (lane == 0) *(volatile int *)&S.done[wi] = uw + 1;
        }
        if (from_cta && step < uw) {
            __threadfence_block();
            if (lane == 0) *(volatile int *)&S.used[wi] = step + 1;
        }
    }
}

template <int NW>
__device__ void deblock_pair_chroma(const PicDesc &p, int pair, int wi, int nw, DbChromaSmem &s, DbFrameShared<NW> &S,
                                    const LaunchState &st)
{
    const int lane = threadIdx.x & 31;
    const int h = lane >> 4, k = lane & 15, comp = k >> 3, ck = k & 7;
    const int uw = (int)p.units_w, rows = (int)p.units_h, Wc = p.cs;
    const int row = 2 * pair + h;
    const bool row_ok = row < rows;
    const bool has_second = 2 * pair + 1 < rows;
    const int steps = has_second ? uw + 1 : uw;
    const bool from_cta = wi > 0;
    const bool to_cta = wi + 1 < nw && has_second;
    int *prog = p.progress + p.units_h;
    uint8_t *C = plane_c(p, comp);
    uint8_t(*t)[8] = s.t[h][comp];
    const uint32_t stop = p.deblock_stop;
    int left[4] = {0, 0, 0, 0};
    int seen = 0, seen_used = 0;
    uint2 nl = make_uint2(0, 0);
    uint4 npc = make_uint4(0, 0, 0, 0);
    uint32_t ncv = 0, nch = 0;
    auto fetch = [&](int u) {
        const int cur = row * uw + u;
        const uint8_t *bs = p.bs + (size_t)cur * kBsBytes;
        nl = __ldcg((const uint2 *)(C + (size_t)(row * 8 + ck) * Wc + u * 8));
        ncv = __ldcg((const uint16_t *)(bs + bs_cv(0, ck)));
        nch = __ldcg((const uint16_t *)(bs + bs_ch(0, ck)));
        npc = __ldcg((const uint4 *)(bs + kBsParams + 16 + 16 * comp));
    };
    if (row_ok && h == 0) fetch(0);
    for (int step = 0; step < steps; step++) {
        const int u = step - h;
        const bool act = row_ok && u >= 0 && u < uw;
        const uint2 line = nl;
        const uint4 prm = npc;
        uint32_t cv = ncv, ch = nch;
        if (row_ok && u + 1 >= 0 && u + 1 < uw) fetch(u + 1);
        if (to_cta && step >= 1 && !cta_wait(st, &S.used[wi + 1], min(step - kDbXRing, uw), seen_used)) return;
        const int x0 = u * 8, y0 = row * 8;
        if (act) {
            const int cur = row * uw + u;
            if ((uint32_t)cur >= (stop >> 10)) {
                if ((uint32_t)cur > (stop >> 10)) cv = ch = 0;
                else {
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        if (stop_key(cur, (e == 0 ? SEQ_CBV0 : SEQ_CBV4) + comp, ck) >= stop) cv &= ~(0xFFu << (8 * e));
                        if (stop_key(cur, (e == 0 ? SEQ_CBH0 : SEQ_CBH4) + comp, ck) >= stop) ch &= ~(0xFFu << (8 * e));
                    }
                }
            }
            int w[12];
#pragma unroll
            for (int i = 0; i < 4; i++) w[i] = left[i];
            unpack8(line, &w[4]);
            db_chroma<4, true>(w, cv & 255, prm.x);
            db_chroma<8, false>(w, (cv >> 8) & 255, prm.z);
            if (u > 0) {
                const uint32_t cw = pack4(w[0], w[1], w[2], w[3]);
                *(uint32_t *)(C + (size_t)(y0 + ck) * Wc + x0 - 4) = cw;
                if (h == 0 && ck >= 4) s.ring[(u - 1) % 3][comp][ck - 4].y = cw;
                if (h == 1 && to_cta && ck >= 4) S.x.c[wi][(u - 1) % kDbXRing][comp][ck - 4].y = cw;
            }
            *(uint2 *)&t[ck + 4][0] = pack8(&w[4]);
        }
        if (to_cta && step >= 1) {
            __syncwarp();
            __threadfence_block();
            if (lane == 0) *(volatile int *)&S.done[wi] = step;
        }
        if (2 * pair > 0 && step < uw) {
            const bool ok = from_cta ? cta_wait(st, &S.done[wi - 1], step + 2, seen)
                                     : db_wait(st, prog + 2 * pair - 2, min(step + 2, uw), seen);
            if (!ok) return;
        }
        __syncwarp();  // the first row's vertical edges of this step updated the ring
        if (act && row > 0 && ck < 4)
            *(uint2 *)&t[ck][0] = h == 1 ? s.ring[u % 3][comp][ck]
                                         : (from_cta ? S.x.c[wi - 1][u % kDbXRing][comp][ck]
                                                     : __ldcg((const uint2 *)(C + (size_t)(y0 - 4 + ck) * Wc + x0)));
        __syncwarp();
        if (act) {
            int w[12];
#pragma unroll
            for (int i = 0; i < 12; i++) w[i] = t[i][ck];
            db_chroma<4, true>(w, ch & 255, prm.y);
            db_chroma<8, false>(w, (ch >> 8) & 255, prm.z);
            t[3][ck] = (uint8_t)w[3];
            t[4][ck] = (uint8_t)w[4];
            t[7][ck] = (uint8_t)w[7];
            t[8][ck] = (uint8_t)w[8];
        }
        __syncwarp();
        if (act) {
            const uint2 cr = *(const uint2 *)&t[ck + 4][0];
            *(uint2 *)(C + (size_t)(y0 + ck) * Wc + x0) = cr;
#pragma unroll
            for (int i = 0; i < 4; i++) left[i] = (cr.y >> (8 * i)) & 255;
            if (h == 0 && ck >= 4) s.ring[u % 3][comp][ck - 4] = cr;
            if (h == 1 && to_cta && ck >= 4) S.x.c[wi][u % kDbXRing][comp][ck - 4] = cr;
            if (row > 0 && ck < 3) *(uint2 *)(C + (size_t)(y0 - 3 + ck) * Wc + x0) = *(const uint2 *)&t[1 + ck][0];
        }
        __syncwarp();
        if (has_second && step >= 1 && !to_cta && lane == 0) st_release(prog + 2 * pair, step);
        if (to_cta && step == uw) {
            __syncwarp();
            __threadfence_block();
            if (lane == 0) *(volatile int *)&S.done[wi] = uw + 1;
        }
        if (from_cta && step < uw) {
            __threadfence_block();
            if (lane == 0) *(volatile int *)&S.used[wi] = step + 1;
        }
    }
}

// MBAFF pictures: a block of kMbWarps warps per kMbWarps MB-pair rows of one
// plane (even block tickets luma, odd ones chroma); see DbMbaffShared.
__global__ void __launch_bounds__(32 * kMbWarps, 24 / kMbWarps) k_deblock(const PicDesc *__restrict__ pics, int npics,
                                                                        uint32_t total_units, LaunchState st)
{
    __shared__ DbMbaffShared S;
    __shared__ uint32_t s_unit;
    if (threadIdx.x == 0) s_unit = atomicAdd(&st.ticket[1], 1u);
    if (threadIdx.x < kMbWarps) {
        S.done[threadIdx.x] = 0;
        S.used[threadIdx.x] = 0;
    }
    __syncthreads();
    const uint32_t g = s_unit;
    if (g >= total_units) return;
    const int pi = find_pic_by_db(pics, npics, g);
    const PicDesc p = pics[pi];
    if (!p.deblock || !p.mbaff) return;
    const int unit = (int)(g - p.db_base);
    const int wi = threadIdx.x >> 5;
    const int first = (unit >> 1) * kMbWarps;
    const int nw = min(kMbWarps, (int)p.units_h - first);
    if (wi >= nw) return;
    if ((unit & 1) == 0) mbaff_luma_row(p, first + wi, wi, nw, S, st);
    else mbaff_chroma_row(p, first + wi, wi, nw, S, st);
}

// Frame pictures: a block of kDbWarps warps per kDbWarps MB-row pairs of one
// plane (even block tickets luma, odd ones chroma); see DbFrameShared.
template <int W>
__device__ __forceinline__ void deblock_frame_body(DbFrameShared<W> &S, uint32_t &s_unit, const PicDesc *__restrict__ pics,
                                                   int npics, uint32_t total_units, const LaunchState &st)
{
    if (threadIdx.x == 0) s_unit = atomicAdd(&st.ticket[2], 1u);
    if (threadIdx.x < W) {
        S.done[threadIdx.x] = 0;
        S.used[threadIdx.x] = 0;
    }
    __syncthreads();
    const uint32_t g = s_unit;
    if (g >= total_units) return;
    const int pi = find_pic_by_dbf(pics, npics, g);
    const PicDesc p = pics[pi];
    if (!p.deblock || p.mbaff) return;
    const int unit = (int)(g - p.dbf_base);
    const int wi = threadIdx.x >> 5;
    const int first = (unit >> 1) * W, pairs = ((int)p.units_h + 1) / 2;
    const int nw = min(W, pairs - first);
    if (wi >= nw) return;
    if ((unit & 1) == 0) deblock_pair_luma<W>(p, first + wi, wi, nw, S.w.l[wi], S, st);
    else deblock_pair_chroma<W>(p, first + wi, wi, nw, S.w.c[wi], S, st);
}

__global__ void __launch_bounds__(32 * kDbWarps, 28 / kDbWarps) k_deblock_frame(const PicDesc *__restrict__ pics, int npics,
                                                                              uint32_t total_units, LaunchState st)
{
    __shared__ DbFrameShared<kDbWarps> S;
    __shared__ uint32_t s_unit;
    deblock_frame_body<kDbWarps>(S, s_unit, pics, npics, total_units, st);
}

// The same with blocks of four MB-row pairs; the picture descriptors of its
// launch count units with deblock_frame_units(mbaff, units_h, 4).
__global__ void __launch_bounds__(128, 7) k_deblock_frame4(const PicDesc *__restrict__ pics, int npics, uint32_t total_units,
                                                           LaunchState st)
{
    __shared__ DbFrameShared<4> S;
    __shared__ uint32_t s_unit;
    deblock_frame_body<4>(S, s_unit, pics, npics, total_units, st);
}

// ======================================================================
// Output: decoded picture to BGR24 rows
// ======================================================================
// CH264PictureBase::convertYuv420pToBgr24 / convertYuv420pToBgr24FlipLines
// (H264PictureBase.cpp:440-499): BT.601 limited-range integer conversion,
// C division (truncation toward zero), clipped.  One thread per 4 pixels of
// a row: one 32-bit luma load, two 16-bit chroma loads, three 32-bit stores.
__global__ void __launch_bounds__(256) k_bgr24(const uint8_t *__restrict__ yuv, int W, int H, uint8_t *__restrict__ out,
                                               int row_bytes, int flip)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (q >= W / 4 || y >= H) return;
    const int x = 4 * q;
    const uint8_t *cb = yuv + (size_t)W * H, *cr = cb + (size_t)W * H / 4;
    const uint32_t yw = __ldg((const uint32_t *)(yuv + (size_t)y * W + x));
    const uint32_t uw = __ldg((const uint16_t *)(cb + (size_t)(y / 2) * (W / 2) + x / 2));
    const uint32_t vw = __ldg((const uint16_t *)(cr + (size_t)(y / 2) * (W / 2) + x / 2));
    uint32_t o[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int Y = (yw >> (8 * k)) & 255, U = (uw >> (8 * (k >> 1))) & 255, V = (vw >> (8 * (k >> 1))) & 255;
        const int b = (1164 * (Y - 16) + 2018 * (U - 128)) / 1000;
        const int g = (1164 * (Y - 16) - 813 * (V - 128) - 391 * (U - 128)) / 1000;
        const int r = (1164 * (Y - 16) + 1596 * (V - 128)) / 1000;
        const int c[3] = {b, g, r};
#pragma unroll
        for (int ch = 0; ch < 3; ch++) {
            const int byte = 3 * k + ch;
            o[byte >> 2] |= (uint32_t)H264R_CLIP3(0, 255, c[ch]) << (8 * (byte & 3));
        }
    }
    uint32_t *dst = (uint32_t *)(out + (size_t)(flip ? H - 1 - y : y) * row_bytes + 3 * x);
    dst[0] = o[0];
    dst[1] = o[1];
    dst[2] = o[2];
}

}  // namespace h264r
