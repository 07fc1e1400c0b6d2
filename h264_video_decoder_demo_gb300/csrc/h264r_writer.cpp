// h264r_writer.cpp — seeded H.264 bitstream writer (include/h264r_writer.h).
//
// The writer is the inverse of the host front end: it draws syntax elements
// from a configuration and writes them with the same code tables the parser
// reads (h264r_cavlc.cpp).  Wherever a syntax element is coded relative to a
// prediction — mvd against mvpLX (8.4.1.3), the Intra4x4 / Intra8x8 mode
// against predIntraNxNPredMode (8.3.1.1, 8.3.2.1), the CAVLC table against nC
// (9.2.1), mb_qp_delta against QPY,PRED — the writer asks a shadow front end
// (the parser's own state and macroblock decoder, h264r_parser_impl.h) for
// the prediction, then feeds every macroblock it has written back through
// that decoder so that the next macroblock's predictions see it.  The stream
// therefore decodes, in the parser and in the reference decoder alike, to
// exactly the motion vectors, modes and levels that were drawn.
#include "../../include/h264r_writer.h"

#include <cstdlib>

#include "h264r_parser_impl.h"

namespace h264r {
int cavlc_write_block(BitWriter &bw, int nC, int start, int end, int max_coeff, const int *coeff);
int cbp_to_code(int cbp, bool intra);
}  // namespace h264r

namespace {

thread_local std::string g_writer_err;

// SplitMix64: the same sequence on every host
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    int range(int lo, int hi) { return hi <= lo ? lo : lo + (int)(next() % (uint64_t)(hi - lo + 1)); }
    bool pct(int p) { return (int)(next() % 100) < p; }
    bool permille(int p) { return (int)(next() % 1000) < p; }
};

struct WriterError {
    std::string msg;
};

[[noreturn]] void die(const char *fmt, ...)
{
    char m[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(m, sizeof(m), fmt, ap);
    va_end(ap);
    throw WriterError{m};
}

enum { kP = 0, kB = 1, kI = 2 };

struct PicPlan {
    int display;
    int type;  // kP, kB, kI
    bool idr;
};

// Table A-1 MaxDpbMbs of the levels the writer picks from
const int kLevels[][2] = {{30, 8100}, {31, 18000}, {32, 20480}, {40, 32768}, {42, 34816}, {50, 110400}, {51, 184320}};

// one inter partition as the writer plans it
struct Part {
    int x, y, w, h;  // luma samples within the MB
    int pred;        // bit 0 list 0, bit 1 list 1; 0: direct 4x4 block
    int ref[2];
    int mv[2][2];    // target motion vector
    int mvd[2][2];
};

struct Writer {
    h264r_writer_cfg cfg;
    Rng rng;
    h264r_parser P;
    std::vector<uint8_t> out;
    BitReader mbr;  // reads each written macroblock back
    int log2_max_frame_num = 8, log2_max_poc_lsb = 10;
    int max_refs = 1;
    int next_frame_num = 0;
    int idr_count = 0;
    int chroma_offset[2] = {0, 0};
    bool high = false;

    explicit Writer(const h264r_writer_cfg &c) : cfg(c), rng(((uint64_t)c.seed << 16) ^ 0x264) {}

    // ------------------------------------------------------------ helpers
    void feed_nal(int ref_idc, int type, const BitWriter &bw)
    {
        const size_t at = out.size();
        put_nal(out, ref_idc, type, bw.buf.data(), bw.buf.size());
        // the shadow front end reads the same NAL unit (without start code)
        const int rc = P.process_nal(out.data() + at + 4, out.size() - at - 4);
        if (rc) die("front end rejected NAL unit type %d: %s", type, P.err.c_str());
    }

    int level_idc() const
    {
        if (cfg.level_idc) return cfg.level_idc;
        const int mbs = cfg.width_mbs * cfg.height_mbs;
        for (const auto &l : kLevels)
            if (l[1] / mbs >= std::max(4, max_refs)) return l[0];
        return 51;
    }

    void write_sps()
    {
        BitWriter b;
        b.u(8, cfg.profile_idc);
        b.u(8, cfg.profile_idc == 66 ? 0x40 : 0x00);  // constraint_set1 for Baseline
        b.u(8, (uint32_t)level_idc());
        b.ue(0);  // seq_parameter_set_id
        if (high) {
            b.ue(1);       // chroma_format_idc 4:2:0
            b.ue(0);       // bit_depth_luma_minus8
            b.ue(0);       // bit_depth_chroma_minus8
            b.u(1, 0);     // qpprime_y_zero_transform_bypass_flag
            b.u(1, 0);     // seq_scaling_matrix_present_flag
        }
        b.ue((uint32_t)(log2_max_frame_num - 4));
        b.ue(0);  // pic_order_cnt_type
        b.ue((uint32_t)(log2_max_poc_lsb - 4));
        b.ue((uint32_t)max_refs);
        b.u(1, 0);  // gaps_in_frame_num_value_allowed_flag
        b.ue((uint32_t)(cfg.width_mbs - 1));
        // pic_height_in_map_units: MB pair rows when frame_mbs_only_flag is 0
        b.ue((uint32_t)((cfg.mbaff ? cfg.height_mbs / 2 : cfg.height_mbs) - 1));
        b.u(1, cfg.mbaff ? 0 : 1);  // frame_mbs_only_flag
        if (cfg.mbaff) b.u(1, 1);   // mb_adaptive_frame_field_flag
        b.u(1, 1);  // direct_8x8_inference_flag
        // a coded height of 1088 for 1080 lines: crop 8 lines (crop units of
        // 2 lines in 4:2:0, 4 when frame_mbs_only_flag is 0)
        const bool crop = cfg.height_mbs == 68;
        b.u(1, crop ? 1 : 0);
        if (crop) {
            b.ue(0);
            b.ue(0);
            b.ue(0);
            b.ue(cfg.mbaff ? 2 : 4);
        }
        b.u(1, 1);  // vui_parameters_present_flag: bitstream restriction only
        for (int i = 0; i < 8; i++) b.u(1, 0);  // aspect, overscan, signal type, chroma loc, timing, nal/vcl hrd, pic_struct
        b.u(1, 1);  // bitstream_restriction_flag
        b.u(1, 1);  // motion_vectors_over_pic_boundaries_flag
        b.ue(0);    // max_bytes_per_pic_denom
        b.ue(0);    // max_bits_per_mb_denom
        b.ue(16);   // log2_max_mv_length_horizontal
        b.ue(16);   // log2_max_mv_length_vertical
        b.ue(cfg.b_pictures ? 1u : 0u);  // max_num_reorder_frames
        b.ue((uint32_t)max_refs);        // max_dec_frame_buffering
        b.trailing();
        feed_nal(3, 7, b);
    }

    void write_pps()
    {
        BitWriter b;
        b.ue(0);    // pic_parameter_set_id
        b.ue(0);    // seq_parameter_set_id
        b.u(1, 0);  // entropy_coding_mode_flag: CAVLC
        b.u(1, cfg.mbaff ? 1 : 0);  // bottom_field_pic_order_in_frame_present_flag
        b.ue(0);    // num_slice_groups_minus1
        b.ue((uint32_t)(cfg.num_refs - 1));
        b.ue(0);
        b.u(1, cfg.weighted == 1 ? 1 : 0);           // weighted_pred_flag
        b.u(2, (uint32_t)(cfg.weighted == 1 ? 1 : cfg.weighted == 2 ? 2 : 0));  // weighted_bipred_idc
        b.se(0);    // pic_init_qp_minus26
        b.se(0);    // pic_init_qs_minus26
        b.se(chroma_offset[0]);
        b.u(1, 1);  // deblocking_filter_control_present_flag
        b.u(1, 0);  // constrained_intra_pred_flag
        b.u(1, 0);  // redundant_pic_cnt_present_flag
        if (high) {
            b.u(1, cfg.transform8x8 ? 1 : 0);
            b.u(1, 0);  // pic_scaling_matrix_present_flag
            b.se(chroma_offset[1]);
        }
        b.trailing();
        feed_nal(3, 8, b);
    }

    // pictures in decoding order
    std::vector<PicPlan> plan() const
    {
        const int n = cfg.num_pictures, step = cfg.b_pictures + 1;
        std::vector<int> anchors;
        for (int d = 0; d < n; d += step) anchors.push_back(d);
        if (anchors.back() != n - 1) anchors.push_back(n - 1);
        std::vector<PicPlan> order;
        int next_i = 0, prev = -1;
        for (int a : anchors) {
            PicPlan p{a, kP, false};
            if (a == 0) {
                p.type = kI;
                p.idr = true;
                next_i = cfg.gop_length ? cfg.gop_length : n + 1;
            } else if (a >= next_i) {
                p.type = kI;
                while (next_i <= a) next_i += cfg.gop_length;
            }
            order.push_back(p);
            for (int d = prev + 1; d < a; d++) order.push_back({d, kB, false});
            prev = a;
        }
        return order;
    }

    int count_refs() const
    {
        int n = 0;
        for (const Pic &p : P.dpb) n += p.is_ref() ? 1 : 0;
        return n;
    }

    // ------------------------------------------------------------ slice header
    struct SliceParams {
        int type, first_mb, nref[2], qp, dbk_alpha, dbk_beta;
        bool idr, ref;
        int frame_num, poc_lsb;
        // explicit weights: [list][ref][Y, Cb, Cr] weight / offset, flags per list entry
        int w[2][16][3], o[2][16][3];
        bool lflag[2][16], cflag[2][16];
    };

    void draw_weights(SliceParams &s)
    {
        const int nl = s.type == kB ? 2 : 1;
        int max0 = -1000;
        for (int l = 0; l < nl; l++) {
            for (int i = 0; i < s.nref[l]; i++) {
                // list 1 weights keep every w0 + w1 <= 128 (8.4.2.3.2 constraint)
                const int hi = (l == 1) ? std::min(127, 128 - max0) : 127;
                s.lflag[l][i] = l == 1 || rng.pct(85);
                s.cflag[l][i] = l == 1 || rng.pct(70);
                for (int c = 0; c < 3; c++) {
                    const bool f = c == 0 ? s.lflag[l][i] : s.cflag[l][i];
                    s.w[l][i][c] = f ? rng.range(-64, hi) : 32;
                    s.o[l][i][c] = f ? rng.range(-32, 32) : 0;
                    if (l == 0) max0 = std::max(max0, s.w[l][i][c]);
                }
            }
        }
    }

    void write_slice_header(BitWriter &b, const SliceParams &s)
    {
        b.ue((uint32_t)(cfg.mbaff ? s.first_mb / 2 : s.first_mb));
        b.ue((uint32_t)(s.type == kI ? 2 : s.type == kB ? 1 : 0));
        b.ue(0);  // pic_parameter_set_id
        b.u(log2_max_frame_num, (uint32_t)s.frame_num);
        if (cfg.mbaff) b.u(1, 0);  // field_pic_flag: a frame (MBAFF)
        if (s.idr) b.ue((uint32_t)(idr_count & 0xFFFF));
        b.u(log2_max_poc_lsb, (uint32_t)s.poc_lsb);
        if (cfg.mbaff) b.se(1);  // delta_pic_order_cnt_bottom: the fields' POCs differ
        if (s.type == kB) b.u(1, cfg.direct_spatial ? 1 : 0);
        if (s.type != kI) {
            b.u(1, 1);  // num_ref_idx_active_override_flag
            b.ue((uint32_t)(s.nref[0] - 1));
            if (s.type == kB) b.ue((uint32_t)(s.nref[1] - 1));
            b.u(1, 0);  // ref_pic_list_modification_flag_l0
            if (s.type == kB) b.u(1, 0);
        }
        if ((cfg.weighted == 1 && s.type == kP) || (cfg.weighted == 1 && s.type == kB)) {
            b.ue(5);  // luma_log2_weight_denom
            b.ue(5);  // chroma_log2_weight_denom
            for (int l = 0; l < (s.type == kB ? 2 : 1); l++)
                for (int i = 0; i < s.nref[l]; i++) {
                    b.u(1, s.lflag[l][i]);
                    if (s.lflag[l][i]) {
                        b.se(s.w[l][i][0]);
                        b.se(s.o[l][i][0]);
                    }
                    b.u(1, s.cflag[l][i]);
                    if (s.cflag[l][i])
                        for (int c = 1; c < 3; c++) {
                            b.se(s.w[l][i][c]);
                            b.se(s.o[l][i][c]);
                        }
                }
        }
        if (s.ref) {  // dec_ref_pic_marking( )
            if (s.idr) {
                b.u(1, 0);  // no_output_of_prior_pics_flag
                b.u(1, 0);  // long_term_reference_flag
            } else {
                b.u(1, 0);  // adaptive_ref_pic_marking_mode_flag: sliding window
            }
        }
        b.se(s.qp - 26);  // slice_qp_delta
        b.ue(0);          // disable_deblocking_filter_idc
        b.se(s.dbk_alpha);
        b.se(s.dbk_beta);
    }

    // ------------------------------------------------------------ macroblocks
    bool avail(const MbDecoder &d, int xN, int yN) const
    {
        int xW = 0, yW = 0;
        return d.nb_mb(xN, yN, 16, 16, xW, yW) >= 0;
    }

    int pick(const int *modes, int n) { return modes[rng.range(0, n - 1)]; }

    // an NxN intra mode whose samples are available (8.3.1.2: the modes that
    // need the left, top or top-left neighbours only where they exist; the
    // top-right ones are substituted from the top row)
    int intra_nxn_mode(const MbDecoder &d, int x, int y)
    {
        const bool A = avail(d, x - 1, y), B = avail(d, x, y - 1), D = avail(d, x - 1, y - 1);
        int m[9], n = 0;
        m[n++] = 2;
        if (B) m[n++] = 0, m[n++] = 3, m[n++] = 7;
        if (A) m[n++] = 1, m[n++] = 8;
        if (A && B && D) m[n++] = 4, m[n++] = 5, m[n++] = 6;
        return pick(m, n);
    }

    // Intra16x16 / chroma mode: DC always; others where their samples exist
    int intra_big_mode(const MbDecoder &d, bool chroma)
    {
        const bool A = avail(d, -1, 0), B = avail(d, 0, -1), D = avail(d, -1, -1);
        int m[4], n = 0;
        m[n++] = chroma ? 0 : 2;
        if (A) m[n++] = 1;
        if (B) m[n++] = chroma ? 2 : 0;
        if (A && B && D) m[n++] = 3;
        return pick(m, n);
    }

    int draw_level()
    {
        const int r = rng.range(0, 99);
        const int mag = r < 55 ? 1 : r < 75 ? 2 : r < 88 ? rng.range(3, 4) : r < 97 ? rng.range(5, 12) : rng.range(13, 40);
        return rng.pct(50) ? -mag : mag;
    }

    // n coefficients of one block, low frequencies more likely
    void draw_block(int *c, int n, int max_total)
    {
        for (int i = 0; i < n; i++) c[i] = 0;
        const int r = rng.range(1, 100);
        int total = r <= 50 ? rng.range(1, 2) : r <= 80 ? rng.range(3, 5) : r <= 95 ? rng.range(6, 10) : rng.range(11, 16);
        total = std::min(total, std::min(n, max_total));
        for (int k = 0; k < total; k++) {
            // P(p = n - 1 - j) grows with j: floor(sqrt(u)) of a uniform u
            const int u = rng.range(0, n * n - 1);
            int j = 0;
            while ((j + 1) * (j + 1) <= u) j++;
            int p = n - 1 - j;
            while (c[p]) p = (p + 1) % n;
            c[p] = draw_level();
        }
    }

    void put_block(BitWriter &b, int nC, int start, int end, int max_coeff, const int *c, int &total)
    {
        total = cavlc_write_block(b, nC, start, end, max_coeff, c);
        if (total < 0) die("level outside the CAVLC escape range");
    }

    // mb_qp_delta and residual( ) for a MB of class cls with coded_block_pattern cbp
    void write_residual(BitWriter &b, MbDecoder &d, int cls, int cbp, bool t8)
    {
        MbState *cur = d.cur;
        // mb_qp_delta is in [-26, 25]
        const int target = std::max(d.qp - 26, std::min(d.qp + 25, rng.range(cfg.qp_min, cfg.qp_max)));
        b.se(target - d.qp);
        for (int i = 0; i < 16; i++) cur->tc[i] = 0;
        memset(cur->tcc, 0, sizeof(cur->tcc));
        int c[64], total = 0;
        const bool i16 = cls == H264R_MB_I16x16;
        if (i16) {
            draw_block(c, 16, 16);
            put_block(b, d.nc_luma(0), 0, 15, 16, c, total);
            cur->tc[0] = (uint8_t)total;
        }
        for (int b8 = 0; b8 < 4; b8++) {
            if (!(cbp & (1 << b8))) continue;
            if (t8) {
                int c8[64];
                draw_block(c8, 64, 16);
                // extra levels over the whole 8x8 block
                for (int k = rng.range(0, 6); k > 0; k--) c8[rng.range(0, 63)] = draw_level();
                for (int b4 = 0; b4 < 4; b4++) {
                    for (int k = 0; k < 16; k++) c[k] = c8[4 * k + b4];
                    put_block(b, d.nc_luma(b8 * 4 + b4), 0, 15, 16, c, total);
                    cur->tc[b8 * 4 + b4] = (uint8_t)total;
                }
                continue;
            }
            for (int b4 = 0; b4 < 4; b4++) {
                const int blk = b8 * 4 + b4;
                if (i16) {
                    draw_block(c, 15, 15);
                    put_block(b, d.nc_luma(blk), 0, 14, 15, c, total);
                } else {
                    if (rng.pct(20)) for (int k = 0; k < 16; k++) c[k] = 0;
                    else draw_block(c, 16, 16);
                    put_block(b, d.nc_luma(blk), 0, 15, 16, c, total);
                }
                cur->tc[blk] = (uint8_t)total;
            }
        }
        const int chroma = cbp >> 4;
        if (chroma) {
            for (int cc = 0; cc < 2; cc++) {
                draw_block(c, 4, 4);
                if (rng.pct(25)) c[rng.range(0, 3)] = 0;
                put_block(b, -1, 0, 3, 4, c, total);
            }
        }
        if (chroma & 2) {
            for (int cc = 0; cc < 2; cc++)
                for (int k = 0; k < 4; k++) {
                    if (rng.pct(30)) for (int i = 0; i < 15; i++) c[i] = 0;
                    else draw_block(c, 15, 15);
                    put_block(b, d.nc_chroma(cc, k), 0, 14, 15, c, total);
                    cur->tcc[cc][k] = (uint8_t)total;
                }
        }
    }

    int draw_cbp(bool luma_allowed = true)
    {
        int cbp = 0;
        if (luma_allowed)
            for (int b8 = 0; b8 < 4; b8++)
                if (rng.pct(cfg.coef_density)) cbp |= 1 << b8;
        if (rng.pct(cfg.coef_density)) cbp |= (rng.pct(50) ? 2 : 1) << 4;
        return cbp;
    }

    // intra MB of slice type st (I_PCM, Intra_16x16 or I_NxN)
    void write_intra(BitWriter &b, MbDecoder &d, int st)
    {
        MbState *cur = d.cur;
        const int base = st == kI ? 0 : st == kP ? 5 : 23;
        const int r = rng.range(0, 99);
        if (rng.permille(cfg.pcm_permille)) {
            b.ue((uint32_t)(base + 25));
            while (!b.byte_aligned()) b.u(1, 0);
            for (int i = 0; i < 384; i++) b.u(8, (uint32_t)rng.range(1, 255));
            return;
        }
        if (r < 30) {  // Intra_16x16
            cur->cls = H264R_MB_I16x16;
            const int mode = intra_big_mode(d, false);
            const int cm = intra_big_mode(d, true);
            const int chroma = rng.pct(cfg.coef_density) ? rng.range(1, 2) : 0;
            const int luma = rng.pct(cfg.coef_density) ? 15 : 0;
            b.ue((uint32_t)(base + 1 + mode + 4 * chroma + (luma ? 12 : 0)));
            b.ue((uint32_t)cm);
            write_residual(b, d, H264R_MB_I16x16, luma | (chroma << 4), false);
            return;
        }
        const bool t8 = high && cfg.transform8x8 && r < 60;
        cur->cls = t8 ? H264R_MB_I8x8 : H264R_MB_I4x4;
        b.ue((uint32_t)base);  // I_NxN
        if (high && cfg.transform8x8) b.u(1, t8 ? 1 : 0);
        for (int i = 0; i < 16; i++) cur->ipm4[i] = 2;
        for (int i = 0; i < 4; i++) cur->ipm8[i] = 2;
        const int nb = t8 ? 4 : 16;
        for (int k = 0; k < nb; k++) {
            const int x = t8 ? (k & 1) * 8 : kBlkX[k] * 4, y = t8 ? (k >> 1) * 8 : kBlkY[k] * 4;
            const int mode = intra_nxn_mode(d, x, y);
            const int pred = d.derive_mode(x, y, t8, 1, 0);
            if (mode == pred) {
                b.u(1, 1);
            } else {
                b.u(1, 0);
                b.u(3, (uint32_t)(mode < pred ? mode : mode - 1));
            }
            if (t8) {
                cur->ipm8[k] = (int8_t)mode;
                for (int j = 0; j < 4; j++) cur->ipm4[k * 4 + j] = (int8_t)mode;
            } else {
                cur->ipm4[k] = (int8_t)mode;
            }
        }
        b.ue((uint32_t)intra_big_mode(d, true));
        const int cbp = draw_cbp();
        b.ue((uint32_t)cbp_to_code(cbp, true));
        if (cbp) write_residual(b, d, cur->cls, cbp, t8);
    }

    // target motion vector of a partition at (px, py) (picture luma samples)
    int pic_h_ = 0;       // height of the picture the current MB predicts from
    bool field_mb_ = false;  // the current MB is a field MB of an MBAFF frame
    void draw_mv(int px, int py, int w, int h, int mv[2])
    {
        const int W = cfg.width_mbs * 16, H = pic_h_;
        if (rng.pct(cfg.edge_mv_percent)) {
            // the reference block lies wholly or partly past one picture edge
            int rx = px + rng.range(-cfg.mv_range, cfg.mv_range) / 4, ry = py + rng.range(-cfg.mv_range, cfg.mv_range) / 4;
            switch (rng.range(0, 3)) {
            case 0: rx = -w - rng.range(-w / 2, 24); break;
            case 1: rx = W + rng.range(-w / 2, 24); break;
            case 2: ry = -h - rng.range(-h / 2, 24); break;
            default: ry = H + rng.range(-h / 2, 24); break;
            }
            mv[0] = std::max(-8192, std::min(8191, (rx - px) * 4 + rng.range(0, 3)));
            mv[1] = std::max(-8192, std::min(8191, (ry - py) * 4 + rng.range(0, 3)));
        } else {
            mv[0] = rng.range(-cfg.mv_range, cfg.mv_range);
            mv[1] = rng.range(-cfg.mv_range, cfg.mv_range);
        }
        // a field MB reads its reference field with x clamped to the doubled
        // field-view width (Q3): past the right edge of the last lines the
        // reference decoder reads beyond its chroma plane, so field MBs keep
        // their prediction (6-tap and chroma support included) left of the edge
        if (field_mb_) mv[0] = std::min(mv[0], 4 * (W - 8 - (px + w)));
    }

    // derive the partitions' mvd in decoding order, as MbDecoder::inter_pred does
    void plan_motion(MbDecoder &d, std::vector<Part> &parts, int shape)
    {
        for (Part &p : parts) {
            if (p.pred == 0) {  // direct 4x4 block
                Blk b;
                if (d.direct_block(p.x >> 2, p.y >> 2, b)) die("direct prediction failed: %s", P.err.c_str());
                d.set_blocks(p.x, p.y, 4, 4, b);
                continue;
            }
            Blk b;
            const int part = (shape == 1) ? (p.y ? 1 : 0) : (shape == 2) ? (p.x ? 1 : 0) : 0;
            for (int l = 0; l < 2; l++) {
                b.ref[l] = (int8_t)p.ref[l];
                b.mv[l][0] = b.mv[l][1] = 0;
                if (p.ref[l] < 0) continue;
                int m[2];
                d.mvp(p.x, p.y, p.w, shape == 1 || shape == 2 ? shape : 0, part, l, p.ref[l], m);
                for (int k = 0; k < 2; k++) {
                    p.mvd[l][k] = p.mv[l][k] - m[k];
                    b.mv[l][k] = (int16_t)p.mv[l][k];
                }
            }
            d.set_blocks(p.x, p.y, p.w, p.h, b);
        }
    }

    // implicit weighting of a bi-predicted block whose two references are
    // the same picture: the reference decoder divides by their POC distance
    // before it tests it for zero (H264InterPrediction.cpp:2955-2960)
    bool same_picture(const MbDecoder &d, int ref0, int ref1) const
    {
        return ref0 >= 0 && ref1 >= 0 && d.ref_pic(0, ref0) && d.ref_pic(1, ref1) &&
               d.ref_poc(0, ref0) == d.ref_poc(1, ref1);
    }

    // a 4x4 block of a field MB of an MBAFF frame at (bx, by) (4-sample
    // units) predicts from left of the right picture edge in luma and chroma
    // (interpolation support included): past it the reference decoder's
    // doubled-width clamp (Q3) reads beyond its chroma plane on the last lines
    bool field_block_ok(const MbDecoder &d, int bx, const Blk &b) const
    {
        if (!d.fld) return true;
        const int W = cfg.width_mbs * 16, px = ((d.addr >> 1) % cfg.width_mbs) * 16 + 4 * bx;
        for (int l = 0; l < 2; l++)
            if (b.ref[l] >= 0) {
                const int mvx = b.mv[l][0];
                if (px + 3 + (mvx >> 2) + 3 > W - 2 || px / 2 + 1 + (mvx >> 3) + 1 > W / 2 - 2) return false;
            }
        return true;
    }

    // direct blocks the reference decodes as the standard does: explicit
    // weighting never meets a list-1-only block (the reference reads its
    // weights out of range, H264InterPrediction.cpp:2756-2771), implicit
    // weighting never a bi-predicted block from one picture twice, a field MB
    // never reads right of the picture edge
    bool direct_ok(MbDecoder &d, int quadrant_mask)
    {
        if (!d.fld && (cfg.weighted == 0 || (cfg.weighted == 1 && !cfg.direct_spatial))) return true;
        for (int q = 0; q < 4; q++) {
            if (!(quadrant_mask & (1 << q))) continue;
            for (int s = 0; s < 4; s++) {
                Blk b;
                const int x = (q & 1) * 8 + 4 * (s & 1), y = (q >> 1) * 8 + 4 * (s >> 1);
                if (d.direct_block(x >> 2, y >> 2, b)) die("direct prediction failed: %s", P.err.c_str());
                if (cfg.weighted == 1 && b.ref[0] < 0) return false;
                if (cfg.weighted == 2 && same_picture(d, b.ref[0], b.ref[1])) return false;
                if (!field_block_ok(d, x >> 2, b)) return false;
            }
        }
        return true;
    }

    // P_Skip of a field MB predicts from left of the right picture edge
    bool p_skip_ok(MbDecoder &d)
    {
        if (!d.fld) return true;
        const MbDecoder::Nb A = d.nb_motion(-1, 0, 0), B = d.nb_motion(0, -1, 0);
        Blk b;
        b.ref[0] = 0;
        b.ref[1] = -1;
        b.mv[0][0] = b.mv[0][1] = b.mv[1][0] = b.mv[1][1] = 0;
        if (!(!A.avail || !B.avail || (A.ref == 0 && A.mv[0] == 0 && A.mv[1] == 0) || (B.ref == 0 && B.mv[0] == 0 && B.mv[1] == 0))) {
            int m[2];
            d.mvp(0, 0, 16, 0, 0, 0, 0, m);
            b.mv[0][0] = (int16_t)m[0];
        }
        return field_block_ok(d, 3, b);
    }

    // reference indices of a partition predicted from lists `pred`
    void draw_refs(const MbDecoder &d, int pred, const int nref[2], int ref[2])
    {
        for (int tries = 0;; tries++) {
            for (int l = 0; l < 2; l++) ref[l] = (pred & (1 << l)) ? rng.range(0, nref[l] - 1) : -1;
            if (cfg.weighted != 2 || pred != 3 || !same_picture(d, ref[0], ref[1])) return;
            if (tries > 16) {  // every pair names one picture: predict from list 0 only
                ref[1] = -1;
                return;
            }
        }
    }

    void reset_mb_motion(MbDecoder &d)
    {
        for (int i = 0; i < 16; i++) {
            d.decoded4x4[i] = false;
            d.blk[i].ref[0] = d.blk[i].ref[1] = -1;
            d.blk[i].mv[0][0] = d.blk[i].mv[0][1] = d.blk[i].mv[1][0] = d.blk[i].mv[1][1] = 0;
        }
        d.spatial_ready = false;
    }

    void write_inter(BitWriter &b, MbDecoder &d, int st, const int nref[2])
    {
        MbState *cur = d.cur;
        cur->cls = H264R_MB_INTER;
        // the MB's origin in the picture it predicts from (a field MB: its field)
        int px, py;
        if (!d.mbaff) {
            px = (d.addr % cfg.width_mbs) * 16;
            py = (d.addr / cfg.width_mbs) * 16;
        } else {
            const int pair = d.addr >> 1;
            px = (pair % cfg.width_mbs) * 16;
            py = d.fld ? (pair / cfg.width_mbs) * 16 : (pair / cfg.width_mbs) * 32 + (d.addr & 1) * 16;
        }
        pic_h_ = d.fld ? cfg.height_mbs * 8 : cfg.height_mbs * 16;
        field_mb_ = d.fld;
        const bool is_b = st == kB;
        const bool explicit_b = is_b && cfg.weighted == 1;
        std::vector<Part> parts;
        int mb_type = 0, shape = 0, sub[4] = {0, 0, 0, 0};
        bool no_sub_lt8 = true, direct16 = false;
        reset_mb_motion(d);
        // partition shape
        int shapes[4], ns = 0;
        shapes[ns++] = 0;
        if (cfg.min_partition >= 1) shapes[ns++] = 1, shapes[ns++] = 2;
        if (cfg.min_partition >= 2) shapes[ns++] = 3;
        shape = pick(shapes, ns);
        auto lists_of = [&](bool allow_l1_only) {
            if (!is_b) return 1;
            int opts[3], n = 0;
            opts[n++] = 1;
            opts[n++] = 3;
            if (allow_l1_only) opts[n++] = 2;
            return pick(opts, n);
        };
        if (is_b && rng.pct(12) && direct_ok(d, 15)) {
            direct16 = true;
            mb_type = 0;
            shape = 3;
            for (int q = 0; q < 4; q++)
                for (int s = 0; s < 4; s++)
                    parts.push_back({(q & 1) * 8 + 4 * (s & 1), (q >> 1) * 8 + 4 * (s >> 1), 4, 4, 0, {-1, -1}, {{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}});
        } else if (shape < 3) {
            const int np = shape == 0 ? 1 : 2;
            int pred[2] = {lists_of(!explicit_b), lists_of(!explicit_b)};
            int refs[2][2];
            for (int p = 0; p < np; p++) {
                draw_refs(d, pred[p], nref, refs[p]);
                pred[p] = (refs[p][0] >= 0 ? 1 : 0) | (refs[p][1] >= 0 ? 2 : 0);
            }
            if (np == 1) pred[1] = pred[0];
            if (!is_b) {
                mb_type = shape;
            } else if (shape == 0) {
                mb_type = pred[0];
            } else {
                // B_X_Y_16x8 / 8x16: types 4..21 as (X, Y) pairs
                static const int pairs[9][2] = {{1, 1}, {2, 2}, {1, 2}, {2, 1}, {1, 3}, {2, 3}, {3, 1}, {3, 2}, {3, 3}};
                int j = 0;
                while (pairs[j][0] != pred[0] || pairs[j][1] != pred[1]) j++;
                mb_type = 4 + 2 * j + (shape == 2 ? 1 : 0);
            }
            for (int p = 0; p < np; p++) {
                Part q{shape == 2 ? 8 * p : 0, shape == 1 ? 8 * p : 0, shape == 2 ? 8 : 16, shape == 1 ? 8 : 16,
                       pred[p], {-1, -1}, {{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}};
                q.ref[0] = refs[p][0];
                q.ref[1] = refs[p][1];
                for (int l = 0; l < 2; l++)
                    if (q.ref[l] >= 0) draw_mv(px + q.x, py + q.y, q.w, q.h, q.mv[l]);
                parts.push_back(q);
            }
        } else {
            mb_type = is_b ? 22 : 3;
            int ref[4][2];
            for (int q = 0; q < 4; q++) {
                // sub_mb_type: P 0..3 (8x8, 8x4, 4x8, 4x4); B 0 direct, then
                // (lists, shape) as in Table 7-18
                // B_8x8 quadrants stay 8x8 or direct: the reference fails every
                // B sub_mb_type above 3 (H264MacroBlock.cpp:985-1004)
                int subshape = (cfg.min_partition >= 3 && !is_b) ? rng.range(0, 3) : 0;
                int pred = 1;
                if (is_b) {
                    if (rng.pct(20) && direct_ok(d, 1 << q)) {
                        sub[q] = 0;
                        pred = 0;
                    } else {
                        pred = lists_of(!explicit_b);
                        draw_refs(d, pred, nref, ref[q]);
                        pred = (ref[q][0] >= 0 ? 1 : 0) | (ref[q][1] >= 0 ? 2 : 0);
                        // sub_mb_type of (shape, lists): 8x8 L0 1, L1 2, Bi 3; 8x4 L0 4, L1 6, Bi 8;
                        // 4x8 L0 5, L1 7, Bi 9; 4x4 L0 10, L1 11, Bi 12
                        static const int tab[4][4] = {{0, 1, 2, 3}, {0, 4, 6, 8}, {0, 5, 7, 9}, {0, 10, 11, 12}};
                        sub[q] = tab[subshape][pred];
                    }
                } else {
                    sub[q] = subshape;
                }
                if (pred == 0) {
                    subshape = 3;
                } else if (subshape) {
                    no_sub_lt8 = false;
                }
                shape |= subshape << (2 + 2 * q);
                if (!is_b) draw_refs(d, pred, nref, ref[q]);
                if (pred == 0) ref[q][0] = ref[q][1] = -1;
                const int qx = (q & 1) * 8, qy = (q >> 1) * 8;
                const int nsub = pred == 0 ? 4 : (subshape == 0 ? 1 : subshape == 3 ? 4 : 2);
                for (int s = 0; s < nsub; s++) {
                    int sx, sy, w, h;
                    switch (pred == 0 ? 3 : subshape) {
                    case 0: sx = 0; sy = 0; w = 8; h = 8; break;
                    case 1: sx = 0; sy = 4 * s; w = 8; h = 4; break;
                    case 2: sx = 4 * s; sy = 0; w = 4; h = 8; break;
                    default: sx = 4 * (s & 1); sy = 4 * (s >> 1); w = 4; h = 4; break;
                    }
                    Part p{qx + sx, qy + sy, w, h, pred, {ref[q][0], ref[q][1]}, {{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}};
                    for (int l = 0; l < 2; l++)
                        if (pred & (1 << l)) draw_mv(px + p.x, py + p.y, w, h, p.mv[l]);
                    parts.push_back(p);
                }
            }
            shape = (shape & ~3) | 3;
        }
        // mvd against the predictions, in decoding order
        reset_mb_motion(d);
        plan_motion(d, parts, shape & 3);
        // ---- syntax
        b.ue((uint32_t)mb_type);
        if (!direct16) {
            if ((shape & 3) == 3) {
                for (int q = 0; q < 4; q++) b.ue((uint32_t)sub[q]);
                for (int l = 0; l < 2; l++)
                    for (int q = 0; q < 4; q++) {
                        const Part *first = nullptr;
                        for (const Part &p : parts)
                            if (((p.y >> 3) * 2 + (p.x >> 3)) == q) {
                                first = &p;
                                break;
                            }
                        if (first->pred & (1 << l))
                            if (nref[l] > 1) b.te(nref[l] - 1, (uint32_t)first->ref[l]);
                    }
                for (int l = 0; l < 2; l++)
                    for (const Part &p : parts)
                        if (p.pred & (1 << l)) {
                            b.se(p.mvd[l][0]);
                            b.se(p.mvd[l][1]);
                        }
            } else {
                for (int l = 0; l < 2; l++)
                    for (const Part &p : parts)
                        if ((p.pred & (1 << l)) && nref[l] > 1) b.te(nref[l] - 1, (uint32_t)p.ref[l]);
                for (int l = 0; l < 2; l++)
                    for (const Part &p : parts)
                        if (p.pred & (1 << l)) {
                            b.se(p.mvd[l][0]);
                            b.se(p.mvd[l][1]);
                        }
            }
        }
        const int cbp = draw_cbp();
        b.ue((uint32_t)cbp_to_code(cbp, false));
        bool t8 = false;
        if ((cbp & 15) && high && cfg.transform8x8 && no_sub_lt8) {
            t8 = rng.pct(50);
            b.u(1, t8 ? 1 : 0);
        }
        if (cbp) write_residual(b, d, H264R_MB_INTER, cbp, t8);
        planned_ = parts;
    }
    std::vector<Part> planned_;

    // ------------------------------------------------------------ pictures
    void write_picture(const PicPlan &pp)
    {
        const int nmbs = cfg.width_mbs * cfg.height_mbs;
        SliceParams s;
        memset(&s, 0, sizeof(s));
        s.type = pp.type;
        s.idr = pp.idr;
        s.ref = pp.type != kB;
        if (pp.idr) next_frame_num = 0;
        s.frame_num = next_frame_num;
        s.poc_lsb = (2 * pp.display) & ((1 << log2_max_poc_lsb) - 1);
        const int refs = count_refs();
        if (pp.type == kP) s.nref[0] = std::min((int)cfg.num_refs, refs);
        if (pp.type == kB) {
            s.nref[0] = std::min((int)cfg.num_refs, refs);
            s.nref[1] = std::min(2, refs);
        }
        if (pp.type != kI && s.nref[0] < 1) die("no reference picture for a %s picture", pp.type == kB ? "B" : "P");
        if (cfg.weighted == 1 && pp.type != kI) draw_weights(s);
        // slices of whole MB pairs in MBAFF frames
        const int unit = cfg.mbaff ? 2 : 1, nunits = nmbs / unit;
        const int nslices = std::max(1, std::min((int)cfg.slices, nunits));
        for (int si = 0; si < nslices; si++) {
            s.first_mb = unit * (int)((int64_t)nunits * si / nslices);
            const int end_mb = unit * (int)((int64_t)nunits * (si + 1) / nslices);
            s.qp = rng.range(cfg.qp_min, cfg.qp_max);
            s.dbk_alpha = rng.range(-cfg.filter_offset_max, cfg.filter_offset_max);
            s.dbk_beta = rng.range(-cfg.filter_offset_max, cfg.filter_offset_max);
            write_slice(s, end_mb);
        }
        if (s.ref) next_frame_num = (s.frame_num + 1) & ((1 << log2_max_frame_num) - 1);
        else next_frame_num = s.frame_num;
        if (pp.idr) idr_count++;
        // the picture is complete: its marking enters the shadow DPB before
        // the next picture's lists are built
        const int rc = P.finish_picture(false);
        if (rc) die("front end: %s", P.err.c_str());
        P.done.clear();
    }

    void write_slice(const SliceParams &s, int end_mb)
    {
        const int nal_type = s.idr ? 5 : 1, ref_idc = s.ref ? 3 : 0;
        BitWriter b;
        b.buf.reserve((size_t)(end_mb - s.first_mb) * 256 + 64);
        write_slice_header(b, s);
        // the front end takes the header: picture boundary, lists, slice record
        std::vector<uint8_t> hdr_nal;
        {
            BitWriter h = b;
            h.trailing();
            put_nal(hdr_nal, ref_idc, nal_type, h.buf.data(), h.buf.size());
        }
        SliceCtx sc;
        BitReader hbr;
        const int rb = P.begin_slice(hdr_nal.data() + 4, hdr_nal.size() - 4, sc, hbr);
        if (rb != 1) die("front end rejected a slice header: %s", P.err.c_str());
        if (hbr.pos != b.nbits) die("slice header length differs (%zu read, %zu written)", hbr.pos, b.nbits);
        MbDecoder d(P, sc, mbr);
        d.mbaff = cfg.mbaff != 0;
        int skip_run = 0;
        const int W = cfg.width_mbs;
        bool pair_field = false, top_skipped = false;
        // the field flag a decoder infers for a pair with both MBs skipped
        auto inferred = [&](int a) {
            const int pair = a >> 1;
            if (pair % W > 0 && P.mbs[a - 2].slice == sc.index) return P.mbs[a - 2].field;
            if (pair >= W && P.mbs[a - 2 * W].slice == sc.index) return P.mbs[a - 2 * W].field;
            return false;
        };
        bool want_skip[2] = {false, false};
        for (int addr = s.first_mb; addr < end_mb; addr++) {
            const bool top = d.mbaff && (addr & 1) == 0;
            if (!d.mbaff) {
                want_skip[0] = s.type != kI && rng.pct(cfg.skip_percent);
            } else if (top) {
                // the pair's kind, and which of its MBs to skip: a pair with
                // both MBs skipped has the kind a decoder infers (the top MB
                // is decoded before the bottom one is known)
                pair_field = rng.pct(cfg.field_percent);
                want_skip[0] = s.type != kI && rng.pct(cfg.skip_percent);
                want_skip[1] = s.type != kI && rng.pct(cfg.skip_percent);
                if (want_skip[0] && want_skip[1]) pair_field = inferred(addr);
            }
            P.mbs[addr].slice = sc.index;
            P.mbs[addr].skip = false;
            P.mbs[addr].field = pair_field;
            d.set_mb(addr);
            bool skip = false;
            if (want_skip[d.mbaff ? (addr & 1) : 0]) {
                reset_mb_motion(d);
                skip = s.type == kP ? p_skip_ok(d) : direct_ok(d, 15);
            }
            if (skip) {
                skip_run++;
                if (decode_skip(d, P.rec[addr])) die("front end: skipped MB %d: %s", addr, P.err.c_str());
                if (d.fld) P.rec[addr].flags |= H264R_MBF_FIELD;
                if (top) top_skipped = true;
                continue;
            }
            if (s.type != kI) {
                b.ue((uint32_t)skip_run);
                skip_run = 0;
            }
            // mb_field_decoding_flag before the first coded MB of a pair
            if (d.mbaff && (top || top_skipped)) b.u(1, pair_field ? 1 : 0);
            if (top) top_skipped = false;
            const size_t start = b.nbits;
            const bool intra = s.type == kI || rng.pct(cfg.intra_percent);
            planned_.clear();
            const int nref[2] = {d.ref_limit(0), d.ref_limit(1)};
            if (intra) write_intra(b, d, s.type);
            else write_inter(b, d, s.type, nref);
            // read the MB back: the front end's state now holds it
            mbr.reset(b.buf.data(), b.buf.size());
            mbr.pos = start;
            d.cur->skip = false;
            if (d.decode()) die("front end rejected MB %d: %s", addr, P.err.c_str());
            if (d.fld) P.rec[addr].flags |= H264R_MBF_FIELD;
            top_skipped = false;
            if (mbr.pos != b.nbits) die("MB %d: %zu bits read back, %zu written", addr, mbr.pos - start, b.nbits - start);
            for (const Part &p : planned_) {
                if (p.pred == 0) continue;
                const int bi = (p.y >> 2) * 4 + (p.x >> 2);
                for (int l = 0; l < 2; l++)
                    if (p.ref[l] >= 0 && (d.cur->mv[l][bi][0] != p.mv[l][0] || d.cur->mv[l][bi][1] != p.mv[l][1]))
                        die("MB %d: motion vector read back differs from the one written", addr);
            }
        }
        if (skip_run) b.ue((uint32_t)skip_run);
        b.trailing();
        put_nal(out, ref_idc, nal_type, b.buf.data(), b.buf.size());
    }

    void run()
    {
        if (cfg.width_mbs < 1 || cfg.height_mbs < 1 || cfg.width_mbs > 512 || cfg.height_mbs > 512 || cfg.num_pictures < 1)
            die("picture size or count out of range");
        if (cfg.profile_idc != 66 && cfg.profile_idc != 100) die("profile_idc must be 66 or 100");
        high = cfg.profile_idc == 100;
        if (!high && (cfg.b_pictures || cfg.transform8x8 || cfg.weighted))
            die("Baseline streams have no B pictures, 8x8 transforms or weighted prediction");
        if (cfg.num_refs < 1 || cfg.num_refs > 15) die("num_refs out of range");
        if (cfg.qp_min > cfg.qp_max || cfg.qp_max > 51) die("QP range out of range");
        if (cfg.weighted > 2 || cfg.min_partition > 3 || cfg.filter_offset_max > 6 || cfg.chroma_qp_offset_max > 12)
            die("configuration field out of range");
        if (cfg.mv_range > 2048) die("mv_range above 2048 quarter samples");
        if (cfg.mbaff && (!high || (cfg.height_mbs & 1))) die("MBAFF needs High profile and an even height");
        max_refs = cfg.num_refs;
        chroma_offset[0] = rng.range(-cfg.chroma_qp_offset_max, cfg.chroma_qp_offset_max);
        chroma_offset[1] = high ? rng.range(-cfg.chroma_qp_offset_max, cfg.chroma_qp_offset_max) : chroma_offset[0];
        write_sps();
        write_pps();
        for (const PicPlan &pp : plan()) write_picture(pp);
    }
};

}  // namespace

extern "C" int h264r_write_stream(const h264r_writer_cfg *cfg, uint8_t **data, size_t *size)
{
    if (!cfg || !data || !size) return H264R_ERR_INVALID_ARG;
    *data = nullptr;
    *size = 0;
    try {
        std::unique_ptr<Writer> w(new Writer(*cfg));
        w->run();
        uint8_t *buf = (uint8_t *)malloc(w->out.size() ? w->out.size() : 1);
        if (!buf) return H264R_ERR_NO_MEMORY;
        memcpy(buf, w->out.data(), w->out.size());
        *data = buf;
        *size = w->out.size();
        g_writer_err.clear();
        return H264R_OK;
    } catch (const WriterError &e) {
        g_writer_err = e.msg;
        return H264R_ERR_INVALID_ARG;
    } catch (const std::bad_alloc &) {
        g_writer_err = "out of memory";
        return H264R_ERR_NO_MEMORY;
    }
}

extern "C" void h264r_writer_free(uint8_t *data) { free(data); }

extern "C" const char *h264r_writer_last_error(void) { return g_writer_err.c_str(); }
