// h264r_synth.cpp — seeded synthetic records (see include/h264r_synth.h).
//
// Deterministic on every host: a splitmix64 generator and integer-only
// arithmetic, no library distributions.
#include "../../include/h264r_synth.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

namespace {

struct Rng {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    int range(int lo, int hi) { return lo + (int)(next() % (uint64_t)(hi - lo + 1)); }  // inclusive
    bool pct(int p) { return (int)(next() % 100) < p; }
};

enum PicType { PIC_I, PIC_P, PIC_B };

struct Plan {
    int display;
    PicType type;
    int slot;
    std::vector<int> l0, l1;  // reference slots, nearest first
    std::vector<int> poc0, poc1;
    int poc;
    int group;
    int structure = H264R_STRUCT_FRAME;  // field pictures: H264R_STRUCT_TOP / _BOTTOM
};

inline int clip3(int lo, int hi, int v) { return v < lo ? lo : (v > hi ? hi : v); }

}  // namespace

struct h264r_synth {
    h264r_synth_cfg cfg;
    Rng rng;
    std::vector<Plan> plan;
    size_t next = 0;
    int dpb_slots = 0;
    // current picture buffers
    std::vector<h264r_mb> mbs;
    std::vector<h264r_slice> slices;
    std::vector<h264r_weight> weights;
    std::vector<uint8_t> motion, coef, pcm;
    // explicit weight tables of the current picture, per list and ref index
    int wl[2][4][3], ol[2][4][3];
};

static void build_plan(h264r_synth *g)
{
    const h264r_synth_cfg &c = g->cfg;
    const int n = c.num_pictures, R = c.num_refs < 1 ? 1 : (c.num_refs > 4 ? 4 : c.num_refs);
    const int gop = c.gop_length ? c.gop_length : 15;
    const int ring = R + 2;
    g->dpb_slots = ring + 4;
    int ring_next = 0, bslot = 0, group = 0;
    std::vector<int> anchor_slots, anchor_pocs;  // decoded anchors, oldest first
    auto add_anchor = [&](int d, int grp) {
        Plan p;
        p.display = d;
        p.poc = 2 * d;
        p.type = (d % gop == 0) ? PIC_I : PIC_P;
        p.slot = ring_next;
        ring_next = (ring_next + 1) % ring;
        if (p.type == PIC_P)
            for (int k = (int)anchor_slots.size() - 1; k >= 0 && (int)p.l0.size() < R; k--) {
                p.l0.push_back(anchor_slots[k]);
                p.poc0.push_back(anchor_pocs[k]);
            }
        p.group = grp;
        g->plan.push_back(p);
        anchor_slots.push_back(p.slot);
        anchor_pocs.push_back(p.poc);
    };
    if (c.gop_kind == H264R_SYNTH_GOP_IPPP) {
        for (int d = 0; d < n; d++) add_anchor(d, group++);
        return;
    }
    // IBBP: anchors at display 0, 3, 6, ...; pictures after the last anchor
    // that has no successor become anchors too
    std::vector<int> anchors;
    for (int d = 0; d < n; d += 3) anchors.push_back(d);
    int last = anchors.back();
    for (int d = last + 1; d < n; d++) anchors.push_back(d);
    add_anchor(anchors[0], group++);
    if (anchors.size() > 1) add_anchor(anchors[1], group++);
    for (size_t k = 1; k < anchors.size(); k++) {
        // B pictures between anchors k-1 and k, then anchor k+1: one group
        int a0 = anchors[k - 1], a1 = anchors[k];
        int grp = group++;
        // anchor_slots holds anchors 0..k (and maybe k+1 is not yet added)
        int idx1 = (int)k;
        for (int d = a0 + 1; d < a1; d++) {
            Plan p;
            p.display = d;
            p.poc = 2 * d;
            p.type = PIC_B;
            p.slot = ring + (bslot++ % 4);
            for (int q = idx1 - 1; q >= 0 && (int)p.l0.size() < (R > 1 ? R - 1 : 1); q--) {
                p.l0.push_back(anchor_slots[q]);
                p.poc0.push_back(anchor_pocs[q]);
            }
            p.l1.push_back(anchor_slots[idx1]);
            p.poc1.push_back(anchor_pocs[idx1]);
            p.group = grp;
            g->plan.push_back(p);
        }
        if (k + 1 < anchors.size()) add_anchor(anchors[k + 1], grp);
    }
}

// PAFF: frames coded as a top and a bottom field picture (top first) in
// the same slot.  The fields reference fields of the frames the frame would
// reference; the second field of a P or B frame may also reference the first
// (the slot itself, at the front of list 0).  Dependency groups are then
// recomputed from the slots each picture reads and writes: a picture comes
// after the writers of what it reads, after the readers and the writer of
// the slot it writes.
static void split_fields(h264r_synth *g)
{
    const h264r_synth_cfg &c = g->cfg;
    std::vector<Plan> out;
    for (const Plan &f : g->plan) {
        if (!g->rng.pct(c.paff_percent)) {
            out.push_back(f);
            continue;
        }
        Plan t = f, b = f;
        t.structure = H264R_STRUCT_TOP;
        b.structure = H264R_STRUCT_BOTTOM;
        b.poc = f.poc + 1;
        if (f.type != PIC_I) {
            b.l0.insert(b.l0.begin(), f.slot);
            b.poc0.insert(b.poc0.begin(), f.poc);
        }
        out.push_back(t);
        out.push_back(b);
    }
    std::vector<int> writer(g->dpb_slots, -1), reader(g->dpb_slots, -1);
    for (Plan &p : out) {
        int grp = std::max(writer[p.slot], reader[p.slot]) + 1;
        for (int sl : p.l0) grp = std::max(grp, writer[sl] + 1);
        for (int sl : p.l1) grp = std::max(grp, writer[sl] + 1);
        for (int sl : p.l0) reader[sl] = std::max(reader[sl], grp);
        for (int sl : p.l1) reader[sl] = std::max(reader[sl], grp);
        writer[p.slot] = grp;
        reader[p.slot] = -1;
        p.group = grp;
    }
    g->plan.swap(out);
}

// ---- intra mode choice: modes whose neighbours exist (single slice, no CIP)
static int pick4(Rng &r, bool top, bool left, bool corner)
{
    int modes[9], n = 0;
    modes[n++] = 2;
    if (top) { modes[n++] = 0; modes[n++] = 3; modes[n++] = 7; }
    if (left) { modes[n++] = 1; modes[n++] = 8; }
    if (top && left && corner) { modes[n++] = 4; modes[n++] = 5; modes[n++] = 6; }
    return modes[r.range(0, n - 1)];
}

// ---- coefficients
struct CoefBuilder {
    uint32_t mask = 0;
    std::vector<uint16_t> sig;
    std::vector<int16_t> lv;
};

static int level_value(Rng &r, bool dc)
{
    int mag = 1;
    while (mag < 40 && r.pct(dc ? 45 : 30)) mag += r.range(1, 3);
    return r.pct(50) ? mag : -mag;
}

// one block of `npos` scan positions starting at `first`; returns true if coded
static bool make_block(Rng &r, CoefBuilder &cb, int bit, int first, int npos, int density, int words)
{
    if (!r.pct(density)) return false;
    int k = 1;
    while (k < npos && r.pct(55)) k++;
    uint16_t s[4] = {0, 0, 0, 0};
    int vals[64];
    int nv = 0;
    for (int i = 0; i < k; i++) {
        // low scan positions are more likely
        int span = npos;
        int pos = first + (int)((r.next() % (uint64_t)span) * (r.next() % (uint64_t)span) / (uint64_t)span);
        if (s[pos >> 4] & (1u << (pos & 15))) continue;
        s[pos >> 4] |= (uint16_t)(1u << (pos & 15));
    }
    for (int w = 0; w < words; w++)
        for (int b = 0; b < 16; b++)
            if (s[w] & (1u << b)) vals[nv++] = level_value(r, (16 * w + b) == 0);
    if (nv == 0) return false;
    cb.mask |= 1u << bit;
    for (int w = 0; w < words; w++) cb.sig.push_back(s[w]);
    for (int i = 0; i < nv; i++) cb.lv.push_back((int16_t)vals[i]);
    return true;
}

static uint32_t emit_coef(h264r_synth *g, CoefBuilder &cb)
{
    if (!cb.mask) return H264R_NONE;
    auto &c = g->coef;
    while (c.size() & 3) c.push_back(0);
    uint32_t off = (uint32_t)c.size();
    const uint8_t *pm = (const uint8_t *)&cb.mask;
    c.insert(c.end(), pm, pm + 4);
    const uint8_t *ps = (const uint8_t *)cb.sig.data();
    c.insert(c.end(), ps, ps + 2 * cb.sig.size());
    while (c.size() & 3) c.push_back(0);
    const uint8_t *pl = (const uint8_t *)cb.lv.data();
    c.insert(c.end(), pl, pl + 2 * cb.lv.size());
    return off;
}

static uint16_t add_weight(h264r_synth *g, const h264r_weight &w)
{
    for (size_t i = 0; i < g->weights.size(); i++)
        if (memcmp(&g->weights[i], &w, sizeof(w)) == 0) return (uint16_t)i;
    g->weights.push_back(w);
    return (uint16_t)(g->weights.size() - 1);
}

// implicit weights of 8.4.3 (Derivation_process_for_prediction_weights,
// H264InterPrediction.cpp:2955-2991) for frame MBs
static void implicit_w(int poc, int poc0, int poc1, int &w0, int &w1)
{
    int tb = clip3(-128, 127, poc - poc0), td = clip3(-128, 127, poc1 - poc0);
    if (td == 0) { w0 = w1 = 32; return; }
    int tx = (16384 + abs(td / 2)) / td;
    int dsf = clip3(-1024, 1023, (tb * tx + 32) >> 6);
    if ((dsf >> 2) < -64 || (dsf >> 2) > 128) { w0 = w1 = 32; return; }
    w0 = 64 - (dsf >> 2);
    w1 = dsf >> 2;
}

static void make_picture(h264r_synth *g, const Plan &pl)
{
    const h264r_synth_cfg &c = g->cfg;
    Rng &r = g->rng;
    // a field picture is a grid of W x H/2 field MBs
    const bool fpic = pl.structure != H264R_STRUCT_FRAME;
    const int W = c.width_mbs, H = fpic ? c.height_mbs / 2 : c.height_mbs, n = W * H;
    g->mbs.assign(n, h264r_mb());
    g->slices.clear();
    g->weights.clear();
    g->motion.clear();
    g->coef.clear();
    g->pcm.clear();
    h264r_weight wdef;
    memset(&wdef, 0, sizeof(wdef));
    g->weights.push_back(wdef);
    h264r_slice s;
    memset(&s, 0, sizeof(s));
    s.chroma_qp_offset[0] = (int8_t)r.range(-2, 2);
    s.chroma_qp_offset[1] = (int8_t)r.range(-2, 2);
    s.filter_offset_a = (int8_t)(2 * r.range(-c.filter_offset_max, c.filter_offset_max));
    s.filter_offset_b = (int8_t)(2 * r.range(-c.filter_offset_max, c.filter_offset_max));
    s.disable_deblocking_filter_idc = 0;
    s.slice_type = pl.type == PIC_I ? 2 : (pl.type == PIC_P ? 0 : 1);
    g->slices.push_back(s);
    // further slices every slice_rows MB rows (MB-pair rows for MBAFF), and
    // constrained intra prediction; the extra draws happen only when asked
    // for, so streams without them are unchanged
    const bool mbaff = c.mbaff != 0 && !fpic;
    const int unit_rows = mbaff ? H / 2 : H;
    if (c.slice_rows > 0) {
        const int nslices = (unit_rows + c.slice_rows - 1) / c.slice_rows;
        for (int k = 0; k < nslices; k++) {
            h264r_slice t = s;
            if (k > 0) {
                t.chroma_qp_offset[0] = (int8_t)r.range(-2, 2);
                t.chroma_qp_offset[1] = (int8_t)r.range(-2, 2);
                t.filter_offset_a = (int8_t)(2 * r.range(-c.filter_offset_max, c.filter_offset_max));
                t.filter_offset_b = (int8_t)(2 * r.range(-c.filter_offset_max, c.filter_offset_max));
            }
            const int roll = r.range(0, 99);
            t.disable_deblocking_filter_idc = (uint8_t)(roll < 50 ? 0 : (roll < 85 ? 2 : 1));
            if (k == 0) g->slices[0] = t;
            else g->slices.push_back(t);
        }
    }
    const bool cip = c.cip_percent > 0 && pl.type != PIC_I && r.pct(c.cip_percent);

    const bool explicit_p = c.weighted != H264R_SYNTH_WP_NONE && pl.type == PIC_P;
    const bool explicit_b = c.weighted == H264R_SYNTH_WP_EXPLICIT && pl.type == PIC_B;
    const bool implicit_b = c.weighted == H264R_SYNTH_WP_IMPLICIT && pl.type == PIC_B;
    const int logwd = 5;
    if (explicit_p || explicit_b) {
        int maxw0 = -64;
        for (int l = 0; l < 2; l++)
            for (int i = 0; i < 4; i++)
                for (int cc = 0; cc < 3; cc++) {
                    int hi = (explicit_b && l == 1) ? 127 - maxw0 : 127;
                    if (hi < -64) hi = -64;
                    g->wl[l][i][cc] = r.range(-64, hi);
                    if (l == 0) maxw0 = g->wl[0][i][cc] > maxw0 ? g->wl[0][i][cc] : maxw0;
                    g->ol[l][i][cc] = r.range(-32, 32);
                }
        if (explicit_b) {  // redraw list 1 under the pairwise sum constraint
            for (int i = 0; i < 4; i++)
                for (int cc = 0; cc < 3; cc++) g->wl[1][i][cc] = r.range(-64, 127 - maxw0 < -64 ? -64 : 127 - maxw0);
        }
    }
    const int nl0 = (int)pl.l0.size(), nl1 = (int)pl.l1.size();

    auto weight_for = [&](int r0, int r1) -> uint16_t {
        h264r_weight w;
        memset(&w, 0, sizeof(w));
        if (explicit_p || explicit_b) {
            w.weighted = 1;
            for (int cc = 0; cc < 3; cc++) {
                w.log_wd[cc] = (int8_t)logwd;
                w.w0[cc] = (int16_t)(r0 >= 0 ? g->wl[0][r0][cc] : 1);
                w.o0[cc] = (int16_t)(r0 >= 0 ? g->ol[0][r0][cc] : 0);
                w.w1[cc] = (int16_t)(r1 >= 0 ? g->wl[1][r1][cc] : 1);
                w.o1[cc] = (int16_t)(r1 >= 0 ? g->ol[1][r1][cc] : 0);
            }
        } else if (implicit_b && r0 >= 0 && r1 >= 0) {
            int w0, w1;
            implicit_w(pl.poc, pl.poc0[r0], pl.poc1[r1], w0, w1);
            w.weighted = 1;
            for (int cc = 0; cc < 3; cc++) {
                w.log_wd[cc] = 5;
                w.w0[cc] = (int16_t)w0;
                w.w1[cc] = (int16_t)w1;
            }
        }
        return add_weight(g, w);
    };

    // MBAFF: MBs in pair order (top, bottom); the pair's field decision is
    // taken at its top MB
    bool pair_field = false;
    for (int a = 0; a < n; a++) {
        const int mx = mbaff ? (a / 2) % W : a % W;
        const int my = mbaff ? 2 * ((a / 2) / W) + (a & 1) : a / W;
        h264r_mb &m = g->mbs[a];
        memset(&m, 0, sizeof(m));
        m.coef = H264R_NONE;
        m.aux = H264R_NONE;
        if (mbaff && (a & 1) == 0) pair_field = r.pct(c.field_percent);
        const bool field = mbaff && pair_field;
        if (field) m.flags |= H264R_MBF_FIELD;
        const bool field_refs = field || fpic;  // predicts from fields
        m.qpy = (uint8_t)r.range(c.qp_min, c.qp_max);
        m.slice = (uint16_t)(c.slice_rows > 0 ? (mbaff ? (a / 2) / W : a / W) / c.slice_rows : 0);
        if (cip) m.flags |= H264R_MBF_CIP;
        bool intra = pl.type == PIC_I || r.pct(c.intra_percent);
        CoefBuilder cb;
        const int dens = c.coef_density;
        if (intra) {
            int roll = r.range(0, 999);
            if (roll < 2) m.type = H264R_MB_IPCM;
            else if (roll < 450) m.type = H264R_MB_I4x4;
            else if (roll < 750) m.type = c.transform8x8 ? H264R_MB_I8x8 : H264R_MB_I4x4;
            else m.type = H264R_MB_I16x16;
            // neighbours usable for intra prediction: same slice, and not an
            // inter MB under constrained intra prediction
            auto usable = [&](int nb) {
                const h264r_mb &q = g->mbs[nb];
                return q.slice == m.slice && !(cip && q.type == H264R_MB_INTER);
            };
            bool A, B, D;
            if (!mbaff) {
                A = mx > 0 && usable(a - 1);
                B = my > 0 && usable(a - W);
                D = mx > 0 && my > 0 && usable(a - W - 1);
            } else {
                // MBAFF (6.4.12.2, Table 6-4): the left samples lie in the
                // left pair; the samples above a top MB, or above a field MB,
                // in the pair above; above a bottom frame MB in the top MB of
                // its own pair; the corner sample of a bottom frame MB in the
                // left pair, of any other MB in the pair above-left.  A pair
                // counts as usable when both its MBs are (under constrained
                // intra prediction the samples of a frame MB beside a field
                // pair come from both MBs).
                const int pa = a / 2, pc = pa % W, pr = pa / W;
                auto pair_ok = [&](int q) { return usable(2 * q) && usable(2 * q + 1); };
                const bool upper = (a & 1) == 0 || field;
                A = pc > 0 && pair_ok(pa - 1);
                B = upper ? pr > 0 && pair_ok(pa - W) : usable(a - 1);
                D = upper ? pc > 0 && pr > 0 && pair_ok(pa - W - 1) : A;
            }
            if (m.type == H264R_MB_IPCM) {
                m.aux = (uint32_t)(g->pcm.size() / 384);
                for (int i = 0; i < 384; i++) g->pcm.push_back((uint8_t)r.range(0, 255));
                m.nz4x4 = 0xFFFF;
                m.nz8x8 = 0xF;
            } else if (m.type == H264R_MB_I4x4) {
                static const int bx[16] = {0, 1, 0, 1, 2, 3, 2, 3, 0, 1, 0, 1, 2, 3, 2, 3};
                static const int by[16] = {0, 0, 1, 1, 0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 3, 3};
                for (int b = 0; b < 16; b++) {
                    bool left = bx[b] > 0 || A, top = by[b] > 0 || B, corner = left && top && (bx[b] > 0 || by[b] > 0 || D);
                    const int md = pick4(r, top, left, corner);
                    m.ipred[b >> 3] |= (uint32_t)md << (4 * (b & 7));
                    if (make_block(r, cb, b, 0, 16, dens, 1)) m.nz4x4 |= (uint16_t)(1u << b);
                }
            } else if (m.type == H264R_MB_I8x8) {
                m.flags |= H264R_MBF_T8x8;
                for (int b = 0; b < 4; b++) {
                    int x8 = b & 1, y8 = b >> 1;
                    bool left = x8 > 0 || A, top = y8 > 0 || B, corner = left && top && (x8 > 0 || y8 > 0 || D);
                    const int md = pick4(r, top, left, corner);
                    m.ipred[0] |= (uint32_t)md << (4 * b);
                    if (make_block(r, cb, b, 0, 64, dens, 4)) m.nz8x8 |= (uint8_t)(1u << b);
                }
            } else {
                int modes[4], nm = 0;
                modes[nm++] = 2;
                if (B) modes[nm++] = 0;
                if (A) modes[nm++] = 1;
                if (A && B && D) modes[nm++] = 3;
                m.i16_mode = (uint8_t)modes[r.range(0, nm - 1)];
                for (int b = 0; b < 16; b++)
                    if (make_block(r, cb, b, 1, 15, dens / 2, 1)) m.nz4x4 |= (uint16_t)(1u << b);
                make_block(r, cb, 16, 0, 16, 80, 1);
            }
            if (m.type != H264R_MB_IPCM) {
                int cm[4], nc = 0;
                cm[nc++] = 0;
                if (A) cm[nc++] = 1;
                if (B) cm[nc++] = 2;
                if (A && B && D) cm[nc++] = 3;
                m.chroma_mode = (uint8_t)cm[r.range(0, nc - 1)];
            }
        } else {
            m.type = H264R_MB_INTER;
            bool skip = r.pct(c.skip_percent);
            // partition shape
            int shape = 0;
            if (!skip) {
                int roll = r.range(0, 99);
                if (c.min_partition >= 1 && roll >= 40 && roll < 55) shape = 1;
                else if (c.min_partition >= 1 && roll >= 55 && roll < 70) shape = 2;
                else if (c.min_partition >= 2 && roll >= 70) {
                    shape = 3;
                    for (int q = 0; q < 4; q++) {
                        int sc = c.min_partition >= 3 ? r.range(0, 3) : 0;
                        shape |= sc << (2 + 2 * q);
                    }
                }
            }
            bool direct16 = skip && pl.type == PIC_B;
            if (direct16) shape = 3 | (3 << 2) | (3 << 4) | (3 << 6) | (3 << 8);
            int nparts;
            {
                int mp = shape & 3;
                if (mp == 0) nparts = 1;
                else if (mp != 3) nparts = 2;
                else {
                    nparts = 0;
                    for (int q = 0; q < 4; q++) {
                        int sc = (shape >> (2 + 2 * q)) & 3;
                        nparts += (sc == 0) ? 1 : (sc == 3 ? 4 : 2);
                    }
                }
            }
            while (g->motion.size() & 3) g->motion.push_back(0);
            m.aux = (uint32_t)g->motion.size();
            uint16_t hdr[2] = {(uint16_t)shape, (uint16_t)nparts};
            const uint8_t *ph = (const uint8_t *)hdr;
            g->motion.insert(g->motion.end(), ph, ph + 4);
            // partition-level prediction choices: one per 8x8 quadrant for
            // sub-partitioned MBs (all sub-partitions share refs), else per part
            int qref[4][2];
            for (int q = 0; q < 4; q++) {
                int r0 = -1, r1 = -1;
                if (pl.type == PIC_P) {
                    r0 = r.range(0, nl0 - 1);
                } else {
                    int k = r.range(0, 2);  // L0, L1, Bi
                    if (explicit_b && k == 1) k = 2;  // avoid explicit list-1-only partitions
                    if (k == 0 || k == 2) r0 = r.range(0, nl0 - 1);
                    if (k == 1 || k == 2) r1 = r.range(0, nl1 - 1);
                }
                qref[q][0] = r0;
                qref[q][1] = r1;
            }
            int mvq[4][2][2];
            for (int e = 0; e < nparts; e++) {
                // quadrant of the entry (for 16x16/16x8/8x16 use the entry index)
                int q = ((shape & 3) == 3) ? 0 : e;
                if ((shape & 3) == 3) {
                    int base = 0;
                    for (int qq = 0; qq < 4; qq++) {
                        int sc = (shape >> (2 + 2 * qq)) & 3;
                        int cnt = (sc == 0) ? 1 : (sc == 3 ? 4 : 2);
                        if (e < base + cnt) { q = qq; break; }
                        base += cnt;
                    }
                }
                h264r_part p;
                memset(&p, 0, sizeof(p));
                int rr[2] = {qref[q][0], qref[q][1]};
                for (int l = 0; l < 2; l++) {
                    p.ref[l] = -1;
                    p.dref[l] = -1;
                    if (rr[l] < 0) continue;
                    int slot = l == 0 ? pl.l0[rr[l]] : pl.l1[rr[l]];
                    p.ref[l] = (int8_t)slot;
                    p.dref[l] = (int8_t)slot;
                    if (field_refs) {  // a field of the reference frame, either parity
                        // (the first field of the current frame, for a second field)
                        const bool bot = slot == pl.slot ? false : r.pct(50);
                        p.ref[l] = (int8_t)(slot | H264R_REF_FIELD | (bot ? H264R_REF_BOTTOM : 0));
                        p.dref[l] = (int8_t)(p.ref[l] & 0x7F);
                    }
                    int mvx, mvy;
                    bool same_as_quadrant = direct16 && (e % 4) != 0;
                    if (same_as_quadrant) {
                        mvx = mvq[q][l][0];
                        mvy = mvq[q][l][1];
                    } else if (skip && !direct16) {
                        mvx = r.range(-16, 16);
                        mvy = r.range(-16, 16);
                    } else if (r.pct(c.edge_mv_percent)) {
                        // point beyond a picture edge
                        int side = r.range(0, 3);
                        mvx = r.range(-c.mv_range, c.mv_range);
                        mvy = r.range(-c.mv_range, c.mv_range);
                        if (side == 0) mvx = -(mx * 16 + 16 + r.range(0, 48)) * 4;
                        if (side == 1) mvx = ((W - mx) * 16 + r.range(0, 48)) * 4;
                        if (side == 2) mvy = -(my * 16 + 16 + r.range(0, 48)) * 4;
                        if (side == 3) mvy = ((H - my) * 16 + r.range(0, 48)) * 4;
                        mvx = clip3(-2048, 2047, mvx);
                        mvy = clip3(-512, 511, mvy);
                        if (field) mvy /= 2;  // field rows (a field picture's grid is in field rows already)
                    } else {
                        mvx = r.range(-c.mv_range, c.mv_range);
                        mvy = r.range(-c.mv_range, c.mv_range);
                    }
                    if (direct16 && (e % 4) == 0) {
                        mvq[q][l][0] = mvx;
                        mvq[q][l][1] = mvy;
                    }
                    p.mv[l][0] = (int16_t)mvx;
                    p.mv[l][1] = (int16_t)mvy;
                }
                p.wt = weight_for(rr[0], rr[1]);
                const uint8_t *pp = (const uint8_t *)&p;
                g->motion.insert(g->motion.end(), pp, pp + sizeof(p));
            }
            if (!skip) {
                if (c.transform8x8 && r.pct(40) && (shape & 3) != 3) {
                    m.flags |= H264R_MBF_T8x8;
                    for (int b = 0; b < 4; b++)
                        if (make_block(r, cb, b, 0, 64, dens, 4)) m.nz8x8 |= (uint8_t)(1u << b);
                } else {
                    for (int b = 0; b < 16; b++)
                        if (make_block(r, cb, b, 0, 16, dens, 1)) m.nz4x4 |= (uint16_t)(1u << b);
                }
            }
        }
        if (m.type != H264R_MB_IPCM && !(m.type == H264R_MB_INTER && cb.mask == 0 && r.pct(30))) {
            int cd = (m.type == H264R_MB_INTER) ? dens / 2 : dens;
            make_block(r, cb, 17, 0, 4, cd, 1);
            make_block(r, cb, 18, 0, 4, cd, 1);
            for (int b = 0; b < 4; b++) make_block(r, cb, H264R_CM_CB_AC0 + b, 1, 15, cd / 3, 1);
            for (int b = 0; b < 4; b++) make_block(r, cb, H264R_CM_CR_AC0 + b, 1, 15, cd / 3, 1);
        }
        // make_block calls above run in ascending mask-bit order, the order
        // the payload requires
        m.coef = emit_coef(g, cb);
    }
}

extern "C" int h264r_synth_create(const h264r_synth_cfg *cfg, h264r_synth **out)
{
    if (!cfg || !out || cfg->width_mbs == 0 || cfg->height_mbs == 0 || cfg->num_pictures == 0 || cfg->qp_min > cfg->qp_max ||
        cfg->qp_max > 51 || ((cfg->mbaff || cfg->paff_percent) && (cfg->height_mbs & 1)))
        return H264R_ERR_INVALID_ARG;
    h264r_synth *g = new (std::nothrow) h264r_synth();
    if (!g) return H264R_ERR_NO_MEMORY;
    g->cfg = *cfg;
    if (g->cfg.num_refs < 1) g->cfg.num_refs = 1;
    if (g->cfg.num_refs > 4) g->cfg.num_refs = 4;
    g->rng.s = 0x5EED0000ull ^ cfg->seed;
    build_plan(g);
    if (cfg->paff_percent > 0) split_fields(g);
    *out = g;
    return H264R_OK;
}

extern "C" int h264r_synth_dpb_slots(const h264r_synth *g) { return g ? g->dpb_slots : 0; }

extern "C" int h264r_synth_next(h264r_synth *g, h264r_picture *pic, int *dependency_group)
{
    if (!g || !pic) return H264R_ERR_INVALID_ARG;
    if (g->next >= g->plan.size()) return 1;
    const Plan &pl = g->plan[g->next++];
    make_picture(g, pl);
    memset(pic, 0, sizeof(*pic));
    pic->width_mbs = g->cfg.width_mbs;
    pic->height_mbs = g->cfg.height_mbs;
    pic->structure = (uint8_t)pl.structure;
    pic->mbaff = g->cfg.mbaff && pl.structure == H264R_STRUCT_FRAME ? 1 : 0;
    pic->dst_slot = (uint8_t)pl.slot;
    pic->deblock = 1;
    pic->num_slices = (uint16_t)g->slices.size();
    pic->num_weights = (uint16_t)g->weights.size();
    pic->num_mbs = (uint32_t)g->mbs.size();
    pic->motion_bytes = (uint32_t)g->motion.size();
    pic->coef_bytes = (uint32_t)g->coef.size();
    pic->num_pcm = (uint32_t)(g->pcm.size() / 384);
    memset(pic->scaling4x4, 16, sizeof(pic->scaling4x4));
    memset(pic->scaling8x8, 16, sizeof(pic->scaling8x8));
    pic->mbs = g->mbs.data();
    pic->slices = g->slices.data();
    pic->weights = g->weights.data();
    pic->motion = g->motion.data();
    pic->coef = g->coef.data();
    pic->pcm = g->pcm.data();
    if (dependency_group) *dependency_group = pl.group;
    return 0;
}

extern "C" int h264r_synth_destroy(h264r_synth *g)
{
    delete g;
    return H264R_OK;
}
