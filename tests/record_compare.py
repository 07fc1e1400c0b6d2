"""Record-by-record comparison of two decodes of the same stream (test
infrastructure): the records the host front end produced against the records
the reference decoder produced (oracle/_ref/ref_dump), picture by picture.

DPB slot numbers are private to each decoder, so references are compared by
the decoding-order index of the picture they name; weights are compared where
a partition uses them.  Returns a list of (picture index, [differences]).
"""
import struct

import numpy as np

from h264_video_decoder_demo_gb300 import records as R

NONE = 0xFFFFFFFF


def _coef_equal(a, ao, b, bo, t8):
    if (ao == NONE) != (bo == NONE):
        return False
    if ao == NONE:
        return True
    ra, rb = a.coef.tobytes(), b.coef.tobytes()
    mask = struct.unpack_from("<I", ra, ao)[0]
    if mask != struct.unpack_from("<I", rb, bo)[0]:
        return False
    nsig = sum((4 if (t8 and bit < 4) else 1) for bit in range(27) if mask >> bit & 1)
    sa, sb = ra[ao + 4: ao + 4 + 2 * nsig], rb[bo + 4: bo + 4 + 2 * nsig]
    if sa != sb:
        return False
    nl = sum(bin(int(x)).count("1") for x in np.frombuffer(sa, np.uint16))
    la, lb = (ao + 4 + 2 * nsig + 3) & ~3, (bo + 4 + 2 * nsig + 3) & ~3
    return ra[la: la + 2 * nl] == rb[lb: lb + 2 * nl]


def _all_parts(p):
    """(MB index per part, header shape per MB, parts) of a picture's inter MBs."""
    raw = np.frombuffer(p.motion.tobytes(), np.uint8)
    inter = np.nonzero(p.mbs["type"] == 0)[0]
    aux = p.mbs["aux"][inter].astype(np.int64)
    if len(inter) == 0:
        return inter, np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0, R.PART_DTYPE)
    hdr = raw[aux[:, None] + np.arange(4)].copy().view(np.uint16).reshape(-1, 2)
    shape, cnt = hdr[:, 0].astype(np.int64), hdr[:, 1].astype(np.int64)
    first = np.repeat(aux + 4, cnt) + 16 * (np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt))
    parts = raw[first[:, None] + np.arange(16)].copy().view(R.PART_DTYPE).reshape(-1)
    return np.repeat(inter, cnt), shape, cnt, parts


def _lookup(table, slots):
    out = np.full(len(slots), -1, np.int64)
    for s, idx in table.items():
        out[slots == s] = idx
    return out


def _motion_diffs(r, m, ref_slot, my_slot):
    ri, rshape, rcnt, rp = _all_parts(r)
    mi, mshape, mcnt, mp = _all_parts(m)
    if len(rshape) != len(mshape) or np.any(rshape != mshape) or np.any(rcnt != mcnt):
        inter = np.nonzero(r.mbs["type"] == 0)[0]
        n = min(len(rshape), len(mshape))
        bad = inter[:n][(rshape[:n] != mshape[:n]) | (rcnt[:n] != mcnt[:n])]
        return sorted(set(bad.tolist())) or [int(inter[0]) if len(inter) else 0]
    bad = np.zeros(len(rp), bool)
    for li in range(2):
        rr, mm = rp["ref"][:, li].astype(np.int64), mp["ref"][:, li].astype(np.int64)
        used = rr >= 0
        bad |= used != (mm >= 0)
        bad |= used & (_lookup(ref_slot, rr & 31) != _lookup(my_slot, mm & 31))
        bad |= used & np.any(rp["mv"][:, li] != mp["mv"][:, li], axis=1)
        dr, dm = rp["dref"][:, li].astype(np.int64), mp["dref"][:, li].astype(np.int64)
        bad |= (dr < 0) != (dm < 0)
        bad |= (dr >= 0) & (_lookup(ref_slot, dr) != _lookup(my_slot, dm))
    wr, wm = r.weights[rp["wt"]], m.weights[mp["wt"]]
    bad |= wr["weighted"] != wm["weighted"]
    w = wr["weighted"] != 0
    bad |= w & np.any(wr["log_wd"] != wm["log_wd"], axis=1)
    u0, u1 = rp["ref"][:, 0] >= 0, rp["ref"][:, 1] >= 0
    bad |= w & u0 & (np.any(wr["w0"] != wm["w0"], axis=1) | np.any(wr["o0"] != wm["o0"], axis=1))
    bad |= w & u1 & (np.any(wr["w1"] != wm["w1"], axis=1) | np.any(wr["o1"] != wm["o1"], axis=1))
    return sorted(set(ri[bad].tolist()))


def compare_streams(ref_pics, mine, ignore_nz_of=()):
    """ref_pics: pictures read from a reference dump (decoding order);
    mine: list of (Picture, info) from engine.Parser.  ignore_nz_of: (picture,
    MB) pairs whose non-zero counts are not compared."""
    out = []
    ref_slot, my_slot = {}, {}
    for i, (r, (m, info)) in enumerate(zip(ref_pics, mine)):
        ref_slot[r.dst_slot] = i
        my_slot[m.dst_slot] = i
        bad = []
        if r.poc != info["poc"]:
            bad.append("poc %d vs %d" % (r.poc, info["poc"]))
        if len(r.mbs) != len(m.mbs):
            out.append((i, ["MB count"]))
            continue
        for f in ("type", "flags", "qpy", "slice", "nz4x4", "nz8x8"):
            d = r.mbs[f] != m.mbs[f]
            if f in ("nz4x4", "nz8x8"):
                for (pi, a) in ignore_nz_of:
                    if pi == i:
                        d[a] = False
            d = np.nonzero(d)[0]
            if len(d):
                bad.append("%s at %d MBs (first %d)" % (f, len(d), d[0]))
        intra = np.isin(r.mbs["type"], [1, 2, 3])
        d = np.nonzero((r.mbs["chroma_mode"] != m.mbs["chroma_mode"]) & intra)[0]
        if len(d):
            bad.append("chroma_mode at %d MBs" % len(d))
        d = np.nonzero(np.any(r.mbs["ipred"] != m.mbs["ipred"], axis=1) & np.isin(r.mbs["type"], [1, 2]))[0]
        if len(d):
            bad.append("intra modes at %d MBs (first %d)" % (len(d), d[0]))
        d = np.nonzero((r.mbs["i16_mode"] != m.mbs["i16_mode"]) & (r.mbs["type"] == 3))[0]
        if len(d):
            bad.append("Intra16x16 mode at %d MBs" % len(d))
        if not (np.array_equal(r.mbs["coef"], m.mbs["coef"]) and r.coef.tobytes() == m.coef.tobytes()):
            # same packing on both sides: equal arrays mean equal levels; else find the MBs
            nc = [a for a in range(len(r.mbs))
                  if not _coef_equal(r, int(r.mbs["coef"][a]), m, int(m.mbs["coef"][a]), r.mbs["flags"][a] & 1)]
            if nc:
                bad.append("coefficients at %d MBs (first %d)" % (len(nc), nc[0]))
        if r.pcm.tobytes() != m.pcm.tobytes():
            bad.append("I_PCM samples")
        nm = _motion_diffs(r, m, ref_slot, my_slot)
        if nm:
            bad.append("motion at %d MBs (first %d)" % (len(nm), nm[0]))
        if r.slices.tobytes() != m.slices.tobytes():
            bad.append("slice parameters")
        if r.deblock != m.deblock:
            bad.append("deblock flag")
        if bad:
            out.append((i, bad))
    return out
