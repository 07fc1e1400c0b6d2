"""Field pictures (PAFF) in the oracle, pinned to its own frame path.

The reference decoder cannot decode field pictures: on streams whose only
change from streams it decodes is the field picture syntax it aborts with
heap corruption (tests/golden/paff_probe.json, made by
tests/golden/make_paff_probe.py).  So the oracle's field-picture path is a
restatement of the standard, and this test pins it to the oracle's frame
path, which the reference's own output pins.

A field picture whose partitions all read fields of its own parity, with
no residual and no deblocking, predicts exactly like a frame picture of the
field's size whose references are those fields: the same reference samples
with the same clamping (8.4.2.2), no chroma vector offset between fields of
equal parity (Table 8-10), intra neighbours inside the field (6.4.12.1,
8.3), I_PCM samples placed row by row.  Every field picture of a seeded PAFF
stream is rewritten that way (own-parity references; a second field's
reference to the first field of its frame goes to the same parity of the
frame before) and decoded twice: as a field into a DPB of frames, and as a
frame picture into a DPB whose slots hold single fields.  The field must
equal the frame picture, picture after picture.
"""
import numpy as np
import pytest

import h264_video_decoder_demo_gb300 as h
from h264_video_decoder_demo_gb300 import records as R
from oracle_cpu import OracleDPB

TOP, BOTTOM = 1, 2


def own_parity(pic, prev_slot):
    """pic with every field reference moved to pic's parity, no residual,
    no deblocking; a reference to pic's own slot goes to prev_slot."""
    bot = R.H264R_REF_BOTTOM if hasattr(R, "H264R_REF_BOTTOM") else 0x40
    q = R.Picture()
    for k in ("width_mbs", "height_mbs", "structure", "mbaff", "dst_slot", "scaling4x4", "scaling8x8"):
        setattr(q, k, getattr(pic, k))
    q.deblock = 0
    q.mbs, q.slices, q.weights, q.pcm = pic.mbs.copy(), pic.slices.copy(), pic.weights.copy(), pic.pcm.copy()
    q.coef = np.zeros(0, np.uint8)
    q.mbs["coef"] = 0xFFFFFFFF
    q.mbs["nz4x4"] = 0
    q.mbs["nz8x8"] = 0
    motion = pic.motion.copy()
    parity = bot if pic.structure == BOTTOM else 0
    for a in np.nonzero(q.mbs["type"] == R.MB_INTER)[0]:
        off = int(q.mbs[a]["aux"])
        count = int(np.frombuffer(motion.tobytes(), "<u2", 2, off)[1])
        parts = motion[off + 4:off + 4 + 16 * count].view(R.PART_DTYPE)
        for l in range(2):
            r = parts["ref"][:, l].astype(np.int32)
            use = r >= 0
            slot = r & 31
            slot = np.where(slot == pic.dst_slot, prev_slot, slot)
            r2 = np.where(use, slot | 0x20 | parity, -1)
            parts["ref"][:, l] = r2.astype(np.int8)
            parts["dref"][:, l] = r2.astype(np.int8)
    q.motion = motion
    return q


def as_frame(fpic, half_slot):
    """The field picture as a frame picture of the field's size in the DPB
    of single fields: slot (s, parity) is half_slot(s, parity)."""
    q = R.Picture()
    for k in ("width_mbs", "scaling4x4", "scaling8x8"):
        setattr(q, k, getattr(fpic, k))
    q.height_mbs = fpic.height_mbs // 2
    q.structure, q.mbaff, q.deblock = 0, 0, 0
    q.dst_slot = half_slot(fpic.dst_slot, fpic.structure == BOTTOM)
    q.mbs, q.slices, q.weights, q.pcm, q.coef = fpic.mbs, fpic.slices, fpic.weights, fpic.pcm, fpic.coef
    motion = fpic.motion.copy()
    for a in np.nonzero(q.mbs["type"] == R.MB_INTER)[0]:
        off = int(q.mbs[a]["aux"])
        count = int(np.frombuffer(motion.tobytes(), "<u2", 2, off)[1])
        parts = motion[off + 4:off + 4 + 16 * count].view(R.PART_DTYPE)
        for l in range(2):
            r = parts["ref"][:, l].astype(np.int32)
            r2 = np.array([half_slot(v & 31, bool(v & 0x40)) if v >= 0 else -1 for v in r], np.int32)
            parts["ref"][:, l] = r2.astype(np.int8)
            parts["dref"][:, l] = r2.astype(np.int8)
    q.motion = motion
    return q


def field_of(planes, wmb, hmb, bottom):
    W, H = 16 * wmb, 16 * hmb
    y = planes[:W * H].reshape(H, W)[int(bottom)::2]
    cb = planes[W * H:W * H * 5 // 4].reshape(H // 2, W // 2)[int(bottom)::2]
    cr = planes[W * H * 5 // 4:W * H * 3 // 2].reshape(H // 2, W // 2)[int(bottom)::2]
    return np.concatenate([y.reshape(-1), cb.reshape(-1), cr.reshape(-1)])


@pytest.mark.parametrize("seed,over", [
    (3, dict(gop_kind=0)),                                             # I / P field pairs
    (4, dict(gop_kind=1, num_refs=2, min_partition=3, edge_mv_percent=20)),  # with B field pairs, MVs past the edges
    (5, dict(gop_kind=1, num_refs=3, intra_percent=40, mv_range=128)),
])
def test_field_pictures_predict_like_frames_of_the_field(engine_lib, seed, over):
    cfg = dict(num_pictures=6, paff_percent=100, coef_density=0, transform8x8=0)
    cfg.update(over)
    g = h.synth("cif_ippp", seed=seed, **cfg)
    pics = list(g)
    assert pics and all(p.structure in (TOP, BOTTOM) for p in pics)
    wmb, hmb, nslots = pics[0].width_mbs, pics[0].height_mbs, g.dpb_slots
    frames = OracleDPB(wmb, hmb, nslots)
    fields = OracleDPB(wmb, hmb // 2, 2 * nslots)

    def half_slot(s, bottom):
        return 2 * s + int(bottom)

    prev = {}  # parity -> slot of the last completed frame
    done = 0
    intra = inter = 0
    for p in pics:
        fp = own_parity(p, prev.get("frame", p.dst_slot))
        rc, _ = frames.reconstruct(fp)
        assert rc == 0
        fr = as_frame(fp, half_slot)
        rc, _ = fields.reconstruct(fr)
        assert rc == 0
        got = field_of(frames.planes(p.dst_slot), wmb, hmb, p.structure == BOTTOM)
        want = fields.planes(fr.dst_slot)
        assert np.array_equal(got, want), "field picture %d (%s) differs from the frame of its field" % (
            done, "bottom" if p.structure == BOTTOM else "top")
        if p.structure == BOTTOM:
            prev["frame"] = p.dst_slot
        intra += int(np.isin(p.mbs["type"], [1, 2, 3, 4]).sum())
        inter += int((p.mbs["type"] == R.MB_INTER).sum())
        done += 1
    assert intra > 0 and inter > 0
