"""C ABI checks that need no GPU: the engine library loads and exports every
symbol include/*.h declares; the host-side validator; the synthetic
workload generator."""
import ctypes
import os
import re

import numpy as np
import pytest

import h264_video_decoder_demo_gb300 as h
from h264_video_decoder_demo_gb300 import records as R
from conftest import ROOT, load_fixture


def declared_symbols():
    names = set()
    for hdr in ("h264r.h", "h264r_synth.h", "h264r_server.h", "h264r_order.h", "h264r_parser.h", "h264r_decoder.h",
                "h264r_writer.h"):
        with open(os.path.join(ROOT, "include", hdr)) as f:
            src = f.read()
        names |= set(re.findall(r"\b(h264r_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol(engine_lib):
    declared = declared_symbols()
    assert len(declared) >= 20
    for name in sorted(declared):
        assert hasattr(engine_lib, name), name
    assert declared == set(h.engine.EXPORTS)


def test_structure_sizes_match_header():
    assert R.MB_DTYPE.itemsize == 32
    assert R.PART_DTYPE.itemsize == 16
    assert R.WEIGHT_DTYPE.itemsize == 32
    assert R.SLICE_DTYPE.itemsize == 8
    assert ctypes.sizeof(R.CPicture) == 8 * 2 + 4 * 4 + 480 + 6 * 8


def test_dpb_bytes(engine_lib):
    cfg = R.CStreamCfg(120, 68, 16, 0)
    per = engine_lib.h264r_stream_dpb_bytes(ctypes.byref(cfg)) // 16
    assert per >= 1920 * 1088 * 3 // 2 and per % 256 == 0


def _fixture_pic():
    pics, _ = load_fixture("heavyhand_cabac_ibp_implicit")
    return pics[1]


def test_validator_accepts_reference_records(engine_lib):
    for p in load_fixture("heavyhand_cabac_mbaff_tff")[0]:
        assert h.validate(p, 16) == 0


@pytest.mark.parametrize("mutation", ["qp", "slice", "type", "coef_off", "motion_off", "ref_slot", "self_ref",
                                      "weight_idx", "mask_bits", "num_mbs", "field_ref_frame_mb", "levels_cut",
                                      "sig_words_cut"])
def test_validator_rejects_bad_records(engine_lib, mutation):
    p = _fixture_pic()
    p.mbs = p.mbs.copy()
    inter = int(np.nonzero((p.mbs["type"] == 0) & (p.mbs["aux"] != R.NONE32))[0][0])
    coded = int(np.nonzero(p.mbs["coef"] != R.NONE32)[0][0])
    if mutation == "qp":
        p.mbs[3]["qpy"] = 52
    elif mutation == "slice":
        p.mbs[3]["slice"] = len(p.slices)
    elif mutation == "type":
        p.mbs[3]["type"] = 9
    elif mutation == "coef_off":
        p.mbs[coded]["coef"] = len(p.coef) + 4
    elif mutation == "motion_off":
        p.mbs[inter]["aux"] = len(p.motion) + 4
    elif mutation in ("ref_slot", "self_ref", "weight_idx", "field_ref_frame_mb"):
        p.motion = p.motion.copy()
        off = int(p.mbs[inter]["aux"]) + 4
        part = np.frombuffer(p.motion[off:off + 16].tobytes(), R.PART_DTYPE).copy()
        if mutation == "ref_slot":
            part["ref"][0, 0] = 20
        elif mutation == "self_ref":
            part["ref"][0, 0] = p.dst_slot
        elif mutation == "weight_idx":
            part["wt"] = len(p.weights)
        else:
            part["ref"][0, 0] = 0x20 | 1
        p.motion[off:off + 16] = np.frombuffer(part.tobytes(), np.uint8)
    elif mutation == "mask_bits":
        p.coef = p.coef.copy()
        off = int(p.mbs[coded]["coef"])
        p.coef[off + 3] = 0x80
    elif mutation == "num_mbs":
        p.mbs = p.mbs[:-1]
    elif mutation in ("levels_cut", "sig_words_cut"):
        # the payload that ends last loses its levels (or most of its
        # significance words): the counts no longer fit the buffer
        last = int(np.argmax(np.where(p.mbs["coef"] != R.NONE32, p.mbs["coef"], 0)))
        off = int(p.mbs[last]["coef"])
        mask = int(np.frombuffer(p.coef[off:off + 4].tobytes(), "<u4")[0])
        t8 = bool(p.mbs[last]["flags"] & 4)
        nw = bin(mask).count("1") + (3 * bin(mask & 15).count("1") if t8 else 0)
        voff = (4 + 2 * nw + 3) & ~3
        p.coef = p.coef[:off + voff] if mutation == "levels_cut" else p.coef[:off + 6]
    assert h.validate(p, 16) in (R.ERR_BAD_RECORD, R.ERR_INVALID_ARG)


def test_validator_field_pictures(engine_lib):
    """Field pictures read fields only; their own slot only for the other
    parity (the first field of the frame)."""
    g = h.synth("cif_ippp", seed=41, num_pictures=4, paff_percent=100, gop_kind=0)
    pics = list(g)
    assert all(h.validate(p, g.dpb_slots) == 0 for p in pics)
    second = next(p for p in pics if p.structure == 2 and (p.mbs["type"] == 0).any())
    inter = int(np.nonzero(second.mbs["type"] == 0)[0][0])
    off = int(second.mbs[inter]["aux"]) + 4
    for bad in (second.dst_slot | 0x20 | 0x40, 1, second.dst_slot):  # own parity, frame ref, own frame
        q = R.Picture.from_c(second.to_c())
        q.motion = q.motion.copy()
        part = np.frombuffer(q.motion[off:off + 16].tobytes(), R.PART_DTYPE).copy()
        part["ref"][0, 0] = bad
        q.motion[off:off + 16] = np.frombuffer(part.tobytes(), np.uint8)
        assert h.validate(q, g.dpb_slots) == R.ERR_BAD_RECORD, bad


def test_synth_is_deterministic(engine_lib):
    a = list(h.synth("cif_ippp", seed=7))
    b = list(h.synth("cif_ippp", seed=7))
    c = list(h.synth("cif_ippp", seed=8))
    assert len(a) == 8
    for x, y in zip(a, b):
        for k in ("mbs", "slices", "weights", "motion", "coef", "pcm"):
            assert np.array_equal(getattr(x, k), getattr(y, k))
    assert not np.array_equal(a[1].coef, c[1].coef)


@pytest.mark.parametrize("name", ["cif_ippp", "1080p_high"])
def test_synth_records_validate(engine_lib, name):
    g = h.synth(name, seed=11, num_pictures=6)
    slots = g.dpb_slots
    pics = list(g)
    assert len(pics) == 6
    for p in pics:
        assert h.validate(p, slots) == 0
    # the workload exercises what its configuration names
    types = set(int(t) for p in pics for t in np.unique(p.mbs["type"]))
    assert {0, 1, 3} <= types
    if name == "1080p_high":
        assert any((p.weights["weighted"] != 0).any() for p in pics)
        assert any((p.mbs["flags"] & 1).any() for p in pics)


def test_synth_slice_and_cip_options_leave_default_streams_unchanged():
    """The generator draws for slices and constrained intra prediction only
    when asked, so existing seeds keep their streams."""
    import numpy as np
    import h264_video_decoder_demo_gb300 as h
    a = list(h.synth("1080p_high", seed=5, width_mbs=20, height_mbs=12, num_pictures=4))
    b = list(h.synth("1080p_high", seed=5, width_mbs=20, height_mbs=12, num_pictures=4, slice_rows=0, cip_percent=0))
    assert all(np.array_equal(x.mbs, y.mbs) and np.array_equal(x.coef, y.coef) and np.array_equal(x.motion, y.motion)
               for x, y in zip(a, b))
    c = list(h.synth("1080p_high", seed=5, width_mbs=20, height_mbs=12, num_pictures=4, slice_rows=3, cip_percent=100))
    assert all(len(p.slices) == 4 for p in c)
    assert all(set(np.unique(p.mbs["slice"]).tolist()) == {0, 1, 2, 3} for p in c)
