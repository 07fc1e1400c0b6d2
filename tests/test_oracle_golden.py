"""The CPU oracle against the reference decoder's own output.

Each golden fixture holds the records of the first pictures of one of the
reference's bundled streams, as the unmodified reference decoded them, and
the md5 of the reference's planes before and after deblocking
(tests/golden/make_fixtures.py).  The oracle must reproduce both exactly.
"""
import hashlib

import pytest

from conftest import fixture_names, load_fixture
from oracle_cpu import OracleDPB


@pytest.mark.parametrize("name", fixture_names())
def test_oracle_matches_reference(name):
    pics, meta = load_fixture(name)
    dpb = OracleDPB(pics[0].width_mbs, pics[0].height_mbs)
    for i, (p, m) in enumerate(zip(pics, meta["pictures"])):
        rc, pre = dpb.reconstruct(p, want_pre=True)
        assert rc == 0, "oracle error %d on picture %d" % (rc, i)
        assert hashlib.md5(pre.tobytes()).hexdigest() == m["pre_md5"], "pre-deblock picture %d" % i
        post = dpb.planes(p.dst_slot)
        assert hashlib.md5(post.tobytes()).hexdigest() == m["post_md5"], "post-deblock picture %d" % i


def test_fixtures_cover_the_hot_path_tools():
    """The fixtures together exercise every reconstruction tool the
    reference's streams use (so the pin is not vacuous)."""
    import numpy as np
    seen_types, mbaff, t8, weighted, bipred, none_mbs, slices = set(), False, False, False, False, False, 1
    for name in fixture_names():
        pics, _ = load_fixture(name)
        for p in pics:
            seen_types |= set(int(t) for t in np.unique(p.mbs["type"]))
            mbaff |= bool(p.mbaff)
            t8 |= bool((p.mbs["flags"] & 1).any())
            weighted |= bool((p.weights["weighted"] != 0).any())
            slices = max(slices, len(p.slices))
            none_mbs |= bool((p.mbs["type"] == 5).any())
            for a in np.nonzero(p.mbs["type"] == 0)[0][:2000]:
                _, parts = p.parts(int(a))
                bipred |= bool(((parts["ref"][:, 0] >= 0) & (parts["ref"][:, 1] >= 0)).any())
    assert {0, 1, 2, 3} <= seen_types
    assert mbaff and t8 and weighted and bipred and none_mbs and slices > 1


@pytest.mark.parametrize("name", fixture_names())
def test_bgr24_and_bmp_writer_match_reference_bmp(name, tmp_path):
    """The reference's BMP output of each fixture picture
    (CH264PictureBase::saveToBmpFile: YUV420P -> BGR24 -> BMP) against the
    oracle's conversion of its planes written by the library's BMP writer
    (host code, no GPU)."""
    import h264_video_decoder_demo_gb300 as h
    from oracle_cpu import bgr24
    pics, meta = load_fixture(name)
    W, H = pics[0].width_mbs * 16, pics[0].height_mbs * 16
    dpb = OracleDPB(pics[0].width_mbs, pics[0].height_mbs)
    for i, (p, m) in enumerate(zip(pics, meta["pictures"])):
        assert dpb.reconstruct(p)[0] == 0
        rows = bgr24(dpb.planes(p.dst_slot), W, H)
        path = tmp_path / ("pic_%d.bmp" % i)
        h.engine.write_bmp(str(path), rows, W, H)
        assert hashlib.md5(path.read_bytes()).hexdigest() == m["bmp_md5"], "picture %d" % i
        flipped = bgr24(dpb.planes(p.dst_slot), W, H, flip=True)
        assert (flipped == rows[::-1]).all()
