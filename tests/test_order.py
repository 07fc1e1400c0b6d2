"""Output order of decoded pictures (include/h264r_order.h), host code, no
GPU.  The golden file tests/golden/output_order.json holds, for each of the
reference's bundled streams, the pictures in the order the reference
completes them (POC, IdrPicFlag, the SPS's reorder depth) and the POCs in the
order its output callback received them (tests/golden/make_fixtures.py);
replaying the first through h264r_order must give the second."""
import json
import os

import pytest

import h264_video_decoder_demo_gb300 as h

HERE = os.path.dirname(os.path.abspath(__file__))


def _fixture():
    with open(os.path.join(HERE, "golden", "output_order.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("stream", sorted(_fixture()))
def test_output_order_matches_reference(stream):
    v = _fixture()[stream]
    q = h.Order(v["max_num_reorder_frames"])
    out = []
    for tag, (poc, idr) in enumerate(v["decoded"]):
        out += q.push(tag, poc, idr)
    out += q.flush()
    assert [v["decoded"][t][0] for t in out] == v["output"]
    assert sorted(out) == list(range(len(v["decoded"])))


def test_reorder_known_answers():
    # depth 0: decoding order is output order
    q = h.Order(0)
    assert q.push(1, 0, True) == [1] and q.push(2, 4) == [2] and q.flush() == []
    # I0 P6 B2 B4 with depth 2, then an IDR that flushes
    q = h.Order(2)
    assert q.push(10, 0, True) == []
    assert q.push(11, 6) == []
    assert q.holds(10) and q.holds(11)
    assert q.push(12, 2) == [10]       # buffer full: lowest POC (0) goes out
    assert q.push(13, 4) == [12]       # 2 < 4 and 6
    assert not q.holds(12)
    assert q.push(14, 0, True) == [13, 11]  # IDR: flush 4, 6; the IDR itself is held
    assert q.flush() == [14]


def test_reorder_depth_inference():
    # Table A-1 MaxDpbMbs / frame size, capped at 16; intra profiles with
    # constraint_set3_flag have none
    assert h.Order.infer_depth(100, 0, 40, 120, 68) == 32768 // 8160
    assert h.Order.infer_depth(100, 0, 51, 120, 68) == 16
    assert h.Order.infer_depth(66, 0, 30, 22, 18) == min(8100 // 396, 16)
    assert h.Order.infer_depth(100, 1, 40, 120, 68) == 0
    assert h.Order.infer_depth(77, 0, 99, 120, 68) == 0
