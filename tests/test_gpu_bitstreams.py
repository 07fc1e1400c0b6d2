"""Whole bitstreams decoded on the GPU against the reference decoder's output.

  - every case of tests/golden/writer_streams.json: the seeded writer's
    streams with the benchmark configurations' tools (CIF IPPP Baseline; the
    1080p High configuration in CAVLC with explicit bi-predictive weights,
    4 references, P sub-partitions to 4x4, I_PCM, MVs past the edges; non-IDR
    I pictures and three slices; implicit weights with three B pictures),
    written again on this host (same bytes) and decoded by h264r_decoder:
    host front end + engine kernels;
  - the two bundled CAVLC streams whole (50 and 76 pictures).
Every output picture must equal the reference's (md5 of its planes), in the
reference's output order.
"""
import hashlib
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

with open(os.path.join(HERE, "golden", "writer_streams.json")) as _f:
    CASES = json.load(_f)["cases"]


def decode(ctx, data):
    from h264_video_decoder_demo_gb300 import Decoder
    got, ends = [], []

    def on_frame(f, code):
        if f is None:
            ends.append(code)
        else:
            got.append((f["poc"], hashlib.md5(f["planes"].tobytes()).hexdigest()))
        return 0

    d = Decoder(ctx, on_frame)
    try:
        d.push(data)
        d.flush()
    finally:
        d.close()
    assert ends == [Decoder.FILE_END]
    return got


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_written_streams_decode_to_reference_frames(gpu_ctx, case):
    import h264_video_decoder_demo_gb300 as h
    cfg = dict(CASES[case]["writer"])
    seed = cfg.pop("seed")
    data = h.write_stream(None, seed=seed, **cfg)
    assert hashlib.md5(data).hexdigest() == CASES[case]["stream_md5"]
    assert decode(gpu_ctx, data) == [(f["poc"], f["yuv_md5"]) for f in CASES[case]["frames"]]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["gop121_cavlc_whole", "heavyhand_cavlc_b4_whole"])
def test_whole_bundled_streams_decode_to_reference_frames(gpu_ctx, name):
    with open(os.path.join(HERE, "golden", name + ".h264"), "rb") as f:
        data = f.read()
    with open(os.path.join(HERE, "golden", name + ".frames.json")) as f:
        meta = json.load(f)
    assert decode(gpu_ctx, data) == [(f["poc"], f["yuv_md5"]) for f in meta["frames"]]
