"""Whole-stream decoding on the GPU (include/h264r_decoder.h and the
reference-compatible C++ interface of include/compat) against the
reference's own output for the committed cut streams (tests/golden/*.h264):
every output picture's planes (md5, output order, POC) and every BMP the
reference's main.cpp writes."""
import hashlib
import json
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

BITSTREAMS = ["gop121_cavlc_4pics", "heavyhand_cavlc_b4_6pics", "heavyhand_cabac_p_6pics", "heavyhand_cabac_ibp_6pics",
              "heavyhand_cabac_mbaff_6pics"]


def _golden(name):
    with open(os.path.join(HERE, "golden", name + ".frames.json")) as f:
        return os.path.join(HERE, "golden", name + ".h264"), json.load(f)


@pytest.mark.gpu
@pytest.mark.parametrize("name", BITSTREAMS)
def test_decoder_matches_reference_frames(gpu_ctx, name):
    from h264_video_decoder_demo_gb300 import Decoder
    path, meta = _golden(name)
    got, ends = [], []

    def on_frame(f, code):
        if f is None:
            ends.append(code)
            return 0
        got.append((f["poc"], hashlib.md5(f["planes"].tobytes()).hexdigest()))
        return 0

    d = Decoder(gpu_ctx, on_frame)
    assert d.open(path) == 0
    assert ends == [Decoder.FILE_END]
    assert got == [(fr["poc"], fr["yuv_md5"]) for fr in meta["frames"]]
    assert d.decoded == meta["pictures"]
    d.close()


@pytest.mark.gpu
def test_decoder_push_in_chunks_and_stop(gpu_ctx):
    from h264_video_decoder_demo_gb300 import Decoder
    path, meta = _golden("heavyhand_cavlc_b4_6pics")
    with open(path, "rb") as f:
        data = f.read()
    got = []
    d = Decoder(gpu_ctx, lambda f, code: got.append(None if f is None else f["poc"]) or False)
    for i in range(0, len(data), 50000):
        d.push(data[i:i + 50000])
    d.flush()
    assert got == [fr["poc"] for fr in meta["frames"]] + [None]
    d.close()
    # a true return stops the decode; the final call still comes
    seen = []
    d = Decoder(gpu_ctx, lambda f, code: seen.append(code) or f is not None)
    d.open(path)
    assert seen == [0, Decoder.FILE_END]
    d.close()
    # a missing file: one OPEN_FILE_FAILED call
    codes = []
    d = Decoder(gpu_ctx, lambda f, code: codes.append(code) or False)
    assert d.open(os.path.join(HERE, "golden", "no_such_stream.h264")) == -10
    assert codes == [Decoder.OPEN_FILE_FAILED]
    d.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", BITSTREAMS)
def test_compat_interface_writes_reference_bmps(gpu_ctx, name, tmp_path):
    """A program written against the reference's CH264VideoDecoder /
    CH264Picture interface (tests/compat/compat_main.cpp, the pattern of the
    reference's main.cpp) writes the reference's BMP files byte for byte."""
    from h264_video_decoder_demo_gb300 import build
    path, meta = _golden(name)
    exe = str(tmp_path / "compat_main")
    lib_dir = os.path.dirname(build.LIB)
    subprocess.run(["g++", "-std=c++11", "-O1", "-I", os.path.join(ROOT, "include", "compat"),
                    os.path.join(HERE, "compat", "compat_main.cpp"), "-o", exe, "-L" + lib_dir, "-lh264r",
                    "-Wl,-rpath," + lib_dir], check=True)
    out = tmp_path / "bmp"
    out.mkdir()
    r = subprocess.run([exe, path, str(out)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    got = []
    for k in range(len(meta["frames"])):
        with open(out / ("out_1920x1088.%d.bmp" % k), "rb") as f:
            got.append(hashlib.md5(f.read()).hexdigest())
    assert got == [fr["bmp_md5"] for fr in meta["frames"]]
