"""The seeded bitstream writer (include/h264r_writer.h) against the reference.

tests/golden/writer_streams.json holds, for every case of
tests/golden/make_writer_fixtures.py, the writer's configuration, the md5 of
the stream it wrote and the reference decoder's own output for that stream
(every output picture's planes, and every picture before and after
deblocking).  Here, on the CPU:
  - the writer writes the same bytes again (deterministic on every host);
  - the front end (parser) plus the CPU oracle reproduce every output picture
    of the reference, in the reference's output order;
  - where the reference is built here (oracle/_ref), its records of the CIF
    streams equal the front end's, field by field;
  - configurations outside the writer's ranges are refused.
The whole bundled CAVLC streams (tests/golden/*_whole.h264) are checked the
same way, and the oracle is replayed against the reference's own dumps of all
five bundled streams (oracle/check_dump).
"""
import hashlib
import json
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DUMPER = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
CHECK = os.path.join(ROOT, "oracle", "check_dump")

with open(os.path.join(HERE, "golden", "writer_streams.json")) as _f:
    CASES = json.load(_f)["cases"]


def write(case):
    import h264_video_decoder_demo_gb300 as h
    cfg = dict(CASES[case]["writer"])
    seed = cfg.pop("seed")
    return h.write_stream(None, seed=seed, **cfg)


def oracle_frames(data):
    """(POC, md5) of every output picture: parser records reconstructed by
    the CPU oracle, in the parser's output order."""
    from h264_video_decoder_demo_gb300.engine import Parser
    from oracle_cpu import OracleDPB
    dpb, got = None, []
    for pic, info in Parser().pictures(data):
        if dpb is None:
            dpb = OracleDPB(pic.width_mbs, pic.height_mbs)
        rc, _ = dpb.reconstruct(pic)
        assert rc == 0
        for s, poc in zip(info["output_slots"], info["output_poc"]):
            got.append((int(poc), hashlib.md5(dpb.planes(int(s)).tobytes()).hexdigest()))
    return got


@pytest.mark.parametrize("case", sorted(CASES))
def test_writer_is_deterministic(engine_lib, case):
    data = write(case)
    assert len(data) == CASES[case]["stream_bytes"]
    assert hashlib.md5(data).hexdigest() == CASES[case]["stream_md5"]


@pytest.mark.parametrize("case", sorted(CASES))
def test_written_streams_reconstruct_to_reference_frames(engine_lib, case):
    got = oracle_frames(write(case))
    assert got == [(f["poc"], f["yuv_md5"]) for f in CASES[case]["frames"]]


@pytest.mark.parametrize("name", ["gop121_cavlc_whole", "heavyhand_cavlc_b4_whole"])
def test_whole_bundled_streams_reconstruct_to_reference_frames(engine_lib, name):
    with open(os.path.join(HERE, "golden", name + ".h264"), "rb") as f:
        data = f.read()
    with open(os.path.join(HERE, "golden", name + ".frames.json")) as f:
        meta = json.load(f)
    assert oracle_frames(data) == [(f["poc"], f["yuv_md5"]) for f in meta["frames"]]


def _reference_built():
    if not os.path.exists(DUMPER):
        pytest.skip("the reference is not built here (oracle/_ref)")


@pytest.mark.parametrize("case", [c for c in sorted(CASES) if c.startswith("cif")])
def test_written_records_match_reference(engine_lib, case, tmp_path):
    _reference_built()
    from h264_video_decoder_demo_gb300.engine import Parser
    from h264r_dump import read_dump
    from record_compare import compare_streams
    data = write(case)
    path, dmp = str(tmp_path / "s.h264"), str(tmp_path / "s.dmp")
    with open(path, "wb") as f:
        f.write(data)
    subprocess.run([DUMPER, path, dmp, "100000", "--no-planes"], stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL, check=True)
    ref = read_dump(dmp)
    mine = list(Parser().pictures(data))
    assert len(mine) == len(ref) + 1
    assert not compare_streams(ref, mine)


BUNDLED = ["gop121.naluCnt453.h264", "HeavyHand_1080p.B_frames.cabac.h264", "HeavyHand_1080p.B_frames_cabac_tff.h264",
           "HeavyHand_1080p.no_B_frames.cabac.no_tff.h264", "HeavyHand_1080p.B_frames_4.no_cabac.no_tff.h264"]


@pytest.mark.parametrize("stream", BUNDLED)
def test_oracle_replays_reference_dumps_of_bundled_streams(stream, tmp_path):
    """The first 16 pictures of every bundled stream (CABAC and CAVLC, IP, IBP,
    four B pictures, MBAFF, nine slices with a lost one): the reference's own
    records replayed through the oracle give the reference's planes before
    and after deblocking, each picture alone and all of them chained."""
    _reference_built()
    from conftest import reference_dir
    src = os.path.join(reference_dir(), "data", stream)
    if not os.path.exists(src):
        pytest.skip("reference streams not present")
    if not os.path.exists(CHECK):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "-s", "check_dump"])
    dmp = str(tmp_path / "s.dmp")
    subprocess.run([DUMPER, src, dmp, "16"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    assert os.path.getsize(dmp) > 0
    for mode in ([], ["--chain"]):
        r = subprocess.run([CHECK, dmp, "--quiet"] + mode, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert r.returncode == 0, r.stdout[-2000:]


@pytest.mark.parametrize("bad", [dict(width_mbs=0), dict(profile_idc=77), dict(num_refs=0), dict(qp_min=40, qp_max=30),
                                 dict(profile_idc=66, b_pictures=2), dict(mv_range=4096), dict(weighted=3)])
def test_writer_rejects_configurations_outside_its_ranges(engine_lib, bad):
    import h264_video_decoder_demo_gb300 as h
    from h264_video_decoder_demo_gb300.engine import EngineError
    with pytest.raises(EngineError) as e:
        h.write_stream("cif_ippp", seed=1, **bad)
    assert e.value.code == -1
