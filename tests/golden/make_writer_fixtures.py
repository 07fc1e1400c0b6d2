"""Reference outputs of the seeded writer's streams (tests/golden/writer_streams.json).

Each case is a configuration of the library's bitstream writer
(include/h264r_writer.h, h264_video_decoder_demo_gb300.write_stream): the
benchmark configurations and variants that reach the constructs no bundled
stream has (explicit bi-predictive weights, motion vectors past the picture
edges, P sub-partitions down to 4x4, I_PCM, non-IDR I pictures, several
slices, implicit weights with three B pictures, CAVLC MBAFF frames).  For every case the script
writes the stream, decodes it with the unmodified reference decoder
(oracle/_ref/ref_dump, built from the reference's own sources by
`make -C oracle ref`) and records:

  writer          the configuration and seed (the tests write the stream again)
  stream_md5      md5 of the written bytes (the writer is deterministic)
  frames          every picture the reference outputs, in output order: POC and
                  md5 of its planes at coded size
  pictures        every picture the reference deblocks, in decoding order: POC
                  and md5 of its planes before and after deblocking

Usage: python tests/golden/make_writer_fixtures.py
Needs the reference sources; the fixture is committed.
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from h264r_dump import read_dump  # noqa: E402

# (case, named writer configuration, seed, overrides)
CASES = [
    # the CPU-runnable configuration as specified: CIF IPPP, Baseline CAVLC
    ("cif_ippp", "cif_ippp", 1, {}),
    # CIF, 20 pictures, two slices per picture, I_PCM MBs
    ("cif_ippp_2slices_pcm", "cif_ippp", 12, dict(num_pictures=20, slices=2, pcm_permille=50)),
    # the 1080p High configuration in CAVLC: IBBP, explicit bi-predictive
    # weights, 4 references, P sub-partitions to 4x4, 5% MVs past the edges
    # (seed 1000: stream 0 of the benchmark)
    ("1080p_high", "1080p_high", 1000, {}),
    # non-IDR I pictures every 5 pictures and three slices per picture
    ("1080p_high_gop5_3slices", "1080p_high", 4, dict(num_pictures=12, gop_length=5, slices=3)),
    # implicit bi-predictive weights, three B pictures between anchors
    ("1080p_implicit_b3", "1080p_high", 5, dict(num_pictures=16, weighted=2, b_pictures=3)),
    # no weighted prediction, one B picture, two references
    ("1080p_default_wp_b1", "1080p_high", 6, dict(num_pictures=16, weighted=0, b_pictures=1, num_refs=2)),
    # MBAFF frames (the MBAFF half of the interlaced configuration): half the
    # MB pairs field pairs, IBP, two references
    ("1080i_mbaff", "1080i_mbaff", 7, dict(num_pictures=12)),
    # MBAFF with explicit bi-predictive weights and four references
    ("1080i_mbaff_explicit", "1080p_high", 8, dict(num_pictures=8, mbaff=1, field_percent=60)),
    # CIF MBAFF, High, two slices, I_PCM
    ("cif_mbaff_2slices_pcm", "cif_ippp", 9, dict(profile_idc=100, mbaff=1, field_percent=50, num_pictures=10,
                                                  slices=2, pcm_permille=50)),
]


def md5(b):
    return hashlib.md5(b).hexdigest()


def main():
    import h264_video_decoder_demo_gb300 as h
    from h264_video_decoder_demo_gb300.engine import STREAMS
    dumper = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
    if not os.path.exists(dumper):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref"])
    out = {"cases": {}}
    with tempfile.TemporaryDirectory() as tmp:
        for name, preset, seed, over in CASES:
            cfg = dict(STREAMS[preset])
            cfg.update(over)
            data = h.write_stream(None, seed=seed, **cfg)
            path = os.path.join(tmp, name + ".h264")
            with open(path, "wb") as f:
                f.write(data)
            dmp, yuv, order = (os.path.join(tmp, name + ext) for ext in (".dmp", ".yuv", ".order"))
            r = subprocess.run([dumper, path, dmp, "1000000", "--yuv", yuv, "--order", order],
                               stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            if r.returncode != 0:
                raise RuntimeError("the reference failed on %s (status %d)" % (name, r.returncode))
            pics = read_dump(dmp)
            pocs = [int(l.split()[1]) for l in open(order) if l.startswith("O ")]
            frame = cfg["width_mbs"] * cfg["height_mbs"] * 384
            with open(yuv, "rb") as f:
                raw = f.read()
            assert len(raw) == frame * len(pocs) == frame * cfg["num_pictures"], (name, len(raw), len(pocs))
            out["cases"][name] = {
                "writer": dict(cfg, seed=seed), "stream_md5": md5(data), "stream_bytes": len(data),
                "frames": [{"poc": p, "yuv_md5": md5(raw[k * frame:(k + 1) * frame])} for k, p in enumerate(pocs)],
                "pictures": [{"poc": p.poc, "pre_md5": md5(p.pre.tobytes()), "post_md5": md5(p.post.tobytes())}
                             for p in pics],
            }
            print(name, len(data), "bytes,", len(pocs), "frames,", len(pics), "pictures deblocked")
            os.remove(dmp)
    with open(os.path.join(HERE, "writer_streams.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
