"""Generate the golden fixtures in tests/golden from the reference decoder.

Runs oracle/_ref/ref_dump (the unmodified reference, built from its own
sources by `make -C oracle ref`) on the reference's bundled streams and keeps
the first pictures of each stream, in decoding order from the IDR:

  <name>.h264r.gz   records of those pictures (dump container, no planes)
  <name>.json       md5 of the reference's pre- and post-deblocking planes,
                    and of the BMP file the reference writes for each picture
                    (CH264PictureBase::saveToBmpFile: YUV420P -> BGR24 -> BMP)

Usage: python tests/golden/make_fixtures.py [--ref-data DIR]
The fixtures are committed; this script needs the reference sources and is
only run where they are present.
"""
import argparse
import gzip
import hashlib
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
from h264r_dump import read_dump, write_dump  # noqa: E402

# (fixture name, stream file, pictures kept, coding tools covered)
FIXTURES = [
    ("gop121_baseline_multislice", "gop121.naluCnt453.h264", 3,
     "Baseline CAVLC, 9 slices/picture, a lost slice (undecoded MBs), P"),
    ("heavyhand_cabac_ibp_implicit", "HeavyHand_1080p.B_frames.cabac.h264", 4,
     "High CABAC, 8x8 transform, B pictures, implicit weights, explicit P weights"),
    ("heavyhand_cabac_mbaff_tff", "HeavyHand_1080p.B_frames_cabac_tff.h264", 3,
     "High CABAC, MBAFF frame/field MB pairs, B pictures"),
    ("heavyhand_cabac_p_explicit", "HeavyHand_1080p.no_B_frames.cabac.no_tff.h264", 2,
     "High CABAC, explicit weighted P prediction"),
]


def md5(a):
    return hashlib.md5(a.tobytes()).hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-data", default="/root/reference/data")
    args = ap.parse_args()
    dumper = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
    if not os.path.exists(dumper):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref"])
    with tempfile.TemporaryDirectory(dir=os.path.join(ROOT, "_work") if os.path.isdir(os.path.join(ROOT, "_work")) else None) as tmp:
        for name, stream, n, tools in FIXTURES:
            dmp = os.path.join(tmp, name + ".dmp")
            bmp_dir = os.path.join(tmp, name + "_bmp")
            os.makedirs(bmp_dir)
            subprocess.run([dumper, os.path.join(args.ref_data, stream), dmp, str(n), "--bmp", bmp_dir],
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, check=True)
            pics = read_dump(dmp)
            meta = {"stream": stream, "coding_tools": tools, "pictures": []}
            for i, p in enumerate(pics):
                with open(os.path.join(bmp_dir, "pic_%03d.bmp" % i), "rb") as f:
                    bmp_md5 = hashlib.md5(f.read()).hexdigest()
                meta["pictures"].append({"poc": p.poc, "dst_slot": p.dst_slot, "mbaff": p.mbaff,
                                         "pre_md5": md5(p.pre), "post_md5": md5(p.post), "bmp_md5": bmp_md5})
            raw = os.path.join(tmp, name + ".raw")
            write_dump(raw, pics, planes=False)
            with open(raw, "rb") as f, gzip.open(os.path.join(HERE, name + ".h264r.gz"), "wb", 9) as g:
                g.write(f.read())
            with open(os.path.join(HERE, name + ".json"), "w") as f:
                json.dump(meta, f, indent=1)
            print(name, len(pics), "pictures")


if __name__ == "__main__":
    main()
