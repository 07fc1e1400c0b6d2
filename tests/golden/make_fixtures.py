"""Generate the golden fixtures in tests/golden from the reference decoder.

Runs oracle/_ref/ref_dump (the unmodified reference, built from its own
sources by `make -C oracle ref`) on the reference's bundled streams and keeps
the first pictures of each stream, in decoding order from the IDR:

  <name>.h264r.gz   records of those pictures (dump container, no planes)
  <name>.json       md5 of the reference's pre- and post-deblocking planes,
                    and of the BMP file the reference writes for each picture
                    (CH264PictureBase::saveToBmpFile: YUV420P -> BGR24 -> BMP)

  output_order.json for every bundled stream: the pictures in decoding order
                    as the reference completes them (POC, IdrPicFlag, reorder
                    depth of the SPS) and the POCs in the order its output
                    callback receives them

  <name>.h264       for the two CAVLC, the two frame-coded CABAC and the MBAFF CABAC streams: the stream cut before the first
                    slice of picture N (parameter sets included), and each
                    stream whole, with
  <name>.frames.json  every picture the reference outputs for that cut stream,
                    in output order: POC, md5 of its planes (ref_dump --yuv) and
                    md5 of the BMP the reference's own main.cpp writes for it
                    (oracle/_ref/h264dec)

Usage: python tests/golden/make_fixtures.py [--ref-data DIR] [--bitstreams-only]
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
from conftest import reference_dir  # noqa: E402
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


ORDER_STREAMS = ["gop121.naluCnt453.h264", "HeavyHand_1080p.B_frames.cabac.h264",
                 "HeavyHand_1080p.B_frames_cabac_tff.h264", "HeavyHand_1080p.no_B_frames.cabac.no_tff.h264",
                 "HeavyHand_1080p.B_frames_4.no_cabac.no_tff.h264"]


def make_order_fixture(dumper, ref_data, tmp):
    """Decoding and output order of whole streams.  The reference completes
    every picture but the last through its deblocking call (where the dumper
    records it); the last one is output without deblocking, so its POC is the
    one output that was never recorded in decoding order."""
    procs = []
    for stream in ORDER_STREAMS:
        path = os.path.join(tmp, stream + ".order")
        procs.append((stream, path, subprocess.Popen(
            [dumper, os.path.join(ref_data, stream), os.devnull, "1000000", "--no-planes", "--order", path],
            stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)))
    fixture = {}
    for stream, path, p in procs:
        if p.wait() != 0:
            raise RuntimeError("ref_dump failed on " + stream)
        decoded, output = [], []
        depth = None
        with open(path) as f:
            for line in f:
                kind, *vals = line.split()
                if kind == "D":
                    decoded.append([int(vals[0]), int(vals[1])])
                    depth = int(vals[2])
                elif kind == "O":
                    output.append(int(vals[0]))
        # POCs restart at every IDR picture: compare as multisets
        from collections import Counter
        last = list((Counter(output) - Counter(poc for poc, _ in decoded)).elements())
        assert len(last) == 1, (stream, last)
        decoded.append([last[0], 0])
        fixture[stream] = {"max_num_reorder_frames": depth, "decoded": decoded, "output": output}
    with open(os.path.join(HERE, "output_order.json"), "w") as f:
        json.dump(fixture, f)
    print("output_order.json:", {k: len(v["output"]) for k, v in fixture.items()})


# (fixture name, stream file, pictures kept)
BITSTREAMS = [
    ("gop121_cavlc_4pics", "gop121.naluCnt453.h264", 4),
    ("heavyhand_cavlc_b4_6pics", "HeavyHand_1080p.B_frames_4.no_cabac.no_tff.h264", 6),
    ("heavyhand_cabac_p_6pics", "HeavyHand_1080p.no_B_frames.cabac.no_tff.h264", 6),
    ("heavyhand_cabac_ibp_6pics", "HeavyHand_1080p.B_frames.cabac.h264", 6),
    ("heavyhand_cabac_mbaff_6pics", "HeavyHand_1080p.B_frames_cabac_tff.h264", 6),
    # the two CAVLC streams whole (50 and 76 pictures)
    ("gop121_cavlc_whole", "gop121.naluCnt453.h264", 1 << 20),
    ("heavyhand_cavlc_b4_whole", "HeavyHand_1080p.B_frames_4.no_cabac.no_tff.h264", 1 << 20),
]


def cut_stream(data, pictures):
    """The bytes before the start code of the first slice of picture `pictures`."""
    i, n = 0, 0
    while True:
        j = data.find(b"\x00\x00\x01", i)
        if j < 0:
            return data
        t = data[j + 3] & 31
        if t in (1, 5) and (data[j + 4] & 0x80):  # first_mb_in_slice == 0
            if n == pictures:
                while j > 0 and data[j - 1] == 0:  # the start code's zero_byte
                    j -= 1
                return data[:j]
            n += 1
        i = j + 3


def make_bitstream_fixtures(ref_data, tmp):
    dumper = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
    h264dec = os.path.join(ROOT, "oracle", "_ref", "h264dec")
    for name, stream, n in BITSTREAMS:
        with open(os.path.join(ref_data, stream), "rb") as f:
            cut = cut_stream(f.read(), n)
        path = os.path.join(HERE, name + ".h264")
        with open(path, "wb") as f:
            f.write(cut)
        yuv = os.path.join(tmp, name + ".yuv")
        order = os.path.join(tmp, name + ".order")
        subprocess.run([dumper, path, os.path.join(tmp, name + ".dmp"), "100000", "--no-planes", "--yuv", yuv,
                        "--order", order], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, check=True)
        bmp_dir = os.path.join(tmp, name + "_bmp")
        os.makedirs(bmp_dir)
        subprocess.run([h264dec, path, bmp_dir], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        pocs = [int(l.split()[1]) for l in open(order) if l.startswith("O ")]
        with open(yuv, "rb") as f:
            raw = f.read()
        frame = 1920 * 1088 * 3 // 2
        assert len(raw) == frame * len(pocs), (len(raw), len(pocs))
        frames = []
        for k, poc in enumerate(pocs):
            with open(os.path.join(bmp_dir, "out_1920x1088.%d.bmp" % k), "rb") as f:
                bmp = hashlib.md5(f.read()).hexdigest()
            frames.append({"poc": poc, "yuv_md5": hashlib.md5(raw[k * frame:(k + 1) * frame]).hexdigest(),
                           "bmp_md5": bmp})
        decoded = sum(1 for l in open(order) if l.startswith("D "))
        with open(os.path.join(HERE, name + ".frames.json"), "w") as f:
            # pictures: decoded pictures (the last one is output without
            # deblocking and not in the decoding-order lines)
            json.dump({"stream": stream, "pictures": min(n, decoded + 1), "width": 1920, "height": 1088,
                       "frames": frames}, f, indent=1)
        print(name, len(cut), "bytes", len(frames), "frames")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-data", default=os.path.join(reference_dir(), "data"))
    ap.add_argument("--bitstreams-only", action="store_true", help="only the cut streams and their frame md5s")
    args = ap.parse_args()
    dumper = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
    if not os.path.exists(dumper):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref"])
    with tempfile.TemporaryDirectory() as tmp:
        for name, stream, n, tools in ([] if args.bitstreams_only else FIXTURES):
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
        if not args.bitstreams_only:
            make_order_fixture(dumper, args.ref_data, tmp)
        make_bitstream_fixtures(args.ref_data, tmp)


if __name__ == "__main__":
    main()
