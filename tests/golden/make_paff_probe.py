"""Does the reference decode field pictures (PAFF)?  (tests/golden/paff_probe.json)

The reference allocates a field picture's frame buffer from the field's own
slice header (PicHeightInMbs = FrameHeightInMbs / 2,
H264SliceHeader.cpp:468, H264PictureBase.cpp:140-182), halves that height
again for the field views (H264PictureBase.cpp:205) and starts a fresh DPB
entry for the second field of a pair (H264VideoDecoder.cpp:107-131).  This
script measures what that does to a stream whose right answer is known
without any field-picture decoder:

  1. the library's writer writes an intra-only stream of HALF-height frames
     (High profile, CAVLC, Intra 4x4 / 8x8 / 16x16 / I_PCM, one slice);
  2. the stream is rewritten, headers only, into a field stream with the
     same slice data bits: every pair of half-height pictures becomes the top
     and the bottom field of one full-height frame (SPS frame_mbs_only_flag
     0 and mb_adaptive_frame_field_flag 0, so pic_height_in_map_units now
     counts field MB rows; slice headers with field_pic_flag 1,
     bottom_field_flag, frame_num and POC per field pair; header lengths kept
     modulo 8, so I_PCM alignment is unchanged).  An intra field picture
     decodes exactly like a frame of the field's size (8.3: neighbours, and
     so CAVLC nC and intra mode prediction, lie in the same field).  QP stays
     at 15 or below with zero filter offsets, so indexA < 16 and alpha is 0:
     the deblocking filter changes no sample in either stream (where the bS
     of field and frame MBs differ, it does not matter);
  3. the reference (oracle/_ref/ref_dump, built from its own sources) decodes
     the written stream and the field stream; the expected output of the field stream is every pair of decoded
     half-height frames interleaved line by line (top field on even lines).

Two cases: "intra" (Intra 4x4 / 8x8 / 16x16 and a few I_PCM MBs) and "pcm"
(every MB I_PCM, so that no neighbour is read and only where the reference
puts a field's samples counts).  paff_probe.json records, per case, the
reference's output for the field stream (exit status, first error message,
output POCs, md5 of every frame-sized output picture and its share of bytes
equal to the expected frame) next to the expected frames, and whether they
agree.

Usage: python tests/golden/make_paff_probe.py   (needs the reference sources)
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

WRITER = dict(width_mbs=22, height_mbs=9, num_pictures=8, profile_idc=100, gop_length=1, b_pictures=0,
              num_refs=1, transform8x8=1, weighted=0, min_partition=0, intra_percent=100, skip_percent=0,
              qp_min=10, qp_max=15, coef_density=40, slices=1, pcm_permille=20, chroma_qp_offset_max=0,
              filter_offset_max=0, mv_range=16)
SEED = 31


# ---------------------------------------------------------------- bits
def split_nals(data):
    """(nal header byte, RBSP bytes) of every NAL unit of an Annex B stream."""
    out, i, n = [], 0, len(data)
    starts = []
    while i + 3 <= n:
        if data[i] == 0 and data[i + 1] == 0 and data[i + 2] == 1:
            starts.append(i + 3)
            i += 3
        else:
            i += 1
    for k, s in enumerate(starts):
        e = starts[k + 1] - 3 if k + 1 < len(starts) else n
        while e > s and data[e - 1] == 0:
            e -= 1
        ebsp = data[s:e]
        rbsp, zeros = bytearray(), 0
        for b in ebsp[1:]:
            if zeros >= 2 and b == 3:
                zeros = 0
                continue
            rbsp.append(b)
            zeros = zeros + 1 if b == 0 else 0
        out.append((ebsp[0], bytes(rbsp)))
    return out


def join_nal(header, rbsp):
    out, zeros = bytearray(b"\x00\x00\x00\x01"), 0
    out.append(header)
    for b in rbsp:
        if zeros >= 2 and b <= 3:
            out.append(3)
            zeros = 0
        out.append(b)
        zeros = zeros + 1 if b == 0 else 0
    return bytes(out)


class Reader:
    def __init__(self, data):
        self.bits = "".join(format(b, "08b") for b in data)
        self.pos = 0

    def u(self, n):
        v = int(self.bits[self.pos:self.pos + n], 2) if n else 0
        self.pos += n
        return v

    def ue(self):
        z = 0
        while self.bits[self.pos + z] == "0":
            z += 1
        self.pos += z
        return self.u(z + 1) - 1

    def se(self):
        k = self.ue()
        return (k + 1) // 2 if k & 1 else -(k // 2)

    def rest(self):
        """The remaining bits up to (not including) rbsp_trailing_bits."""
        s = self.bits[self.pos:].rstrip("0")
        assert s.endswith("1")
        return s[:-1]


class Writer:
    def __init__(self):
        self.bits = []

    def u(self, n, v):
        if n:
            self.bits.append(format(v, "0%db" % n))

    def ue(self, v):
        b = format(v + 1, "b")
        self.bits.append("0" * (len(b) - 1) + b)

    def se(self, v):
        self.ue(2 * v - 1 if v > 0 else -2 * v)

    def raw(self, s):
        self.bits.append(s)

    def bytes(self):
        s = "".join(self.bits) + "1"  # rbsp_trailing_bits
        s += "0" * (-len(s) % 8)
        assert len(s) % 8 == 0, "RBSP not byte aligned"
        return bytes(int(s[i:i + 8], 2) for i in range(0, len(s), 8))


# ---------------------------------------------------------------- rewriting
def rewrite_sps(rbsp, fields):
    """The writer's High-profile SPS, with frame_mbs_only_flag 0,
    mb_adaptive_frame_field_flag 0 and a frame_num 2 bits shorter when fields
    is set.  Returns the RBSP and the written stream's frame_num and POC
    lengths."""
    r, w = Reader(rbsp), Writer()
    for n in (8, 8, 8):
        w.u(n, r.u(n))
    w.ue(r.ue())                      # seq_parameter_set_id
    w.ue(r.ue())                      # chroma_format_idc
    w.ue(r.ue())
    w.ue(r.ue())                      # bit depths
    w.u(1, r.u(1))                    # transform bypass
    assert r.u(1) == 0                # no scaling matrices
    w.u(1, 0)
    log2_fn = r.ue()
    w.ue(log2_fn - 2 if fields else log2_fn)
    assert r.ue() == 0                # pic_order_cnt_type 0
    w.ue(0)
    log2_poc = r.ue()
    w.ue(log2_poc)
    w.ue(r.ue())                      # max_num_ref_frames
    w.u(1, r.u(1))                    # gaps
    w.ue(r.ue())                      # pic_width_in_mbs_minus1
    w.ue(r.ue())                      # pic_height_in_map_units_minus1
    assert r.u(1) == 1                # frame_mbs_only_flag
    if fields:
        w.u(1, 0)
        w.u(1, 0)                     # mb_adaptive_frame_field_flag
    else:
        w.u(1, 1)
    w.raw(r.rest())
    return w.bytes(), log2_fn + 4, log2_poc + 4


def parse_slice_header(rbsp, nal_type, log2_fn, log2_poc):
    r = Reader(rbsp)
    h = dict(first_mb=r.ue(), slice_type=r.ue(), pps_id=r.ue(), frame_num=r.u(log2_fn))
    h["idr"] = nal_type == 5
    if h["idr"]:
        h["idr_pic_id"] = r.ue()
    h["poc_lsb"] = r.u(log2_poc)
    assert h["slice_type"] % 5 == 2, "intra-only streams"
    h["marking"] = [r.u(1), r.u(1)] if h["idr"] else [r.u(1)]
    assert h["idr"] or h["marking"] == [0]          # sliding window
    h["qp_delta"] = r.se()
    h["dbk"] = [r.ue()]
    if h["dbk"][0] != 1:
        h["dbk"] += [r.se(), r.se()]
    h["header_bits"] = r.pos
    h["data"] = r.rest()                             # slice data
    return h


def write_field_slice(h, log2_fn, log2_poc, pps_id, frame_num, poc_lsb, idr, bottom):
    """The slice as a field: field_pic_flag 1, bottom_field_flag, the field
    pair's frame_num and the field's POC; everything else as written.  The
    header keeps its length modulo 8 (pps_id pads it), so the slice data
    keeps its byte alignment (pcm_alignment_zero_bit): frame_num is 2 bits
    shorter than in the written stream, as long as the two flags."""
    w = Writer()
    w.ue(h["first_mb"])
    w.ue(h["slice_type"])
    w.ue(pps_id)
    w.u(log2_fn - 2, frame_num)
    w.u(1, 1)                         # field_pic_flag
    w.u(1, bottom)                    # bottom_field_flag
    if idr:
        w.ue(h["idr_pic_id"])
    w.u(log2_poc, poc_lsb)
    for b in (h["marking"] if idr else [0]):
        w.u(1, b)
    w.se(h["qp_delta"])
    w.ue(h["dbk"][0])
    for v in h["dbk"][1:]:
        w.se(v)
    assert (len("".join(w.bits)) - h["header_bits"]) % 8 == 0, "slice data would lose its alignment"
    w.raw(h["data"])
    return w.bytes()


def make_streams(data):
    """(the written stream, its field-picture version, pictures)."""
    fields = []
    log2_fn = log2_poc = None
    k = 0                             # picture index (one slice per picture)
    for hdr, rbsp in split_nals(data):
        t = hdr & 31
        if t == 7:
            b, log2_fn, log2_poc = rewrite_sps(rbsp, True)
            fields.append(join_nal(hdr, b))
        elif t == 8:
            fields.append(join_nal(hdr, rbsp))
        elif t in (1, 5):
            h = parse_slice_header(rbsp, t, log2_fn, log2_poc)
            assert h["first_mb"] == 0 and h["pps_id"] == 0
            j, bottom = k // 2, k & 1
            idr = k == 0
            nh = (hdr & 0x60) | (5 if idr else 1)
            fields.append(join_nal(nh, write_field_slice(h, log2_fn, log2_poc, 0, j, 4 * j + bottom, idr, bottom)))
            k += 1
    return data, b"".join(fields), k


def reference_decode(dumper, stream, tmp, name):
    path = os.path.join(tmp, name + ".h264")
    with open(path, "wb") as f:
        f.write(stream)
    yuv, order, dmp = (os.path.join(tmp, name + e) for e in (".yuv", ".order", ".dmp"))
    r = subprocess.run([dumper, path, dmp, "1000", "--no-planes", "--yuv", yuv, "--order", order],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
    raw = open(yuv, "rb").read() if os.path.exists(yuv) else b""
    pocs = [int(l.split()[1]) for l in open(order) if l.startswith("O ")] if os.path.exists(order) else []
    return r.returncode, r.stdout, raw, pocs


def md5(b):
    return hashlib.md5(b).hexdigest()


def first_error(log):
    for line in log.splitlines():
        if "rror" in line or "[ERR]" in line:
            return line.split("h264_video_decoder_demo/", 1)[-1].strip()
    return None


def probe(h, dumper, tmp, name, over):
    cfg = dict(WRITER, **over)
    data = h.write_stream(None, seed=SEED, **cfg)
    frames, fields, npics = make_streams(data)
    W, Hh = 16 * cfg["width_mbs"], 16 * cfg["height_mbs"]
    half = W * Hh * 3 // 2
    out = {"writer": dict(cfg, seed=SEED), "half_height_pictures": npics,
           "frames_stream_md5": md5(frames), "fields_stream_md5": md5(fields)}
    rc, log, raw, pocs = reference_decode(dumper, frames, tmp, name + "_frames")
    assert rc == 0 and len(raw) == half * npics, ("the half-height frames did not decode", rc, log)
    pics = [np.frombuffer(raw[i * half:(i + 1) * half], np.uint8) for i in range(npics)]
    expected = []
    for j in range(npics // 2):
        planes = []
        for (off, w, hh) in ((0, W, Hh), (W * Hh, W // 2, Hh // 2), (W * Hh * 5 // 4, W // 2, Hh // 2)):
            top = pics[2 * j][off:off + w * hh].reshape(hh, w)
            bot = pics[2 * j + 1][off:off + w * hh].reshape(hh, w)
            fr = np.empty((2 * hh, w), np.uint8)
            fr[0::2], fr[1::2] = top, bot
            planes.append(fr.tobytes())
        expected.append(b"".join(planes))
    out["expected_frames"] = [md5(e) for e in expected]
    rc, log, raw, pocs = reference_decode(dumper, fields, tmp, name + "_fields")
    full = 2 * half
    got = [raw[i * full:(i + 1) * full] for i in range(len(raw) // full)]
    lines = [l.strip() for l in log.splitlines() if l.strip()]
    out["reference"] = {"exit_status": rc, "first_error": first_error(log),
                        "last_line": lines[-1].split("h264_video_decoder_demo/", 1)[-1] if lines else None,
                        "output_pocs": pocs,
                        "output_bytes": len(raw), "frame_md5s": [md5(g) for g in got]}
    out["reference"]["equal_byte_share"] = [
        round(float(np.mean(np.frombuffer(g, np.uint8) == np.frombuffer(e, np.uint8))), 4)
        for g, e in zip(got, expected)]
    out["reference_equals_expected"] = len(got) == len(expected) and all(a == b for a, b in zip(got, expected))
    return out


# intra: Intra 4x4 / 8x8 / 16x16 and a few I_PCM MBs (CAVLC contexts and
# intra prediction from neighbours in the field); pcm: every MB I_PCM (no
# neighbour is read: only the field's placement in the frame buffer counts)
CASES = {"intra": {}, "pcm": dict(pcm_permille=1000)}


def main():
    import h264_video_decoder_demo_gb300 as h
    dumper = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
    if not os.path.exists(dumper):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref"])
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, over in CASES.items():
            out[name] = probe(h, dumper, tmp, name, over)
    with open(os.path.join(HERE, "paff_probe.json"), "w") as f:
        json.dump(out, f, indent=1)
    for name, r in out.items():
        print(name, json.dumps(r["reference"]), "equal:", r["reference_equals_expected"])


if __name__ == "__main__":
    main()
