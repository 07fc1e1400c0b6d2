"""Reader/writer for the record dump container (oracle/dumpfmt.h) and numpy
views of the record structures declared in include/h264r.h.

Test infrastructure: used by the fixture generator, the CPU tests and the GPU
parity tests.
"""
import os
import struct
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from h264_video_decoder_demo_gb300.records import MB_DTYPE, PART_DTYPE, SLICE_DTYPE, WEIGHT_DTYPE  # noqa: E402

MAGIC = b"H264RDMP"
PIC_TAG = 0x31434950
# h264r_dump_pic without the scaling lists: tag, w, h, structure, mbaff,
# dst_slot, deblock, num_slices, num_weights, num_mbs, motion_bytes,
# coef_bytes, num_pcm, [scaling 96 + 384], poc, pic_num_cnt, flags, plane_bytes
_HDR1 = struct.Struct("<IHHBBBBHHIIII")
_HDR2 = struct.Struct("<iiII")
HDR_SIZE = _HDR1.size + 96 + 384 + _HDR2.size
HAS_PRE, HAS_POST = 1, 2


from h264_video_decoder_demo_gb300.records import Picture as _RecPicture  # noqa: E402


class Picture(_RecPicture):
    """Records of one picture plus the dump's reference planes."""

    def __init__(self):
        super().__init__()
        self.poc = self.pic_num_cnt = 0
        self.pre = None
        self.post = None


def read_dump(path, max_pictures=None):
    import gzip
    pics = []
    opener = gzip.open if path.endswith(".gz") else open
    with opener(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError("not a record dump")
        f.read(8)
        while max_pictures is None or len(pics) < max_pictures:
            raw = f.read(HDR_SIZE)
            if len(raw) < HDR_SIZE:
                break
            (tag, w, h, structure, mbaff, slot, deblock, nsl, nwt, nmb, mbytes, cbytes,
             npcm) = _HDR1.unpack_from(raw, 0)
            if tag != PIC_TAG:
                raise ValueError("corrupt dump")
            p = Picture()
            p.width_mbs, p.height_mbs, p.structure, p.mbaff = w, h, structure, mbaff
            p.dst_slot, p.deblock = slot, deblock
            o = _HDR1.size
            p.scaling4x4 = np.frombuffer(raw, np.uint8, 96, o).reshape(6, 16).copy()
            p.scaling8x8 = np.frombuffer(raw, np.uint8, 384, o + 96).reshape(6, 64).copy()
            p.poc, p.pic_num_cnt, flags, plane_bytes = _HDR2.unpack_from(raw, o + 480)
            p.mbs = np.frombuffer(f.read(32 * nmb), MB_DTYPE).copy()
            p.slices = np.frombuffer(f.read(8 * nsl), SLICE_DTYPE).copy()
            p.weights = np.frombuffer(f.read(32 * nwt), WEIGHT_DTYPE).copy()
            p.motion = np.frombuffer(f.read(mbytes), np.uint8).copy()
            p.coef = np.frombuffer(f.read(cbytes), np.uint8).copy()
            p.pcm = np.frombuffer(f.read(384 * npcm), np.uint8).copy()
            if flags & HAS_PRE:
                p.pre = np.frombuffer(f.read(plane_bytes), np.uint8).copy()
            if flags & HAS_POST:
                p.post = np.frombuffer(f.read(plane_bytes), np.uint8).copy()
            pics.append(p)
    return pics


def write_dump(path, pics, planes=True):
    with open(path, "wb") as f:
        f.write(MAGIC + struct.pack("<II", 1, 0))
        for p in pics:
            flags = 0
            if planes and p.pre is not None:
                flags |= HAS_PRE
            if planes and p.post is not None:
                flags |= HAS_POST
            f.write(_HDR1.pack(PIC_TAG, p.width_mbs, p.height_mbs, p.structure, p.mbaff,
                               p.dst_slot, p.deblock, len(p.slices), len(p.weights),
                               len(p.mbs), len(p.motion), len(p.coef), len(p.pcm) // 384))
            f.write(np.ascontiguousarray(p.scaling4x4, np.uint8).tobytes())
            f.write(np.ascontiguousarray(p.scaling8x8, np.uint8).tobytes())
            f.write(_HDR2.pack(p.poc, p.pic_num_cnt, flags, p.plane_bytes))
            for a in (p.mbs, p.slices, p.weights, p.motion, p.coef, p.pcm):
                f.write(np.ascontiguousarray(a).tobytes())
            if flags & HAS_PRE:
                f.write(p.pre.tobytes())
            if flags & HAS_POST:
                f.write(p.post.tobytes())
