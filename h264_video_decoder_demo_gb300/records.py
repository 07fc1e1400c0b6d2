"""numpy views of the reconstruction records declared in include/h264r.h and
their ctypes mirror.  A Picture holds one decoded picture's records in host
memory; Picture.to_c() returns the h264r_picture the C ABI takes.
"""
import ctypes

import numpy as np

MB_DTYPE = np.dtype([
    ("type", "u1"), ("flags", "u1"), ("qpy", "u1"), ("i16_mode", "u1"),
    ("chroma_mode", "u1"), ("nz8x8", "u1"), ("nz4x4", "<u2"), ("slice", "<u2"),
    ("reserved", "<u2"), ("ipred", "<u4", (2,)), ("coef", "<u4"), ("aux", "<u4"),
    ("reserved2", "<u4")])
SLICE_DTYPE = np.dtype([
    ("chroma_qp_offset", "i1", (2,)), ("filter_offset_a", "i1"), ("filter_offset_b", "i1"),
    ("disable_deblocking_filter_idc", "u1"), ("slice_type", "u1"), ("reserved", "u1", (2,))])
WEIGHT_DTYPE = np.dtype([
    ("weighted", "i1"), ("log_wd", "i1", (3,)), ("w0", "<i2", (3,)), ("w1", "<i2", (3,)),
    ("o0", "<i2", (3,)), ("o1", "<i2", (3,)), ("reserved", "<i2", (2,))])
PART_DTYPE = np.dtype([
    ("mv", "<i2", (2, 2)), ("ref", "i1", (2,)), ("dref", "i1", (2,)), ("wt", "<u2"),
    ("reserved", "<u2")])
assert MB_DTYPE.itemsize == 32 and SLICE_DTYPE.itemsize == 8
assert WEIGHT_DTYPE.itemsize == 32 and PART_DTYPE.itemsize == 16

MB_INTER, MB_I4x4, MB_I8x8, MB_I16x16, MB_IPCM, MB_NONE = range(6)
MBF_T8x8, MBF_FIELD, MBF_CIP = 1, 2, 4
NONE32 = 0xFFFFFFFF

# error codes (include/h264r.h)
OK = 0
ERR_INVALID_ARG, ERR_BAD_RECORD, ERR_UNSUPPORTED, ERR_CUDA = -1, -2, -3, -4
ERR_NO_MEMORY, ERR_BUDGET, ERR_DEVICE_TIMEOUT, ERR_BUSY = -5, -6, -7, -8
ERR_TOO_LARGE, ERR_IO = -9, -10


class CPicture(ctypes.Structure):
    """struct h264r_picture"""
    _fields_ = [("width_mbs", ctypes.c_uint16), ("height_mbs", ctypes.c_uint16),
                ("structure", ctypes.c_uint8), ("mbaff", ctypes.c_uint8),
                ("dst_slot", ctypes.c_uint8), ("deblock", ctypes.c_uint8),
                ("num_slices", ctypes.c_uint16), ("num_weights", ctypes.c_uint16),
                ("num_mbs", ctypes.c_uint32), ("motion_bytes", ctypes.c_uint32),
                ("coef_bytes", ctypes.c_uint32), ("num_pcm", ctypes.c_uint32),
                ("scaling4x4", ctypes.c_uint8 * 96), ("scaling8x8", ctypes.c_uint8 * 384),
                ("mbs", ctypes.c_void_p), ("slices", ctypes.c_void_p),
                ("weights", ctypes.c_void_p), ("motion", ctypes.c_void_p),
                ("coef", ctypes.c_void_p), ("pcm", ctypes.c_void_p)]



class CParsed(ctypes.Structure):
    """struct h264r_parsed (include/h264r_parser.h)"""
    _fields_ = [("pic", CPicture), ("poc", ctypes.c_int32), ("index", ctypes.c_uint32),
                ("idr", ctypes.c_uint8), ("reference", ctypes.c_uint8), ("slice_type", ctypes.c_uint8),
                ("reserved", ctypes.c_uint8), ("num_output", ctypes.c_uint32),
                ("output_slots", ctypes.c_void_p), ("output_poc", ctypes.c_void_p),
                ("output_index", ctypes.c_void_p)]



class CFrame(ctypes.Structure):
    """struct h264r_frame (include/h264r_decoder.h)"""
    _fields_ = [("y", ctypes.c_void_p), ("cb", ctypes.c_void_p), ("cr", ctypes.c_void_p),
                ("width", ctypes.c_int32), ("height", ctypes.c_int32), ("poc", ctypes.c_int32),
                ("output_count", ctypes.c_int32), ("decode_index", ctypes.c_uint32),
                ("slice_type", ctypes.c_uint8), ("reserved", ctypes.c_uint8 * 3),
                ("slot", ctypes.c_int32), ("stream", ctypes.c_void_p)]


FRAME_CALLBACK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(CFrame), ctypes.c_void_p, ctypes.c_int)


class Picture:
    """One picture's records in host memory (numpy arrays)."""

    _ARRAYS = ("mbs", "slices", "weights", "motion", "coef", "pcm")

    def __init__(self):
        self.width_mbs = self.height_mbs = 0
        self.structure = self.mbaff = self.dst_slot = 0
        self.deblock = 1
        self.scaling4x4 = np.full((6, 16), 16, np.uint8)
        self.scaling8x8 = np.full((6, 64), 16, np.uint8)
        self.mbs = np.zeros(0, MB_DTYPE)
        self.slices = np.zeros(0, SLICE_DTYPE)
        self.weights = np.zeros(1, WEIGHT_DTYPE)
        self.motion = np.zeros(0, np.uint8)
        self.coef = np.zeros(0, np.uint8)
        self.pcm = np.zeros(0, np.uint8)

    @property
    def plane_bytes(self):
        return self.width_mbs * self.height_mbs * 384

    @property
    def record_bytes(self):
        return sum(np.asarray(getattr(self, a)).nbytes for a in self._ARRAYS)

    def to_c(self):
        """ctypes h264r_picture pointing at this object's arrays (host memory).
        The arrays must stay alive while the struct is used."""
        c = CPicture()
        c.width_mbs, c.height_mbs = self.width_mbs, self.height_mbs
        c.structure, c.mbaff, c.dst_slot, c.deblock = self.structure, self.mbaff, self.dst_slot, self.deblock
        c.num_slices, c.num_weights, c.num_mbs = len(self.slices), len(self.weights), len(self.mbs)
        c.motion_bytes, c.coef_bytes, c.num_pcm = len(self.motion), len(self.coef), len(self.pcm) // 384
        ctypes.memmove(c.scaling4x4, np.ascontiguousarray(self.scaling4x4, np.uint8).tobytes(), 96)
        ctypes.memmove(c.scaling8x8, np.ascontiguousarray(self.scaling8x8, np.uint8).tobytes(), 384)
        for name in self._ARRAYS:
            a = getattr(self, name)
            if not a.flags["C_CONTIGUOUS"]:
                a = np.ascontiguousarray(a)
                setattr(self, name, a)
            setattr(c, name, a.ctypes.data if a.size else None)
        return c

    def ref_slots(self):
        """DPB slots the picture's inter partitions read (motion payload)."""
        inter = np.nonzero(self.mbs["type"] == MB_INTER)[0]
        if len(inter) == 0:
            return set()
        raw = np.ascontiguousarray(self.motion).view(np.uint8)
        aux = self.mbs["aux"][inter].astype(np.int64)
        cnt = raw[aux[:, None] + np.array([2, 3])].astype(np.int64)
        cnt = cnt[:, 0] | (cnt[:, 1] << 8)
        first = np.repeat(aux + 4, cnt) + 16 * (np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt))
        refs = raw[first[:, None] + np.array([8, 9])].view(np.int8).reshape(-1)
        return set(int(r) & 31 for r in np.unique(refs[refs >= 0]))

    @classmethod
    def from_c(cls, c):
        """Copy an h264r_picture with host pointers into numpy arrays."""
        p = cls()
        p.width_mbs, p.height_mbs = c.width_mbs, c.height_mbs
        p.structure, p.mbaff, p.dst_slot, p.deblock = c.structure, c.mbaff, c.dst_slot, c.deblock
        p.scaling4x4 = np.frombuffer(bytes(c.scaling4x4), np.uint8).reshape(6, 16).copy()
        p.scaling8x8 = np.frombuffer(bytes(c.scaling8x8), np.uint8).reshape(6, 64).copy()

        def grab(ptr, n, dtype):
            if n == 0 or not ptr:
                return np.zeros(0, dtype)
            buf = (ctypes.c_uint8 * (n * np.dtype(dtype).itemsize)).from_address(ptr)
            return np.frombuffer(bytes(buf), dtype).copy()

        p.mbs = grab(c.mbs, c.num_mbs, MB_DTYPE)
        p.slices = grab(c.slices, c.num_slices, SLICE_DTYPE)
        p.weights = grab(c.weights, c.num_weights, WEIGHT_DTYPE)
        p.motion = grab(c.motion, c.motion_bytes, np.uint8)
        p.coef = grab(c.coef, c.coef_bytes, np.uint8)
        p.pcm = grab(c.pcm, c.num_pcm * 384, np.uint8)
        return p

    def parts(self, addr):
        """(shape, parts) of an inter MB's motion payload."""
        off = int(self.mbs[addr]["aux"])
        raw = self.motion.tobytes()
        shape, count = np.frombuffer(raw, "<u2", 2, off)
        return int(shape), np.frombuffer(raw, PART_DTYPE, int(count), off + 4)


class CStreamCfg(ctypes.Structure):
    _fields_ = [("width_mbs", ctypes.c_uint16), ("height_mbs", ctypes.c_uint16),
                ("dpb_slots", ctypes.c_uint16), ("reserved", ctypes.c_uint16)]


class CCfg(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("dpb_budget_bytes", ctypes.c_uint64),
                ("max_batch_pictures", ctypes.c_uint32), ("flags", ctypes.c_uint32)]


class CTuning(ctypes.Structure):
    """struct h264r_tuning (include/h264r.h): launch shapes and graph replay"""
    _fields_ = [("inter_mbs_per_cta", ctypes.c_int32), ("deblock_pairs_per_cta", ctypes.c_int32),
                ("graphs", ctypes.c_int32), ("reserved", ctypes.c_int32)]

    def as_dict(self):
        return {"inter_mbs_per_cta": self.inter_mbs_per_cta,
                "deblock_pairs_per_cta": self.deblock_pairs_per_cta, "graphs": self.graphs}


class CSynthCfg(ctypes.Structure):
    """struct h264r_synth_cfg (include/h264r_synth.h)"""
    _fields_ = [("seed", ctypes.c_uint32), ("width_mbs", ctypes.c_uint16),
                ("height_mbs", ctypes.c_uint16), ("num_pictures", ctypes.c_uint16),
                ("gop_length", ctypes.c_uint16), ("gop_kind", ctypes.c_uint8),
                ("num_refs", ctypes.c_uint8), ("transform8x8", ctypes.c_uint8),
                ("weighted", ctypes.c_uint8), ("min_partition", ctypes.c_uint8),
                ("intra_percent", ctypes.c_uint8), ("skip_percent", ctypes.c_uint8),
                ("qp_min", ctypes.c_uint8), ("qp_max", ctypes.c_uint8),
                ("edge_mv_percent", ctypes.c_uint8), ("mv_range", ctypes.c_int16),
                ("filter_offset_max", ctypes.c_int8), ("coef_density", ctypes.c_uint8),
                ("mbaff", ctypes.c_uint8), ("field_percent", ctypes.c_uint8),
                ("slice_rows", ctypes.c_uint8), ("cip_percent", ctypes.c_uint8),
                ("paff_percent", ctypes.c_uint8)]


class CWriterCfg(ctypes.Structure):
    """struct h264r_writer_cfg (include/h264r_writer.h)"""
    _fields_ = [("seed", ctypes.c_uint32), ("width_mbs", ctypes.c_uint16), ("height_mbs", ctypes.c_uint16),
                ("num_pictures", ctypes.c_uint16), ("profile_idc", ctypes.c_uint8), ("level_idc", ctypes.c_uint8),
                ("gop_length", ctypes.c_uint8), ("b_pictures", ctypes.c_uint8), ("num_refs", ctypes.c_uint8),
                ("transform8x8", ctypes.c_uint8), ("weighted", ctypes.c_uint8), ("direct_spatial", ctypes.c_uint8),
                ("min_partition", ctypes.c_uint8), ("intra_percent", ctypes.c_uint8),
                ("skip_percent", ctypes.c_uint8), ("edge_mv_percent", ctypes.c_uint8), ("qp_min", ctypes.c_uint8),
                ("qp_max", ctypes.c_uint8), ("filter_offset_max", ctypes.c_uint8), ("coef_density", ctypes.c_uint8),
                ("slices", ctypes.c_uint8), ("pcm_permille", ctypes.c_uint8),
                ("chroma_qp_offset_max", ctypes.c_uint8), ("mbaff", ctypes.c_uint8), ("field_percent", ctypes.c_uint8),
                ("reserved", ctypes.c_uint8),
                ("mv_range", ctypes.c_uint16), ("reserved2", ctypes.c_uint16)]


class CServerCfg(ctypes.Structure):
    """struct h264r_server_cfg (include/h264r_server.h)"""
    _fields_ = [("max_batch_pictures", ctypes.c_uint32), ("queue_depth", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("lanes", ctypes.c_uint32)]


class CServerDone(ctypes.Structure):
    """struct h264r_server_done"""
    _fields_ = [("stream", ctypes.c_int32), ("status", ctypes.c_int32), ("tag", ctypes.c_uint64),
                ("latency_ms", ctypes.c_double)]


class CServerStats(ctypes.Structure):
    """struct h264r_server_stats"""
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "pictures_done", "streams_open", "streams_waiting", "streams_done", "batches", "batch_pictures",
        "dpb_bytes_in_use", "dpb_bytes_peak", "waiting_peak")] + [
        ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double)]
