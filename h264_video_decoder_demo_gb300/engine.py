"""Python binding of the engine's C ABI (include/h264r.h) over ctypes.

The CUDA engine lives in libh264r.so next to this file (built in-tree by
h264_video_decoder_demo_gb300.build).  There is no fallback: when the library
is missing, loading fails with an error that says how to build it.
"""
import ctypes
import os
import threading

import numpy as np

from . import records as R

_LIB = None
_LIB_LOCK = threading.Lock()
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libh264r.so")

# every symbol include/h264r.h, h264r_synth.h, h264r_server.h, h264r_order.h, h264r_parser.h and
# h264r_decoder.h declare
EXPORTS = [
    "h264r_ctx_create", "h264r_ctx_destroy", "h264r_last_error", "h264r_stream_open",
    "h264r_stream_close", "h264r_stream_reset", "h264r_stream_dpb_bytes", "h264r_submit_picture",
    "h264r_submit_picture_device", "h264r_submit_batch_device", "h264r_submit_batch_device_on", "h264r_output",
    "h264r_output_async", "h264r_output_async_on",
    "h264r_load_slot", "h264r_slot_device_ptr", "h264r_stream_sync", "h264r_ctx_sync",
    "h264r_stream_cuda_stream", "h264r_stream_output_cuda_stream", "h264r_validate_picture", "h264r_ctx_kernel_launches",
    "h264r_ctx_set_timing", "h264r_ctx_last_timing", "h264r_ctx_kernel_timing", "h264r_ctx_set_wait_test",
    "h264r_ctx_host_stats",
    "h264r_synth_create", "h264r_synth_dpb_slots", "h264r_synth_next", "h264r_synth_destroy",
    "h264r_submit_batch", "h264r_picture_bytes", "h264r_ctx_cuda_stream",
    "h264r_deblock_picture_noalloc",
    "h264r_ctx_device", "h264r_ctx_dpb_budget", "h264r_ctx_max_batch",
    "h264r_ctx_set_tuning", "h264r_ctx_get_tuning", "h264r_ctx_set_mix_tuning", "h264r_autotune_batch_device",
    "h264r_ctx_graph_replays", "h264r_ctx_graphs_captured",
    "h264r_output_bgr24", "h264r_output_bgr24_device", "h264r_write_bmp", "h264r_write_yuv",
    "h264r_order_create", "h264r_order_destroy", "h264r_order_push", "h264r_order_flush",
    "h264r_order_holds", "h264r_order_infer_depth",
    "h264r_server_create", "h264r_server_destroy", "h264r_server_open", "h264r_server_push",
    "h264r_server_end", "h264r_server_poll", "h264r_server_pending", "h264r_server_get_stats",
    "h264r_parser_create", "h264r_parser_destroy", "h264r_parser_last_error", "h264r_parser_feed",
    "h264r_parser_end", "h264r_parser_next", "h264r_parser_geometry",
    "h264r_probe_coeff_token", "h264r_probe_total_zeros", "h264r_probe_run_before", "h264r_probe_cbp",
    "h264r_probe_cabac_init", "h264r_probe_cabac_decision",
    "h264r_decoder_create", "h264r_decoder_destroy", "h264r_decoder_last_error", "h264r_decoder_set_callback",
    "h264r_decoder_push", "h264r_decoder_flush", "h264r_decoder_open", "h264r_decoder_decoded",
    "h264r_decoder_output", "h264r_write_stream", "h264r_writer_free", "h264r_writer_last_error",
]


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("h264r error %d: %s" % (code, msg))
        self.code = code


def lib():
    """Load libh264r.so (once) and declare the C signatures."""
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LIB_LOCK:
        if _LIB is None:
            _LIB = _load()
    return _LIB


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libh264r.so is not built: run `python -m h264_video_decoder_demo_gb300.build` "
                          "(or __graft_entry__.build()) first")
    L = ctypes.CDLL(LIB_PATH)
    vp, i32, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64
    P = ctypes.POINTER
    sig = {
        "h264r_ctx_create": (i32, [P(R.CCfg), P(vp)]),
        "h264r_ctx_destroy": (i32, [vp]),
        "h264r_last_error": (ctypes.c_char_p, [vp]),
        "h264r_stream_open": (i32, [vp, P(R.CStreamCfg), P(vp)]),
        "h264r_stream_close": (i32, [vp]),
        "h264r_stream_reset": (i32, [vp]),
        "h264r_stream_dpb_bytes": (u64, [P(R.CStreamCfg)]),
        "h264r_submit_picture": (i32, [vp, P(R.CPicture)]),
        "h264r_submit_picture_device": (i32, [vp, P(R.CPicture)]),
        "h264r_submit_batch_device": (i32, [vp, i32, P(vp), P(R.CPicture)]),
        "h264r_submit_batch_device_on": (i32, [vp, vp, i32, P(vp), P(R.CPicture)]),
        "h264r_output": (i32, [vp, i32, vp, vp, vp]),
        "h264r_output_async": (i32, [vp, i32, vp, vp, vp]),
        "h264r_output_async_on": (i32, [vp, i32, vp, vp, vp, vp]),
        "h264r_stream_output_cuda_stream": (vp, [vp]),
        "h264r_load_slot": (i32, [vp, i32, vp, vp, vp]),
        "h264r_slot_device_ptr": (i32, [vp, i32, P(vp)]),
        "h264r_stream_sync": (i32, [vp]),
        "h264r_ctx_sync": (i32, [vp]),
        "h264r_stream_cuda_stream": (vp, [vp]),
        "h264r_ctx_cuda_stream": (vp, [vp]),
        "h264r_deblock_picture_noalloc": (i32, [P(R.CPicture), vp, vp]),
        "h264r_validate_picture": (i32, [P(R.CPicture), i32]),
        "h264r_ctx_kernel_launches": (u64, [vp]),
        "h264r_ctx_set_timing": (i32, [vp, i32]),
        "h264r_ctx_set_wait_test": (i32, [vp, u64, i32]),
        "h264r_ctx_kernel_timing": (i32, [vp, P(ctypes.c_float), P(i32)]),
        "h264r_ctx_host_stats": (i32, [vp, P(ctypes.c_double)]),
        "h264r_write_stream": (i32, [P(R.CWriterCfg), P(P(ctypes.c_uint8)), P(ctypes.c_size_t)]),
        "h264r_writer_free": (None, [P(ctypes.c_uint8)]),
        "h264r_writer_last_error": (ctypes.c_char_p, []),
        "h264r_ctx_last_timing": (i32, [vp, P(ctypes.c_float), P(i32)]),
        "h264r_submit_batch": (i32, [vp, i32, P(vp), P(R.CPicture)]),
        "h264r_picture_bytes": (i32, [P(R.CPicture), P(ctypes.c_uint64)]),
        "h264r_synth_create": (i32, [P(R.CSynthCfg), P(vp)]),
        "h264r_synth_dpb_slots": (i32, [vp]),
        "h264r_synth_next": (i32, [vp, P(R.CPicture), P(i32)]),
        "h264r_synth_destroy": (i32, [vp]),
        "h264r_output_bgr24": (i32, [vp, i32, vp, ctypes.c_uint32, i32]),
        "h264r_output_bgr24_device": (i32, [vp, i32, vp, ctypes.c_uint32, i32]),
        "h264r_write_bmp": (i32, [ctypes.c_char_p, vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]),
        "h264r_write_yuv": (i32, [ctypes.c_char_p, vp, vp, vp, ctypes.c_uint32, ctypes.c_uint32]),
        "h264r_order_create": (i32, [i32, P(vp)]),
        "h264r_order_destroy": (i32, [vp]),
        "h264r_order_push": (i32, [vp, u64, ctypes.c_int32, i32, P(u64), i32]),
        "h264r_order_flush": (i32, [vp, P(u64), i32]),
        "h264r_order_holds": (i32, [vp, u64]),
        "h264r_order_infer_depth": (i32, [i32, i32, i32, i32, i32]),
        "h264r_ctx_device": (i32, [vp]),
        "h264r_ctx_dpb_budget": (u64, [vp]),
        "h264r_ctx_max_batch": (i32, [vp]),
        "h264r_ctx_set_tuning": (i32, [vp, P(R.CTuning)]),
        "h264r_ctx_get_tuning": (i32, [vp, i32, P(R.CPicture), P(R.CTuning)]),
        "h264r_ctx_set_mix_tuning": (i32, [vp, i32, P(R.CPicture), P(R.CTuning)]),
        "h264r_autotune_batch_device": (i32, [vp, i32, P(vp), P(R.CPicture), i32, P(R.CTuning),
                                              P(ctypes.c_float)]),
        "h264r_ctx_graph_replays": (u64, [vp]),
        "h264r_ctx_graphs_captured": (u64, [vp]),
        "h264r_server_create": (i32, [vp, P(R.CServerCfg), P(vp)]),
        "h264r_server_destroy": (i32, [vp]),
        "h264r_server_open": (i32, [vp, P(R.CStreamCfg), P(i32)]),
        "h264r_server_push": (i32, [vp, i32, P(R.CPicture), i32, u64, vp]),
        "h264r_server_end": (i32, [vp, i32]),
        "h264r_server_poll": (i32, [vp, P(R.CServerDone), i32, i32]),
        "h264r_server_pending": (i32, [vp, i32]),
        "h264r_server_get_stats": (i32, [vp, P(R.CServerStats)]),
        "h264r_parser_create": (i32, [P(vp)]),
        "h264r_parser_destroy": (i32, [vp]),
        "h264r_parser_last_error": (ctypes.c_char_p, [vp]),
        "h264r_parser_feed": (i32, [vp, vp, ctypes.c_size_t]),
        "h264r_parser_end": (i32, [vp]),
        "h264r_parser_next": (i32, [vp, P(R.CParsed)]),
        "h264r_parser_geometry": (i32, [vp, P(i32), P(i32), P(i32)]),
        "h264r_probe_coeff_token": (i32, [i32, ctypes.c_uint32, P(i32)]),
        "h264r_probe_total_zeros": (i32, [i32, i32, ctypes.c_uint32, P(i32)]),
        "h264r_probe_run_before": (i32, [i32, ctypes.c_uint32, P(i32)]),
        "h264r_probe_cbp": (i32, [ctypes.c_uint32, i32]),
        "h264r_probe_cabac_init": (i32, [i32, i32, P(i32)]),
        "h264r_probe_cabac_decision": (i32, [i32, i32, i32, i32, P(i32)]),
        "h264r_decoder_create": (i32, [vp, P(vp)]),
        "h264r_decoder_destroy": (i32, [vp]),
        "h264r_decoder_last_error": (ctypes.c_char_p, [vp]),
        "h264r_decoder_set_callback": (i32, [vp, R.FRAME_CALLBACK, vp]),
        "h264r_decoder_push": (i32, [vp, vp, ctypes.c_size_t]),
        "h264r_decoder_flush": (i32, [vp]),
        "h264r_decoder_open": (i32, [vp, ctypes.c_char_p]),
        "h264r_decoder_decoded": (ctypes.c_uint32, [vp]),
        "h264r_decoder_output": (ctypes.c_uint32, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def picture_bytes(pic):
    """Algorithmic bytes [inter, intra, deblock, records] of a Picture."""
    c = pic.to_c()
    out = (ctypes.c_uint64 * 4)()
    rc = lib().h264r_picture_bytes(ctypes.byref(c), out)
    if rc != 0:
        raise EngineError(rc, "h264r_picture_bytes")
    return list(out)


def bgr_row_bytes(width):
    """Bytes per BGR24 row as the reference's bitmaps pad them (multiple of 4)."""
    return (3 * width + 3) // 4 * 4


def write_bmp(path, bgr, width, height):
    """24-bit BMP of top-down BGR24 rows (numpy uint8, height x row_bytes)."""
    bgr = np.ascontiguousarray(bgr, np.uint8)
    rb = bgr.size // height
    rc = lib().h264r_write_bmp(os.fsencode(path), bgr.ctypes.data, width, height, rb)
    if rc != 0:
        raise EngineError(rc, "write_bmp")


def write_yuv(path, planes, width, height):
    """Planar YUV 4:2:0 file (planes: numpy uint8 of width*height*3/2)."""
    planes = np.ascontiguousarray(planes, np.uint8)
    base = planes.ctypes.data
    rc = lib().h264r_write_yuv(os.fsencode(path), base, base + width * height, base + width * height * 5 // 4, width, height)
    if rc != 0:
        raise EngineError(rc, "write_yuv")


def validate(pic, dpb_slots):
    c = pic.to_c()
    return lib().h264r_validate_picture(ctypes.byref(c), dpb_slots)


class Context:
    """An engine context on one GPU (h264r_ctx)."""

    def __init__(self, device=0, dpb_budget_bytes=0, max_batch=64, records_ready=False):
        # records_ready: H264R_CFG_DEVICE_RECORDS_READY (device records are
        # complete when a *_device submit is made)
        cfg = R.CCfg(device, dpb_budget_bytes, max_batch, 1 if records_ready else 0)
        h = ctypes.c_void_p()
        rc = lib().h264r_ctx_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != 0:
            raise EngineError(rc, "h264r_ctx_create failed")
        self.h = h

    def check(self, rc, what):
        if rc != 0:
            raise EngineError(rc, "%s: %s" % (what, lib().h264r_last_error(self.h).decode()))
        return rc

    def last_error(self):
        return lib().h264r_last_error(self.h).decode()

    def kernel_launches(self):
        return int(lib().h264r_ctx_kernel_launches(self.h))

    def set_timing(self, on):
        self.check(lib().h264r_ctx_set_timing(self.h, 1 if on else 0), "set_timing")

    def set_wait_test(self, spin_limit=0, withhold_first_rows=False):
        """Failure-path tests: a small device spin limit and/or launches that
        withhold their wavefronts' first rows (h264r_ctx_set_wait_test);
        set_wait_test() restores normal operation."""
        self.check(lib().h264r_ctx_set_wait_test(self.h, int(spin_limit), 1 if withhold_first_rows else 0),
                   "set_wait_test")

    def last_timing(self):
        """(summed ms of [inter, intra, deblock], launch sequences) since set_timing(True)."""
        t = (ctypes.c_float * 3)()
        n = ctypes.c_int()
        self.check(lib().h264r_ctx_last_timing(self.h, t, ctypes.byref(n)), "last_timing")
        return list(t), n.value

    def kernel_timing(self):
        """(summed ms of [k_inter, k_intra, k_bs, deblocking filter], launch
        sequences) since set_timing(True); k_bs runs in line while timing."""
        t = (ctypes.c_float * 4)()
        n = ctypes.c_int()
        self.check(lib().h264r_ctx_kernel_timing(self.h, t, ctypes.byref(n)), "kernel_timing")
        return list(t), n.value

    def host_stats(self):
        """Host seconds of h264r_submit_batch: (waiting for a launch slot,
        validating and packing, upload and launch, packing threads)."""
        s = (ctypes.c_double * 4)()
        self.check(lib().h264r_ctx_host_stats(self.h, s), "host_stats")
        return list(s)

    def sync(self):
        return self.check(lib().h264r_ctx_sync(self.h), "ctx_sync")

    def cuda_stream(self):
        """cudaStream_t (int) of the context's batch stream."""
        return lib().h264r_ctx_cuda_stream(self.h)

    def submit_batch(self, streams, pics):
        """Batched reconstruction from host records (list of Picture)."""
        n = len(streams)
        arr = (ctypes.c_void_p * n)(*[s.h.value for s in streams])
        cpics = (R.CPicture * n)(*[p.to_c() for p in pics])
        return self.check(lib().h264r_submit_batch(self.h, n, arr, cpics), "submit_batch")

    def prepare_batch(self, streams, pics):
        """The C arguments of a host-record batch (streams and h264r_picture
        descriptors pointing into the Pictures' arrays), built once for
        submit_prepared, as a C caller keeps the descriptors its parser
        emitted.  The Pictures must stay alive and unchanged."""
        n = len(streams)
        arr = (ctypes.c_void_p * n)(*[s.h.value for s in streams])
        cpics = (R.CPicture * n)(*[p.to_c() for p in pics])
        return n, arr, cpics, list(pics)

    def submit_prepared(self, prep):
        """h264r_submit_batch of a prepare_batch result: validation, packing
        and the host-to-device copy of the records happen on every call."""
        n, arr, cpics, _ = prep
        return self.check(lib().h264r_submit_batch(self.h, n, arr, cpics), "submit_batch")

    def submit_batch_device(self, streams, cpics):
        n = len(streams)
        arr = (ctypes.c_void_p * n)(*[s.h.value for s in streams])
        pics = (R.CPicture * n)(*cpics)
        return lib().h264r_submit_batch_device(self.h, n, arr, pics)

    def set_tuning(self, inter_mbs_per_cta=4, deblock_pairs_per_cta=8, graphs=False):
        """Default launch shapes and graph replay of every batch (h264r_ctx_set_tuning)."""
        t = R.CTuning(inter_mbs_per_cta, deblock_pairs_per_cta, 1 if graphs else 0, 0)
        return self.check(lib().h264r_ctx_set_tuning(self.h, ctypes.byref(t)), "set_tuning")

    def tuning(self, cpics=()):
        """The tuning a batch of these pictures (CPicture) launches with, as a dict."""
        n = len(cpics)
        pics = (R.CPicture * max(n, 1))(*cpics)
        t = R.CTuning()
        self.check(lib().h264r_ctx_get_tuning(self.h, n, pics, ctypes.byref(t)), "get_tuning")
        return t.as_dict()

    def set_mix_tuning(self, cpics, inter_mbs_per_cta=4, deblock_pairs_per_cta=8, graphs=False):
        """Tuning of the geometry mix of these pictures (CPicture), e.g. a kept autotuner result."""
        n = len(cpics)
        pics = (R.CPicture * n)(*cpics)
        t = R.CTuning(inter_mbs_per_cta, deblock_pairs_per_cta, 1 if graphs else 0, 0)
        return self.check(lib().h264r_ctx_set_mix_tuning(self.h, n, pics, ctypes.byref(t)), "set_mix_tuning")

    def autotune_batch_device(self, streams, cpics, reps=5):
        """Time every launch shape on this batch and keep the fastest for its
        geometry mix (h264r_autotune_batch_device); returns (tuning dict, ms per batch)."""
        n = len(streams)
        arr = (ctypes.c_void_p * n)(*[s.h.value for s in streams])
        pics = (R.CPicture * n)(*cpics)
        t = R.CTuning()
        ms = ctypes.c_float()
        self.check(lib().h264r_autotune_batch_device(self.h, n, arr, pics, reps, ctypes.byref(t), ctypes.byref(ms)),
                   "autotune_batch_device")
        return t.as_dict(), ms.value

    def graph_counts(self):
        """(launch sequences replayed from captured graphs, graphs captured)."""
        return int(lib().h264r_ctx_graph_replays(self.h)), int(lib().h264r_ctx_graphs_captured(self.h))

    def close(self):
        if self.h:
            lib().h264r_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Stream:
    """A stream with a device-resident DPB (h264r_stream)."""

    def __init__(self, ctx, width_mbs, height_mbs, dpb_slots):
        self.ctx = ctx
        self.width_mbs, self.height_mbs, self.dpb_slots = width_mbs, height_mbs, dpb_slots
        cfg = R.CStreamCfg(width_mbs, height_mbs, dpb_slots, 0)
        h = ctypes.c_void_p()
        rc = lib().h264r_stream_open(ctx.h, ctypes.byref(cfg), ctypes.byref(h))
        ctx.check(rc, "stream_open")
        self.h = h

    @property
    def plane_bytes(self):
        return self.width_mbs * self.height_mbs * 384

    def submit(self, pic):
        """Reconstruct a picture from host records (Picture)."""
        c = pic.to_c()
        return self.ctx.check(lib().h264r_submit_picture(self.h, ctypes.byref(c)), "submit_picture")

    def submit_device(self, cpic):
        return self.ctx.check(lib().h264r_submit_picture_device(self.h, ctypes.byref(cpic)), "submit_picture_device")

    def output(self, slot, out=None):
        """Decoded planes of a DPB slot as one uint8 array (Y, Cb, Cr)."""
        W, H = self.width_mbs * 16, self.height_mbs * 16
        if out is None:
            out = np.empty(W * H * 3 // 2, np.uint8)
        base = out.ctypes.data
        self.ctx.check(lib().h264r_output(self.h, slot, base, base + W * H, base + W * H + W * H // 4), "output")
        self.sync()
        return out

    def output_async(self, slot, out):
        """Copy a slot into `out` (numpy uint8, pinned for overlap) on the
        stream's copy stream (h264r_output_async); sync before reading."""
        W, H = self.width_mbs * 16, self.height_mbs * 16
        base = out.ctypes.data
        return self.ctx.check(lib().h264r_output_async(self.h, slot, base, base + W * H, base + W * H + W * H // 4),
                              "output_async")

    def output_bgr24(self, slot, flip=False):
        """The picture in a slot as BGR24 rows (height x row_bytes, numpy)."""
        W, H = self.width_mbs * 16, self.height_mbs * 16
        rb = bgr_row_bytes(W)
        out = np.empty((H, rb), np.uint8)
        self.ctx.check(lib().h264r_output_bgr24(self.h, slot, out.ctypes.data, rb, int(flip)), "output_bgr24")
        self.sync()
        return out

    def load_slot(self, slot, planes):
        W, H = self.width_mbs * 16, self.height_mbs * 16
        planes = np.ascontiguousarray(planes, np.uint8)
        base = planes.ctypes.data
        self.ctx.check(lib().h264r_load_slot(self.h, slot, base, base + W * H, base + W * H + W * H // 4), "load_slot")

    def slot_ptr(self, slot):
        p = ctypes.c_void_p()
        self.ctx.check(lib().h264r_slot_device_ptr(self.h, slot, ctypes.byref(p)), "slot_ptr")
        return p.value

    def cuda_stream(self):
        return lib().h264r_stream_cuda_stream(self.h)

    def sync(self):
        return self.ctx.check(lib().h264r_stream_sync(self.h), "stream_sync")

    def reset(self):
        """Ready for a new bitstream of the same geometry (buffers cleared)."""
        return self.ctx.check(lib().h264r_stream_reset(self.h), "stream_reset")

    def close(self):
        if self.h:
            lib().h264r_stream_close(self.h)
            self.h = None


class Order:
    """Output order of decoded pictures (include/h264r_order.h): the
    reference's reorder buffer of max_num_reorder_frames pictures."""

    def __init__(self, max_num_reorder_frames):
        h = ctypes.c_void_p()
        rc = lib().h264r_order_create(max_num_reorder_frames, ctypes.byref(h))
        if rc != 0:
            raise EngineError(rc, "order_create")
        self.h = h
        self._buf = (ctypes.c_uint64 * 32)()

    def push(self, tag, poc, idr=False):
        """A picture finished decoding; returns the tags to output now."""
        n = lib().h264r_order_push(self.h, tag, poc, int(bool(idr)), self._buf, 32)
        if n < 0:
            raise EngineError(n, "order_push")
        return [self._buf[i] for i in range(n)]

    def flush(self):
        n = lib().h264r_order_flush(self.h, self._buf, 32)
        if n < 0:
            raise EngineError(n, "order_flush")
        return [self._buf[i] for i in range(n)]

    def holds(self, tag):
        return lib().h264r_order_holds(self.h, tag) == 1

    @staticmethod
    def infer_depth(profile_idc, constraint_set3_flag, level_idc, width_mbs, frame_height_mbs):
        return lib().h264r_order_infer_depth(profile_idc, constraint_set3_flag, level_idc, width_mbs, frame_height_mbs)

    def close(self):
        if self.h:
            lib().h264r_order_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Parser:
    """Host-side front end (include/h264r_parser.h): Annex B bytes in,
    completed pictures (records plus DPB slot and output list) out."""

    def __init__(self):
        h = ctypes.c_void_p()
        rc = lib().h264r_parser_create(ctypes.byref(h))
        if rc != 0:
            raise EngineError(rc, "parser_create")
        self.h = h
        self._out = R.CParsed()

    def _check(self, rc, what):
        if rc < 0:
            raise EngineError(rc, "%s: %s" % (what, lib().h264r_parser_last_error(self.h).decode()))
        return rc

    def feed(self, data):
        buf = (ctypes.c_uint8 * len(data)).from_buffer_copy(data)
        self._check(lib().h264r_parser_feed(self.h, buf, len(data)), "parser_feed")

    def end(self):
        self._check(lib().h264r_parser_end(self.h), "parser_end")

    def geometry(self):
        w, hh, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        lib().h264r_parser_geometry(self.h, ctypes.byref(w), ctypes.byref(hh), ctypes.byref(s))
        return w.value, hh.value, s.value

    def next(self):
        """The next completed picture as (records.Picture, info dict), or None."""
        rc = self._check(lib().h264r_parser_next(self.h, ctypes.byref(self._out)), "parser_next")
        if rc == 0:
            return None
        o = self._out
        c = o.pic
        p = R.Picture()
        p.width_mbs, p.height_mbs, p.structure, p.mbaff = c.width_mbs, c.height_mbs, c.structure, c.mbaff
        p.dst_slot, p.deblock = c.dst_slot, c.deblock
        p.scaling4x4 = np.frombuffer(bytes(c.scaling4x4), np.uint8).reshape(6, 16).copy()
        p.scaling8x8 = np.frombuffer(bytes(c.scaling8x8), np.uint8).reshape(6, 64).copy()

        def arr(ptr, n, dtype):
            if n == 0 or not ptr:
                return np.zeros(0, dtype)
            nbytes = n * np.dtype(dtype).itemsize
            return np.frombuffer(ctypes.string_at(ptr, nbytes), dtype).copy()

        p.mbs = arr(c.mbs, c.num_mbs, R.MB_DTYPE)
        p.slices = arr(c.slices, c.num_slices, R.SLICE_DTYPE)
        p.weights = arr(c.weights, c.num_weights, R.WEIGHT_DTYPE)
        p.motion = arr(c.motion, c.motion_bytes, np.uint8)
        p.coef = arr(c.coef, c.coef_bytes, np.uint8)
        p.pcm = arr(c.pcm, c.num_pcm * 384, np.uint8)
        n = o.num_output
        info = {"poc": o.poc, "index": o.index, "idr": bool(o.idr), "reference": bool(o.reference),
                "slice_type": o.slice_type,
                "output_slots": list(arr(o.output_slots, n, np.uint8)),
                "output_poc": list(arr(o.output_poc, n, np.int32)),
                "output_index": list(arr(o.output_index, n, np.uint32))}
        return p, info

    def pictures(self, data, chunk=1 << 20):
        """Parse a whole byte stream; yields (Picture, info) in decoding order."""
        for i in range(0, len(data), chunk):
            self.feed(data[i:i + chunk])
            while True:
                r = self.next()
                if r is None:
                    break
                yield r
        self.end()
        while True:
            r = self.next()
            if r is None:
                break
            yield r

    def close(self):
        if self.h:
            lib().h264r_parser_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Decoder:
    """Whole-stream decoding on the context's GPU (include/h264r_decoder.h):
    on_frame(frame, error_code) is called per output picture in output order
    (frame: dict with poc, decode_index, slice_type, width, height, planes =
    one uint8 array Y|Cb|Cr copied out of the callback), then once with
    frame None and H264R_DECODE_FILE_END.  A true return value stops the
    decode, as the reference's callback convention has it."""

    FILE_END, OPEN_FILE_FAILED = 1, 2

    def __init__(self, ctx, on_frame, copy_planes=True):
        self.ctx = ctx
        h = ctypes.c_void_p()
        rc = lib().h264r_decoder_create(ctx.h, ctypes.byref(h))
        if rc != 0:
            raise EngineError(rc, "decoder_create")
        self.h = h
        self._user = on_frame

        def trampoline(fp, user, code):
            if not fp:
                return int(bool(self._user(None, code)))
            f = fp.contents
            n = f.width * f.height * 3 // 2
            planes = np.frombuffer(ctypes.string_at(f.y, n), np.uint8).copy() if copy_planes else None
            info = {"poc": f.poc, "decode_index": f.decode_index, "slice_type": f.slice_type,
                    "output_count": f.output_count, "width": f.width, "height": f.height, "planes": planes,
                    "slot": f.slot}
            return int(bool(self._user(info, code)))

        self._cb = R.FRAME_CALLBACK(trampoline)
        lib().h264r_decoder_set_callback(self.h, self._cb, None)

    def _check(self, rc, what):
        if rc < 0:
            raise EngineError(rc, "%s: %s" % (what, lib().h264r_decoder_last_error(self.h).decode()))
        return rc

    def push(self, data):
        buf = (ctypes.c_uint8 * len(data)).from_buffer_copy(data)
        return self._check(lib().h264r_decoder_push(self.h, buf, len(data)), "decoder_push")

    def flush(self):
        return self._check(lib().h264r_decoder_flush(self.h), "decoder_flush")

    def open(self, path):
        return lib().h264r_decoder_open(self.h, path.encode())

    @property
    def decoded(self):
        return lib().h264r_decoder_decoded(self.h)

    def close(self):
        if self.h:
            lib().h264r_decoder_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching server on a context (include/h264r_server.h): streams
    are admitted by the context's DPB budget, pictures pushed as their records
    are complete, finished pictures polled with their latency."""

    def __init__(self, ctx, max_batch=0, queue_depth=0, lanes=0):
        self.ctx = ctx
        h = ctypes.c_void_p()
        cfg = R.CServerCfg(max_batch, queue_depth, 0, lanes)
        ctx.check(lib().h264r_server_create(ctx.h, ctypes.byref(cfg), ctypes.byref(h)), "server_create")
        self.h = h
        self._keep = {}

    def open(self, width_mbs, height_mbs, dpb_slots):
        sid = ctypes.c_int()
        cfg = R.CStreamCfg(width_mbs, height_mbs, dpb_slots, 0)
        rc = lib().h264r_server_open(self.h, ctypes.byref(cfg), ctypes.byref(sid))
        if rc != 0:
            raise EngineError(rc, "server_open")
        return sid.value

    def push(self, stream, pic, group, tag, out=None):
        """Queue a Picture; `out` (numpy uint8, W*H*3/2, ideally pinned) receives the planes."""
        c = pic.to_c()
        ptr = out.ctypes.data if out is not None else None
        if out is not None:
            self._keep[(stream, tag)] = out
        return lib().h264r_server_push(self.h, stream, ctypes.byref(c), group, tag, ptr)

    def push_c(self, stream, cpic, group, tag, out_ptr):
        """push() with the C arguments built by the caller: a CPicture whose
        arrays the caller keeps alive, and the address of the output planes
        (kept alive by the caller until the picture is polled)."""
        return lib().h264r_server_push(self.h, stream, ctypes.byref(cpic), group, tag, out_ptr)

    def end(self, stream):
        return lib().h264r_server_end(self.h, stream)

    def poll(self, max_items=256, wait_ms=10):
        buf = (R.CServerDone * max_items)()
        n = lib().h264r_server_poll(self.h, buf, max_items, wait_ms)
        if n < 0:
            raise EngineError(n, "server_poll")
        out = []
        for i in range(n):
            d = buf[i]
            self._keep.pop((d.stream, d.tag), None)
            out.append((d.stream, d.tag, d.status, d.latency_ms))
        return out

    def pending(self, stream):
        return lib().h264r_server_pending(self.h, stream)

    def stats(self):
        st = R.CServerStats()
        lib().h264r_server_get_stats(self.h, ctypes.byref(st))
        return {name: getattr(st, name) for name, _ in R.CServerStats._fields_}

    def close(self):
        if self.h:
            lib().h264r_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Synth:
    """Seeded synthetic stream generator (include/h264r_synth.h)."""

    GOP_IPPP, GOP_IBBP = 0, 1
    WP_NONE, WP_EXPLICIT, WP_IMPLICIT = 0, 1, 2

    def __init__(self, **kw):
        cfg = R.CSynthCfg()
        defaults = dict(seed=1, width_mbs=22, height_mbs=18, num_pictures=8, gop_length=15,
                        gop_kind=0, num_refs=1, transform8x8=0, weighted=0, min_partition=2,
                        intra_percent=10, skip_percent=10, qp_min=20, qp_max=36,
                        edge_mv_percent=0, mv_range=64, filter_offset_max=0, coef_density=40)
        defaults.update(kw)
        for k, v in defaults.items():
            setattr(cfg, k, v)
        self.cfg = cfg
        h = ctypes.c_void_p()
        rc = lib().h264r_synth_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != 0:
            raise EngineError(rc, "h264r_synth_create")
        self.h = h

    @property
    def dpb_slots(self):
        return lib().h264r_synth_dpb_slots(self.h)

    def __iter__(self):
        return self

    def __next__(self):
        c = R.CPicture()
        grp = ctypes.c_int()
        rc = lib().h264r_synth_next(self.h, ctypes.byref(c), ctypes.byref(grp))
        if rc == 1:
            raise StopIteration
        if rc != 0:
            raise EngineError(rc, "h264r_synth_next")
        pic = R.Picture.from_c(c)
        pic.group = grp.value
        return pic

    def close(self):
        if self.h:
            lib().h264r_synth_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# named workloads: the reference's benchmark configurations as synthetic
# record streams (shapes, sizes and value distributions of each config)
WORKLOADS = {
    # CIF 352x288, 8 pictures IPPP, Baseline CAVLC, 1 ref, QP 20..36, 10% I4x4
    "cif_ippp": dict(width_mbs=22, height_mbs=18, num_pictures=8, gop_kind=0, num_refs=1,
                     transform8x8=0, weighted=0, min_partition=2, intra_percent=10,
                     skip_percent=5, qp_min=20, qp_max=36, mv_range=64, filter_offset_max=0),
    # 1080p High: 1920x1088, 30 pictures, GOP 15 IBBP, 8x8 transform, partitions
    # to 4x4, 4 refs, explicit weights, MVs +-256 qpel with 5% past the edges,
    # QP 22..40, alpha/beta offsets +-6
    "1080p_high": dict(width_mbs=120, height_mbs=68, num_pictures=30, gop_length=15, gop_kind=1,
                       num_refs=4, transform8x8=1, weighted=1, min_partition=3, intra_percent=5,
                       skip_percent=10, qp_min=22, qp_max=40, edge_mv_percent=5, mv_range=256,
                       filter_offset_max=6, coef_density=40),
    # interlaced 1080i: MBAFF frame/field MB pairs (half the pairs field),
    # I/P anchors with B between, MVs +-128 qpel, no weighted prediction
    "1080i_mbaff": dict(width_mbs=120, height_mbs=68, num_pictures=20, gop_length=12, gop_kind=1,
                        num_refs=2, transform8x8=1, weighted=0, min_partition=3, intra_percent=5,
                        skip_percent=10, qp_min=22, qp_max=40, edge_mv_percent=5, mv_range=128,
                        filter_offset_max=6, coef_density=40, mbaff=1, field_percent=50),
    "720p_high": dict(width_mbs=80, height_mbs=45, num_pictures=60, gop_length=15, gop_kind=1,
                      num_refs=4, transform8x8=1, weighted=2, min_partition=3, intra_percent=5,
                      skip_percent=10, qp_min=22, qp_max=40, edge_mv_percent=5, mv_range=256,
                      filter_offset_max=6, coef_density=40),
}


def synth(name, seed=1, **over):
    kw = dict(WORKLOADS[name])
    kw.update(over)
    return Synth(seed=seed, **kw)


# named bitstream configurations of the seeded writer (include/h264r_writer.h):
# the reference's benchmark configurations as CAVLC Annex B streams
STREAMS = {
    # CIF 352x288, 8 pictures IPPP, Baseline CAVLC, one slice, 1 reference,
    # partitions 16x16 / 16x8 / 8x16 / 8x8, MVs +-64 qpel, QP 20..36, 10% intra
    "cif_ippp": dict(width_mbs=22, height_mbs=18, num_pictures=8, profile_idc=66, gop_length=0, b_pictures=0,
                     num_refs=1, transform8x8=0, weighted=0, direct_spatial=1, min_partition=2, intra_percent=10,
                     skip_percent=5, edge_mv_percent=0, qp_min=20, qp_max=36, filter_offset_max=0,
                     coef_density=40, slices=1, pcm_permille=0, chroma_qp_offset_max=0, mv_range=64),
    # 1080p High (coded 1920x1088), 30 pictures, GOP 15 IBBP, 8x8 transforms,
    # partitions down to 4x4, up to 4 references, explicit weighted prediction
    # (weights -64..127, every bi-predictive sum <= 128, offsets +-32), spatial
    # direct, MVs +-256 qpel with 5% past the edges, QP 22..40, alpha / beta
    # offsets +-6; CAVLC (the writer has no CABAC)
    "1080p_high": dict(width_mbs=120, height_mbs=68, num_pictures=30, profile_idc=100, gop_length=15, b_pictures=2,
                       num_refs=4, transform8x8=1, weighted=1, direct_spatial=1, min_partition=3, intra_percent=5,
                       skip_percent=10, edge_mv_percent=5, qp_min=22, qp_max=40, filter_offset_max=6,
                       coef_density=40, slices=1, pcm_permille=2, chroma_qp_offset_max=3, mv_range=256),
    # interlaced 1080i as MBAFF frames (the MBAFF half of the interlaced
    # configuration): 1920x1088, 20 pictures, GOP 12 with one B picture
    # between anchors, half the MB pairs field pairs, 2 references, no weighted
    # prediction, MVs +-128 qpel, CAVLC
    "1080i_mbaff": dict(width_mbs=120, height_mbs=68, num_pictures=20, profile_idc=100, gop_length=12, b_pictures=1,
                        num_refs=2, transform8x8=1, weighted=0, direct_spatial=1, min_partition=3, intra_percent=5,
                        skip_percent=10, edge_mv_percent=5, qp_min=22, qp_max=40, filter_offset_max=6,
                        coef_density=40, slices=1, pcm_permille=2, chroma_qp_offset_max=3, mv_range=128, mbaff=1,
                        field_percent=50),
}


class GroupTracker:
    """Dependency groups of a stream's pictures, one picture at a time in
    decoding order, as the batched entry points and the server need them: a
    picture comes after the pictures it reads (its references), after every
    reader of the picture its DPB slot held before, and after that picture."""

    def __init__(self):
        self.writer, self.readers = {}, {}

    def next(self, pic):
        refs = pic.ref_slots()
        g = 0
        for sl in refs:
            g = max(g, self.writer.get(sl, -1) + 1)
        g = max(g, self.readers.get(pic.dst_slot, -1) + 1, self.writer.get(pic.dst_slot, -1) + 1)
        for sl in refs:
            self.readers[sl] = max(self.readers.get(sl, -1), g)
        self.writer[pic.dst_slot] = g
        self.readers[pic.dst_slot] = -1
        pic.group = g
        return g


def assign_groups(pics):
    """Sets pic.group of every picture (decoding order); returns the count."""
    t = GroupTracker()
    return max((t.next(p) for p in pics), default=-1) + 1


def parse_stream(data):
    """Records of every picture of an Annex B stream (front end), with their
    dependency groups: (list of Picture, DPB slots the stream needs)."""
    p = Parser()
    try:
        pics = [pic for pic, _ in p.pictures(data)]
        p.end()
        while True:
            r = p.next()
            if r is None:
                break
            pics.append(r[0])
        slots = p.geometry()[2]
    finally:
        p.close()
    assign_groups(pics)
    return pics, slots


def write_stream(name=None, seed=1, **over):
    """Annex B bytes of a seeded stream (h264r_write_stream): a named
    configuration of STREAMS with fields overridden, or fields alone."""
    kw = dict(STREAMS[name]) if name else {}
    kw.update(over)
    cfg = R.CWriterCfg()
    cfg.seed = seed
    for k, v in kw.items():
        setattr(cfg, k, v)
    data = ctypes.POINTER(ctypes.c_uint8)()
    size = ctypes.c_size_t()
    rc = lib().h264r_write_stream(ctypes.byref(cfg), ctypes.byref(data), ctypes.byref(size))
    if rc != 0:
        raise EngineError(rc, "h264r_write_stream: %s" % lib().h264r_writer_last_error().decode())
    try:
        return ctypes.string_at(data, size.value)
    finally:
        lib().h264r_writer_free(data)
