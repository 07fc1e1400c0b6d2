"""ctypes binding of the CPU oracle (oracle/liboracle.so).

Test infrastructure: the checker the GPU engine is compared with.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "liboracle.so")
_L = None


def lib():
    global _L
    if _L is None:
        if not os.path.exists(LIB):
            subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "-s", "liboracle.so"])
        L = ctypes.CDLL(LIB)
        L.h264o_slot_bytes.restype = ctypes.c_uint64
        L.h264o_slot_bytes.argtypes = [ctypes.c_int, ctypes.c_int]
        L.h264o_reconstruct.restype = ctypes.c_int
        L.h264o_reconstruct.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.h264o_bgr24.restype = None
        L.h264o_bgr24.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        _L = L
    return _L


class OracleDPB:
    """Host DPB of the oracle: nslots picture buffers in the engine's layout."""

    def __init__(self, width_mbs, height_mbs, nslots=32):
        self.width_mbs, self.height_mbs = width_mbs, height_mbs
        self.plane_bytes = width_mbs * height_mbs * 384
        sb = lib().h264o_slot_bytes(width_mbs, height_mbs)
        self.slots = [np.zeros(sb, np.uint8) for _ in range(nslots)]
        self._ptrs = (ctypes.c_void_p * nslots)(*[s.ctypes.data for s in self.slots])

    def reconstruct(self, pic, want_pre=False):
        """Reconstruct pic into its slot; returns (rc, pre-deblock planes or None)."""
        c = pic.to_c()
        pre = np.zeros(self.plane_bytes, np.uint8) if want_pre else None
        rc = lib().h264o_reconstruct(ctypes.byref(c), self._ptrs, len(self.slots),
                                     pre.ctypes.data if pre is not None else None)
        return rc, pre

    def planes(self, slot):
        return self.slots[slot][:self.plane_bytes]


def bgr24(planes, width, height, flip=False):
    """The oracle's BGR24 rows of YUV 4:2:0 planes (height x row_bytes)."""
    rb = (3 * width + 3) // 4 * 4
    out = np.zeros((height, rb), np.uint8)
    planes = np.ascontiguousarray(planes, np.uint8)
    lib().h264o_bgr24(width, height, planes.ctypes.data, out.ctypes.data, rb, int(flip))
    return out
