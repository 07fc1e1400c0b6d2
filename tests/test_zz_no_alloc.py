"""The no-allocation deblocking entry point against the engine's own.

h264r_deblock_picture_noalloc serves callers that cannot let the library
allocate device memory (processes whose GPU memory is all in a pool of their
own, real-time loops that must not stall other streams on a cudaMalloc): it
filters a picture in place using only a static device array compiled into
the library.  Here it must give exactly the planes the engine's regular
deblocking gives, on two different pictures in a row (the shared scratch
keeps the first call's contents, so this also checks it is re-initialised).
Collected last on purpose: a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

import h264_video_decoder_demo_gb300 as h
from h264_video_decoder_demo_gb300 import records as R

pytestmark = pytest.mark.gpu


def device_picture(pic, keep):
    """CPicture whose record pointers are device copies (torch tensors)."""
    import torch
    c = pic.to_c()
    for name in R.Picture._ARRAYS:
        a = np.ascontiguousarray(getattr(pic, name)).view(np.uint8).reshape(-1)
        t = torch.from_numpy(a.copy()).cuda() if a.size else torch.empty(1, dtype=torch.uint8, device="cuda")
        keep.append(t)
        setattr(c, name, t.data_ptr())
    return c


@pytest.mark.parametrize("workload,seed", [("1080p_high", 77), ("1080i_mbaff", 78)])
def test_noalloc_deblock_matches_engine_two_calls(gpu_ctx, workload, seed):
    """Frame pictures go through the frame deblocking kernel; MBAFF pictures
    (half the MB pairs field pairs) through the MB-pair-row kernel, whose
    progress counters span three per pair row."""
    import torch
    lib = h.lib()
    gen = h.synth(workload, seed=seed, num_pictures=4)
    pics = list(gen)
    if workload == "1080i_mbaff":
        assert all(p.mbaff for p in pics)
    s = h.Stream(gpu_ctx, pics[0].width_mbs, pics[0].height_mbs, gen.dpb_slots)
    keep = []
    try:
        checked = 0
        for i, p in enumerate(pics):
            if i in (1, 2):  # a P picture then a B picture
                p.deblock = 0
                s.submit(p)
                pre = s.output(p.dst_slot).copy()
                p.deblock = 1
                s.submit(p)
                post = s.output(p.dst_slot).copy()
                assert not np.array_equal(pre, post)
                planes = torch.from_numpy(pre).cuda()
                cpic = device_picture(p, keep)
                torch.cuda.synchronize()
                rc = lib.h264r_deblock_picture_noalloc(ctypes.byref(cpic), ctypes.c_void_p(planes.data_ptr()),
                                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
                assert rc == 0
                got = planes.cpu().numpy()
                diff = np.nonzero(got != post)[0]
                assert len(diff) == 0, "picture %d: %d samples differ, first at %d" % (i, len(diff), diff[0])
                checked += 1
            else:
                s.submit(p)
                s.sync()
        assert checked == 2
    finally:
        s.close()


def test_noalloc_rejects_pictures_beyond_its_scratch(gpu_ctx):
    lib = h.lib()
    p = next(iter(h.synth("cif_ippp", seed=3, num_pictures=1)))
    c = p.to_c()
    c.width_mbs, c.height_mbs = 128, 128
    c.num_mbs = 128 * 128
    rc = lib.h264r_deblock_picture_noalloc(ctypes.byref(c), ctypes.c_void_p(16), None)
    assert rc == R.ERR_TOO_LARGE
