"""The engine's failure path, made to run without a fault or a hang.

The reference prints and returns a negative code when a step fails
(RETURN_IF_FAILED, h264_video_decoder_demo/CommonFunction.h:40-47).  On the
GPU the wavefront kernels wait for the rows above them; each wait spins at
most a bounded number of times, then records H264R_ERR_DEVICE_TIMEOUT and
returns.  Here a launch withholds its wavefronts' first tickets
(h264r_ctx_set_wait_test), so the first row of the first picture never runs
and the rows below it wait on progress that is never published.  With a short
spin limit every kernel of the launch returns, the sync reports the timeout
once, and the same context then decodes the stream bit-exactly.
"""
import time

import numpy as np
import pytest

import h264_video_decoder_demo_gb300 as h
from h264_video_decoder_demo_gb300 import records as R

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("workload", ["1080p_high", "1080i_mbaff"])
def test_withheld_progress_times_out_and_the_context_recovers(engine_lib, workload):
    import torch
    from oracle_cpu import OracleDPB
    assert torch.cuda.is_available()
    gen = h.synth(workload, seed=91, num_pictures=3)
    pics = list(gen)
    assert sum(1 for m in pics[0].mbs if m["type"] in (1, 2, 3)) > 0  # the first picture has intra rows
    ctx = h.Context(0)
    s = h.Stream(ctx, pics[0].width_mbs, pics[0].height_mbs, gen.dpb_slots)
    try:
        ctx.set_wait_test(spin_limit=1 << 12, withhold_first_rows=True)
        t0 = time.perf_counter()
        s.submit(pics[0])
        with pytest.raises(h.engine.EngineError) as e:
            s.sync()
        assert e.value.code == R.ERR_DEVICE_TIMEOUT
        assert time.perf_counter() - t0 < 30.0
        assert "bounded wait expired" in ctx.last_error()
        s.sync()  # the error is reported once
        # normal operation on the same context and stream
        ctx.set_wait_test()
        dpb = OracleDPB(pics[0].width_mbs, pics[0].height_mbs, gen.dpb_slots)
        for i, p in enumerate(pics):
            s.submit(p)
            got = s.output(p.dst_slot)
            rc, _ = dpb.reconstruct(p)
            assert rc == 0
            assert np.array_equal(got, dpb.planes(p.dst_slot)), "picture %d differs from the oracle" % i
    finally:
        ctx.set_wait_test()
        s.close()
        ctx.close()
