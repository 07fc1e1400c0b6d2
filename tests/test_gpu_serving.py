"""The continuous-batching server (include/h264r_server.h) against the engine
run one stream at a time.

Streams of three sizes (CIF IPPP, 720p and 1080p IBBP) arrive one after
another under a DPB memory budget that holds only a few of them, so later
streams wait for earlier ones to finish; their pictures are pushed as the
per-stream window allows and batched with whatever else is ready.  Every
decoded picture must equal, byte for byte (tolerance 0: the path is integer
arithmetic), the same stream decoded alone through h264r_submit_picture.
"""
import hashlib
import time

import numpy as np
import pytest

import h264_video_decoder_demo_gb300 as h
from h264_video_decoder_demo_gb300 import records as R

pytestmark = pytest.mark.gpu

MIX = [("cif_ippp", 11, 8), ("1080p_high", 31, 6), ("720p_high", 21, 6), ("cif_ippp", 12, 8),
       ("1080p_high", 32, 6), ("720p_high", 22, 6), ("cif_ippp", 13, 8)]


def md5(a):
    return hashlib.md5(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_streams():
    out = []
    for name, seed, n in MIX:
        g = h.synth(name, seed=seed, num_pictures=n)
        pics = list(g)
        out.append((pics, g.dpb_slots))
        g.close()
    return out


def alone(streams):
    """md5 of every picture, each stream decoded on its own."""
    ref = []
    with h.Context(0) as ctx:
        for pics, slots in streams:
            s = h.Stream(ctx, pics[0].width_mbs, pics[0].height_mbs, slots)
            ref.append([])
            for p in pics:
                s.submit(p)
                ref[-1].append(md5(s.output(p.dst_slot)))
            s.close()
    return ref


def test_server_results_equal_alone_and_in_the_mix():
    import torch
    streams = make_streams()
    ref = alone(streams)
    dpb = [R.CStreamCfg(p[0].width_mbs, p[0].height_mbs, slots, 0) for p, slots in streams]
    sizes = [h.lib().h264r_stream_dpb_bytes(c) for c in dpb]
    budget = max(sizes) + sorted(sizes)[len(sizes) // 2]  # a 1080p DPB and a bit more
    window = 3
    with h.Context(0, dpb_budget_bytes=budget) as ctx, h.Server(ctx, queue_depth=window) as srv:
        ids, cursor, ended = [None] * len(streams), [0] * len(streams), [False] * len(streams)
        outs = {}
        got = {}
        t0 = time.perf_counter()
        arrivals = [0.004 * i for i in range(len(streams))]
        deadline = t0 + 120
        while len(got) < sum(len(p) for p, _ in streams):
            assert time.perf_counter() < deadline, "server made no progress"
            now = time.perf_counter() - t0
            for i, (pics, slots) in enumerate(streams):
                if ids[i] is None and now >= arrivals[i]:
                    ids[i] = srv.open(pics[0].width_mbs, pics[0].height_mbs, slots)
                if ids[i] is None or ended[i]:
                    continue
                while cursor[i] < len(pics) and srv.pending(ids[i]) < window:
                    p = pics[cursor[i]]
                    buf = torch.empty(p.plane_bytes, dtype=torch.uint8, pin_memory=True).numpy()
                    outs[(ids[i], cursor[i])] = buf
                    assert srv.push(ids[i], p, p.group, cursor[i], buf) == 0
                    cursor[i] += 1
                if cursor[i] == len(pics):
                    srv.end(ids[i])
                    ended[i] = True
            for sid, tag, status, lat in srv.poll(wait_ms=2):
                assert status == 0, (sid, tag, status)
                got[(sid, tag)] = md5(outs[(sid, tag)])
        st = srv.stats()
    for i, (pics, _) in enumerate(streams):
        for k in range(len(pics)):
            assert got[(ids[i], k)] == ref[i][k], "stream %d (%s) picture %d differs in the mix" % (i, MIX[i][0], k)
    assert st["pictures_done"] == len(got)
    assert st["waiting_peak"] >= 1, "the budget never made a stream wait"
    assert st["dpb_bytes_peak"] <= budget
    assert st["batch_pictures"] > st["batches"], "no batch held more than one picture"
    assert st["streams_done"] == len(streams)
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]


def test_server_rejects_a_stream_larger_than_the_budget():
    with h.Context(0, dpb_budget_bytes=8 << 20) as ctx, h.Server(ctx) as srv:
        with pytest.raises(h.EngineError) as e:
            srv.open(120, 68, 4)
        assert e.value.code == R.ERR_BUDGET
        sid = srv.open(22, 18, 4)  # CIF fits
        assert sid >= 0
        srv.end(sid)
