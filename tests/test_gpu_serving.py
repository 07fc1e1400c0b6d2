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

# (generator, seed, pictures[, overrides]): progressive streams of three sizes,
# a stream of field pictures (every frame a top and a bottom field, each its
# own dependency group) and one of MBAFF frames
MIX = [("cif_ippp", 11, 8), ("1080p_high", 31, 6), ("720p_high", 21, 6), ("cif_ippp", 12, 8),
       ("1080p_high", 32, 6), ("720p_high", 22, 6), ("cif_ippp", 13, 8),
       ("cif_ippp", 41, 5, dict(paff_percent=100)), ("1080i_mbaff", 42, 6, dict(width_mbs=22, height_mbs=18))]


def md5(a):
    return hashlib.md5(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_streams():
    out = []
    for name, seed, n, *over in MIX:
        g = h.synth(name, seed=seed, num_pictures=n, **(over[0] if over else {}))
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


@pytest.mark.parametrize("lanes", [1, 0])
def test_server_results_equal_alone_and_in_the_mix(lanes):
    """lanes 1: every stream in one chain of batches, which must hold pictures
    of several streams; 0: the default lanes (streams split by id)."""
    import torch
    streams = make_streams()
    ref = alone(streams)
    dpb = [R.CStreamCfg(p[0].width_mbs, p[0].height_mbs, slots, 0) for p, slots in streams]
    sizes = [h.lib().h264r_stream_dpb_bytes(c) for c in dpb]
    budget = max(sizes) + sorted(sizes)[len(sizes) // 2]  # a 1080p DPB and a bit more
    window = 3
    with h.Context(0, dpb_budget_bytes=budget) as ctx, h.Server(ctx, queue_depth=window, lanes=lanes) as srv:
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
    if lanes == 1:
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


def test_server_fed_by_parser_threads_matches_reference():
    """A host parser thread per stream, as the reference runs its decoder on a
    thread of its own (SDH264Player/MyVideoPlayer.cpp:126-169): each thread
    parses one of the writer's bitstreams and pushes every picture as soon as
    its records are complete; the server batches the streams' pictures
    together.  Every decoded picture equals the reference decoder's own
    planes of that stream (tests/golden/writer_streams.json)."""
    import json
    import os
    import threading

    import torch

    from h264_video_decoder_demo_gb300.engine import GroupTracker, Parser
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "writer_streams.json")) as f:
        cases = json.load(f)["cases"]
    names = ["cif_ippp", "cif_ippp_2slices_pcm", "1080p_default_wp_b1", "1080p_high_gop5_3slices"]
    datas = []
    for nm in names:
        cfg = dict(cases[nm]["writer"])
        seed = cfg.pop("seed")
        datas.append(h.write_stream(None, seed=seed, **cfg))
    window = 4
    got = [dict() for _ in names]
    errors = []
    with h.Context(0) as ctx, h.Server(ctx, queue_depth=window) as srv:
        lock = threading.Lock()
        pending = {}
        outs = {}

        def parser_thread(i):
            try:
                p = Parser()
                groups = GroupTracker()
                sid = None
                k = 0

                def push(pic):
                    nonlocal sid, k
                    if sid is None:
                        sid = srv.open(pic.width_mbs, pic.height_mbs, p.geometry()[2])
                        with lock:
                            pending[sid] = 0
                    while pending[sid] >= window:
                        time.sleep(0.0002)
                    buf = torch.empty(pic.plane_bytes, dtype=torch.uint8, pin_memory=True).numpy()
                    with lock:
                        outs[(sid, k)] = (i, buf)
                        pending[sid] += 1
                    assert srv.push(sid, pic, groups.next(pic), k, buf) == 0
                    k += 1

                data = datas[i]
                for off in range(0, len(data), 1 << 16):  # the bytes arrive in pieces
                    p.feed(data[off:off + (1 << 16)])
                    while True:
                        r = p.next()
                        if r is None:
                            break
                        push(r[0])
                p.end()
                while True:
                    r = p.next()
                    if r is None:
                        break
                    push(r[0])
                srv.end(sid)
                p.close()
            except Exception as exc:  # reported below
                errors.append(exc)

        threads = [threading.Thread(target=parser_thread, args=(i,)) for i in range(len(names))]
        for t in threads:
            t.start()
        total = sum(len(c["pictures"]) + 1 for c in (cases[n] for n in names))
        done = 0
        deadline = time.perf_counter() + 120
        while done < total and not errors:
            assert time.perf_counter() < deadline, "server made no progress"
            for sid, tag, status, lat in srv.poll(wait_ms=2):
                assert status == 0
                with lock:
                    i, buf = outs.pop((sid, tag))
                    pending[sid] -= 1
                got[i][tag] = md5(buf)
                done += 1
        for t in threads:
            t.join()
        st = srv.stats()
    assert not errors, errors[0]
    assert st["pictures_done"] == total and st["streams_done"] == len(names)
    for i, nm in enumerate(names):
        c = cases[nm]
        want = [pic["post_md5"] for pic in c["pictures"]]  # decoding order, deblocked
        n = len(want) + 1
        assert sorted(got[i]) == list(range(n))
        assert [got[i][k] for k in range(n - 1)] == want, nm
        # the last picture is output without deblocking
        last_poc = [f for f in c["frames"] if f["yuv_md5"] == got[i][n - 1]]
        assert last_poc, "%s: last picture differs from the reference's output" % nm


def test_batches_on_a_callers_stream_match_oracle():
    """h264r_submit_batch_device_on / h264r_output_async_on (what the server's
    lanes use): the pictures of two streams batched per dependency group on
    one CUDA stream of the caller's, with no ordering through the streams' own
    CUDA streams, and every frame copied out on a second one; a slot rewritten
    by a later batch waits for its copy.  Every frame equals the oracle's."""
    import ctypes

    import torch

    from oracle_cpu import OracleDPB
    gens = [h.synth("cif_ippp", seed=s, num_pictures=14, gop_kind=1, gop_length=14) for s in (21, 22)]  # slots reused
    pics = [list(g) for g in gens]
    slots = [g.dpb_slots for g in gens]
    dev = torch.device("cuda", 0)
    keep = []

    def to_dev(p):
        c = p.to_c()
        for name in R.Picture._ARRAYS:
            a = np.ascontiguousarray(getattr(p, name)).view(np.uint8).reshape(-1)
            t = torch.from_numpy(a.copy()).to(dev) if a.size else torch.empty(1, dtype=torch.uint8, device=dev)
            keep.append(t)
            setattr(c, name, t.data_ptr())
        return c

    L = h.engine.lib()
    with h.Context(0) as ctx:
        streams = [h.Stream(ctx, ps[0].width_mbs, ps[0].height_mbs, sl) for ps, sl in zip(pics, slots)]
        cp = [[to_dev(p) for p in ps] for ps in pics]
        torch.cuda.synchronize()
        lane, copy = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
        for st in streams:  # the buffer clear queued at open, before the lane
            ev = torch.cuda.Event()
            ev.record(torch.cuda.ExternalStream(st.cuda_stream(), device=dev))
            lane.wait_event(ev)
        outs = {}
        for g in range(max(p.group for ps in pics for p in ps) + 1):
            items = [(i, k, p) for i, ps in enumerate(pics) for k, p in enumerate(ps) if p.group == g]
            n = len(items)
            arr = (ctypes.c_void_p * n)(*[streams[i].h.value for i, _, _ in items])
            pa = (R.CPicture * n)(*[cp[i][k] for i, k, _ in items])
            assert L.h264r_submit_batch_device_on(ctx.h, ctypes.c_void_p(lane.cuda_stream), n, arr, pa) == 0
            ev = torch.cuda.Event()
            ev.record(lane)
            copy.wait_event(ev)
            for i, k, p in items:
                buf = torch.empty(p.plane_bytes, dtype=torch.uint8, pin_memory=True).numpy()
                y, wh = buf.ctypes.data, p.width_mbs * p.height_mbs * 256
                assert L.h264r_output_async_on(streams[i].h, p.dst_slot, y, y + wh, y + wh + wh // 4,
                                               ctypes.c_void_p(copy.cuda_stream)) == 0
                outs[(i, k)] = buf
        copy.synchronize()
        lane.synchronize()
        for st in streams:
            st.close()
    for i, ps in enumerate(pics):
        dpb = OracleDPB(ps[0].width_mbs, ps[0].height_mbs, slots[i])
        for k, p in enumerate(ps):
            rc, _ = dpb.reconstruct(p)
            assert rc == 0
            assert np.array_equal(outs[(i, k)], dpb.planes(p.dst_slot)), "stream %d picture %d" % (i, k)
