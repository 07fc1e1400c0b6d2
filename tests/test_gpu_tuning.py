"""GPU: launch shapes, captured launch graphs and the autotuner.

Decoded samples must not depend on how a launch sequence is shaped or
launched: every k_inter block size (2, 4, 8 MBs), every frame-deblocking
block size (4, 8 MB-row pairs), with and without graph replay, must give the
oracle's pictures byte for byte.  All calls go through the C ABI.
"""
import numpy as np
import pytest

import h264_video_decoder_demo_gb300 as h
from h264_video_decoder_demo_gb300 import records as R
from oracle_cpu import OracleDPB

pytestmark = pytest.mark.gpu

SHAPES = [(iw, dw, g) for g in (0, 1) for iw in (2, 4, 8) for dw in (4, 8)]


@pytest.fixture(scope="module")
def mixed_workload():
    """CIF, 720p and 1080p streams (6 pictures each) with the oracle's planes
    of every picture, and the dependency-group batches that mix them."""
    specs = [("cif_ippp", 61, 6), ("720p_high", 62, 6), ("1080p_high", 63, 6)]
    pics, slots, expect = [], [], []
    for name, seed, n in specs:
        g = h.synth(name, seed=seed, num_pictures=n)
        ps = list(g)
        slots.append(g.dpb_slots)
        g.close()
        o = OracleDPB(ps[0].width_mbs, ps[0].height_mbs, slots[-1])
        planes = []
        for p in ps:
            rc, _ = o.reconstruct(p)
            assert rc == 0
            planes.append(o.planes(p.dst_slot).copy())
        pics.append(ps)
        expect.append(planes)
    batches = []
    cursor = [0] * len(specs)
    while any(c < len(p) for c, p in zip(cursor, pics)):
        grp = []
        for i, ps in enumerate(pics):
            if cursor[i] >= len(ps):
                continue
            g0 = ps[cursor[i]].group
            while cursor[i] < len(ps) and ps[cursor[i]].group == g0:
                grp.append((i, cursor[i]))
                cursor[i] += 1
        batches.append(grp)
    return pics, slots, expect, batches


def _decode_mixed(ctx, work, repeats=1):
    pics, slots, expect, batches = work
    streams = [h.Stream(ctx, ps[0].width_mbs, ps[0].height_mbs, sl) for ps, sl in zip(pics, slots)]
    try:
        for _ in range(repeats):
            for grp in batches:
                ctx.submit_batch([streams[i] for i, _ in grp], [pics[i][k] for i, k in grp])
                for i, k in grp:
                    out = streams[i].output(pics[i][k].dst_slot)
                    assert np.array_equal(out, expect[i][k]), "stream %d picture %d differs from the oracle" % (i, k)
    finally:
        for s in streams:
            s.close()


@pytest.mark.parametrize("iw,dw,graphs", SHAPES)
def test_every_launch_shape_matches_oracle(engine_lib, mixed_workload, iw, dw, graphs):
    ctx = h.Context(0)
    try:
        ctx.set_tuning(iw, dw, graphs=bool(graphs))
        assert ctx.tuning() == {"inter_mbs_per_cta": iw, "deblock_pairs_per_cta": dw, "graphs": graphs}
        # with graphs, repeat so that launch buffers see their shapes again
        _decode_mixed(ctx, mixed_workload, repeats=3 if graphs else 1)
        replays, captured = ctx.graph_counts()
        if not graphs:
            assert replays == 0 and captured == 0
    finally:
        ctx.close()


def _synth_cif(seed):
    return h.synth("cif_ippp", seed=seed)


def _synth_cif_mbaff(seed):
    # MBAFF frames: k_bs in line and the MBAFF deblocking kernel in the graph
    return h.synth("cif_ippp", seed=seed, num_pictures=8, mbaff=1, field_percent=50, gop_kind=1, num_refs=2,
                   transform8x8=1, mv_range=128, edge_mv_percent=10)


@pytest.mark.parametrize("make", [_synth_cif, _synth_cif_mbaff], ids=["frame", "mbaff"])
def test_graph_replay_per_picture_matches_oracle(engine_lib, make):
    """One CIF stream, one picture per launch, decoded three times over: the
    per-stream launch buffers see each shape again and replay graphs; every
    picture equals the oracle's."""
    g = make(64)
    ps = list(g)
    slots = g.dpb_slots
    g.close()
    o = OracleDPB(ps[0].width_mbs, ps[0].height_mbs, slots)
    expect = []
    for p in ps:
        assert o.reconstruct(p)[0] == 0
        expect.append(o.planes(p.dst_slot).copy())
    ctx = h.Context(0)
    s = h.Stream(ctx, ps[0].width_mbs, ps[0].height_mbs, slots)
    try:
        ctx.set_tuning(4, 8, graphs=True)
        launches0 = ctx.kernel_launches()
        for rep in range(3):
            for k, p in enumerate(ps):
                s.submit(p)
                assert np.array_equal(s.output(p.dst_slot), expect[k]), "repeat %d picture %d" % (rep, k)
        replays, captured = ctx.graph_counts()
        assert captured >= 1 and replays >= captured
        # replayed sequences count their kernels like direct launches
        assert ctx.kernel_launches() - launches0 >= 3 * 2 * len(ps)
    finally:
        s.close()
        ctx.close()


def test_autotuner_keeps_a_valid_shape_per_mix(engine_lib):
    """h264r_autotune_batch_device on a batch of device-resident 720p
    pictures: returns one of the launch shapes, stores it for that geometry
    mix only, and decoding under it still equals the oracle."""
    import torch

    dev = torch.device("cuda", 0)
    g = h.synth("720p_high", seed=65, num_pictures=4)
    ps = list(g)
    slots = g.dpb_slots
    g.close()
    ctx = h.Context(0)
    streams = [h.Stream(ctx, ps[0].width_mbs, ps[0].height_mbs, slots) for _ in range(2)]
    keep = []
    try:
        def dev_pic(p):
            c = p.to_c()
            for name in R.Picture._ARRAYS:
                a = np.ascontiguousarray(getattr(p, name)).view(np.uint8).reshape(-1)
                t = torch.from_numpy(a.copy()).to(dev) if a.size else torch.empty(1, dtype=torch.uint8, device=dev)
                keep.append(t)
                setattr(c, name, t.data_ptr())
            return c
        cps = [dev_pic(p) for p in ps]
        # the first picture (an I picture) of two streams: a batch that can run again
        best, ms = ctx.autotune_batch_device(streams, [cps[0], cps[0]], reps=3)
        assert (best["inter_mbs_per_cta"], best["deblock_pairs_per_cta"], best["graphs"]) in SHAPES
        assert ms > 0
        assert ctx.tuning([cps[0], cps[0]]) == best
        assert ctx.tuning() == {"inter_mbs_per_cta": 4, "deblock_pairs_per_cta": 8, "graphs": 0}
        assert ctx.tuning([cps[0]]) == ctx.tuning()
        # decode both streams in order under the tuned shape
        o = OracleDPB(ps[0].width_mbs, ps[0].height_mbs, slots)
        for c, p in zip(cps, ps):
            assert ctx.submit_batch_device(streams, [c, c]) == 0
            assert o.reconstruct(p)[0] == 0
            ref = o.planes(p.dst_slot)
            for s in streams:
                assert np.array_equal(s.output(p.dst_slot), ref)
    finally:
        for s in streams:
            s.close()
        ctx.close()


def test_tuning_rejects_unknown_shapes(engine_lib):
    ctx = h.Context(0)
    try:
        for iw, dw in [(3, 8), (16, 8), (4, 2), (4, 16), (-1, 8)]:
            with pytest.raises(h.EngineError) as e:
                ctx.set_tuning(iw, dw)
            assert e.value.code == R.ERR_INVALID_ARG
        assert ctx.tuning() == {"inter_mbs_per_cta": 4, "deblock_pairs_per_cta": 8, "graphs": 0}
        ctx.set_tuning(0, 0, graphs=True)  # 0 selects the default shapes
        assert ctx.tuning() == {"inter_mbs_per_cta": 4, "deblock_pairs_per_cta": 8, "graphs": 1}
        # a kept choice for one geometry mix (one CIF picture) leaves other mixes alone
        g = h.synth("cif_ippp", seed=66, num_pictures=1)
        p = next(iter(g))
        c = p.to_c()
        ctx.set_mix_tuning([c], 2, 4, graphs=False)
        assert ctx.tuning([c]) == {"inter_mbs_per_cta": 2, "deblock_pairs_per_cta": 4, "graphs": 0}
        assert ctx.tuning([c, c]) == ctx.tuning()
        with pytest.raises(h.EngineError):
            ctx.set_mix_tuning([c], 5, 8)
        g.close()
    finally:
        ctx.close()


def test_prepared_batches_match_oracle(engine_lib, mixed_workload):
    """Batch arguments built once (Context.prepare_batch) and submitted on
    every pass, as the end-to-end benchmark does: each pass re-validates,
    packs and uploads the records; every picture of both passes equals the
    oracle's."""
    pics, slots, expect, batches = mixed_workload
    ctx = h.Context(0)
    streams = [h.Stream(ctx, ps[0].width_mbs, ps[0].height_mbs, sl) for ps, sl in zip(pics, slots)]
    try:
        prepared = [(ctx.prepare_batch([streams[i] for i, _ in grp], [pics[i][k] for i, k in grp]), grp)
                    for grp in batches]
        for rep in range(2):
            for prep, grp in prepared:
                ctx.submit_prepared(prep)
                for i, k in grp:
                    out = streams[i].output(pics[i][k].dst_slot)
                    assert np.array_equal(out, expect[i][k]), "pass %d stream %d picture %d" % (rep, i, k)
    finally:
        for s in streams:
            s.close()
        ctx.close()
