"""Picture geometries at the edges of the wavefront kernels, against the CPU
oracle: one MB wide or tall, a single MB, MBAFF pairs one pair wide, the
largest width and height a stream accepts (512 MBs), a 3840x2160 picture, and
degenerate pictures batched together in one launch.  Also the batch entry
points' argument checks (empty and oversized batches)."""
import ctypes

import numpy as np
import pytest

from test_gpu_parity import run_against_oracle

import h264_video_decoder_demo_gb300 as h
from h264_video_decoder_demo_gb300.engine import lib

# every tool of the 1080p configuration, on small pictures
SMALL = dict(num_pictures=6, gop_length=6, gop_kind=1, num_refs=2, transform8x8=1, weighted=1, min_partition=3,
             intra_percent=30, skip_percent=10, edge_mv_percent=30, mv_range=96, filter_offset_max=6, coef_density=50)


@pytest.mark.gpu
@pytest.mark.parametrize("w,hgt", [(1, 1), (1, 6), (6, 1), (2, 3), (3, 17), (17, 3)])
def test_degenerate_sizes_match_oracle(gpu_ctx, w, hgt):
    g = h.synth("1080p_high", seed=300 + 7 * w + hgt, width_mbs=w, height_mbs=hgt, **SMALL)
    assert run_against_oracle(gpu_ctx, g) == SMALL["num_pictures"]


@pytest.mark.gpu
@pytest.mark.parametrize("w,hgt", [(1, 2), (3, 4)])
def test_degenerate_mbaff_sizes_match_oracle(gpu_ctx, w, hgt):
    g = h.synth("1080i_mbaff", seed=400 + w, width_mbs=w, height_mbs=hgt, num_pictures=5, gop_length=5, num_refs=2,
                field_percent=50, intra_percent=30, mv_range=64)
    assert run_against_oracle(gpu_ctx, g) == 5


@pytest.mark.gpu
@pytest.mark.parametrize("w,hgt", [(512, 64), (64, 512)])
def test_largest_stream_width_and_height_match_oracle(gpu_ctx, w, hgt):
    """512 MBs is the widest / tallest picture h264r_stream_open accepts."""
    g = h.synth("1080p_high", seed=500 + w, width_mbs=w, height_mbs=hgt, num_pictures=3, gop_length=3, gop_kind=0,
                num_refs=1, intra_percent=20, edge_mv_percent=10, mv_range=256, coef_density=30)
    assert run_against_oracle(gpu_ctx, g) == 3


@pytest.mark.gpu
def test_uhd_picture_matches_oracle(gpu_ctx):
    g = h.synth("1080p_high", seed=600, width_mbs=240, height_mbs=135, num_pictures=3, gop_length=3, gop_kind=1)
    assert run_against_oracle(gpu_ctx, g) == 3


@pytest.mark.gpu
def test_degenerate_sizes_batched_together(gpu_ctx):
    """Pictures of six degenerate sizes, one per stream, in one launch per
    dependency step; each stream against its own oracle DPB."""
    from oracle_cpu import OracleDPB
    sizes = [(1, 1), (1, 6), (6, 1), (2, 3), (3, 17), (17, 3)]
    gens = [list(h.synth("1080p_high", seed=700 + i, width_mbs=w, height_mbs=hh, **SMALL)) for i, (w, hh) in enumerate(sizes)]
    slots = 8
    streams = [h.Stream(gpu_ctx, w, hh, slots) for w, hh in sizes]
    dpbs = [OracleDPB(w, hh, slots) for w, hh in sizes]
    try:
        for k in range(SMALL["num_pictures"]):
            pics = [g[k] for g in gens]
            gpu_ctx.submit_batch(streams, pics)
            gpu_ctx.sync()
            for s, d, p in zip(streams, dpbs, pics):
                rc, _ = d.reconstruct(p)
                assert rc == 0
                assert np.array_equal(s.output(p.dst_slot), d.planes(p.dst_slot)), (p.width_mbs, p.height_mbs, k)
    finally:
        for s in streams:
            s.close()


@pytest.mark.gpu
def test_batch_argument_checks(gpu_ctx):
    L = lib()
    empty_streams = (ctypes.c_void_p * 1)()
    empty_pics = (h.records.CPicture * 1)()
    assert L.h264r_submit_batch(gpu_ctx.h, 0, empty_streams, empty_pics) == -1
    assert L.h264r_submit_batch_device(gpu_ctx.h, 0, empty_streams, empty_pics) == -1
    n = L.h264r_ctx_max_batch(gpu_ctx.h) + 1
    many_streams = (ctypes.c_void_p * n)()
    many_pics = (h.records.CPicture * n)()
    assert L.h264r_submit_batch(gpu_ctx.h, n, many_streams, many_pics) < 0
    # a stream wider than the engine's limit is refused at open
    with pytest.raises(h.EngineError):
        h.Stream(gpu_ctx, 513, 4, 4)


@pytest.mark.gpu
@pytest.mark.parametrize("slice_rows,cip", [(1, 0), (3, 0), (2, 100), (0, 100)])
def test_slices_and_constrained_intra_match_oracle(gpu_ctx, slice_rows, cip):
    """Several slices per picture (their own QP and filter offsets, deblocking
    modes 0, 1 and 2) and constrained intra prediction: intra neighbour
    availability and the deblocking edges at slice boundaries."""
    g = h.synth("1080p_high", seed=800 + 7 * slice_rows + cip, width_mbs=20, height_mbs=12, num_pictures=8,
                gop_length=8, gop_kind=1, num_refs=2, intra_percent=40, filter_offset_max=6,
                slice_rows=slice_rows, cip_percent=cip)
    assert run_against_oracle(gpu_ctx, g) == 8


@pytest.mark.gpu
def test_mbaff_slices_and_constrained_intra_match_oracle(gpu_ctx):
    g = h.synth("1080i_mbaff", seed=900, width_mbs=12, height_mbs=8, num_pictures=5, gop_length=5, num_refs=2,
                field_percent=50, intra_percent=30, slice_rows=2, cip_percent=100)
    assert run_against_oracle(gpu_ctx, g) == 5


@pytest.mark.gpu
def test_output_async_copies_survive_slot_reuse(gpu_ctx):
    """h264r_output_async copies on the stream's copy stream while the stream
    goes on reconstructing; a later picture that reuses a slot waits for the
    slot's copy.  Twelve pictures submitted back to back, each copied out
    right after its submission, one sync at the end: every copy equals the
    oracle's picture."""
    import torch
    from oracle_cpu import OracleDPB
    w, hh = 20, 12
    g = h.synth("1080p_high", seed=950, width_mbs=w, height_mbs=hh, num_pictures=12, gop_length=12, gop_kind=1,
                num_refs=2, intra_percent=20)
    pics = list(g)
    slots = g.dpb_slots
    s = h.Stream(gpu_ctx, w, hh, slots)
    d = OracleDPB(w, hh, slots)
    n = w * 16 * hh * 16 * 3 // 2
    outs = [torch.empty(n, dtype=torch.uint8, pin_memory=True).numpy() for _ in pics]
    expected = []
    try:
        for k, p in enumerate(pics):
            s.submit(p)
            s.output_async(p.dst_slot, outs[k])
            rc, _ = d.reconstruct(p)
            assert rc == 0
            expected.append(d.planes(p.dst_slot).copy())
        s.sync()
        for k in range(len(pics)):
            assert np.array_equal(outs[k], expected[k]), k
    finally:
        s.close()


@pytest.mark.gpu
def test_reset_stream_decodes_like_a_new_one(gpu_ctx):
    """h264r_stream_reset clears the picture buffers as h264r_stream_open
    does: a P picture decoded first after a reset reads cleared references,
    exactly as on a freshly opened stream (not the pictures decoded before)."""
    g = h.synth("cif_ippp", seed=77, num_pictures=4, gop_length=4, gop_kind=0, intra_percent=0, skip_percent=0)
    pics = list(g)
    p = next(q for q in pics if q.group > 0)
    fresh = h.Stream(gpu_ctx, p.width_mbs, p.height_mbs, g.dpb_slots)
    fresh.submit(p)
    want = fresh.output(p.dst_slot).copy()
    fresh.close()
    s = h.Stream(gpu_ctx, p.width_mbs, p.height_mbs, g.dpb_slots)
    for q in pics:
        s.submit(q)
    s.sync()
    stale = s.output(p.dst_slot).copy()
    s.reset()
    s.submit(p)
    got = s.output(p.dst_slot).copy()
    s.close()
    assert not np.array_equal(stale, want), "the P picture does not depend on its reference"
    assert np.array_equal(got, want)
