"""CABAC tables and arithmetic decoding engine of the host front end against
the reference decoder's own (CPU; skipped where the reference is not built
here, oracle/_ref/libref_probe.so):

  - the context initialisation values (m, n) of Tables 9-12 to 9-33 for I
    slices and every cabac_init_idc, over every ctxIdx the parser uses
    (CH264Cabac::get_m_and_n, H264Cabac.cpp:36);
  - one DecodeDecision (9.3.3.2.1, rangeTabLPS and the state transitions of
    Tables 9-44 / 9-45) from every context state, both MPS values, every
    range quarter and offsets on both sides of the LPS boundary
    (CH264Cabac::DecodeDecision, H264Cabac.cpp:2577).
Record-for-record equality of whole CABAC streams is in tests/test_parser.py.
"""
import ctypes
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
PROBE = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libref_probe.so")


@pytest.fixture(scope="module")
def probe():
    if not os.path.exists(PROBE):
        pytest.skip("the reference is not built here (oracle/_ref)")
    return ctypes.CDLL(PROBE)


def test_context_initialisation_table_matches_reference(engine_lib, probe):
    mine, ref = (ctypes.c_int * 2)(), (ctypes.c_int * 2)()
    for model in range(4):
        for slice_type in ((2,) if model == 0 else (0, 1)):
            idc = 0 if model == 0 else model - 1
            for ctx in range(460):
                assert engine_lib.h264r_probe_cabac_init(model, ctx, mine) == 0
                if probe.ref_probe_cabac_mn(ctx, slice_type, idc, ref) != 0:
                    continue  # a context the reference does not define for this slice type
                assert (mine[0], mine[1]) == (ref[0], ref[1]), (model, slice_type, ctx)


def test_decision_engine_matches_reference(engine_lib, probe):
    mine, ref = (ctypes.c_int * 5)(), (ctypes.c_int * 5)()
    for state in range(63):
        for mps in (0, 1):
            for q in range(4):
                rng = 256 + 64 * q + 17
                # every offset from below the largest LPS range to the top,
                # and some below (every LPS boundary is crossed)
                for off in [0, 1, rng // 4] + list(range(max(0, rng - 260), rng)):
                    assert engine_lib.h264r_probe_cabac_decision(state, mps, rng, off, mine) == 0
                    assert probe.ref_probe_cabac_decision(state, mps, rng, off, ref) == 0
                    assert list(mine) == list(ref), (state, mps, rng, off)
