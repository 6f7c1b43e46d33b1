"""Sweep shapes on the GPU: the persistent tile-queue sweep (one launch per
pass; CTAs claim (solve, hyperplane) tiles from an atomic ticket and wait
for the tiles holding their cells' swept-side neighbours) gives the same
result bit for bit as one launch per hyperplane, for scalar and block
LU-SGS, one and several sweeps, laminar and SST, single solves and batches;
and its bounded waits report ATH_ERR_TIMEOUT without faulting, leaving the
context usable."""
import numpy as np
import pytest

from conftest import golden_case, set_states

pytestmark = pytest.mark.gpu

ATH_ERR_TIMEOUT = -7


@pytest.fixture(scope="module")
def ctx():
    from aither_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _inputs(tmp, name):
    from aither_gb300 import cases
    if name == "bump_batch":
        return [cases.bump_channel(str(tmp / f"b{q}"), ni, nj, nk, h, m, name=f"b{q}")[0]
                for q, (ni, nj, nk, h, m) in enumerate([(24, 12, 6, 0.06, 0.5),
                                                         (16, 16, 8, 0.09, 0.75),
                                                         (30, 10, 4, 0.04, 0.4)])], None
    inp, st, _ = golden_case(name, str(tmp))
    return inp, st


def _run(ctx, inp, st, precision, shape, iters):
    from aither_gb300 import Batch, Setup
    s = Setup(inp)
    set_states(s, st)
    b = Batch(ctx, s, precision)
    if shape is not None:
        b.set_sweep_shape(*shape)
    b.iterate(iters)
    out = [b.field(k, "STATE") for k in range(s.counts()[1])]
    b.close()
    return out


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["bump_batch", "bump_sweeps3_it1", "plate_blusgs_sw2_it1",
                                  "sst_plate2_blusgs_it1", "sst_weno_ausm_it1",
                                  "pair_sst_o4_it1"])
def test_tile_queue_sweep_matches_per_plane_sweeps(ctx, name, precision, tmp_path):
    inp, st = _inputs(tmp_path, name)
    ref = _run(ctx, inp, st, precision, (0, 64, 0), 6)
    for tile in (32, 256):
        got = _run(ctx, inp, st, precision, (3, tile, 0), 6)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b), (name, tile)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["bump_batch", "bump_sweeps3_it1"])
def test_lane_group_and_hybrid_sweeps_match_thread_per_cell(ctx, name, precision, tmp_path):
    """Lane groups on every plane (mode 2), lane groups below a plane size
    with a thread per cell above it (mode 4; a threshold of 40 cells splits
    these grids' planes between the two), and the solves' chains run as 2
    or 4 concurrent chains, each launch chained to the previous plane's by
    programmatic dependent launch: the same result bit for bit as one chain
    with a thread per cell on every plane."""
    inp, st = _inputs(tmp_path, name)
    ref = _run(ctx, inp, st, precision, (0, 64, 0), 6)
    for shape in ((2, 32, 0), (4, 32, 40), (4, 64, 1), (2, 32, 2), (2, 64, 4), (0, 64, 4)):
        got = _run(ctx, inp, st, precision, shape, 6)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b), (name, shape)


def test_tile_queue_wait_limit_reports_timeout_and_context_survives(ctx, tmp_path):
    from aither_gb300 import Batch, Setup
    from aither_gb300._lib import AthError
    inp, _ = _inputs(tmp_path, "bump_batch")
    ref = _run(ctx, inp, None, 0, (3, 64, 0), 3)
    b = Batch(ctx, Setup(inp))
    b.set_sweep_shape(3, 64, 0)
    b.sweep_wait_test(2000, True)  # every wait polls a flag nothing sets
    with pytest.raises(AthError) as e:
        b.iterate(1)
    assert e.value.code == ATH_ERR_TIMEOUT
    b.close()
    # the context keeps working: a new batch reproduces the reference run
    got = _run(ctx, inp, None, 0, (3, 64, 0), 3)
    for a, r in zip(got, ref):
        assert np.array_equal(a, r)
