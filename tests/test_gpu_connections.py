"""Interblock connections in every patch orientation on the GPU (FP64),
through the C ABI: against the reference's fixtures where the reference is
self-consistent, against the oracle in every orientation, and the residual's
independence of the second block's indexing (tests/test_connections.py
states the cases and why the reference is checked by invariance only in
some orientations).

Tolerances (relative, flow variables on one scale, k and omega each on its
own): 1e-12 per cell after one iteration; after ten, 1e-12 for the state
and 1e-10 for the residual and update (differences of large fluxes, as in
tests/test_gpu_parity.py).
"""
import numpy as np
import pytest

from conftest import golden_case, set_states
from test_connections import INV_TOL, REF_CONSISTENT, _cols_err, to_aligned

pytestmark = pytest.mark.gpu

CELL_TOL = 1e-12
NORM_TOL = 1e-10


@pytest.fixture(scope="module")
def ctx():
    from aither_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _batch(ctx, inp, st):
    from aither_gb300 import Batch, Setup
    s = Setup(inp)
    set_states(s, st)
    return s, Batch(ctx, s)


@pytest.mark.parametrize("name", [f"pair_{ph}_o{o}_it{n}" for ph, os_ in REF_CONSISTENT.items()
                                  for o in os_ for n in (1, 10)])
def test_gpu_matches_reference_on_orientation(ctx, name, tmp_path):
    inp, st, g = golden_case(name, str(tmp_path))
    _, b = _batch(ctx, inp, st)
    n = int(g["iterations"])
    norms = b.iterate(n)
    tol = CELL_TOL if n == 1 else NORM_TOL
    for k in range(2):
        p = f"b{k}_"
        assert _cols_err(b.field(k, "STATE"), g[p + "state"]) <= CELL_TOL
        assert _cols_err(b.field(k, "RESID"), g[p + "resid"]) <= tol
        assert _cols_err(b.field(k, "DU"), g[p + "du"]) <= tol
    nv = g["l2"].shape[1]
    l2 = np.array([[x.l2[v] for v in range(nv)] for x in norms])
    assert np.abs(l2 - g["l2"]).max() / np.abs(g["l2"]).max() <= NORM_TOL
    b.close()


@pytest.mark.parametrize("physics", ["euler", "ns", "sst"])
@pytest.mark.parametrize("orient", range(8))
def test_gpu_matches_oracle_in_every_orientation(ctx, physics, orient, tmp_path):
    from aither_gb300 import Setup, cases
    from pyoracle import Oracle
    inp, st = cases.block_pair(str(tmp_path), orient=orient, physics=physics, name="pair")
    s, b = _batch(ctx, inp, st)
    b.iterate(10)
    so = Setup(inp)
    set_states(so, st)
    o = Oracle(so)
    o.iterate(10)
    for k in range(2):
        assert _cols_err(b.field(k, "STATE"), o.field(k, "STATE")) <= CELL_TOL
        assert _cols_err(b.field(k, "RESID"), o.field(k, "RESID")) <= NORM_TOL
        assert _cols_err(b.field(k, "DU"), o.field(k, "DU")) <= NORM_TOL
    o.close()
    b.close()


@pytest.mark.parametrize("physics", ["euler", "sst"])
def test_gpu_residual_independent_of_block_orientation(ctx, physics, tmp_path):
    from aither_gb300 import cases
    ref = None
    for orient in range(8):
        inp, st = cases.block_pair(str(tmp_path / f"o{orient}"), orient=orient, physics=physics,
                                   name="pair")
        _, b = _batch(ctx, inp, st)
        b.iterate(1)
        a = [b.field(0, "RESID"), to_aligned(b.field(1, "RESID"), orient)]
        b.close()
        if ref is None:
            ref = a
            continue
        for k in range(2):
            assert _cols_err(a[k], ref[k]) <= INV_TOL, (orient, k)
