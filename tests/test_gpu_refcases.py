"""The reference's own test cases on the GPU (FP64), through the C ABI:
per-cell fields against the reference build's fixtures and the last row of
the residual history against the reference's regression truth table
(tests/test_refcases.py describes the cases; they are read from
tests/golden/refcases/, which is copied from the reference by
tests/golden/make_golden.py and skipped where absent).

Tolerances: 1e-12 relative per cell after one iteration; after twenty (or
four bdf2 time steps) 1e-12 for the state and time step and 1e-10 for the
residual and update; the L2 history 1e-10; uniformFlow on physical scales
(refcases_common.uniform_flow_errors); the truth table at its own 1 %.
"""
import numpy as np
import pytest

from conftest import rel_err
from refcases_common import (FIXTURES, TRUTH, case_input, cols_err, fixture, fixture_fields,
                             have_case, resid_row, truth_failures, uniform_flow_errors)

pytestmark = pytest.mark.gpu

CELL_TOL = 1e-12
NORM_TOL = 1e-10


# Residual and update after many iterations of turbFlatPlate (Wilcox k-omega
# 2006 at CFL 1e5 on the 137x97 grid with cells of aspect ratio ~1e3 at the
# wall): the state agrees at 1e-12, but the residual and update are small
# differences of large fluxes near convergence and carry the last-bit
# differences of pow() in Sutherland's law (CUDA against the host libm)
# amplified by the implicit coupling; 1e-9 relative to their largest
# entries.
LOOSE = {"turbFlatPlate": 1e-9}

@pytest.fixture(scope="module")
def ctx():
    from aither_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _l2(norms, nv):
    return np.array([[x.l2[v] for v in range(nv)] for x in norms])


@pytest.mark.parametrize("case,n", [(c, n) for c, ns in FIXTURES for n in ns])
def test_gpu_matches_reference_case(ctx, case, n):
    if not have_case(case):
        pytest.skip("reference test cases not copied to this machine")
    from aither_gb300 import Batch, Setup
    g = fixture(case, n)
    s = Setup(case_input(case))
    nl = max(1, s.solve_view(0).nl_iters)
    b = Batch(ctx, s)
    norms = b.iterate(n * nl)
    assert all(x.status == 0 for x in norms)
    steps = n * nl
    for k in range(int(g["nblocks"])):
        for key, f in (("state", "STATE"), ("resid", "RESID"), ("du", "DU"), ("dt", "DT")):
            a, ref = fixture_fields(g, k, key, b.field(k, f))
            if case == "uniformFlow" and key in ("state", "resid", "du"):
                flow, turb = uniform_flow_errors(a, ref, key)
                assert flow <= 1e-14, (k, key, flow)
                if n == 1:
                    assert turb <= 1e-6, (k, key, turb)
            elif case == "uniformFlow":
                assert cols_err(a, ref) <= (CELL_TOL if n == 1 else 1e-7), (k, key)
            else:
                tol = CELL_TOL if (steps == 1 or key in ("state", "dt")) else NORM_TOL
                if case in LOOSE and steps > 1 and key in ("resid", "du"):
                    tol = LOOSE[case]
                assert cols_err(a, ref) <= tol, (k, key)
    nv = g["l2"].shape[1]
    l2 = _l2(norms, nv)
    if case == "uniformFlow":
        assert rel_err(l2[:, 5:], g["l2"][:, 5:]) <= (1e-12 if n == 1 else 1e-5)
    else:
        assert rel_err(l2, g["l2"]) <= (LOOSE.get(case, NORM_TOL) if n > 1 else NORM_TOL)
    b.close()


@pytest.mark.parametrize("case", sorted(TRUTH))
def test_gpu_reproduces_regression_truth(ctx, case, tmp_path):
    """The GPU path run as the reference's regression script runs the
    reference: the same iterations, the residual history written by this
    build's writer, its last row within 1 % of the truth table."""
    if not have_case(case):
        pytest.skip("reference test cases not copied to this machine")
    from aither_gb300 import Batch, Setup
    iters = TRUTH[case][0]
    s = Setup(case_input(case))
    nl = max(1, s.solve_view(0).nl_iters)
    b = Batch(ctx, s)
    norms = list(b.iterate(iters * nl))
    b.close()
    path = str(tmp_path / "r.resid")
    s.write_resid(0, path, norms, 0, np.zeros(7))
    row = resid_row(path, len(TRUTH[case][1]))
    assert truth_failures(case, row) == []
