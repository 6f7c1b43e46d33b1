"""The reference's own test cases on the CPU: the oracle against the
reference build's fixtures, and both against the reference's regression
truth table (testCases/regressionTests.py).

Cases: uniformFlow (SST, ten blocks joined in all 8 patch orientations),
subsonicCylinder (Euler, stagnation inlet and pressure outlet),
multiblockCylinder (two blocks, AUSMPW+), couette (periodic, moving
isothermal walls), viscousFlatPlate (laminar), rae2822 (SST airfoil on a
C-grid whose wake cut is a connection of the block with itself) and
shockTube (bdf2 dual time, WENO, two blocks).

Tolerances: 1e-13 relative per cell (the oracle restates the reference
operation by operation); uniformFlow on physical scales (see
refcases_common.uniform_flow_errors); the regression table at its own 1 %.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import REF_SRC, ROOT, rel_err
from refcases_common import (FIXTURES, TRUTH, case_input, cols_err, copy_case, fixture,
                             fixture_fields, have_case, resid_row, truth_failures,
                             uniform_flow_errors)

TOL = 1e-13
REF_AITHER = os.path.join(ROOT, "oracle", "_ref", "aither")


def _oracle(inp):
    from aither_gb300 import Setup
    from pyoracle import Oracle
    s = Setup(inp)
    return s, Oracle(s)


@pytest.mark.parametrize("case,n", [(c, n) for c, ns in FIXTURES for n in ns])
def test_oracle_matches_reference_case(case, n):
    if not have_case(case):
        pytest.skip("reference test cases not copied to this machine")
    g = fixture(case, n)
    s, o = _oracle(case_input(case))
    nl = max(1, s.solve_view(0).nl_iters)
    l2 = o.iterate(n * nl)
    for b in range(int(g["nblocks"])):
        for key, f in (("state", "STATE"), ("resid", "RESID"), ("du", "DU"), ("dt", "DT")):
            a, ref = fixture_fields(g, b, key, o.field(b, f))
            if case == "uniformFlow" and key in ("state", "resid", "du"):
                flow, turb = uniform_flow_errors(a, ref, key)
                assert flow <= 1e-14, (b, key, flow)
                if n == 1:
                    assert turb <= 1e-6, (b, key, turb)
            elif case == "uniformFlow":  # the time step follows k and omega
                assert cols_err(a, ref) <= (TOL if n == 1 else 1e-7), (b, key)
            else:
                assert cols_err(a, ref) <= TOL, (b, key)
    nv = g["l2"].shape[1]
    if case == "uniformFlow":
        # the k and omega equations' L2 (sources of a decaying free stream;
        # after one iteration exact, later moved by the roundoff of the flow)
        assert rel_err(l2[:, 0, 5:nv], g["l2"][:, 5:]) <= (1e-12 if n == 1 else 1e-5)
        assert float(np.abs(l2[:, 0, :5] - g["l2"][:, :5]).max()) <= 1e-14
    else:
        assert rel_err(l2[:, 0, :nv], g["l2"]) <= TOL
    o.close()


@pytest.mark.skipif(not (os.path.exists(REF_AITHER) and REF_SRC),
                    reason="reference build not available on this machine")
@pytest.mark.parametrize("case", sorted(TRUTH) + ["uniformFlow"])
def test_reference_build_reproduces_regression_truth(case, tmp_path):
    """The reference build here (oracle/ref_build, single rank) run as the
    reference's regression script runs it: the last residual row within 1 %
    of the truth table (uniformFlow: runs to completion)."""
    if not have_case(case):
        pytest.skip("reference test cases not copied to this machine")
    iters = TRUTH[case][0] if case in TRUTH else 20
    copy_case(case, str(tmp_path), iters)
    r = subprocess.run([REF_AITHER, case + ".inp"], cwd=str(tmp_path), capture_output=True,
                       text=True, env=dict(os.environ, AITHER_INSTALL_DIRECTORY=REF_SRC))
    assert r.returncode == 0, r.stderr[-2000:]
    if case in TRUTH:
        row = resid_row(str(tmp_path / f"{case}.resid"), len(TRUTH[case][1]))
        assert truth_failures(case, row) == []


@pytest.mark.parametrize("case", sorted(TRUTH))
def test_oracle_reproduces_regression_truth(case, tmp_path):
    """This build's setup and residual-history writer around the oracle:
    the same iterations, the last row of the residual file within 1 % of the
    reference's truth table."""
    if not have_case(case):
        pytest.skip("reference test cases not copied to this machine")
    from aither_gb300._lib import Norms
    iters = TRUTH[case][0]
    s, o = _oracle(case_input(case))
    nl = max(1, s.solve_view(0).nl_iters)
    l2 = o.iterate(iters * nl)[:, 0, :]
    o.close()
    rows = []
    for k in range(len(l2)):
        x = Norms()
        for v in range(l2.shape[1]):
            x.l2[v] = l2[k, v]
        rows.append(x)
    path = str(tmp_path / "r.resid")
    s.write_resid(0, path, rows, 0, np.zeros(7))
    row = resid_row(path, len(TRUTH[case][1]))
    assert truth_failures(case, row) == []
