"""Full-size configurations on the CPU oracle against the reference: the
256x192x4 SST-2003 flat plate (WENO, AUSMPW+, block LU-SGS), one iteration.
The fixture keeps the per-cell fields of the 16 cells nearest the wall in
every column and per-variable sums of |value| over all cells
(tests/golden/make_golden.py ROWCASES)."""
import numpy as np
import pytest

from conftest import load_golden, rel_err
from refcases_common import cols_err, fixture_fields

TOL = 1e-13


def c3_setup(tmp):
    import ast

    from aither_gb300 import Setup, cases
    g = load_golden("sst_c3_it1")
    inp, _ = cases.sst_plate(str(tmp), name="sst_c3", **ast.literal_eval(str(g["kwargs"])))
    return g, Setup(inp)


def abssum(a):
    a = np.asarray(a)
    return np.abs(a).reshape(a.shape[0] * a.shape[1] * a.shape[2], -1).sum(0)


def test_oracle_full_sst_plate_one_iteration(tmp_path):
    from pyoracle import Oracle
    g, s = c3_setup(tmp_path)
    o = Oracle(s)
    l2 = o.iterate(1)
    for key, f in (("state", "STATE"), ("resid", "RESID"), ("du", "DU"), ("dt", "DT"),
                   ("specrad", "SPECRAD")):
        full = o.field(0, f)
        if key == "dt":
            full = full[..., 0]
        a, ref = fixture_fields(g, 0, key, full)
        assert cols_err(a, ref) <= TOL, key
        assert rel_err(abssum(full), g[f"b0_{key}_abssum"]) <= 1e-12, key
    assert rel_err(l2[:, 0, :], g["l2"]) <= TOL
    o.close()
