"""Full-size configurations on the GPU (FP64) against the reference and the
oracle: the 256x192x4 SST-2003 flat plate after one iteration, per cell
(the 16 cells nearest the wall in every column, as the fixture keeps them)
and per-variable sums of |value| over all 196,608 cells at 1e-12 relative,
and every cell against the oracle run here at 1e-12."""
import pytest

from conftest import rel_err
from refcases_common import cols_err, fixture_fields
from test_fullsize import abssum, c3_setup

pytestmark = pytest.mark.gpu

TOL = 1e-12


def test_gpu_full_sst_plate_one_iteration(tmp_path):
    from aither_gb300 import Batch, Context
    from pyoracle import Oracle
    g, s = c3_setup(tmp_path)
    ctx = Context(0)
    b = Batch(ctx, s)
    norms = b.iterate(1)
    o = Oracle(s)
    o.iterate(1)
    for key, f in (("state", "STATE"), ("resid", "RESID"), ("du", "DU"), ("dt", "DT"),
                   ("specrad", "SPECRAD")):
        full = b.field(0, f)
        want = o.field(0, f)
        if key == "dt":
            full, want = full[..., 0], want[..., 0]
        assert cols_err(full, want) <= TOL, key
        a, ref = fixture_fields(g, 0, key, full)
        assert cols_err(a, ref) <= TOL, key
        assert rel_err(abssum(full), g[f"b0_{key}_abssum"]) <= TOL, key
    l2 = [[x.l2[v] for v in range(7)] for x in norms]
    assert rel_err(l2, g["l2"]) <= 1e-10
    o.close()
    b.close()
    ctx.close()
