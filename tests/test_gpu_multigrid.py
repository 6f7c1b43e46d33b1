"""Multigrid batches on the device beyond the per-cell parity of
test_gpu_parity.py: the iteration graph holds the coarse levels' launches,
the mixed-precision cycle converges to the FP64 one, and a batch whose
solves differ in their multigrid schedule is refused."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from aither_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _bump(path, **kw):
    from aither_gb300 import cases
    args = dict(ni=24, nj=12, nk=4, height=0.08, mach=0.7, multigrid=(3, "W"))
    args.update(kw)
    inp, _ = cases.bump_channel(str(path), **args)
    return inp


def test_multigrid_launches_and_mixed_convergence(ctx, tmp_path):
    """A W cycle over three levels: more kernel launches per iteration than
    the same batch without multigrid (the coarse levels' residual, sweeps
    and transfers), and the mixed-precision cycle's state after 300
    iterations within 1e-6 of the FP64 cycle's."""
    from aither_gb300 import PREC_FP64, PREC_MIXED, Batch, Setup
    s = Setup(_bump(tmp_path / "mg"))
    s1 = Setup(_bump(tmp_path / "one", multigrid=None))
    b1 = Batch(ctx, s1, PREC_FP64)
    b1.iterate(2)
    n1 = b1.stats().kernel_launches / 2
    b1.close()
    out = {}
    for prec in (PREC_FP64, PREC_MIXED):
        b = Batch(ctx, s, prec)
        norms = b.iterate(300)
        assert all(x.status == 0 for x in norms)
        if prec == PREC_FP64:
            assert b.stats().kernel_launches / 300 > n1
            l2 = np.array([sum(v * v for v in n.l2[:5]) ** 0.5 for n in norms])
            assert l2[-1] < 1e-3 * l2[0]
        out[prec] = b.field(0, "STATE")
        b.close()
    assert rel_err(out[PREC_MIXED], out[PREC_FP64]) <= 1e-6


def test_batch_refuses_mixed_multigrid_schedules(ctx, tmp_path):
    from aither_gb300 import PREC_FP64, AthError, Batch, Setup
    s = Setup([_bump(tmp_path / "a"), _bump(tmp_path / "b", multigrid=(2, "V"))])
    with pytest.raises(AthError, match="multigrid"):
        Batch(ctx, s, PREC_FP64)
