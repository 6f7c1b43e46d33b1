"""The allocation-free residual entry point refuses, before touching the
GPU, every solve view whose residual it does not form: it implements the
steady Euler residual with MUSCL and the Roe flux and the scalar diagonal
of lusgs/dplur, and must not hand back that arithmetic for a viscous, RANS,
block-solver, global-time-step or dual-time view (ATH_ERR_UNSUPPORTED).
These checks run on the host (no GPU needed)."""
import ctypes as C

import pytest

ATH_ERR_UNSUPPORTED = -3


def _block():
    from aither_gb300._lib import BlockDev
    b = BlockDev()
    b.ni, b.nj, b.nk, b.ng = 8, 6, 4, 2
    for name in ("W", "vol", "R", "lam", "dt", "ainv"):
        setattr(b, name, 256)
    for d in range(3):
        b.width[d] = 256
        b.farea[d] = 256
    return b


def _view(**kw):
    from aither_gb300._lib import SolveView
    v = SolveView()
    v.eqn, v.recon, v.limiter, v.flux, v.solver, v.turb = 0, 1, 1, 0, 0, 0
    v.nv, v.ng, v.sweeps = 5, 2, 1
    for k, x in kw.items():
        setattr(v, k, x)
    return v


@pytest.mark.parametrize("field,value,words", [
    ("eqn", 1, b"Euler"), ("eqn", 2, b"Euler"), ("turb", 1, b"turbulence"),
    ("solver", 1, b"block diagonal"), ("solver", 3, b"block diagonal"),
    ("dt_global", 1e-3, b"global timeStep"), ("dual_cfl", 5.0, b"dual-time"),
    ("recon", 2, b"MUSCL"), ("flux", 1, b"Roe")])
def test_noalloc_refuses_unsupported_views(field, value, words):
    from aither_gb300._lib import lib
    rc = lib().ath_block_residual_noalloc(C.byref(_block()), C.byref(_view(**{field: value})),
                                          1.0, None)
    assert rc == ATH_ERR_UNSUPPORTED
    assert words in lib().ath_last_error()
