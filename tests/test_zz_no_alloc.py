"""The allocation-free residual entry point, through the C ABI.

Callers that cannot allocate device memory while the solver step runs
(graph-recording hosts, serving loops with a fixed HBM budget, plugin hosts
owning the allocator) call ath_block_residual_noalloc with their own device
arrays; its face-flux scratch is a fixed array inside the library.  This
checks, on two calls in a row, that it reproduces ath_batch_residual's
residual, spectral radius, time step and inverse diagonal (FP64 tolerance of
the other parity tests, 1e-12 relative), and that oversized blocks are
rejected.  Device arrays here are allocated by the test (the caller), with
PyTorch.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _device_layout_faces(g, d):
    """Host face arrays (one extra entry along d) -> face i stored at cell i."""
    a = g[["fareai", "fareaj", "fareak"][d]]
    sl = [slice(None)] * 4
    sl[3 - d] = slice(0, a.shape[3 - d] - 1)
    return np.ascontiguousarray(a[tuple(sl)]).reshape(-1)


def test_noalloc_residual_matches_batch(tmp_path):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    from aither_gb300 import Batch, Context, Setup, cases
    from aither_gb300._lib import BlockDev, check, lib

    inp, _ = cases.bump_channel(str(tmp_path), 40, 20, 10, 0.08, 0.7, name="na")
    setup = Setup(inp)
    ctx = Context(0)
    batch = Batch(ctx, setup)
    batch.iterate(2)
    batch.stage("fill_ghosts")
    batch.stage("residual")
    want = {f: batch.field(0, f) for f in ("RESID", "DT", "SPECRAD", "AINV")}
    n = batch.pool_cells()
    W = np.empty(5 * n)
    batch.copy_state(W, to_device=False)

    v = setup.block_view(0)
    g = setup.geometry(0)
    ni, nj, nk, ng = v.ni, v.nj, v.nk, v.ng
    assert n == v.ncell_padded
    dev = torch.device("cuda", 0)

    def up(a):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)

    t_W = up(W)
    t_vol = up(g["vol"].reshape(-1))
    t_w = [up(g["width"][d].reshape(-1)) for d in range(3)]
    t_fa = [up(_device_layout_faces(g, d)) for d in range(3)]
    phys = setup.solve_view(0)
    stream = torch.cuda.current_stream(dev).cuda_stream

    def phys_cells(t, w):
        a = t.cpu().numpy().reshape(w, nk + 2 * ng, nj + 2 * ng, ni + 2 * ng)
        return np.moveaxis(a[:, ng:-ng, ng:-ng, ng:-ng], 0, -1)

    for call in range(2):
        t_R = torch.full((5 * n,), float("nan"), dtype=torch.float64, device=dev)
        t_lam = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        t_dt = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        t_ai = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        b = BlockDev()
        b.ni, b.nj, b.nk, b.ng = ni, nj, nk, ng
        b.W = t_W.data_ptr()
        b.vol = t_vol.data_ptr()
        for d in range(3):
            b.width[d] = t_w[d].data_ptr()
            b.farea[d] = t_fa[d].data_ptr()
        b.R, b.lam, b.dt, b.ainv = (t_R.data_ptr(), t_lam.data_ptr(), t_dt.data_ptr(),
                                    t_ai.data_ptr())
        check(lib().ath_block_residual_noalloc(C.byref(b), C.byref(phys), phys.cfl_start,
                                               C.c_void_p(stream)))
        torch.cuda.synchronize(dev)
        assert rel_err(phys_cells(t_R, 5), want["RESID"]) <= TOL, call
        assert rel_err(phys_cells(t_dt, 1), want["DT"]) <= TOL, call
        assert rel_err(phys_cells(t_lam, 1)[..., 0], want["SPECRAD"][..., 0]) <= TOL, call
        assert rel_err(phys_cells(t_ai, 1), want["AINV"]) <= TOL, call
    batch.close()
    ctx.close()


def test_noalloc_rejects_oversized_block():
    from aither_gb300._lib import ATH_OK, BlockDev, SolveView, lib
    b = BlockDev()
    b.ni, b.nj, b.nk, b.ng = 100, 100, 20, 2  # 104*104*24 padded cells > maximum
    for name in ("W", "vol", "R", "lam", "dt", "ainv"):
        setattr(b, name, 16)
    for d in range(3):
        b.width[d] = 16
        b.farea[d] = 16
    phys = SolveView()
    rc = lib().ath_block_residual_noalloc(C.byref(b), C.byref(phys), 1.0, None)
    assert rc != ATH_OK
    assert b"at most" in lib().ath_last_error()
