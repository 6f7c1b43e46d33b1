"""Runs to convergence with per-solve retirement on the device.

A solve retires in the iteration where its total L2 norm (over the five
equations) first falls to `drop` times its first-iteration value; its
kernels then skip their work.  Because the decision is taken on the device
per solve, a solve's result is the same whether it runs alone or next to
other solves, and whatever the host's polling interval."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

RETIRED = 1


@pytest.fixture(scope="module")
def ctx():
    from aither_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _cases(tmp):
    from aither_gb300 import cases
    a, _ = cases.bump_channel(str(tmp / "a"), 16, 8, 4, 0.06, 0.55, name="a")
    b, _ = cases.bump_channel(str(tmp / "b"), 20, 10, 3, 0.09, 0.75, name="b")
    c, _ = cases.bump_channel(str(tmp / "c"), 12, 12, 5, 0.04, 0.40, name="c")
    return [a, b, c]


def _total(norms, nsolves, s):
    a = np.array([[n.l2[v] for v in range(5)] for n in norms]).reshape(-1, nsolves, 5)[:, s]
    return np.sqrt((a ** 2).sum(axis=1))


@pytest.mark.parametrize("precision", [0, 1])
def test_retirement_happens_in_the_iteration_the_drop_is_reached(ctx, precision, tmp_path):
    from aither_gb300 import Batch, Setup
    inp = _cases(tmp_path)[0]
    b = Batch(ctx, Setup(inp), precision)
    info = b.converge(5000, 1e-3, check_every=97)
    n = info[0].iterations
    assert info[0].converged == 1 and info[0].drop <= 1e-3 and n > 10
    w_conv = b.field(0, "STATE")
    # a retired solve does no work: its state stays, its status says so
    after = b.iterate(3)
    assert all(x.status == RETIRED for x in after)
    assert np.array_equal(b.field(0, "STATE"), w_conv)
    b.close()
    # the same number of plain iterations gives the same state, and n is
    # the first iteration whose drop reaches the target
    b2 = Batch(ctx, Setup(inp), precision)
    tot = _total(b2.iterate(n), 1, 0)
    r = tot / tot[0]
    assert r[n - 1] <= 1e-3 < r[n - 2]
    assert np.array_equal(b2.field(0, "STATE"), w_conv)
    b2.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_converged_result_is_the_same_alone_and_in_a_batch(ctx, precision, tmp_path):
    from aither_gb300 import Batch, Setup
    inps = _cases(tmp_path)
    mix = Batch(ctx, Setup(inps), precision)
    info = mix.converge(6000, 1e-3, check_every=64)
    assert all(x.converged == 1 for x in info)
    # the three solves converge at different iterations
    assert len({x.iterations for x in info}) > 1
    for s, inp in enumerate(inps):
        alone = Batch(ctx, Setup(inp), precision)
        ia = alone.converge(6000, 1e-3, check_every=31)
        assert ia[0].iterations == info[s].iterations
        assert np.array_equal(alone.field(0, "STATE"), mix.field(s, "STATE"))
        alone.close()
    mix.close()


@pytest.mark.parametrize("case", [0, 1])
def test_mixed_precision_converged_state_against_fp64(ctx, case, tmp_path):
    """Mixed precision (FP32 limiter, Roe dissipation, spectral radii and
    sweeps; FP64 face states, central fluxes, residual sums, update and
    norms) against FP64 at a 1e-6 drop: same iteration count within 1 %, and
    the converged states agree to 1e-6 relative (measured ~1e-8)."""
    from aither_gb300 import Batch, Setup
    inp = _cases(tmp_path)[case]
    out = {}
    for prec in (0, 1):
        b = Batch(ctx, Setup(inp), prec)
        info = b.converge(20000, 1e-6, check_every=200)
        assert info[0].converged == 1
        out[prec] = (b.field(0, "STATE"), info[0].iterations)
        b.close()
    err = rel_err(out[1][0], out[0][0])
    print(f"mixed vs FP64 converged state: rel err {err:.2e}, iterations "
          f"{out[1][1]} vs {out[0][1]}")
    assert err <= 1e-6
    assert abs(out[1][1] - out[0][1]) <= max(2, 0.01 * out[0][1])


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_leaves_the_solution_unchanged(ctx, precision, tmp_path):
    """The launch-shape autotuner times real iterations, then restores the
    solution and the per-solve counters: the results are those of an
    untuned batch."""
    from aither_gb300 import Batch, Setup
    inps = _cases(tmp_path)
    ref = Batch(ctx, Setup(inps), precision)
    ref.iterate(7)
    tuned = Batch(ctx, Setup(inps), precision)
    tuned.iterate(3)
    t = tuned.autotune(2)
    assert t in (32, 64, 128, 256)
    tuned.iterate(4)
    for s in range(3):
        assert np.array_equal(tuned.field(s, "STATE"), ref.field(s, "STATE"))
    ref.close()
    tuned.close()


def test_sst_mixed_precision_converged_state_against_fp64(ctx, tmp_path):
    """SST-2003 RANS bump channel (seven equations) to a 1e-6 drop of the
    total L2 over all seven: the mixed path retires within 1 % of the FP64
    iteration count, and its converged flow variables and each turbulence
    variable agree with FP64 to 1e-6 relative (each to its own scale)."""
    from aither_gb300 import Batch, Setup, cases
    inp, _ = cases.wall_channel(str(tmp_path / "sst"), 32, 16, 4, "bump", 0.08, 0.6,
                                alpha=2.0, rans=True, stretch=1.1, name="sst")
    out = {}
    for prec in (0, 1):
        b = Batch(ctx, Setup(inp), prec)
        info = b.converge(20000, 1e-6, check_every=100)
        assert info[0].converged == 1
        out[prec] = (b.field(0, "STATE"), info[0].iterations)
        b.close()
    a, ref = out[1][0], out[0][0]
    assert ref.shape[-1] == 7
    errs = [rel_err(a[..., :5], ref[..., :5])] + [rel_err(a[..., v], ref[..., v])
                                                  for v in (5, 6)]
    print(f"SST mixed vs FP64: rel err flow {errs[0]:.2e} k {errs[1]:.2e} "
          f"omega {errs[2]:.2e}; iterations {out[1][1]} vs {out[0][1]}")
    assert max(errs) <= 1e-6
    assert abs(out[1][1] - out[0][1]) <= max(2, 0.01 * out[0][1])


@pytest.mark.parametrize("solver", ["dplur", "bdplur"])
def test_jacobi_relaxation_reaches_the_lusgs_steady_state(ctx, solver, tmp_path):
    """DP-LUR (Jacobi sweeps, every cell at once) and LU-SGS relax the same
    linear system differently but drive the same residual to zero: at a
    1e-8 drop their converged states agree to 1e-6."""
    from aither_gb300 import Batch, Setup, cases
    out = {}
    for ms in ("lusgs", solver):
        inp, _ = cases.bump_channel(str(tmp_path / ms), 16, 8, 4, 0.06, 0.55, name=ms,
                                    matrix_solver=ms, sweeps=1 if ms == "lusgs" else 4)
        b = Batch(ctx, Setup(inp), 0)
        info = b.converge(20000, 1e-8, check_every=200)
        assert info[0].converged == 1
        out[ms] = (b.field(0, "STATE"), info[0].iterations)
        b.close()
    err = rel_err(out[solver][0], out["lusgs"][0])
    print(f"{solver} vs lusgs: rel err {err:.2e}, iterations {out[solver][1]} vs "
          f"{out['lusgs'][1]}")
    assert err <= 1e-6


@pytest.mark.parametrize("kind", ["laminar", "sst"])
def test_mixed_precision_converged_wall_forces_against_fp64(ctx, kind, tmp_path):
    """Integrated wall forces (pressure and shear over the viscous wall) of
    the converged mixed-precision solution against the FP64 one: within
    1e-6 relative to the largest force component, at a 1e-8 drop (laminar
    Navier-Stokes bump channel) and a 1e-7 drop (SST-2003 RANS).  The forces
    of a converged state are taken from one more iteration of the retired
    solve, reactivated."""
    from aither_gb300 import Batch, Setup, cases
    if kind == "laminar":
        inp, _ = cases.wall_channel(str(tmp_path / kind), 24, 16, 2, "bump", 0.06, 0.5,
                                    alpha=1.0, viscous=True, reynolds=2e4, stretch=1.1,
                                    cfl=50.0, name=kind)
        drop = 1e-8
    else:
        inp, _ = cases.wall_channel(str(tmp_path / kind), 32, 16, 4, "bump", 0.08, 0.6,
                                    alpha=2.0, rans=True, stretch=1.1, name=kind)
        drop = 1e-7
    forces, states = {}, {}
    for prec in (0, 1):
        b = Batch(ctx, Setup(inp), prec)
        info = b.converge(40000, drop, check_every=200)
        assert info[0].converged == 1, (kind, prec, info[0].drop, info[0].iterations)
        b.set_target(0, 0.0, active=True)
        f = np.array(b.iterate(1)[0].force[:])
        assert np.abs(f).max() > 0
        forces[prec], states[prec] = f, b.field(0, "STATE")
        b.close()
    err = float(np.abs(forces[1] - forces[0]).max() / np.abs(forces[0]).max())
    serr = rel_err(states[1][..., :5], states[0][..., :5])
    print(f"{kind}: mixed vs FP64 wall forces rel err {err:.2e}, state {serr:.2e}")
    assert err <= 1e-6
