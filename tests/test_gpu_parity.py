"""Parity of the sm_103a path with the reference, through the C ABI.

Tolerances (relative to the largest magnitude of the compared field):
  * FP64 path, per cell, after one iteration: 1e-12 for every field;
  * after tens of iterations: 1e-12 for the state, time step and flow
    spectral radius; 1e-10 for the residual, the implicit update and the
    turbulence spectral radius (it carries the omega source), which are small
    differences of large fluxes once the solution converges and amplify the
    last-bit differences of pow() between CUDA and the host libm (Sutherland's
    law) and of FMA-free reordering;
  * FP64 path, L2 residual histories (incl. 200 iterations of the full
    64x32x8 vortex box) and integrated wall forces: 1e-10.
"""
import numpy as np
import pytest

from conftest import golden_case, rel_err, total_iterations

pytestmark = pytest.mark.gpu

CELL_TOL = 1e-12
NORM_TOL = 1e-10


# multigrid: V and W cycles over 2 and 3 levels, LU-SGS (1 and 3 sweeps),
# DP-LUR, block LU-SGS and block DP-LUR (two-block laminar plates)
MG_CASES = [f"{c}_it{n}" for c in ("bump_mg_v", "bump_mg_w3", "bump_mg_dplur",
                                   "plate_mg_blusgs", "plate_mg_bdplur") for n in (1, 15)]


@pytest.fixture(scope="module")
def ctx():
    from aither_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _batch(ctx, inp, st, precision=0):
    from aither_gb300 import Batch, Setup
    s = Setup(inp)
    if st is not None:
        s.set_state(0, st[0])
    return s, Batch(ctx, s, precision)


def _l2(norms, nsolves=1, solve=0, nv=5):
    a = np.array([[n.l2[v] for v in range(nv)] for n in norms])
    return a.reshape(-1, nsolves, nv)[:, solve, :]


def _cols_err(a, b):
    """Largest relative error of the flow variables (one scale for the
    five) and of each turbulence variable (its own scale: k and omega
    differ from the flow and from each other by orders of magnitude)."""
    a, b = np.asarray(a), np.asarray(b)
    errs = [rel_err(a[..., :5], b[..., :5])]
    errs += [rel_err(a[..., v], b[..., v]) for v in range(5, b.shape[-1])]
    return max(errs)


@pytest.mark.parametrize("name", ["vortex16_it1", "vortex16_it20", "bump24_it1",
                                  "bump24_it30", "bump_sup_it1", "bump_sup_it40",
                                  "bump_weno_it1", "bump_weno_it20", "bump_wenoz_ausm_it1",
                                  "bump_wenoz_ausm_it20", "bump_const_ausm_it20",
                                  "bump_vanalbada_ausm_it20", "plate_adiabatic_it1",
                                  "plate_adiabatic_it20", "plate_isothermal_it1",
                                  "plate_isothermal_it20", "bump_blusgs_it1",
                                  "bump_blusgs_it20", "bump_sweeps3_it1", "bump_sweeps3_it20",
                                  "bump_blusgs_weno_sw2_it1", "bump_blusgs_weno_sw2_it20",
                                  "plate_blusgs_it1", "plate_blusgs_it20",
                                  "plate_blusgs_sw2_it1", "plate_blusgs_sw2_it20",
                                  "bump_dplur_it1", "bump_dplur_it20", "plate_bdplur_it1",
                                  "plate_bdplur_it20", "bump_stag_pout_it1",
                                  "bump_stag_pout_it20", "bump_inlet_pout_it1",
                                  "bump_inlet_pout_it20", "bump_nr_it1", "bump_nr_it20",
                                  "bump_nr_bdf2_it1", "bump_nr_bdf2_it12", "plate_heatflux_it1",
                                  "plate_heatflux_it20", "vortex_bdf2_it1", "vortex_bdf2_it4",
                                  "vortex_cn_dual_it1", "vortex_cn_dual_it4",
                                  "plate_bdf2_blusgs_it1", "plate_bdf2_blusgs_it4",
                                  "bump_nr_out_it1", "bump_nr_out_it20", "bump_nr_both_bdf2_it1",
                                  "bump_nr_both_bdf2_it8", "chan_nr_out_visc_it1",
                                  "chan_nr_out_visc_it10", *MG_CASES])
def test_fp64_matches_reference_fixture(ctx, name, tmp_path):
    inp, st, g = golden_case(name, str(tmp_path))
    s, b = _batch(ctx, inp, st)
    n = total_iterations(g)
    norms = b.iterate(n)
    diff_tol = CELL_TOL if n == 1 else NORM_TOL
    for k in range(int(g["nblocks"])):
        p = f"b{k}_"
        assert rel_err(b.field(k, "STATE"), g[p + "state"]) <= CELL_TOL
        assert rel_err(b.field(k, "RESID"), g[p + "resid"]) <= diff_tol
        assert rel_err(b.field(k, "DT")[..., 0], g[p + "dt"]) <= CELL_TOL
        assert rel_err(b.field(k, "SPECRAD")[..., 0], g[p + "specrad"][..., 0]) <= CELL_TOL
        assert rel_err(b.field(k, "DU"), g[p + "du"]) <= diff_tol
    assert rel_err(_l2(norms), g["l2"]) <= NORM_TOL
    assert all(x.status == 0 for x in norms)
    if "forces" in g and np.abs(g["forces"]).max() > 0:
        assert rel_err(np.array(norms[-1].force[:]), g["forces"]) <= NORM_TOL
    b.close()


SST_CASES = ["sst_plate_it1", "sst_plate_it20", "sst_plate2_blusgs_it1",
             "sst_plate2_blusgs_it10", "sst_weno_ausm_it1", "sst_weno_ausm_it10",
             "sst_plate_dplur_it1", "sst_plate_dplur_it10", "sst_chan_stag_pout_it1",
             "sst_chan_stag_pout_it10", "sst_plate_bdf2_it1", "sst_plate_bdf2_it4",
             "wk_plate_it1", "wk_plate_it15", "wk_plate2_blusgs_it1", "wk_plate2_blusgs_it15"]


@pytest.mark.parametrize("name", SST_CASES)
def test_fp64_sst_matches_reference_fixture(ctx, name, tmp_path):
    """SST-2003 k-omega RANS flat plate (seven equations): one 12x10x2 block
    with scalar LU-SGS and MUSCL/Roe, two blocks with an interblock
    connection and block LU-SGS, and WENO/AUSM; state, residual, time step,
    flow and turbulence spectral radii, update, L2 history and wall forces
    against the reference."""
    inp, st, g = golden_case(name, str(tmp_path))
    s, b = _batch(ctx, inp, None)
    for k in range(int(g["nblocks"])):
        s_k = g[f"b{k}_state0"]
        assert rel_err(b.field(k, "STATE"), s_k) == 0.0
    n = total_iterations(g)
    norms = b.iterate(n)
    diff_tol = CELL_TOL if n == 1 else NORM_TOL
    for k in range(int(g["nblocks"])):
        p = f"b{k}_"
        assert b.field(k, "STATE").shape[-1] == 7
        assert _cols_err(b.field(k, "STATE"), g[p + "state"]) <= CELL_TOL
        assert _cols_err(b.field(k, "RESID"), g[p + "resid"]) <= diff_tol
        assert rel_err(b.field(k, "DT")[..., 0], g[p + "dt"]) <= CELL_TOL
        sr = b.field(k, "SPECRAD")
        assert rel_err(sr[..., 0], g[p + "specrad"][..., 0]) <= CELL_TOL
        # the turbulence radius carries the source radius 2 beta* omega V,
        # which amplifies last-bit differences of omega over many iterations
        # like the residual does
        assert rel_err(sr[..., 1], g[p + "specrad"][..., 1]) <= diff_tol
        assert _cols_err(b.field(k, "DU"), g[p + "du"]) <= diff_tol
    assert _cols_err(_l2(norms, nv=7), g["l2"]) <= NORM_TOL
    assert all(x.status == 0 for x in norms)
    if np.abs(g["forces"]).max() > 0:
        assert rel_err(np.array(norms[-1].force[:]), g["forces"]) <= NORM_TOL
    b.close()


@pytest.mark.parametrize("name", ["vortex16_it20", "bump24_it30", "bump_sup_it40",
                                  "bump_blusgs_it20", "bump_sweeps3_it20",
                                  "plate_blusgs_sw2_it20", "sst_plate_it20",
                                  "sst_plate2_blusgs_it10", "bump_dplur_it20",
                                  "plate_bdplur_it20", "vortex_bdf2_it4", "vortex_cn_dual_it4"])
def test_fp64_matrix_residual(ctx, name, tmp_path):
    """flags bit 0: the logged matrix residual of every iteration; it is a
    log-only quantity, so the solution is unchanged."""
    from aither_gb300 import Batch, Setup
    inp, st, g = golden_case(name, str(tmp_path))
    s = Setup(inp)
    if st is not None:
        s.set_state(0, st[0])
    b = Batch(ctx, s, 0, flags=1)
    norms = b.iterate(total_iterations(g))
    mres = np.array([n.matrix_resid for n in norms])
    assert rel_err(mres, g["matrix_resid"]) <= NORM_TOL
    assert _cols_err(b.field(0, "STATE"), g["b0_state"]) <= CELL_TOL
    b.close()


@pytest.mark.parametrize("name", ["plate_c2_it20", "plate_c2b_it20"])
def test_fp64_laminar_plate_two_blocks(ctx, name, tmp_path):
    """Laminar flat plate, two 128x64x2 blocks with an interblock connection,
    scalar LU-SGS (plate_c2) and block LU-SGS with 4 sweeps (plate_c2b): 20
    iterations against the reference's L2 history and state statistics."""
    inp, st, g = golden_case(name, str(tmp_path))
    s, b = _batch(ctx, inp, st)
    norms = b.iterate(20)
    assert rel_err(_l2(norms), g["l2"]) <= NORM_TOL
    assert rel_err(np.array(norms[-1].force[:]), g["forces"]) <= NORM_TOL
    for k in range(2):
        w = b.field(k, "STATE")
        assert rel_err(w.reshape(-1, 5).sum(axis=0), g[f"b{k}_state_sum"]) <= NORM_TOL
        assert rel_err(w[::3, ::7, ::11], g[f"b{k}_state_samples"]) <= CELL_TOL * 100
    b.close()


def test_fp64_full_vortex_box_200_iterations(ctx, tmp_path):
    inp, st, g = golden_case("vortex_c1_it200", str(tmp_path))
    s, b = _batch(ctx, inp, st)
    norms = b.iterate(200)
    assert rel_err(_l2(norms), g["l2"]) <= NORM_TOL
    w = b.field(0, "STATE")
    assert rel_err(w.reshape(-1, 5).sum(axis=0), g["b0_state_sum"]) <= NORM_TOL
    assert rel_err(w[::3, ::7, ::11], g["b0_state_samples"]) <= CELL_TOL * 100
    b.close()


def test_stages_match_oracle(ctx, tmp_path):
    """Each stage of one iteration against the CPU oracle on a bump channel."""
    from aither_gb300 import cases
    from pyoracle import Oracle
    inp, _ = cases.bump_channel(str(tmp_path), 30, 14, 5, 0.09, 0.8, name="stg")
    s, b = _batch(ctx, inp, None)
    o = Oracle(s)
    b.iterate(3)
    o.iterate(3)
    b.stage("fill_ghosts")
    o.stage("fill_ghosts")
    assert rel_err(b.field(0, "STATE_GHOSTS"), o.field(0, "STATE_GHOSTS")) <= CELL_TOL
    b.stage("residual")
    o.stage("residual")
    assert rel_err(b.field(0, "RESID"), o.field(0, "RESID")) <= CELL_TOL
    for nm in ("timestep", "diag_invert"):
        b.stage(nm)
        o.stage(nm)
    assert rel_err(b.field(0, "DT"), o.field(0, "DT")) <= CELL_TOL
    assert rel_err(b.field(0, "AINV"), o.field(0, "AINV")) <= CELL_TOL
    b.stage("relax")
    o.stage("relax")
    assert rel_err(b.field(0, "DU"), o.field(0, "DU")) <= CELL_TOL
    nb = b.stage("update")
    no = o.stage("update")
    assert rel_err(b.field(0, "STATE"), o.field(0, "STATE")) <= CELL_TOL
    assert rel_err(np.array([nb[0].l2[v] for v in range(5)]), no[0]) <= CELL_TOL
    b.close()


def test_batched_solves_equal_solves_alone(ctx, tmp_path):
    """Several independent solves of different sizes in one batch give the
    same results as each solve run alone (FP64: bit for bit)."""
    from aither_gb300 import Batch, Setup, cases
    specs = [(20, 10, 4, 0.05, 0.5), (33, 12, 3, 0.08, 0.75), (16, 16, 6, 0.1, 0.4)]
    inps = []
    for q, (ni, nj, nk, h, m) in enumerate(specs):
        d = tmp_path / f"c{q}"
        inp, _ = cases.bump_channel(str(d), ni, nj, nk, h, m, name=f"b{q}")
        inps.append(inp)
    sb = Setup(inps)
    bb = Batch(ctx, sb)
    nb = bb.iterate(15)
    for q, inp in enumerate(inps):
        s1, b1 = _batch(ctx, inp, None)
        n1 = b1.iterate(15)
        assert np.array_equal(_l2(nb, 3, q), _l2(n1))
        assert np.array_equal(bb.field(q, "STATE"), b1.field(0, "STATE"))
        b1.close()
    bb.close()


def test_nonphysical_state_reported(ctx, tmp_path):
    """A negative pressure planted on the host is reported through the
    solve's status; the context stays usable."""
    from aither_gb300 import cases
    inp, st = cases.vortex_box(str(tmp_path), 8, 4, 2, name="bad")
    w = st[0].reshape(2, 4, 8, 5).copy()
    w[1, 2, 3, 4] = -1.0
    s, b = _batch(ctx, inp, [w.reshape(-1)])
    norms = b.iterate(1)
    assert norms[0].status != 0
    b.close()
    inp2, st2 = cases.vortex_box(str(tmp_path / "ok"), 8, 4, 2, name="ok")
    s2, b2 = _batch(ctx, inp2, st2)
    assert all(n.status == 0 for n in b2.iterate(2))
    b2.close()


def test_memory_budget_is_enforced(tmp_path):
    from aither_gb300 import AthError, Batch, Context, Setup, cases
    c = Context(0, hbm_budget=1 << 20)
    inp, _ = cases.bump_channel(str(tmp_path), 40, 20, 10, 0.05, 0.5, name="big")
    with pytest.raises(AthError) as e:
        Batch(c, Setup(inp))
    assert e.value.code == -5
    c.close()


FAST_CASES = ["vortex16_it1", "vortex16_it20", "bump24_it1", "bump24_it30", "bump_sup_it1",
              "bump_sup_it40", "bump_vanalbada_ausm_it20", "plate_adiabatic_it1",
              "plate_adiabatic_it20", "plate_blusgs_it1", "plate_blusgs_it20",
              "bump_sweeps3_it20", "vortex_bdf2_it4"]


@pytest.mark.parametrize("name", FAST_CASES)
def test_fp64_fast_faces_match_reference_fixture(ctx, name, tmp_path):
    """The fast FP64 faces (MUSCL and Roe rearranged to fewer divisions and
    square roots, ATH_BATCH_FAST_FACES) against the reference: 1e-12 per
    cell after one iteration, 1e-10 for residual and update after many and
    for the L2 history (the same tolerances as the bit-exact path, which
    they meet with roundoff-level differences)."""
    from aither_gb300 import BATCH_FAST_FACES, Batch, Setup
    inp, st, g = golden_case(name, str(tmp_path))
    s = Setup(inp)
    if st is not None:
        s.set_state(0, st[0])
    b = Batch(ctx, s, 0, BATCH_FAST_FACES)
    n = total_iterations(g)
    norms = b.iterate(n)
    diff_tol = CELL_TOL if n == 1 else NORM_TOL
    for k in range(int(g["nblocks"])):
        p = f"b{k}_"
        assert rel_err(b.field(k, "STATE"), g[p + "state"]) <= CELL_TOL
        assert rel_err(b.field(k, "RESID"), g[p + "resid"]) <= diff_tol
        assert rel_err(b.field(k, "DT")[..., 0], g[p + "dt"]) <= CELL_TOL
        assert rel_err(b.field(k, "DU"), g[p + "du"]) <= diff_tol
    assert rel_err(_l2(norms), g["l2"]) <= NORM_TOL
    b.close()


def test_fp64_fast_faces_full_vortex_box_200_iterations(ctx, tmp_path):
    """The 64x32x8 vortex box (200 LU-SGS iterations at CFL 10) with the
    fast faces: L2 history within 1e-10 of the reference's."""
    from aither_gb300 import BATCH_FAST_FACES, Batch, Setup
    inp, st, g = golden_case("vortex_c1_it200", str(tmp_path))
    s = Setup(inp)
    s.set_state(0, st[0])
    b = Batch(ctx, s, 0, BATCH_FAST_FACES)
    norms = b.iterate(200)
    assert rel_err(_l2(norms), g["l2"]) <= NORM_TOL
    w = b.field(0, "STATE")
    assert rel_err(w.reshape(-1, 5).sum(axis=0), g["b0_state_sum"]) <= 1e-12
    b.close()
