"""CPU oracle against the reference: golden fixtures produced by the
reference solver itself (tests/golden/make_golden.py) and, where the
reference sources are present, a live run of the reference build."""
import os
import subprocess

import numpy as np
import pytest

from conftest import REF_HARNESS, REF_SRC, golden_case, rel_err, total_iterations

# The oracle restates the reference operation by operation and is built
# with -ffp-contract=off; it reproduces the reference bit for bit on these
# cases.  The stated tolerance leaves room for a different libm sqrt only.
TOL = 1e-13

FULL = ["vortex16_it1", "vortex16_it20", "bump24_it1", "bump24_it30",
        "bump_sup_it1", "bump_sup_it40", "bump_weno_it1", "bump_weno_it20",
        "bump_wenoz_ausm_it1", "bump_wenoz_ausm_it20", "bump_const_ausm_it20",
        "bump_vanalbada_ausm_it20", "plate_adiabatic_it1", "plate_adiabatic_it20",
        "plate_isothermal_it1", "plate_isothermal_it20", "bump_blusgs_it1", "bump_blusgs_it20",
        "bump_sweeps3_it1", "bump_sweeps3_it20", "bump_blusgs_weno_sw2_it1",
        "bump_blusgs_weno_sw2_it20", "plate_blusgs_it1", "plate_blusgs_it20",
        "plate_blusgs_sw2_it1", "plate_blusgs_sw2_it20", "sst_plate_it1", "sst_plate_it20",
        "sst_plate2_blusgs_it1", "sst_plate2_blusgs_it10", "sst_weno_ausm_it1",
        "sst_weno_ausm_it10", "bump_dplur_it1", "bump_dplur_it20", "plate_bdplur_it1",
        "plate_bdplur_it20", "sst_plate_dplur_it1", "sst_plate_dplur_it10",
        "bump_stag_pout_it1", "bump_stag_pout_it20", "bump_inlet_pout_it1",
        "bump_inlet_pout_it20", "bump_nr_it1", "bump_nr_it20", "bump_nr_bdf2_it1",
        "bump_nr_bdf2_it12", "plate_heatflux_it1", "plate_heatflux_it20",
        "sst_chan_stag_pout_it1", "sst_chan_stag_pout_it10", "vortex_bdf2_it1", "vortex_bdf2_it4",
        "vortex_cn_dual_it1", "vortex_cn_dual_it4", "plate_bdf2_blusgs_it1", "plate_bdf2_blusgs_it4",
        "sst_plate_bdf2_it1", "sst_plate_bdf2_it4", "bump_nr_out_it1", "bump_nr_out_it20",
        "bump_nr_both_bdf2_it1", "bump_nr_both_bdf2_it8", "chan_nr_out_visc_it1",
        "chan_nr_out_visc_it10", "bump_mg_v_it1", "bump_mg_v_it15", "bump_mg_w3_it1",
        "bump_mg_w3_it15", "bump_mg_dplur_it1", "bump_mg_dplur_it15", "plate_mg_blusgs_it1",
        "plate_mg_blusgs_it15", "plate_mg_bdplur_it1", "plate_mg_bdplur_it15",
        "wk_plate_it1", "wk_plate_it15", "wk_plate2_blusgs_it1", "wk_plate2_blusgs_it15"]


def _oracle(inp, st):
    from aither_gb300 import Setup
    from pyoracle import Oracle
    s = Setup(inp)
    if st is not None:
        s.set_state(0, st[0])
    return s, Oracle(s)


@pytest.mark.parametrize("name", FULL)
def test_oracle_matches_reference_fixture(name, tmp_path):
    inp, st, g = golden_case(name, str(tmp_path))
    _, o = _oracle(inp, st)
    l2 = o.iterate(total_iterations(g))
    for b in range(int(g["nblocks"])):
        p = f"b{b}_"
        assert rel_err(o.field(b, "STATE"), g[p + "state"]) <= TOL
        assert rel_err(o.field(b, "RESID"), g[p + "resid"]) <= TOL
        assert rel_err(o.field(b, "DT")[..., 0], g[p + "dt"]) <= TOL
        assert rel_err(o.field(b, "SPECRAD")[..., 0], g[p + "specrad"][..., 0]) <= TOL
        if g[p + "state"].shape[-1] == 7:  # RANS: the turbulence radius too
            assert rel_err(o.field(b, "SPECRAD")[..., 1], g[p + "specrad"][..., 1]) <= TOL
        assert rel_err(o.field(b, "DU"), g[p + "du"]) <= TOL
    assert rel_err(l2[:, 0, :], g["l2"]) <= TOL
    if "forces" in g and np.abs(g["forces"]).max() > 0:
        # integrated wall forces: same terms, summed in another order
        assert rel_err(o.forces[-1, 0], g["forces"]) <= 1e-12


@pytest.mark.parametrize("name", ["vortex16_it20", "bump24_it30", "bump_sup_it40",
                                  "bump_blusgs_it20", "bump_sweeps3_it20",
                                  "plate_blusgs_sw2_it20", "vortex_bdf2_it4",
                                  "vortex_cn_dual_it4", "sst_plate_bdf2_it4",
                                  "bump_mg_w3_it15", "plate_mg_blusgs_it15"])
def test_oracle_matrix_residual(name, tmp_path):
    """The logged linear-system residual (linearSolver::Residual)."""
    from aither_gb300 import Setup
    from pyoracle import Oracle
    inp, st, g = golden_case(name, str(tmp_path))
    s = Setup(inp)
    if st is not None:
        s.set_state(0, st[0])
    o = Oracle(s, matrix_resid=True)
    o.iterate(total_iterations(g))
    assert rel_err(o.mres[:, 0], g["matrix_resid"]) <= TOL


def test_oracle_full_vortex_box_200_iterations(tmp_path):
    """The 64x32x8 vortex box, 200 LU-SGS iterations at CFL 10: L2 history
    and state statistics equal the reference's."""
    inp, st, g = golden_case("vortex_c1_it200", str(tmp_path))
    _, o = _oracle(inp, st)
    l2 = o.iterate(200)
    assert rel_err(l2[:, 0, :], g["l2"]) <= 1e-12
    w = o.field(0, "STATE")
    assert rel_err(w.reshape(-1, 5).sum(axis=0), g["b0_state_sum"]) <= 1e-12
    assert rel_err(w[::3, ::7, ::11], g["b0_state_samples"]) <= 1e-12


@pytest.mark.parametrize("name", ["plate_c2_it20", "plate_c2b_it20"])
def test_oracle_laminar_plate_two_blocks(name, tmp_path):
    """Two 128x64x2 blocks joined by an interblock connection, laminar
    Navier-Stokes at Re_L = 1e5 on a wall-normal geometric grid (first cell
    1e-5, ratio 1.08), scalar LU-SGS and 4-sweep block LU-SGS: 20 iterations
    against the reference."""
    inp, st, g = golden_case(name, str(tmp_path))
    _, o = _oracle(inp, st)
    l2 = o.iterate(20)
    assert rel_err(l2[:, 0, :], g["l2"]) <= 1e-12
    assert rel_err(o.forces[-1, 0], g["forces"]) <= 1e-12
    for b in range(2):
        w = o.field(b, "STATE")
        assert rel_err(w.reshape(-1, 5).sum(axis=0), g[f"b{b}_state_sum"]) <= 1e-12
        assert rel_err(w[::3, ::7, ::11], g[f"b{b}_state_samples"]) <= 1e-12


@pytest.mark.skipif(not (os.path.exists(REF_HARNESS) and os.path.isdir(REF_SRC)),
                    reason="reference build not available on this machine")
@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_matches_live_reference(seed, tmp_path):
    """Random small bump channels, run through the reference build here."""
    from refdump import read_dump

    from aither_gb300 import cases
    rng = np.random.default_rng(seed)
    ni, nj, nk = (int(x) for x in rng.integers([10, 6, 2], [20, 12, 5]))
    inp, _ = cases.bump_channel(str(tmp_path), ni, nj, nk, float(rng.uniform(0.04, 0.1)),
                                float(rng.uniform(0.3, 0.85)), name="live")
    env = dict(os.environ, AITHER_INSTALL_DIRECTORY=REF_SRC)
    r = subprocess.run([REF_HARNESS, "live.inp", "5", "out.bin"], cwd=str(tmp_path),
                       env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    R = read_dump(str(tmp_path / "out.bin"))
    _, o = _oracle(inp, None)
    l2 = o.iterate(5)
    assert rel_err(o.field(0, "STATE"), R["b0_state"][2:-2, 2:-2, 2:-2]) <= TOL
    assert rel_err(o.field(0, "DU"), R["b0_du"]) <= TOL
    assert rel_err(l2[:, 0, :], R["l2"]) <= TOL


def test_oracle_detects_nonphysical_state(tmp_path):
    """A negative pressure planted in the initial state is reported, not
    silently propagated (host-side fault injection)."""
    from aither_gb300 import cases
    inp, st = cases.vortex_box(str(tmp_path), 8, 4, 2, name="bad")
    w = st[0].reshape(2, 4, 8, 5).copy()
    w[1, 2, 3, 4] = -1.0
    _, o = _oracle(inp, [w.reshape(-1)])
    with pytest.raises(RuntimeError):
        o.iterate(1)
