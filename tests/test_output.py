"""Output files in the reference's formats (restart, Plot3D cell-centre
function file and grid, Paraview meta file, residual history) against the
files the reference's own executable wrote on the same cases
(tests/golden/output/, made by make_output_golden.py).  The oracle's state
after N iterations is bit-exact with the reference's, so the library's
writers must reproduce those files byte for byte."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

OUT = os.path.join(GOLDEN, "output")
NAMES = ["plate", "sst", "bump"]


def output_case(name, tmp):
    with open(os.path.join(OUT, name, "case.json")) as f:
        meta = json.load(f)
    from aither_gb300 import cases
    inp, _ = getattr(cases, meta["generator"])(str(tmp), **meta["kwargs"])
    cases.set_output_keys(inp, meta["iterations"], meta["variables"],
                          restart_freq=meta["iterations"])
    return inp, meta


def ref_bytes(name, fn):
    with open(os.path.join(OUT, name, fn), "rb") as f:
        return f.read()


def l2_normalisation(l2):
    """The reference's residual normalisation: the first step's L2, raised
    to each equation's largest over steps 1-4 (PrintResiduals)."""
    first = l2[0].copy()
    for k in range(1, min(5, len(l2))):
        first = np.maximum(first, l2[k])
    return first


@pytest.fixture(scope="module", params=NAMES)
def ran(request, tmp_path_factory):
    from pyoracle import Oracle

    from aither_gb300 import Setup
    name = request.param
    tmp = tmp_path_factory.mktemp(name)
    inp, meta = output_case(name, tmp)
    s = Setup(inp)
    o = Oracle(s, 1, output_grads=True)
    l2 = o.iterate(meta["iterations"])[:, 0, :]
    fields = []
    for b in s.solve_blocks(0):
        fl = {"prim": o.field(b, "STATE"), "dt": o.field(b, "DT"), "resid": o.field(b, "RESID"),
              "aux": o.field(b, "AUX"), "wall_dist": o.field(b, "WALLDIST"),
              "grads": o.field(b, "GRADS")}
        fields.append(fl)
    yield name, meta, s, l2, fields, tmp
    o.close()
    s.close()


def test_function_file_is_the_references(ran):
    name, meta, s, _, fields, tmp = ran
    n, sim = meta["iterations"], meta["sim"]
    path = str(tmp / "out.fun")
    s.write_function(0, fields, path)  # the input file's outputVariables
    assert open(path, "rb").read() == ref_bytes(name, f"{sim}_{n}_center.fun")


def test_restart_file_is_the_references(ran):
    name, meta, s, l2, fields, tmp = ran
    n, sim = meta["iterations"], meta["sim"]
    path = str(tmp / "out.rst")
    s.write_restart(0, n, l2_normalisation(l2), [f["prim"] for f in fields], path)
    assert open(path, "rb").read() == ref_bytes(name, f"{sim}_{n}.rst")


def test_restart_read_back(ran):
    """ReadRestart's arithmetic: values divided by the reference scales,
    species density rho * mass fraction."""
    name, meta, s, l2, fields, _ = ran
    n, sim = meta["iterations"], meta["sim"]
    it, rf, prims = s.read_restart(0, os.path.join(OUT, name, f"{sim}_{n}.rst"))
    assert it == n
    assert np.array_equal(rf, l2_normalisation(l2))
    sv = s.solve_view(0)
    r, a, mu = sv.r_ref, sv.a_ref, sv.mu_ref
    for f, got in zip(fields, prims):
        w = f["prim"]
        want = np.empty_like(w)
        want[..., 0] = 0.0 + (w[..., 0] * r) / r * (w[..., 0] / w[..., 0])
        want[..., 1:4] = (w[..., 1:4] * a) / a
        want[..., 4] = (w[..., 4] * (r * a * a)) / (r * a * a)
        if w.shape[-1] == 7:
            want[..., 5] = (w[..., 5] * (a * a)) / (a * a)
            want[..., 6] = (w[..., 6] * (a * a * r / mu)) / (a * a * r / mu)
        assert np.array_equal(got, want)


def test_center_grid_and_meta_are_the_references(ran):
    name, meta, s, _, _, tmp = ran
    n, sim = meta["iterations"], meta["sim"]
    grid = meta["kwargs"]["name"]
    s.write_center_grid(0, str(tmp / "c.xyz"))
    assert open(tmp / "c.xyz", "rb").read() == ref_bytes(name, f"{grid}_center.xyz")
    s.write_meta(0, n, str(tmp / "m.p3d"))
    assert open(tmp / "m.p3d", "rb").read() == ref_bytes(name, f"{sim}_center.p3d")


def test_residual_history_columns(ran):
    """Header line exact; step, CFL and the normalised L2 columns as the
    reference printed them (the L-infinity location and the matrix residual
    are checked through the device norms in the GPU tests)."""
    from aither_gb300._lib import Norms
    name, meta, s, l2, _, tmp = ran
    sv = s.solve_view(0)
    nv = l2.shape[1]
    rows = []
    for k in range(len(l2)):
        x = Norms()
        for v in range(nv):
            x.l2[v] = l2[k, v]
        x.cfl = min(sv.cfl_start + k * sv.cfl_step, sv.cfl_max)
        rows.append(x)
    rf = np.zeros(7)
    s.write_resid(0, str(tmp / "r.resid"), rows, 0, rf)
    got = open(tmp / "r.resid").read().splitlines()
    want = ref_bytes(name, f"{meta['sim']}.resid").decode().splitlines()
    assert got[0] == want[0]
    assert len(got) == len(want)
    for g, w in zip(got[1:], want[1:]):
        assert g.split()[:3 + nv] == w.split()[:3 + nv]
    assert np.array_equal(rf[:nv], l2_normalisation(l2))


def test_unsupported_variable_is_an_error(ran):
    """A variable the reference does not write, and a gradient variable
    without the kept gradients, are errors and write no file."""
    from aither_gb300._lib import AthError
    _, _, s, _, fields, tmp = ran
    with pytest.raises(AthError):
        s.write_function(0, fields, str(tmp / "x.fun"), variables=["notAVariable"])
    assert not os.path.exists(tmp / "x.fun")
    bare = [{k: v for k, v in f.items() if k != "grads"} for f in fields]
    with pytest.raises(AthError):
        s.write_function(0, bare, str(tmp / "y.fun"), variables=["tempGrad_x"])
    assert not os.path.exists(tmp / "y.fun")


# ---- bdf2 restart files: two time levels -----------------------------------
RESTART_NAMES = ["plate_bdf2_rst", "sst_bdf2_rst"]


def restart_case(name, tmp):
    with open(os.path.join(OUT, name, "case.json")) as f:
        meta = json.load(f)
    from aither_gb300 import cases
    inp, _ = getattr(cases, meta["generator"])(str(tmp), **meta["kwargs"])
    return inp, meta


def time_normalisation(l2, nl):
    """PrintResiduals' normalisation of a time-accurate run: the first
    nonlinear iteration of each of the first five time steps."""
    return l2_normalisation(l2[::nl])


def oracle_restart_fields(o, s):
    prims = [o.field(b, "STATE") for b in s.solve_blocks(0)]
    nm1 = [o.field(b, "CONS_NM1") for b in s.solve_blocks(0)]
    return prims, nm1


@pytest.mark.parametrize("name", RESTART_NAMES)
def test_bdf2_restart_written_and_continued(name, tmp_path):
    """The oracle's state and time n-1 after N time steps, written by the
    library's restart writer, are the reference's file byte for byte; read
    back into a fresh oracle (state and time n-1 from the file) and run M
    more time steps, they give the reference's restarted run's file."""
    from pyoracle import Oracle

    from aither_gb300 import Setup
    inp, meta = restart_case(name, tmp_path)
    n1, n2 = meta["steps"]
    nl, sim = meta["kwargs"]["nl"], meta["sim"]
    s = Setup(inp)
    o = Oracle(s, 1)
    l2 = o.iterate(n1 * nl)[:, 0, :]
    rf = time_normalisation(l2, nl)
    prims, nm1 = oracle_restart_fields(o, s)
    path = str(tmp_path / "a.rst")
    s.write_restart(0, n1, rf, prims, path, nm1=nm1)
    assert open(path, "rb").read() == ref_bytes(name, f"{sim}_{n1}.rst")
    o.close()

    it, rf1, prims1, levels, nm1_1 = s.read_restart(0, os.path.join(OUT, name, f"{sim}_{n1}.rst"),
                                                    levels=True)
    assert it == n1 and levels == 2 and np.array_equal(rf1, rf)
    o2 = Oracle(s, 1)
    for k, b in enumerate(s.solve_blocks(0)):
        o2.set_state(b, prims1[k])
        o2.set_state_nm1(b, nm1_1[k])
    o2.iterate(n2 * nl)
    prims2, nm1_2 = oracle_restart_fields(o2, s)
    path2 = str(tmp_path / "b.rst")
    s.write_restart(0, n1 + n2, rf1, prims2, path2, nm1=nm1_2)
    assert open(path2, "rb").read() == ref_bytes(name, f"{sim}_{n1 + n2}.rst")
    o2.close()
    s.close()


def test_bdf2_restart_needs_time_n_minus_1(tmp_path):
    from aither_gb300 import Setup
    from aither_gb300._lib import AthError
    inp, meta = restart_case("plate_bdf2_rst", tmp_path)
    s = Setup(inp)
    prims = [np.ones((v.nk, v.nj, v.ni, 5)) for v in map(s.block_view, s.solve_blocks(0))]
    with pytest.raises(AthError):
        s.write_restart(0, 1, np.ones(5), prims, str(tmp_path / "x.rst"))
    s.close()


def _norm_rows(l2):
    from aither_gb300._lib import Norms
    rows = []
    for k in range(len(l2)):
        x = Norms()
        for v in range(l2.shape[1]):
            x.l2[v] = l2[k, v]
        rows.append(x)
    return rows


@pytest.mark.parametrize("name", RESTART_NAMES)
def test_bdf2_residual_history(name, tmp_path):
    """Time-accurate residual history: time step and nonlinear iteration
    columns, the input's time step, the normalisation of the first
    nonlinear iterations of time steps 0-4; the restarted run appends a
    header and rows numbered on from the restart, normalised by the file's
    values."""
    from pyoracle import Oracle

    from aither_gb300 import Setup
    inp, meta = restart_case(name, tmp_path)
    n1, n2 = meta["steps"]
    nl, sim = meta["kwargs"]["nl"], meta["sim"]
    s = Setup(inp)
    nv = s.solve_nv(0)
    o = Oracle(s, 1)
    l2 = o.iterate(n1 * nl)[:, 0, :]
    prims, nm1 = oracle_restart_fields(o, s)
    o.close()
    rf = np.zeros(7)
    path = str(tmp_path / "r.resid")
    s.write_resid(0, path, _norm_rows(l2), 0, rf)
    got = open(path).read().splitlines()
    want = ref_bytes(name, f"{sim}_{n1}.resid").decode().splitlines()
    assert got[0] == want[0] and len(got) == len(want)
    for g, w in zip(got[1:], want[1:]):
        assert g.split()[:3 + nv] == w.split()[:3 + nv]
    assert np.array_equal(rf[:nv], time_normalisation(l2, nl))

    o2 = Oracle(s, 1)
    for k, b in enumerate(s.solve_blocks(0)):
        o2.set_state(b, prims[k])
        o2.set_state_nm1(b, nm1[k])
    l2b = o2.iterate(n2 * nl)[:, 0, :]
    o2.close()
    rf_file = rf.copy()
    s.write_resid(0, path, _norm_rows(l2b), n1 * nl, rf, append=True, restarted=True)
    assert np.array_equal(rf, rf_file)
    got = open(path).read().splitlines()
    want_b = ref_bytes(name, f"{sim}_{n1 + n2}.resid").decode().splitlines()
    # the reference prints its header again when a restarted run opens the file
    got = got[:len(want)] + [want[0]] + got[len(want):]
    assert len(got) == len(want_b)
    for g, w in zip(got, want_b):
        assert g.split()[:3 + nv] == w.split()[:3 + nv]
    s.close()
