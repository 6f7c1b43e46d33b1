"""Host-side setup and the C ABI surface (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REF_HARNESS, REF_SRC, ROOT


def _header_functions():
    txt = open(os.path.join(ROOT, "include", "aither_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ath_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from aither_gb300 import _lib
    L = ctypes.CDLL(_lib.LIB_PATH)
    names = _header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_oracle_library_exports():
    import pyoracle
    L = ctypes.CDLL(pyoracle.ORACLE_LIB)
    for n in ("orc_create", "orc_iterate", "orc_residual", "orc_relax", "orc_update"):
        assert hasattr(L, n)


def test_bad_input_reports_error(tmp_path):
    from aither_gb300 import AthError, Setup
    with pytest.raises(AthError) as e:
        Setup(str(tmp_path / "missing.inp"))
    assert "cannot open" in str(e.value)
    p = tmp_path / "x.inp"
    p.write_text("gridName: x\nequationSet: euler\ntimeIntegration: implicitEuler\n"
                 "faceReconstruction: weno\nreferenceTemperature: 288\n"
                 "referenceDensity: 1.2\nboundaryConditions: 0\n")
    with pytest.raises(AthError):
        Setup(str(p))


def test_geometry_of_box(tmp_path):
    from aither_gb300 import Setup, cases
    inp, st = cases.vortex_box(str(tmp_path), 8, 4, 2, name="g")
    s = Setup(inp)
    g = s.geometry(0)
    ng = g["ng"]
    vol = g["vol"][ng:-ng, ng:-ng, ng:-ng]
    assert np.isclose(vol.sum(), 10.0 * 5.0 * 1.25, rtol=1e-14)
    w = g["width"]
    assert np.allclose(w[0][ng:-ng, ng:-ng, :], 10.0 / 8)  # ghost widths too
    fi = g["fareai"]
    assert np.allclose(fi[0][ng:-ng, ng:-ng, ng:-ng - 0], 1.0)


def test_hyperplane_order_and_ghost_ops(tmp_path):
    from aither_gb300 import Setup, cases
    inp, _ = cases.bump_channel(str(tmp_path), 7, 5, 3, 0.05, 0.5, name="h")
    s = Setup(inp)
    v = s.block_view(0)
    ni, nj, nk, ng = v.ni, v.nj, v.nk, v.ng
    NI, NJ = ni + 2 * ng, nj + 2 * ng
    off = np.ctypeslib.as_array(v.plane_offsets, (v.nplanes + 1,))
    cells = np.ctypeslib.as_array(v.plane_cells, (ni * nj * nk,))
    assert v.nplanes == ni + nj + nk - 2
    seen = set()
    for p in range(v.nplanes):
        for c in cells[off[p]:off[p + 1]]:
            i, j, k = c % NI - ng, (c // NI) % NJ - ng, c // (NI * NJ) - ng
            assert i + j + k == p
            seen.add(int(c))
    assert len(seen) == ni * nj * nk
    ops = s.geometry(0)["ops"]
    # every ghost cell of the 6 faces, ng layers deep, is written once
    expect = ng * 2 * (nj * nk + ni * nk + ni * nj)
    assert len(ops) == expect
    assert len(set(int(o["dst"]) for o in ops)) == expect


def test_periodic_connections_pair_interior_cells(tmp_path):
    from aither_gb300 import Setup, cases
    inp, _ = cases.vortex_box(str(tmp_path), 6, 4, 2, name="p")
    s = Setup(inp)
    v = s.block_view(0)
    ng, NI, NJ = v.ng, v.ni + 2 * v.ng, v.nj + 2 * v.ng
    ops = s.geometry(0)["ops"]
    conn = [o for o in ops if o["type"] == 7]
    assert len(conn) == 2 * ng * (v.nj * v.nk + v.ni * v.nk)
    for o in conn:
        src = int(o["src"])
        i, j, k = src % NI - ng, (src // NI) % NJ - ng, src // (NI * NJ) - ng
        assert 0 <= i < v.ni and 0 <= j < v.nj and 0 <= k < v.nk
        dst = int(o["dst"])
        di, dj = dst % NI - ng, (dst // NI) % NJ - ng
        # periodic in i: ghost i=-L <- interior i=ni-L (and vice versa)
        if o["dir"] == 0:
            assert (di - i) % v.ni == 0 and dj == j


@pytest.mark.skipif(not (os.path.exists(REF_HARNESS) and os.path.isdir(REF_SRC)),
                    reason="reference build not available on this machine")
def test_geometry_matches_reference(tmp_path):
    import subprocess

    from refdump import read_dump

    from aither_gb300 import Setup, cases
    inp, _ = cases.bump_channel(str(tmp_path), 12, 6, 3, 0.1, 0.5, name="geo")
    env = dict(os.environ, AITHER_INSTALL_DIRECTORY=REF_SRC)
    r = subprocess.run([REF_HARNESS, "geo.inp", "1", "out.bin"], cwd=str(tmp_path),
                       env=env, capture_output=True, text=True)
    assert r.returncode == 0
    R = read_dump(str(tmp_path / "out.bin"))
    g = Setup(inp).geometry(0)
    ng = g["ng"]
    p = (slice(ng, -ng),) * 3
    assert np.array_equal(g["vol"][p], R["b0_vol"][p])
    assert np.array_equal(np.moveaxis(g["center"], 0, -1)[p], R["b0_center"][p])
    w, rw = np.moveaxis(g["width"], 0, -1), R["b0_width"]
    assert np.array_equal(w[ng:-ng, ng:-ng, :, 0], rw[ng:-ng, ng:-ng, :, 0])
    assert np.array_equal(w[ng:-ng, :, ng:-ng, 1], rw[ng:-ng, :, ng:-ng, 1])
    assert np.array_equal(w[:, ng:-ng, ng:-ng, 2], rw[:, ng:-ng, ng:-ng, 2])
    for d, nm in enumerate(["fareai", "fareaj", "fareak"]):
        a = np.moveaxis(g[nm], 0, -1)
        sl = [slice(ng, -ng)] * 3
        sl[2 - d] = slice(ng, -ng if True else None)
        ext = [slice(ng, -ng)] * 3
        ext[2 - d] = slice(ng, a.shape[2 - d] - ng)
        assert np.array_equal(a[tuple(ext)], R["b0_" + nm][tuple(ext)])


def test_nonreflecting_inlet_and_outlet_parsed(tmp_path):
    """inlet(...; nonreflecting=true; lengthScale=L) is accepted with L over
    the reference length, and so is a nonreflecting pressure outlet;
    nonreflecting without lengthScale is a setup error."""
    from aither_gb300 import Setup, cases
    from aither_gb300._lib import AthError
    kw = dict(ni=8, nj=4, nk=2, height=0.05, mach=0.4, inflow="inlet", outflow="pressure")
    inp, _ = cases.bump_channel(str(tmp_path / "a"), nonreflecting=2.0, **kw)
    s = Setup(inp)
    sv = s.solve_view(0)
    st = [sv.states[i] for i in range(sv.nstates)]
    nr = [x for x in st if x.nonreflecting]
    assert len(nr) == 1 and nr[0].length_scale == 2.0 / sv.l_ref
    assert sum(s.block_view(b).n_nr for b in range(s.counts()[1])) == 4 * 2
    s.close()
    text = open(inp).read()
    bad = text.replace("pressureOutlet(tag=4; pressure=",
                       "pressureOutlet(tag=4; nonreflecting=true; lengthScale=1.0; pressure=")
    open(inp, "w").write(bad)
    s = Setup(inp)
    sv = s.solve_view(0)
    po = [sv.states[i] for i in range(sv.nstates) if sv.states[i].nonreflecting]
    assert len(po) == 2 and po[1].length_scale == 1.0 / sv.l_ref
    s.close()
    bad = re.sub(r"; lengthScale=[^;)]*", "", text)
    assert "nonreflecting=true" in bad and "lengthScale" not in bad
    open(inp, "w").write(bad)
    with pytest.raises(AthError, match="lengthScale"):
        Setup(inp)


def test_multigrid_levels(tmp_path):
    """multigridLevels: each coarser level keeps every node a boundary
    surface starts or ends on and otherwise every other node
    (procBlock::GetCoarseMeshAndBCs); the transfer maps restrict with
    weights that sum to one per coarse cell and prolong with coefficients
    in [0, 1] on these box-like cells; turbulence equations, time-accurate
    solves and nonreflecting boundaries are refused with multigrid."""
    from aither_gb300 import Setup, cases
    from aither_gb300._lib import AthError
    inp, _ = cases.bump_channel(str(tmp_path / "a"), ni=26, nj=14, nk=5, height=0.07, mach=0.6,
                                multigrid=(3, "W"))
    s = Setup(inp)
    assert s.levels() == 3
    dims = [(s.block_view(0, lv).ni, s.block_view(0, lv).nj, s.block_view(0, lv).nk)
            for lv in range(3)]
    assert dims == [(26, 14, 5), (13, 7, 3), (7, 4, 2)]
    assert s.solve_view(0, 1).mg_cycle == 2 and s.solve_view(0, 0).mg_levels == 3
    for lv in range(2):
        m = s.mg_map(lv, 0)
        nc = s.level_counts(lv + 1)[2]
        sums = np.bincount(m["coarse_cell"], weights=m["volfac"], minlength=nc)
        assert np.allclose(sums, 1.0, atol=1e-14)
        assert m["coef"].min() >= -1e-12 and m["coef"].max() <= 1 + 1e-12
    s.close()
    for kw in (dict(time="bdf2", dt=1e-5, nl=3), dict(inflow="inlet", outflow="pressure",
                                                      nonreflecting=1.0)):
        inp, _ = cases.bump_channel(str(tmp_path / "b"), ni=8, nj=4, nk=2, height=0.05, mach=0.4,
                                    multigrid=(2, "V"), **kw)
        with pytest.raises(AthError, match="multigrid"):
            Setup(inp)
    inp, _ = cases.flat_plate(str(tmp_path / "c"), ni=8, nj=6, nk=2, dy0=1e-3, ratio=1.3,
                              rans=True, nblocks=1, multigrid=(2, "V"))
    with pytest.raises(AthError, match="multigrid"):
        Setup(inp)
