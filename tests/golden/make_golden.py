"""Generates the golden fixtures of tests/golden/ by running the reference
solver itself (built from its sources by oracle/ref_build into oracle/_ref)
through oracle/ref_build/ref_harness.cpp on seeded synthetic cases and on
the reference's own test cases.

    python tests/golden/make_golden.py --reference /path/to/aither [--only ...]
    (or AITHER_REFERENCE_SRC=/path/to/aither)

The reference's test cases (testCases/<case>/<case>.inp and its grid) are
copied into tests/golden/refcases/<case>/, which is not committed, so that
the tests can set the same cases up on machines without the reference's
sources; their fixtures are ref_<case>_it<N>.npz.

Each fixture is an .npz with the fields the reference produced:
  <case>_it<N>.npz : state0, state (physical, after N iterations), resid,
                     dt, specrad, du (of iteration N), l2 and matrix_resid
                     (per iteration), forces (wall forces of iteration N)
Small grids keep the fixtures a few hundred kB; the full-size vortex-box
configuration (64x32x8, 200 iterations) stores its L2 history and summary
statistics of the final state only.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from aither_gb300 import cases  # noqa: E402
from refdump import read_dump  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
REFCASE_DIR = os.path.join(HERE, "refcases")

# (fixture name, generator, kwargs, iterations, full fields?)
CASES = [
    # multigrid (coarse-grid correction of the linear system): V and W
    # cycles over 2 and 3 levels with LU-SGS (1 and 3 sweeps), DP-LUR, block
    # LU-SGS and block DP-LUR; the plates have an interblock connection on
    # every level
    ("bump_mg_v", cases.bump_channel,
     dict(ni=24, nj=12, nk=4, height=0.08, mach=0.7, multigrid=(2, "V")), [1, 15], True),
    ("bump_mg_w3", cases.bump_channel,
     dict(ni=26, nj=14, nk=5, height=0.07, mach=0.6, sweeps=3, multigrid=(3, "W")),
     [1, 15], True),
    ("bump_mg_dplur", cases.bump_channel,
     dict(ni=20, nj=12, nk=3, height=0.08, mach=0.7, matrix_solver="dplur", sweeps=3,
          multigrid=(3, "V")), [1, 15], True),
    ("plate_mg_blusgs", cases.flat_plate,
     dict(ni=12, nj=10, nk=2, dy0=1e-3, ratio=1.3, matrix_solver="blusgs", sweeps=2,
          multigrid=(2, "W")), [1, 15], True),
    ("plate_mg_bdplur", cases.flat_plate,
     dict(ni=14, nj=8, nk=2, dy0=1e-3, ratio=1.3, cfl=20.0, matrix_solver="bdplur", sweeps=4,
          multigrid=(3, "V")), [1, 15], True),
    # Wilcox k-omega 2006: scalar LU-SGS on one block, block LU-SGS with 2
    # sweeps on two blocks
    ("wk_plate", cases.flat_plate,
     dict(ni=12, nj=10, nk=2, dy0=1e-4, ratio=1.3, reynolds=5e6, mach=0.2, rans=True,
          nblocks=1, turb_model="kOmegaWilcox2006"), [1, 15], True),
    ("wk_plate2_blusgs", cases.flat_plate,
     dict(ni=10, nj=10, nk=2, dy0=1e-4, ratio=1.3, reynolds=5e6, mach=0.2, rans=True,
          matrix_solver="blusgs", sweeps=2, turb_model="kOmegaWilcox2006"), [1, 15], True),
    ("vortex16", cases.vortex_box, dict(ni=16, nj=8, nk=4), [1, 20], True),
    ("bump24", cases.bump_channel, dict(ni=24, nj=12, nk=4, height=0.08, mach=0.7), [1, 30], True),
    ("bump_sup", cases.bump_channel, dict(ni=20, nj=10, nk=3, height=0.10, mach=0.85), [1, 40], True),
    ("vortex_c1", cases.vortex_box, dict(), [200], False),
    ("bump_weno", cases.bump_channel,
     dict(ni=20, nj=10, nk=4, height=0.1, mach=0.8, recon="weno", limiter="none"), [1, 20], True),
    ("bump_wenoz_ausm", cases.bump_channel,
     dict(ni=18, nj=9, nk=4, height=0.07, mach=0.6, recon="wenoZ", limiter="none", flux="ausm"),
     [1, 20], True),
    ("bump_const_ausm", cases.bump_channel,
     dict(ni=16, nj=8, nk=3, height=0.05, mach=0.5, recon="constant", limiter="none",
          flux="ausm"), [1, 20], True),
    ("plate_adiabatic", cases.flat_plate,
     dict(ni=12, nj=8, nk=2, dy0=1e-3, ratio=1.3), [1, 20], True),
    ("plate_isothermal", cases.flat_plate,
     dict(ni=14, nj=9, nk=2, dy0=5e-4, ratio=1.35, wall_t=300.0, mach=0.5), [1, 20], True),
    ("plate_c2", cases.flat_plate, dict(), [20], False),
    ("bump_vanalbada_ausm", cases.bump_channel,
     dict(ni=22, nj=11, nk=3, height=0.09, mach=0.75, limiter="vanAlbada", flux="ausm"),
     [1, 20], True),
    # block LU-SGS (blusgs) and multi-sweep relaxation
    ("bump_blusgs", cases.bump_channel,
     dict(ni=20, nj=10, nk=3, height=0.08, mach=0.7, matrix_solver="blusgs"), [1, 20], True),
    ("bump_sweeps3", cases.bump_channel,
     dict(ni=18, nj=9, nk=3, height=0.06, mach=0.6, sweeps=3), [1, 20], True),
    ("bump_blusgs_weno_sw2", cases.bump_channel,
     dict(ni=16, nj=8, nk=4, height=0.07, mach=0.8, recon="weno", limiter="none",
          matrix_solver="blusgs", sweeps=2), [1, 20], True),
    ("plate_blusgs", cases.flat_plate,
     dict(ni=12, nj=8, nk=2, dy0=1e-3, ratio=1.3, matrix_solver="blusgs"), [1, 20], True),
    ("plate_blusgs_sw2", cases.flat_plate,
     dict(ni=10, nj=8, nk=2, dy0=5e-4, ratio=1.35, wall_t=300.0, mach=0.5,
          matrix_solver="blusgs", sweeps=2), [1, 20], True),
    ("plate_c2b", cases.flat_plate, dict(matrix_solver="blusgs", sweeps=4), [20], False),
    # RANS, SST-2003 (k, omega as equations 6 and 7)
    ("sst_plate", cases.flat_plate,
     dict(ni=12, nj=10, nk=2, dy0=1e-4, ratio=1.3, reynolds=5e6, mach=0.2, rans=True,
          nblocks=1), [1, 20], True),
    ("sst_plate2_blusgs", cases.flat_plate,
     dict(ni=10, nj=10, nk=2, dy0=1e-4, ratio=1.3, reynolds=5e6, mach=0.2, rans=True,
          matrix_solver="blusgs", sweeps=2), [1, 10], True),
    ("sst_weno_ausm", cases.flat_plate,
     dict(ni=14, nj=12, nk=3, dy0=5e-5, ratio=1.25, reynolds=5e6, mach=0.2, rans=True,
          nblocks=1, recon="weno", limiter="none", flux="ausm", matrix_solver="blusgs"),
     [1, 10], True),
    # DP-LUR and block DP-LUR (Jacobi sweeps)
    ("bump_dplur", cases.bump_channel,
     dict(ni=20, nj=10, nk=3, height=0.08, mach=0.7, matrix_solver="dplur", sweeps=3),
     [1, 20], True),
    ("plate_bdplur", cases.flat_plate,
     dict(ni=12, nj=8, nk=2, dy0=1e-3, ratio=1.3, cfl=20.0, matrix_solver="bdplur", sweeps=4),
     [1, 20], True),
    ("sst_plate_dplur", cases.flat_plate,
     dict(ni=12, nj=10, nk=2, dy0=1e-4, ratio=1.3, reynolds=5e6, mach=0.2, rans=True,
          nblocks=1, cfl=20.0, matrix_solver="dplur", sweeps=2), [1, 10], True),
    # stagnation inlet, reference inlet, pressure outlet, heat-flux wall
    ("bump_stag_pout", cases.bump_channel,
     dict(ni=20, nj=10, nk=3, height=0.08, mach=0.5, inflow="stagnation", outflow="pressure"),
     [1, 20], True),
    ("bump_inlet_pout", cases.bump_channel,
     dict(ni=18, nj=9, nk=3, height=0.06, mach=0.4, inflow="inlet", outflow="pressure",
          back_pressure=1.02, recon="weno", limiter="none"), [1, 20], True),
    # nonreflecting inlet: steady, and bdf2 dual time
    ("bump_nr", cases.bump_channel,
     dict(ni=18, nj=9, nk=3, height=0.06, mach=0.4, inflow="inlet", outflow="pressure",
          back_pressure=1.02, nonreflecting=2.0), [1, 20], True),
    ("bump_nr_bdf2", cases.bump_channel,
     dict(ni=18, nj=9, nk=3, height=0.06, mach=0.4, inflow="inlet", outflow="pressure",
          back_pressure=1.02, nonreflecting=0.5, time="bdf2", dt=2e-5, nl=3), [1, 12], True),
    # nonreflecting pressure outlet (LODI with transverse terms from the
    # previous residual's gradients): steady inviscid, with a nonreflecting
    # inlet in bdf2 dual time, and a laminar viscous channel
    ("bump_nr_out", cases.bump_channel,
     dict(ni=18, nj=9, nk=3, height=0.06, mach=0.4, inflow="inlet", outflow="pressure",
          back_pressure=1.02, nr_outlet=1.5), [1, 20], True),
    ("bump_nr_both_bdf2", cases.bump_channel,
     dict(ni=16, nj=8, nk=3, height=0.08, mach=0.5, inflow="inlet", outflow="pressure",
          back_pressure=0.98, nonreflecting=0.5, nr_outlet=0.8, time="bdf2", dt=2e-5, nl=3),
     [1, 8], True),
    ("chan_nr_out_visc", cases.wall_channel,
     dict(ni=16, nj=10, nk=2, kind="bump", param=0.06, mach=0.4, viscous=True, reynolds=5e4,
          stretch=1.15, cfl=10.0, inflow="stagnation", outflow="pressure", nr_outlet=1.0),
     [1, 10], True),
    ("plate_heatflux", cases.flat_plate,
     dict(ni=12, nj=8, nk=2, dy0=1e-3, ratio=1.3, wall_q=500.0), [1, 20], True),
    ("sst_chan_stag_pout", cases.wall_channel,
     dict(ni=16, nj=10, nk=3, kind="bump", param=0.06, mach=0.5, alpha=2.0, rans=True,
          stretch=1.1, cfl=5.0, inflow="stagnation", outflow="pressure"), [1, 10], True),
    # time-accurate: iterations count time steps, each of nl nonlinear iterations
    ("vortex_bdf2", cases.vortex_box,
     dict(ni=16, nj=8, nk=4, time="bdf2", dt=5e-4, nl=3), [1, 4], True),
    ("vortex_cn_dual", cases.vortex_box,
     dict(ni=16, nj=8, nk=4, time="crankNicholson", dt=5e-4, nl=3, dual_cfl=5.0), [1, 4], True),
    ("plate_bdf2_blusgs", cases.flat_plate,
     dict(ni=12, nj=8, nk=2, dy0=1e-3, ratio=1.3, matrix_solver="blusgs", time="bdf2",
          dt=1e-4, nl=2), [1, 4], True),
    ("sst_plate_bdf2", cases.flat_plate,
     dict(ni=12, nj=10, nk=2, dy0=1e-4, ratio=1.3, reynolds=5e6, mach=0.2, rans=True,
          nblocks=1, time="bdf2", dt=1e-5, nl=2), [1, 4], True),
]
# two blocks joined in each of the 8 patch orientations (block_pair): Euler
# with scalar LU-SGS, and SST-2003 RANS with block LU-SGS
CASES += [(f"pair_{ph}_o{o}", cases.block_pair, dict(orient=o, physics=ph), [1, 10], True)
          for ph in ("euler", "sst") for o in range(8)]

# full-size configurations whose per-cell fields are kept only for the first
# cells along one direction (d, n), with per-variable sums of |value| over
# every cell: (fixture name, generator, kwargs, iteration counts, rows)
ROWCASES = [
    # the 256x192x4 SST-2003 flat plate (WENO, AUSMPW+, block LU-SGS)
    ("sst_c3", cases.sst_plate, dict(), [1], (1, 16)),
]

# the reference's own test cases: (case, iteration counts, rows kept of the
# per-cell fields: None = all; (d, n) = the first n cells along direction d)
REFCASES = [
    ("uniformFlow", [1, 20], None),
    ("subsonicCylinder", [1, 20], None),
    ("multiblockCylinder", [1, 20], None),
    ("couette", [1, 20], None),
    ("viscousFlatPlate", [1, 20], None),
    ("rae2822", [1, 20], (1, 8)),
    ("shockTube", [1, 4], None),
    ("transonicBump", [1, 20], None),
    ("turbFlatPlate", [1, 20], None),
]


def run_case(name, gen, kw, niter, full, ref_dir):
    with tempfile.TemporaryDirectory() as d:
        inp, st = gen(d, name=name, **kw)
        args = [HARNESS, os.path.basename(inp), str(niter), "out.bin"]
        if st is not None:
            np.concatenate([np.asarray(x, dtype="<f8").reshape(-1) for x in st]).tofile(
                os.path.join(d, "state.bin"))
            args.append("state.bin")
        env = dict(os.environ, AITHER_INSTALL_DIRECTORY=ref_dir)
        r = subprocess.run(args, cwd=d, env=env, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference harness failed on {name}: {r.stderr[-2000:]}")
        R = read_dump(os.path.join(d, "out.bin"))
    nblocks = sum(1 for k in R if k.startswith("b") and k.endswith("_resid"))
    out = {"l2": R["l2"], "matrix_resid": R["matrix_resid"], "forces": R["forces"],
           "kwargs": np.array(repr(kw)),
           "iterations": np.array(niter), "nblocks": np.array(nblocks)}
    for b in range(nblocks):
        p = f"b{b}_"
        ng = (R[p + "state"].shape[0] - R[p + "resid"].shape[0]) // 2
        state = R[p + "state"][ng:-ng, ng:-ng, ng:-ng]
        if full:
            out.update({p + "state0": R[p + "state0"], p + "state": state,
                        p + "resid": R[p + "resid"], p + "dt": R[p + "dt"],
                        p + "specrad": R[p + "specrad"], p + "du": R[p + "du"]})
        else:
            out.update({p + "state_sum": state.reshape(-1, 5).sum(axis=0),
                        p + "state_sumsq": (state.reshape(-1, 5) ** 2).sum(axis=0),
                        p + "state_samples": state[::3, ::7, ::11].copy()})
    path = os.path.join(HERE, f"{name}_it{niter}.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


def copy_refcase(case, ref_dir):
    """Copies a reference test case (input file and grid) into
    tests/golden/refcases/<case>/ and returns its input path there."""
    import shutil
    src = os.path.join(ref_dir, "testCases", case)
    dst = os.path.join(REFCASE_DIR, case)
    os.makedirs(dst, exist_ok=True)
    for f in os.listdir(src):
        if f.endswith((".inp", ".xyz")):
            shutil.copy(os.path.join(src, f), dst)
    return os.path.join(dst, case + ".inp")


def run_refcase(case, niter, rows, ref_dir, gen=None, kw=None):
    """A reference test case (gen None) or a generated full-size case, with
    the per-cell fields restricted to `rows`."""
    with tempfile.TemporaryDirectory() as d:
        import shutil
        if gen is None:
            inp = copy_refcase(case, ref_dir)
            for f in os.listdir(os.path.dirname(inp)):
                shutil.copy(os.path.join(os.path.dirname(inp), f), d)
            name = case
        else:
            inp, _ = gen(d, name=case, **kw)
            name = os.path.basename(inp)[:-4]
        env = dict(os.environ, AITHER_INSTALL_DIRECTORY=ref_dir)
        r = subprocess.run([HARNESS, name + ".inp", str(niter), "out.bin"], cwd=d, env=env,
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference harness failed on {case}: {r.stderr[-2000:]}")
        R = read_dump(os.path.join(d, "out.bin"))
    nblocks = sum(1 for k in R if k.startswith("b") and k.endswith("_resid"))
    out = {"l2": R["l2"], "matrix_resid": R["matrix_resid"], "forces": R["forces"],
           "case": np.array(case), "iterations": np.array(niter), "nblocks": np.array(nblocks),
           "rows": np.array(rows if rows else (-1, -1)), "kwargs": np.array(repr(kw or {}))}
    for b in range(nblocks):
        p = f"b{b}_"
        ng = (R[p + "state"].shape[0] - R[p + "resid"].shape[0]) // 2
        fields = {"state": R[p + "state"][ng:-ng, ng:-ng, ng:-ng], "resid": R[p + "resid"],
                  "dt": R[p + "dt"], "specrad": R[p + "specrad"], "du": R[p + "du"]}
        for key, a in fields.items():
            if rows:
                d_, n_ = rows
                sl = [slice(None)] * a.ndim
                sl[2 - d_] = slice(0, n_)
                out[p + key + "_abssum"] = np.abs(a).reshape(
                    a.shape[0] * a.shape[1] * a.shape[2], -1).sum(0)
                a = a[tuple(sl)]
            out[p + key] = np.ascontiguousarray(a)
    path = os.path.join(HERE, f"{'ref_' if gen is None else ''}{case}_it{niter}.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("AITHER_REFERENCE_SRC"),
                    help="the reference's source tree (or AITHER_REFERENCE_SRC)")
    ap.add_argument("--only", nargs="*", help="fixture base names to (re)generate")
    a = ap.parse_args()
    if not a.reference or not os.path.isdir(os.path.join(a.reference, "src")):
        ap.error("--reference (or AITHER_REFERENCE_SRC) must name the reference's source tree")
    if not os.path.exists(HARNESS):
        sys.path.insert(0, ROOT)
        from aither_gb300 import build
        build.build_reference(a.reference)
    for name, gen, kw, iters, full in CASES:
        if a.only and name not in a.only:
            continue
        for n in iters:
            run_case(name, gen, kw, n, full, a.reference)
    for case, iters, rows in REFCASES:
        if a.only and case not in a.only:
            continue
        for n in iters:
            run_refcase(case, n, rows, a.reference)
    for name, gen, kw, iters, rows in ROWCASES:
        if a.only and name not in a.only:
            continue
        for n in iters:
            run_refcase(name, n, rows, a.reference, gen, kw)


if __name__ == "__main__":
    main()
