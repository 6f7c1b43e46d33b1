"""Generates the output-format fixtures of tests/golden/output/ by running
the reference solver's own executable (built from its sources by
oracle/ref_build into oracle/_ref/aither) on small seeded cases with long
outputVariables lists and a restart frequency.  Each case directory keeps
the files the reference wrote after N iterations:

    <sim>_<N>.rst          restart file (WriteRestart)
    <sim>_<N>_center.fun   Plot3D cell-centre function file (WriteFunFile)
    <grid>_center.xyz      cell-centre grid (WriteCellCenter)
    <sim>_center.p3d       Paraview meta file (WriteMeta)
    <sim>.resid            residual history (PrintHeaders / PrintResiduals)
    case.json              generator, arguments, iterations, variables

Restart cases (bdf2, two time levels in the restart file) keep the restart
file after N time steps and the one the reference wrote after M more time
steps of a run restarted from it:

    <sim>_<N>.rst, <sim>_<N+M>.rst, case.json
    <sim>_<N>.resid, <sim>_<N+M>.resid   residual histories of the two runs

    python tests/golden/make_output_golden.py [--reference /path/to/aither]
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from aither_gb300 import cases  # noqa: E402

REF_EXE = os.path.join(ROOT, "oracle", "_ref", "aither")
OUT = os.path.join(HERE, "output")

COMMON = ["density", "vel_x", "vel_y", "vel_z", "pressure", "mach", "sos", "dt", "energy",
          "enthalpy", "cp", "cv", "rank", "globalPosition", "mf_air", "vf_air", "resid_mass",
          "resid_mom_x", "resid_mom_y", "resid_mom_z", "resid_energy"]
VISC = ["temperature", "viscosity", "wallDistance"]
VELGRAD = ["velGrad_" + a + b for b in "xyz" for a in "uvw"]
GRADS = [f"{q}Grad_{a}" for q in ("temp", "density", "press") for a in "xyz"]
TURB_GRADS = [f"{q}Grad_{a}" for q in ("tke", "omega") for a in "xyz"]
SST = ["tke", "sdr", "f1", "f2", "viscosityRatio", "turbulentViscosity", "resid_tke",
       "resid_sdr"]

# (name, generator, kwargs, iterations, variables)
CASES = [
    ("plate", "flat_plate", dict(ni=12, nj=8, nk=2, dy0=1e-3, ratio=1.3, name="plate"), 6,
     COMMON + VISC + VELGRAD + GRADS),
    ("sst", "flat_plate", dict(ni=12, nj=10, nk=2, dy0=1e-4, ratio=1.3, reynolds=5e6, mach=0.2,
                               rans=True, nblocks=1, matrix_solver="blusgs", name="sst"), 4,
     COMMON + VISC + VELGRAD + SST + GRADS + TURB_GRADS),
    ("bump", "bump_channel", dict(ni=16, nj=8, nk=3, height=0.08, mach=0.6, name="bump"), 5,
     COMMON + ["wallDistance"] + VELGRAD + GRADS),
]


# (name, generator, kwargs, time steps before the restart, time steps after)
RESTARTS = [
    ("plate_bdf2_rst", "flat_plate",
     dict(ni=12, nj=8, nk=2, dy0=1e-3, ratio=1.3, time="bdf2", dt=1e-4, nl=2, name="plate"),
     3, 2),
    ("sst_bdf2_rst", "flat_plate",
     dict(ni=12, nj=10, nk=2, dy0=1e-4, ratio=1.3, reynolds=5e6, mach=0.2, rans=True,
          nblocks=1, matrix_solver="blusgs", time="bdf2", dt=1e-5, nl=2, name="sst"), 3, 2),
]


def case_input(tmp: str, gen: str, kw: dict, iterations: int, variables: list) -> str:
    inp, _ = getattr(cases, gen)(tmp, **kw)
    cases.set_output_keys(inp, iterations, variables, restart_freq=iterations)
    return inp


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=REF_EXE)
    ap.add_argument("--install-dir", default=os.environ.get("AITHER_REFERENCE_SRC"),
                    help="directory holding fluidDatabase/ (the reference's source tree, "
                         "or AITHER_REFERENCE_SRC)")
    ap.add_argument("--only", nargs="*", help="case names to (re)generate")
    args = ap.parse_args()
    os.makedirs(OUT, exist_ok=True)
    env = dict(os.environ, AITHER_INSTALL_DIRECTORY=args.install_dir)

    def run(tmp, name, *argv):
        r = subprocess.run([args.reference, *argv], cwd=tmp, env=env, capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{name}: reference failed\n{r.stdout[-2000:]}{r.stderr}")

    for name, gen, kw, n1, n2 in RESTARTS:
        if args.only and name not in args.only:
            continue
        with tempfile.TemporaryDirectory() as tmp:
            inp = case_input(tmp, gen, kw, n1, ["density"])
            cases.set_output_keys(inp, n1, ["density"], restart_freq=n1)
            sim = os.path.splitext(os.path.basename(inp))[0]
            run(tmp, name, os.path.basename(inp))
            shutil.copy(os.path.join(tmp, f"{sim}.resid"), os.path.join(tmp, f"{sim}_{n1}.resid"))
            cases.set_output_keys(inp, n2, ["density"], restart_freq=n2)
            run(tmp, name, os.path.basename(inp), f"{sim}_{n1}.rst")
            shutil.copy(os.path.join(tmp, f"{sim}.resid"),
                        os.path.join(tmp, f"{sim}_{n1 + n2}.resid"))
            dest = os.path.join(OUT, name)
            shutil.rmtree(dest, ignore_errors=True)
            os.makedirs(dest)
            for fn in (f"{sim}_{n1}.rst", f"{sim}_{n1 + n2}.rst", f"{sim}_{n1}.resid",
                       f"{sim}_{n1 + n2}.resid"):
                shutil.copy(os.path.join(tmp, fn), os.path.join(dest, fn))
            with open(os.path.join(dest, "case.json"), "w") as f:
                json.dump({"generator": gen, "kwargs": kw, "steps": [n1, n2], "sim": sim}, f,
                          indent=1)
            print(name, "->", dest, sorted(os.listdir(dest)))

    for name, gen, kw, iters, variables in CASES:
        if args.only is not None and name not in args.only:
            continue
        with tempfile.TemporaryDirectory() as tmp:
            inp = case_input(tmp, gen, kw, iters, variables)
            r = subprocess.run([args.reference, os.path.basename(inp)], cwd=tmp, env=env,
                               capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{name}: reference failed\n{r.stdout[-2000:]}{r.stderr}")
            sim = os.path.splitext(os.path.basename(inp))[0]
            dest = os.path.join(OUT, name)
            shutil.rmtree(dest, ignore_errors=True)
            os.makedirs(dest)
            for fn in (f"{sim}_{iters}.rst", f"{sim}_{iters}_center.fun",
                       f"{kw['name']}_center.xyz", f"{sim}_center.p3d", f"{sim}.resid"):
                shutil.copy(os.path.join(tmp, fn), os.path.join(dest, fn))
            with open(os.path.join(dest, "case.json"), "w") as f:
                json.dump({"generator": gen, "kwargs": kw, "iterations": iters,
                           "variables": variables, "sim": sim}, f, indent=1)
            print(name, "->", dest, sorted(os.listdir(dest)))


if __name__ == "__main__":
    main()
