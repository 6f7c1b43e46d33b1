"""The reference's own test cases: where they live, their fixtures, their
tolerances and the reference's regression truth table.

The cases (input file and grid) are copied from the reference's
testCases/<case>/ into tests/golden/refcases/<case>/ by
tests/golden/make_golden.py; that directory is not committed, so these
tests skip on machines where it is absent.  Fixtures ref_<case>_it<N>.npz
are the reference build's own results (committed).
"""
from __future__ import annotations

import os
import shutil

import numpy as np

from conftest import GOLDEN, REFCASES, load_golden, rel_err

# (case, fixture iteration counts): counts are time steps for the
# time-accurate shockTube (bdf2, 5 nonlinear iterations per step)
FIXTURES = [("uniformFlow", (1, 20)), ("subsonicCylinder", (1, 20)),
            ("multiblockCylinder", (1, 20)), ("couette", (1, 20)),
            ("viscousFlatPlate", (1, 20)), ("rae2822", (1, 20)), ("shockTube", (1, 4)),
            ("transonicBump", (1, 20)), ("turbFlatPlate", (1, 20))]

# testCases/regressionTests.py: normalised L2 of the last residual-file row
# after `iterations` (single-process values), 1 % tolerance; columns in
# `ignore` are not compared (the reference's SetIgnoreIndices).  uniformFlow
# is run-only there (its residual is roundoff of a uniform flow).
TRUTH = {
    "subsonicCylinder": (100, [1.8751e-01, 2.6727e-01, 3.1217e-01, 7.9662e-01, 1.8639e-01], {3}),
    "multiblockCylinder": (100, [2.0529e-01, 3.4540e-01, 5.0153e-01, 1.0180e+00, 1.9997e-01],
                           {3}),
    "shockTube": (100, [4.8537e-01, 4.5855e-01, 1.0000e+00, 1.0000e+00, 2.6434e-01], {2, 3}),
    "viscousFlatPlate": (100, [7.4673e-02, 2.4711e-01, 3.8960e-02, 1.0000e+00, 7.7683e-02],
                         {3}),
    "rae2822": (20, [5.5618e-01, 6.6813e-01, 5.3620e-01, 1.0000e+00, 4.9726e-01, 2.5769e-09,
                     3.4032e-10], {3}),
    "couette": (100, [1.1816e-01, 5.0725e-01, 6.9807e-02, 5.5916e-01, 2.3024e-01], {3}),
    # Wilcox k-omega 2006, 137x97 NASA TMR grid (single-process values)
    "turbFlatPlate": (20, [2.2309e-01, 2.9862e-01, 1.0000e+00, 3.2376e-01, 2.1910e-01,
                           2.5208e-07, 3.3009e-06], {2}),
    # three multigrid levels, W cycle, DP-LUR (single-process values)
    "transonicBump": (100, [2.6152e-02, 1.5984e-02, 9.6803e-03, 1.0000e+00, 1.9215e-02], {3}),
}


def case_input(case: str) -> str:
    return os.path.join(REFCASES, case, case + ".inp")


def have_case(case: str) -> bool:
    return os.path.exists(case_input(case))


def copy_case(case: str, dst: str, iterations: int | None = None) -> str:
    """Copies a case into dst (optionally rewriting its iteration count and
    output frequency as the reference's regression script does) and returns
    the input path there."""
    src = os.path.join(REFCASES, case)
    for f in os.listdir(src):
        shutil.copy(os.path.join(src, f), dst)
    inp = os.path.join(dst, case + ".inp")
    if iterations is not None:
        with open(inp) as f:
            lines = f.readlines()
        with open(inp, "w") as f:
            for ln in lines:
                if "iterations:" in ln and not ln.strip().startswith("nonlinear"):
                    f.write(f"iterations: {iterations}\n")
                elif "outputFrequency:" in ln:
                    f.write(f"outputFrequency: {iterations}\n")
                else:
                    f.write(ln)
    return inp


def fixture(case: str, n: int) -> dict:
    return load_golden(f"ref_{case}_it{n}")


def fixture_fields(g: dict, b: int, key: str, field: np.ndarray) -> tuple:
    """(computed, reference) arrays of one field, restricted to the rows the
    fixture keeps (large cases keep the first cells along one direction)."""
    rows = tuple(int(x) for x in g["rows"])
    ref = g[f"b{b}_{key}"]
    a = np.asarray(field)
    if rows[0] >= 0:
        d, n = rows
        sl = [slice(None)] * a.ndim
        sl[2 - d] = slice(0, n)
        a = a[tuple(sl)]
    if key in ("dt",) and a.ndim == ref.ndim + 1:
        a = a[..., 0]
    return a, ref


def cols_err(a, b):
    """Largest relative error of the flow variables (one scale) and of each
    turbulence variable (its own scale)."""
    a, b = np.asarray(a), np.asarray(b)
    if a.ndim == 3:
        return rel_err(a, b)
    errs = [rel_err(a[..., :5], b[..., :5])]
    errs += [rel_err(a[..., v], b[..., v]) for v in range(5, b.shape[-1])]
    return max(errs)


def uniform_flow_errors(a, b, key):
    """uniformFlow is a uniform stream: its flow residual and update are
    roundoff (~1e-16 of the fluxes) and differ with any change of operation
    order, and through the implicit coupling at CFL 1000 that roundoff moves
    k and omega in their 8th digit after one iteration and in their 2nd
    after twenty (their L2 norms stay within 1e-5).  The comparison uses
    physical scales: flow state, residual and update against 1 (the
    nondimensional density and speed-of-sound scale), turbulence variables
    relative to their own magnitude."""
    a, b = np.asarray(a), np.asarray(b)
    flow = float(np.abs(a[..., :5] - b[..., :5]).max())
    turb = max(rel_err(a[..., v], b[..., v]) for v in range(5, b.shape[-1]))
    return flow, turb


def resid_row(path: str, n: int) -> list[float]:
    """Normalised L2 columns of the last row of a residual file, as the
    reference's regression script reads them (tokens 3.. of the line)."""
    with open(path) as f:
        last = f.readlines()[-1]
    return [float(x) for x in last.split()[3:3 + n]]


def truth_failures(case: str, row: list[float]) -> list:
    _, truth, ignore = TRUTH[case]
    return [(i, r, t) for i, (r, t) in enumerate(zip(row, truth))
            if i not in ignore and abs(r - t) > 0.01 * t]


__all__ = ["FIXTURES", "TRUTH", "GOLDEN", "case_input", "have_case", "copy_case", "fixture",
           "fixture_fields", "cols_err", "uniform_flow_errors", "resid_row", "truth_failures"]
