import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300)")


@pytest.fixture(scope="session", autouse=True)
def built():
    """The native library and the oracle are built once per session."""
    from aither_gb300 import build
    build.build_library()
    build.build_oracle()
    return True


GOLDEN = os.path.join(ROOT, "tests", "golden")
REF_HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
REFCASES = os.path.join(ROOT, "tests", "golden", "refcases")


def _reference_source():
    from aither_gb300 import build
    return build.reference_source() or ""


# the reference's source tree where this machine has it ("" elsewhere)
REF_SRC = _reference_source()


def load_golden(name):
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def golden_case(name, outdir):
    """Regenerates the input files of a golden fixture (seeded, identical)."""
    import ast

    import numpy as np
    from aither_gb300 import cases
    g = load_golden(name)
    kw = ast.literal_eval(str(g["kwargs"]))
    base = name.split("_it")[0]
    gen = (cases.vortex_box if base.startswith("vortex")
           else cases.block_pair if base.startswith("pair_")
           else cases.wall_channel if base.startswith(("sst_chan", "chan_"))
           else cases.flat_plate if base.startswith(("plate", "sst", "wk_"))
           else cases.bump_channel)
    inp, st = gen(outdir, name=base, **kw)
    return inp, st, g


def set_states(setup, st):
    """Sets the analytic initial state of every block of a case (st: one
    array per block, or None)."""
    if st is not None:
        for b, x in enumerate(st):
            setup.set_state(b, x)


def rel_err(a, b):
    import numpy as np
    scale = max(float(np.abs(b).max()), 1e-300)
    return float(np.abs(np.asarray(a) - np.asarray(b)).max()) / scale


def total_iterations(g):
    """Nonlinear iterations a fixture ran: its time steps times the
    nonlinear iterations per step of time-accurate cases."""
    import ast
    kw = ast.literal_eval(str(g["kwargs"]))
    return int(g["iterations"]) * int(kw.get("nl", 1))
