"""Interblock connections in every patch orientation (CPU oracle).

Each case is two blocks of a skewed box joined at x = 1 (cases.block_pair);
the second block's index axes are a signed permutation of the first's, one
case per in-plane patch orientation, with the connecting surface on each
direction and side of the second block.  A three-dimensional vortex crosses
the connection.

Three kinds of check:
  * against the reference's own results (fixtures generated by running the
    reference build, tests/golden/make_golden.py) where the reference is
    self-consistent: bit for bit (1e-13);
  * invariance: the residual of both blocks must not depend on how the
    second block is indexed, so every orientation reproduces the aligned
    one (1e-12 relative: the only difference is the roundoff of face areas
    formed from the nodes in another order).  The implicit update is not
    invariant: the LU-SGS sweeps visit the second block's cells in its own
    hyperplane order, a Gauss-Seidel ordering that changes with the
    indexing, in the reference too; nor, for viscous solves, are the
    spectral radius and time step of the second block (they change by
    ~1e-5 with its orientation, identically in the reference);
  * the reference's fixtures themselves show where it is not
    self-consistent: in the orientations that keep the in-plane axes and
    reverse exactly one of them its first-block residual differs from the
    aligned case by O(1), and for viscous solves every swapped orientation
    differs by 1e-5..1e-3 (the physics is the same in every orientation).
    These orientations are checked by invariance only.
"""
import numpy as np
import pytest

from conftest import golden_case, load_golden, rel_err, set_states

TOL = 1e-13
INV_TOL = 1e-12
# orientations in which the reference's result is independent of the
# second block's indexing (per physics)
REF_CONSISTENT = {"euler": [0, 1, 2, 4, 6, 7], "sst": [0, 2]}


def _cols_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    errs = [rel_err(a[..., :5], b[..., :5])]
    errs += [rel_err(a[..., v], b[..., v]) for v in range(5, b.shape[-1])]
    return max(errs)


def _oracle(inp, st):
    from aither_gb300 import Setup
    from pyoracle import Oracle
    s = Setup(inp)
    set_states(s, st)
    return s, Oracle(s)


@pytest.mark.parametrize("name", [f"pair_{ph}_o{o}_it{n}" for ph, os_ in REF_CONSISTENT.items()
                                  for o in os_ for n in (1, 10)])
def test_oracle_matches_reference_on_orientation(name, tmp_path):
    inp, st, g = golden_case(name, str(tmp_path))
    _, o = _oracle(inp, st)
    l2 = o.iterate(int(g["iterations"]))
    for b in range(2):
        p = f"b{b}_"
        assert _cols_err(o.field(b, "STATE"), g[p + "state"]) <= TOL
        assert _cols_err(o.field(b, "RESID"), g[p + "resid"]) <= TOL
        assert _cols_err(o.field(b, "DU"), g[p + "du"]) <= TOL
        assert rel_err(o.field(b, "DT")[..., 0], g[p + "dt"]) <= TOL
    nv = g["l2"].shape[1]
    assert rel_err(l2[:, 0, :nv], g["l2"]) <= TOL
    o.close()


def to_aligned(f, orient):
    """A second-block field [k][j][i][v] of orientation `orient` in the
    index order of the aligned case (orientation 0)."""
    from aither_gb300 import cases
    ax, sg = cases.orientation_set()[orient]
    a = np.asarray(f)
    for t in range(3):
        if sg[t] < 0:
            a = np.flip(a, axis=2 - t)
    order = [2 - ax.index(2 - q) for q in range(3)] + list(range(3, a.ndim))
    return np.ascontiguousarray(np.transpose(a, order))


@pytest.mark.parametrize("physics", ["euler", "ns", "sst"])
def test_oracle_result_independent_of_block_orientation(physics, tmp_path):
    from aither_gb300 import cases
    ref = None
    for orient in range(8):
        inp, st = cases.block_pair(str(tmp_path / f"o{orient}"), orient=orient, physics=physics,
                                   name="pair")
        _, o = _oracle(inp, st)
        o.iterate(1)
        a = {(b, f): (o.field(b, f) if b == 0 else to_aligned(o.field(b, f), orient))
             for b in (0, 1) for f in ("RESID",)}
        o.close()
        if ref is None:
            ref = a
            continue
        for key in a:
            assert _cols_err(a[key], ref[key]) <= INV_TOL, (orient, key)


def test_reference_fixtures_record_its_orientation_defects():
    """The reference's results differ between orientations that describe the
    same physical problem: O(1) where one in-plane axis is reversed and the
    other kept (orientations 3 and 5, inviscid and viscous), 1e-5 and more
    for viscous solves with swapped in-plane axes.  This build's results are
    orientation-independent (test above) and equal the reference's in its
    consistent orientations."""
    for ph, bad, floor in (("euler", [3, 5], 1e-2), ("sst", [1, 3, 4, 5, 6, 7], 1e-5)):
        g0 = load_golden(f"pair_{ph}_o0_it1")
        for o in bad:
            g = load_golden(f"pair_{ph}_o{o}_it1")
            e = max(_cols_err(g["b0_resid"], g0["b0_resid"]),
                    _cols_err(to_aligned(g["b1_resid"], o), g0["b1_resid"]))
            assert e > floor, (ph, o, e)
        for o in REF_CONSISTENT[ph]:
            g = load_golden(f"pair_{ph}_o{o}_it1")
            e = max(_cols_err(g["b0_resid"], g0["b0_resid"]),
                    _cols_err(to_aligned(g["b1_resid"], o), g0["b1_resid"]))
            assert e <= INV_TOL, (ph, o, e)
