"""ctypes wrapper of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py; never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(_HERE, "liboracle.so")
FIELD = dict(STATE=0, STATE_GHOSTS=1, RESID=2, DT=3, SPECRAD=4, DU=5, AINV=6, AUX=7, VELGRAD=8,
             WALLDIST=9, CONS_N=10, CONS_NM1=11, GRADS=12)
WIDTH = dict(STATE=5, STATE_GHOSTS=5, RESID=5, DT=1, SPECRAD=2, DU=5, AINV=1, AUX=5, VELGRAD=9,
             WALLDIST=1, CONS_N=5, CONS_NM1=5, GRADS=24)

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            raise RuntimeError(f"{ORACLE_LIB} is not built; run `python -m aither_gb300.build`")
        from aither_gb300._lib import BlockView, SolveView
        L = C.CDLL(ORACLE_LIB)
        vp = C.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.c_int, C.POINTER(BlockView), C.c_int, C.POINTER(SolveView)]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_threads.argtypes = [vp, C.c_int]
        for f in ("orc_fill_ghosts", "orc_residual", "orc_timestep", "orc_diag_invert",
                  "orc_relax"):
            getattr(L, f).argtypes = [vp]
        L.orc_update.restype = C.c_int
        L.orc_update.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_iterate.restype = C.c_int
        L.orc_iterate.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
        L.orc_get_field.restype = C.c_int
        L.orc_get_field.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.orc_set_matrix_resid.argtypes = [vp, C.c_int]
        L.orc_set_output_grads.argtypes = [vp, C.c_int]
        L.orc_matrix_resid.restype = C.c_double
        L.orc_matrix_resid.argtypes = [vp, C.c_int]
        L.orc_forces.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
        L.orc_set_state.restype = C.c_int
        L.orc_set_state.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
        L.orc_set_state_nm1.restype = C.c_int
        L.orc_set_state_nm1.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
        from aither_gb300._lib import MgMap
        L.orc_set_coarse.argtypes = [vp, vp, C.c_int, C.POINTER(MgMap)]
        _lib = L
    return _lib


def lib_setup():
    from aither_gb300._lib import lib as product_lib
    return product_lib()


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """CPU oracle instance built from an aither_gb300 Setup."""

    def __init__(self, setup, threads: int = 0, matrix_resid: bool = False,
                 output_grads: bool = False):
        from aither_gb300._lib import BlockView, SolveView
        self.setup = setup
        self.nsolves, self.nblocks, self.ncells = setup.counts()
        bv = (BlockView * self.nblocks)(*[setup.block_view(b) for b in range(self.nblocks)])
        sv = (SolveView * self.nsolves)(*[setup.solve_view(s) for s in range(self.nsolves)])
        # equations per cell: 7 when any solve is RANS (k, omega), else 5
        self.nv = max(x.nv for x in sv)
        self.h = lib().orc_create(self.nblocks, bv, self.nsolves, sv)
        if threads:
            lib().orc_set_threads(self.h, threads)
        if matrix_resid:
            lib().orc_set_matrix_resid(self.h, 1)
        if output_grads:
            lib().orc_set_output_grads(self.h, 1)
        # coarser multigrid levels, each linked to the next finer one
        self.levels = []
        fine = self.h
        for lv in range(1, setup.levels()):
            ns, nb, _ = setup.level_counts(lv)
            lbv = (BlockView * nb)(*[setup.block_view(b, lv) for b in range(nb)])
            lsv = (SolveView * ns)(*[setup.solve_view(s, lv) for s in range(ns)])
            h = lib().orc_create(nb, lbv, ns, lsv)
            if threads:
                lib().orc_set_threads(h, threads)
            nfine = setup.level_counts(lv - 1)[1]
            from aither_gb300._lib import MgMap, check
            maps = (MgMap * nfine)()
            for b in range(nfine):
                check(lib_setup().ath_setup_mg_map(setup.h, lv - 1, b, C.byref(maps[b])))
            cycle = setup.solve_view(0, lv - 1).mg_cycle
            lib().orc_set_coarse(fine, h, cycle, maps)
            self.levels.append(h)
            fine = h

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None
        for h in getattr(self, "levels", []):
            lib().orc_destroy(h)
        self.levels = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def iterate(self, n: int = 1) -> np.ndarray:
        l2 = np.zeros(n * self.nsolves * 7)
        self.mres = np.zeros((n, self.nsolves))
        self.forces = np.zeros((n, self.nsolves, 6))
        for it in range(n):
            rc = lib().orc_iterate(self.h, 1, _dp(l2[it * self.nsolves * 7:]))
            if rc:
                raise RuntimeError(f"oracle reported status {rc}")
            for s in range(self.nsolves):
                self.mres[it, s] = lib().orc_matrix_resid(self.h, s)
                f = np.zeros(6)
                lib().orc_forces(self.h, s, _dp(f))
                self.forces[it, s] = f
        return l2.reshape(n, self.nsolves, 7)[:, :, :self.nv]

    def stage(self, name: str):
        if name == "update":
            l2 = np.zeros(self.nsolves * 7)
            rc = lib().orc_update(self.h, _dp(l2), None)
            if rc:
                raise RuntimeError(f"oracle reported status {rc}")
            return l2.reshape(self.nsolves, 7)[:, :self.nv]
        getattr(lib(), "orc_" + name)(self.h)

    def field(self, b: int, field: str) -> np.ndarray:
        v = self.setup.block_view(b)
        w = WIDTH[field]
        if field in ("STATE", "STATE_GHOSTS", "RESID", "DU", "CONS_N", "CONS_NM1"):
            w = v.nv
        n = (v.ncell_padded if field == "STATE_GHOSTS" else v.ni * v.nj * v.nk) * w
        out = np.empty(n)
        rc = lib().orc_get_field(self.h, b, FIELD[field], _dp(out))
        if rc:
            raise RuntimeError(f"oracle field error {rc}")
        if field == "STATE_GHOSTS":
            return out.reshape(v.nk + 2 * v.ng, v.nj + 2 * v.ng, v.ni + 2 * v.ng, w)
        return out.reshape(v.nk, v.nj, v.ni, w)

    def set_state(self, b: int, prim: np.ndarray) -> None:
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        lib().orc_set_state(self.h, b, _dp(prim))

    def set_state_nm1(self, b: int, cons) -> None:
        """Time n-1 of a bdf2 solve's block (None: the current state)."""
        if cons is None:
            rc = lib().orc_set_state_nm1(self.h, b, None)
        else:
            cons = np.ascontiguousarray(cons, dtype=np.float64)
            rc = lib().orc_set_state_nm1(self.h, b, _dp(cons))
        if rc:
            raise RuntimeError(f"oracle time level error {rc}")
