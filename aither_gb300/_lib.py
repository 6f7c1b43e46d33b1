"""ctypes declarations of include/aither_gb300.h and thin Python wrappers.

The native library is the product; these wrappers only marshal arguments.
Loading fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libaither_gb300.so")

ATH_OK = 0
BC = dict(SLIP_WALL=0, VISCOUS_WALL=1, CHARACTERISTIC=2, STAGNATION_INLET=3,
          PRESSURE_OUTLET=4, SUPERSONIC_INFLOW=5, SUPERSONIC_OUTFLOW=6,
          PERIODIC=7, INTERBLOCK=8)
PREC_FP64, PREC_MIXED = 0, 1
BATCH_MATRIX_RESID, BATCH_FAST_FACES, BATCH_OUTPUT_GRADS = 1, 2, 4
FIELD = dict(STATE=0, STATE_GHOSTS=1, RESID=2, DT=3, SPECRAD=4, DU=5, AINV=6, AUX=7, VELGRAD=8,
             WALLDIST=9, CONS_N=10, CONS_NM1=11, GRADS=12)


class GhostOp(C.Structure):
    _fields_ = [("dst", C.c_int64), ("src", C.c_int64), ("src_block", C.c_int32),
                ("type", C.c_int32), ("layer", C.c_int32), ("dir", C.c_int32),
                ("lower", C.c_int32), ("state", C.c_int32), ("face", C.c_int64),
                ("src2", C.c_int64)]


class BCState(C.Structure):
    _fields_ = [("tag", C.c_int32), ("type", C.c_int32),
                ("rho", C.c_double), ("u", C.c_double), ("v", C.c_double),
                ("w", C.c_double), ("p", C.c_double),
                ("p0", C.c_double), ("t0", C.c_double), ("dir", C.c_double * 3),
                ("p_out", C.c_double),
                ("wall_u", C.c_double), ("wall_v", C.c_double), ("wall_w", C.c_double),
                ("wall_t", C.c_double), ("wall_q", C.c_double),
                ("isothermal", C.c_int32), ("heat_flux", C.c_int32),
                ("turb_intensity", C.c_double), ("eddy_visc_ratio", C.c_double),
                ("nonreflecting", C.c_int32), ("pad_nr", C.c_int32),
                ("length_scale", C.c_double)]


class NrCell(C.Structure):
    _fields_ = [("cell", C.c_int64), ("face", C.c_int64), ("surf", C.c_int32),
                ("dir", C.c_int32), ("lower", C.c_int32), ("pad", C.c_int32)]


class SolveView(C.Structure):
    _fields_ = [("eqn", C.c_int32), ("recon", C.c_int32), ("limiter", C.c_int32),
                ("flux", C.c_int32), ("solver", C.c_int32), ("turb", C.c_int32),
                ("nv", C.c_int32), ("ng", C.c_int32), ("sweeps", C.c_int32),
                ("kappa", C.c_double), ("cfl_start", C.c_double), ("cfl_step", C.c_double),
                ("cfl_max", C.c_double), ("theta", C.c_double), ("zeta", C.c_double),
                ("relax", C.c_double),
                ("gas_r", C.c_double), ("gas_n", C.c_double), ("gas_hf", C.c_double),
                ("mu_c1", C.c_double), ("mu_s", C.c_double), ("mu_ref", C.c_double),
                ("t_ref", C.c_double),
                ("r_ref", C.c_double), ("a_ref", C.c_double), ("l_ref", C.c_double),
                ("visc_scale", C.c_double), ("visc_cfl_coeff", C.c_double),
                ("k_c1", C.c_double), ("k_s", C.c_double), ("k_ref", C.c_double),
                ("nstates", C.c_int32), ("states", C.POINTER(BCState)),
                ("dt_global", C.c_double), ("dual_cfl", C.c_double),
                ("nl_iters", C.c_int32), ("multilevel", C.c_int32),
                ("mg_levels", C.c_int32), ("mg_cycle", C.c_int32)]


class MgMap(C.Structure):
    _fields_ = [("coarse_block", C.c_int32), ("pad", C.c_int32), ("ncells", C.c_int64),
                ("coarse_cell", C.POINTER(C.c_int32)), ("volfac", C.POINTER(C.c_double)),
                ("coef", C.POINTER(C.c_double))]


class BlockView(C.Structure):
    _fields_ = [("ni", C.c_int32), ("nj", C.c_int32), ("nk", C.c_int32),
                ("ng", C.c_int32), ("nv", C.c_int32), ("solve", C.c_int32),
                ("ncell_padded", C.c_int64), ("nface_padded", C.c_int64 * 3),
                ("vol", C.POINTER(C.c_double)), ("center", C.POINTER(C.c_double)),
                ("width", C.POINTER(C.c_double)),
                ("farea", C.POINTER(C.c_double) * 3),
                ("wall_dist", C.POINTER(C.c_double)),
                ("state0", C.POINTER(C.c_double)),
                ("nops", C.c_int32), ("ops", C.POINTER(GhostOp)),
                ("nedge_ops", C.c_int32), ("edge_ops", C.POINTER(GhostOp)),
                ("nvops", C.c_int32), ("vops", C.POINTER(GhostOp)),
                ("nvedge_ops", C.c_int32), ("vedge_ops", C.POINTER(GhostOp)),
                ("nplanes", C.c_int32), ("plane_offsets", C.POINTER(C.c_int32)),
                ("plane_cells", C.POINTER(C.c_int32)),
                ("nbr_mask", C.POINTER(C.c_uint8)),
                ("n_nr", C.c_int32), ("nr", C.POINTER(NrCell))]


class Norms(C.Structure):
    _fields_ = [("l2", C.c_double * 7), ("linf", C.c_double),
                ("linf_block", C.c_int32), ("linf_i", C.c_int32), ("linf_j", C.c_int32),
                ("linf_k", C.c_int32), ("linf_eqn", C.c_int32),
                ("matrix_resid", C.c_double), ("cfl", C.c_double), ("status", C.c_int32),
                ("force", C.c_double * 6)]


class ConvergeInfo(C.Structure):
    """ath_converge_info: per-solve record of a run to convergence."""
    _fields_ = [("iterations", C.c_int64), ("drop", C.c_double), ("ms", C.c_double),
                ("converged", C.c_int32), ("pad", C.c_int32)]


class RequestStatus(C.Structure):
    """ath_request_status: one retired request of a Server."""
    _fields_ = [("id", C.c_int64), ("iterations", C.c_int64), ("drop", C.c_double),
                ("converged", C.c_int32), ("pad", C.c_int32), ("queue_ms", C.c_double),
                ("latency_ms", C.c_double), ("device_ms", C.c_double)]


class BlockDev(C.Structure):
    """ath_block_dev: caller-owned device arrays of one block."""
    _fields_ = [("ni", C.c_int32), ("nj", C.c_int32), ("nk", C.c_int32), ("ng", C.c_int32),
                ("W", C.c_void_p), ("vol", C.c_void_p), ("width", C.c_void_p * 3),
                ("farea", C.c_void_p * 3), ("R", C.c_void_p), ("lam", C.c_void_p),
                ("dt", C.c_void_p), ("ainv", C.c_void_p)]


class BlockFields(C.Structure):
    """ath_block_fields: host fields of one block for the output writers."""
    _fields_ = [("prim", C.c_void_p), ("dt", C.c_void_p), ("resid", C.c_void_p),
                ("aux", C.c_void_p), ("velgrad", C.c_void_p), ("wall_dist", C.c_void_p),
                ("cons_nm1", C.c_void_p), ("grads", C.c_void_p)]


class Stats(C.Structure):
    _fields_ = [("kernel_launches", C.c_int64), ("device_ms", C.c_double)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"native library {LIB_PATH} is not built; run "
                               "`python -m aither_gb300.build`")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        sig = {
            "ath_last_error": (C.c_char_p, []),
            "ath_setup_from_input": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
            "ath_setup_append": (C.c_int, [vp, C.c_char_p]),
            "ath_setup_from_input_dev": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(vp)]),
            "ath_setup_destroy": (C.c_int, [vp]),
            "ath_setup_counts": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                           C.POINTER(C.c_int64)]),
            "ath_setup_block": (C.c_int, [vp, C.c_int, C.POINTER(BlockView)]),
            "ath_setup_solve": (C.c_int, [vp, C.c_int, C.POINTER(SolveView)]),
            "ath_setup_set_state": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double)]),
            "ath_setup_levels": (C.c_int, [vp, C.POINTER(C.c_int)]),
            "ath_batch_flags": (C.c_int, [vp, C.POINTER(C.c_int)]),
            "ath_setup_level_counts": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int),
                                                 C.POINTER(C.c_int), C.POINTER(C.c_int64)]),
            "ath_setup_level_block": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(BlockView)]),
            "ath_setup_level_solve": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(SolveView)]),
            "ath_setup_mg_map": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(MgMap)]),
            "ath_ctx_create": (C.c_int, [C.c_int, C.c_size_t, C.POINTER(vp)]),
            "ath_ctx_destroy": (C.c_int, [vp]),
            "ath_ctx_fp64_peak": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double)]),
            "ath_batch_create": (C.c_int, [vp, vp, C.c_int, C.c_int, C.POINTER(vp)]),
            "ath_batch_destroy": (C.c_int, [vp]),
            "ath_batch_iterate": (C.c_int, [vp, C.c_int, C.POINTER(Norms)]),
            "ath_batch_fill_ghosts": (C.c_int, [vp]),
            "ath_batch_residual": (C.c_int, [vp]),
            "ath_batch_timestep": (C.c_int, [vp]),
            "ath_batch_diag_invert": (C.c_int, [vp]),
            "ath_batch_relax": (C.c_int, [vp]),
            "ath_batch_update": (C.c_int, [vp, C.POINTER(Norms)]),
            "ath_batch_get_field": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]),
            "ath_batch_set_state": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double)]),
            "ath_batch_set_state_nm1": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double)]),
            "ath_batch_field_width": (C.c_int, [vp, C.c_int, C.c_int]),
            "ath_batch_pool_vars": (C.c_int, [vp, C.POINTER(C.c_int)]),
            "ath_output_function": (C.c_int, [vp, C.c_int, C.c_char_p, C.POINTER(BlockFields),
                                              C.c_char_p]),
            "ath_output_restart": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(C.c_double),
                                             C.POINTER(BlockFields), C.c_char_p]),
            "ath_input_restart": (C.c_int, [vp, C.c_int, C.c_char_p, C.POINTER(C.c_int),
                                            C.POINTER(C.c_double),
                                            C.POINTER(C.POINTER(C.c_double)),
                                            C.POINTER(C.c_int),
                                            C.POINTER(C.POINTER(C.c_double))]),
            "ath_output_center_grid": (C.c_int, [vp, C.c_int, C.c_char_p]),
            "ath_output_meta": (C.c_int, [vp, C.c_int, C.c_char_p, C.c_int, C.c_char_p]),
            "ath_output_resid": (C.c_int, [vp, C.c_int, C.c_char_p, C.c_int, C.c_int, C.c_int,
                                           C.POINTER(Norms), C.POINTER(C.c_double)]),
            "ath_batch_write_function": (C.c_int, [vp, vp, C.c_int, C.c_char_p, C.c_char_p]),
            "ath_batch_write_restart": (C.c_int, [vp, vp, C.c_int, C.c_int,
                                                  C.POINTER(C.c_double), C.c_char_p]),
            "ath_batch_read_restart": (C.c_int, [vp, vp, C.c_int, C.c_char_p,
                                                 C.POINTER(C.c_int), C.POINTER(C.c_double)]),
            "ath_batch_stats": (C.c_int, [vp, C.POINTER(Stats)]),
            "ath_batch_pool_cells": (C.c_int, [vp, C.POINTER(C.c_int64)]),
            "ath_batch_copy_state": (C.c_int, [vp, C.POINTER(C.c_double), C.c_int]),
            "ath_batch_profile": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double)]),
            "ath_batch_converge": (C.c_int, [vp, C.c_int, C.c_double, C.c_int,
                                             C.POINTER(ConvergeInfo)]),
            "ath_batch_set_target": (C.c_int, [vp, C.c_int, C.c_double, C.c_int]),
            "ath_batch_solve_info": (C.c_int, [vp, C.POINTER(ConvergeInfo)]),
            "ath_batch_autotune": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int)]),
            "ath_batch_sweep_shape": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                                C.POINTER(C.c_int)]),
            "ath_batch_set_sweep_shape": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
            "ath_batch_sweep_wait_test": (C.c_int, [vp, C.c_longlong, C.c_int]),
            "ath_server_create": (C.c_int, [vp, C.c_int, C.c_double, C.c_int64, C.c_int,
                                            C.c_int, C.POINTER(vp)]),
            "ath_server_submit": (C.c_int, [vp, C.c_char_p, C.POINTER(C.c_int64)]),
            "ath_server_step": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
            "ath_server_poll": (C.c_int, [vp, C.POINTER(RequestStatus), C.c_int,
                                          C.POINTER(C.c_int)]),
            "ath_server_fetch": (C.c_int, [vp, C.c_int64, C.c_int, C.POINTER(C.c_double)]),
            "ath_server_release": (C.c_int, [vp, C.c_int64]),
            "ath_server_destroy": (C.c_int, [vp]),
            "ath_block_residual_noalloc": (C.c_int, [C.POINTER(BlockDev), C.POINTER(SolveView),
                                                     C.c_double, vp]),
        }
        missing = []
        for name, (res, args) in sig.items():
            try:
                f = getattr(L, name)
            except AttributeError:
                missing.append(name)
                continue
            f.restype = res
            f.argtypes = args
        if missing:
            raise RuntimeError(f"{LIB_PATH} lacks exported symbols: {missing}")
        _lib = L
    return _lib


class AthError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"aither_gb300 error {code}: {msg}")
        self.code = code


def check(code: int) -> None:
    if code != ATH_OK:
        raise AthError(code, lib().ath_last_error().decode())


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _arr(ptr, n, dtype=np.float64):
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class Setup:
    """Host-side case setup: parse + geometry + ghost-cell bookkeeping."""

    def __init__(self, inp_paths, device: int | None = None):
        """device: a CUDA device computing the cells' geometry and wall
        distance (None: the host)."""
        if isinstance(inp_paths, str):
            inp_paths = [inp_paths]
        h = C.c_void_p()
        if device is None:
            check(lib().ath_setup_from_input(inp_paths[0].encode(), C.byref(h)))
        else:
            check(lib().ath_setup_from_input_dev(inp_paths[0].encode(), device, C.byref(h)))
        self.h = h
        for p in inp_paths[1:]:
            check(lib().ath_setup_append(self.h, p.encode()))

    def close(self):
        if self.h:
            lib().ath_setup_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def counts(self):
        ns, nb, nc = C.c_int(), C.c_int(), C.c_int64()
        check(lib().ath_setup_counts(self.h, C.byref(ns), C.byref(nb), C.byref(nc)))
        return ns.value, nb.value, nc.value

    # ---- output files in the reference's formats
    def solve_blocks(self, solve: int) -> list:
        return [b for b in range(self.counts()[1]) if self.block_view(b).solve == solve]

    def solve_nv(self, solve: int) -> int:
        return self.block_view(self.solve_blocks(solve)[0]).nv

    @staticmethod
    def _fields(blocks: list) -> "C.Array":
        keep = []
        arr = (BlockFields * len(blocks))()
        for k, fl in enumerate(blocks):
            for name in ("prim", "dt", "resid", "aux", "velgrad", "wall_dist", "cons_nm1",
                         "grads"):
                a = fl.get(name)
                if a is not None:
                    a = np.ascontiguousarray(a, dtype=np.float64)
                    keep.append(a)
                    setattr(arr[k], name, a.ctypes.data)
        arr._keep = keep
        return arr

    def write_function(self, solve: int, fields: list, path: str, variables=None) -> None:
        """Plot3D cell-centre function file from host fields (one dict per
        block of the solve: prim, dt, resid, aux, velgrad, wall_dist)."""
        arr = self._fields(fields)
        v = ",".join(variables).encode() if variables else None
        check(lib().ath_output_function(self.h, solve, v, arr, path.encode()))

    def write_restart(self, solve: int, iteration: int, resid_first, prims: list,
                      path: str, nm1: list | None = None) -> None:
        """Restart file from host states; nm1 (conserved state of time n-1
        per block) is required for bdf2 solves."""
        arr = self._fields([{"prim": p, "cons_nm1": None if nm1 is None else nm1[k]}
                            for k, p in enumerate(prims)])
        rf = np.ascontiguousarray(resid_first, dtype=np.float64)
        check(lib().ath_output_restart(self.h, solve, iteration, dptr(rf), arr, path.encode()))

    def read_restart(self, solve: int, path: str, levels: bool = False):
        """(iteration, L2 normalisation, [primitive state per block]); with
        levels=True also the file's time levels and [conserved state of time
        n-1 per block] (None for a one-level file)."""
        blocks = self.solve_blocks(solve)
        nv = self.solve_nv(solve)
        outs, nm1 = [], []
        for b in blocks:
            v = self.block_view(b)
            outs.append(np.empty((v.nk, v.nj, v.ni, nv)))
            nm1.append(np.empty((v.nk, v.nj, v.ni, nv)))
        ptrs = (C.POINTER(C.c_double) * len(outs))(*[dptr(o) for o in outs])
        ptrs1 = (C.POINTER(C.c_double) * len(nm1))(*[dptr(o) for o in nm1])
        it, nl = C.c_int(), C.c_int()
        rf = np.empty(nv)
        check(lib().ath_input_restart(self.h, solve, path.encode(), C.byref(it), dptr(rf), ptrs,
                                      C.byref(nl), ptrs1))
        if not levels:
            return it.value, rf, outs
        return it.value, rf, outs, nl.value, (nm1 if nl.value >= 2 else None)

    def write_center_grid(self, solve: int, path: str) -> None:
        check(lib().ath_output_center_grid(self.h, solve, path.encode()))

    def write_meta(self, solve: int, iteration: int, path: str, variables=None) -> None:
        v = ",".join(variables).encode() if variables else None
        check(lib().ath_output_meta(self.h, solve, v, iteration, path.encode()))

    def write_resid(self, solve: int, path: str, norms: list, first_step: int,
                    resid_first: np.ndarray, append: bool = False,
                    restarted: bool = False) -> None:
        """Residual history rows of one solve from nonlinear iteration
        first_step on; resid_first (nv values) is the running normalisation,
        updated in place (left as given in a restarted run)."""
        arr = (Norms * len(norms))(*norms)
        flags = (1 if append else 0) | (2 if restarted else 0)
        check(lib().ath_output_resid(self.h, solve, path.encode(), flags,
                                     first_step, len(norms), arr, dptr(resid_first)))

    def block_view(self, b: int, level: int = 0) -> BlockView:
        v = BlockView()
        check(lib().ath_setup_level_block(self.h, level, b, C.byref(v)))
        return v

    def solve_view(self, s: int, level: int = 0) -> SolveView:
        v = SolveView()
        check(lib().ath_setup_level_solve(self.h, level, s, C.byref(v)))
        return v

    # ---- multigrid levels
    def levels(self) -> int:
        n = C.c_int()
        check(lib().ath_setup_levels(self.h, C.byref(n)))
        return n.value

    def level_counts(self, level: int):
        ns, nb, nc = C.c_int(), C.c_int(), C.c_int64()
        check(lib().ath_setup_level_counts(self.h, level, C.byref(ns), C.byref(nb),
                                           C.byref(nc)))
        return ns.value, nb.value, nc.value

    def mg_map(self, level: int, b: int) -> dict:
        """Transfer of block b of `level` to the next coarser level: the
        coarse block, and per fine physical cell (k, j, i order) its coarse
        cell, restriction weight and 7 prolongation coefficients."""
        m = MgMap()
        check(lib().ath_setup_mg_map(self.h, level, b, C.byref(m)))
        n = m.ncells
        return {"coarse_block": m.coarse_block,
                "coarse_cell": np.ctypeslib.as_array(m.coarse_cell, (n,)).copy(),
                "volfac": np.ctypeslib.as_array(m.volfac, (n,)).copy(),
                "coef": np.ctypeslib.as_array(m.coef, (n, 7)).copy()}

    def set_state(self, b: int, prim: np.ndarray) -> None:
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        check(lib().ath_setup_set_state(self.h, b, dptr(prim)))

    def geometry(self, b: int) -> dict:
        """Copies of the padded geometry arrays of block b."""
        v = self.block_view(b)
        nc = v.ncell_padded
        NI, NJ, NK = v.ni + 2 * v.ng, v.nj + 2 * v.ng, v.nk + 2 * v.ng
        g = {"vol": _arr(v.vol, nc).reshape(NK, NJ, NI),
             "center": _arr(v.center, 3 * nc).reshape(3, NK, NJ, NI),
             "width": _arr(v.width, 3 * nc).reshape(3, NK, NJ, NI)}
        shp = [(NK, NJ, NI + 1), (NK, NJ + 1, NI), (NK + 1, NJ, NI)]
        for d, nm in enumerate(["fareai", "fareaj", "fareak"]):
            nf = v.nface_padded[d]
            g[nm] = _arr(v.farea[d], 4 * nf).reshape((4,) + shp[d])
        g["ops"] = np.ctypeslib.as_array(v.ops, shape=(v.nops,)).copy() if v.nops else None
        g["ng"] = v.ng
        return g


class Context:
    def __init__(self, device: int = 0, hbm_budget: int = 0):
        h = C.c_void_p()
        check(lib().ath_ctx_create(device, hbm_budget, C.byref(h)))
        self.h = h

    def fp64_peak(self, reps: int = 5) -> float:
        """Measured FP64 FMA issue rate of the context's GPU, TFLOP/s."""
        t = C.c_double()
        check(lib().ath_ctx_fp64_peak(self.h, reps, C.byref(t)))
        return t.value

    def close(self):
        if self.h:
            lib().ath_ctx_destroy(self.h)
            self.h = None


class Batch:
    """Device-resident blocks of one or more solves."""

    def __init__(self, ctx: Context, setup: Setup, precision: int = PREC_FP64,
                 flags: int = 0):
        h = C.c_void_p()
        check(lib().ath_batch_create(ctx.h, setup.h, precision, flags, C.byref(h)))
        self.h = h
        self.setup = setup
        self.nsolves, self.nblocks, self.ncells = setup.counts()

    def close(self):
        if self.h:
            lib().ath_batch_destroy(self.h)
            self.h = None

    def iterate(self, n: int = 1) -> np.ndarray:
        norms = (Norms * (n * self.nsolves))()
        check(lib().ath_batch_iterate(self.h, n, norms))
        return norms

    def converge(self, max_iters: int, drop: float, check_every: int = 50):
        """Iterates until every solve has retired (total L2 drop reached or
        nonphysical state) or max_iters; returns per-solve ConvergeInfo."""
        info = (ConvergeInfo * self.nsolves)()
        check(lib().ath_batch_converge(self.h, max_iters, drop, check_every, info))
        return info

    def autotune(self, reps: int = 3) -> int:
        """Picks the sweep CTA size by timing; the solves are not advanced."""
        t = C.c_int()
        check(lib().ath_batch_autotune(self.h, reps, C.byref(t)))
        return t.value

    def set_target(self, solve: int, drop: float, active: bool = True) -> None:
        check(lib().ath_batch_set_target(self.h, solve, drop, 1 if active else 0))

    def solve_info(self):
        info = (ConvergeInfo * self.nsolves)()
        check(lib().ath_batch_solve_info(self.h, info))
        return info

    def stage(self, name: str, norms=None):
        f = getattr(lib(), "ath_batch_" + name)
        if name == "update":
            out = (Norms * self.nsolves)()
            check(f(self.h, out))
            return out
        check(f(self.h))

    def field(self, b: int, field: str) -> np.ndarray:
        v = self.setup.block_view(b)
        fid = FIELD[field]
        w = lib().ath_batch_field_width(self.h, b, fid)
        if w < 0:
            check(w)
        n = (v.ncell_padded if field == "STATE_GHOSTS" else v.ni * v.nj * v.nk) * w
        out = np.empty(n, dtype=np.float64)
        check(lib().ath_batch_get_field(self.h, b, fid, dptr(out)))
        if field == "STATE_GHOSTS":
            return out.reshape(v.nk + 2 * v.ng, v.nj + 2 * v.ng, v.ni + 2 * v.ng, w)
        return out.reshape(v.nk, v.nj, v.ni, w)

    def set_state(self, b: int, prim: np.ndarray) -> None:
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        check(lib().ath_batch_set_state(self.h, b, dptr(prim)))

    def set_state_nm1(self, b: int, cons: np.ndarray | None) -> None:
        """Time n-1 of a bdf2 solve's block (conserved, nv per cell), kept
        through the first time step; None copies the current state."""
        if cons is None:
            check(lib().ath_batch_set_state_nm1(self.h, b, None))
            return
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        check(lib().ath_batch_set_state_nm1(self.h, b, dptr(cons)))

    def pool_cells(self) -> int:
        n = C.c_int64()
        check(lib().ath_batch_pool_cells(self.h, C.byref(n)))
        return n.value

    def write_function(self, solve: int, path: str, variables=None) -> None:
        """Plot3D cell-centre function file of a solve's resident solution."""
        v = ",".join(variables).encode() if variables else None
        check(lib().ath_batch_write_function(self.h, self.setup.h, solve, v, path.encode()))

    def write_restart(self, solve: int, iteration: int, resid_first, path: str) -> None:
        rf = np.ascontiguousarray(resid_first, dtype=np.float64)
        check(lib().ath_batch_write_restart(self.h, self.setup.h, solve, iteration, dptr(rf),
                                            path.encode()))

    def read_restart(self, solve: int, path: str):
        """Loads a restart file into the solve's resident state; returns
        (iteration, L2 normalisation)."""
        it = C.c_int()
        rf = np.empty(7)
        check(lib().ath_batch_read_restart(self.h, self.setup.h, solve, path.encode(),
                                           C.byref(it), dptr(rf)))
        return it.value, rf[:self.setup.solve_nv(solve)]

    def sweep_shape(self) -> dict:
        """LU-SGS sweep shape: mode 1 persistent cluster sweep (cluster CTAs
        per solve), 0 one launch per hyperplane, 2 the same with a group of
        lanes per scalar cell, 3 persistent tile queue (threads = cells per
        tile)."""
        m, t, c = C.c_int(), C.c_int(), C.c_int()
        check(lib().ath_batch_sweep_shape(self.h, C.byref(m), C.byref(t), C.byref(c)))
        return {"mode": m.value, "threads": t.value, "cluster": c.value}

    def set_sweep_shape(self, mode: int, threads: int, cluster: int = 0) -> None:
        check(lib().ath_batch_set_sweep_shape(self.h, mode, threads, cluster))

    def sweep_wait_test(self, poll_limit: int, wait_never: bool) -> None:
        """Poll limit of the tile-queue sweep's waits; wait_never makes every
        wait poll a flag nothing sets (tests of the bounded wait)."""
        check(lib().ath_batch_sweep_wait_test(self.h, poll_limit, 1 if wait_never else 0))

    def pool_vars(self) -> int:
        """Values per cell of the copy_state snapshot (5, or 7 with SST)."""
        n = C.c_int()
        check(lib().ath_batch_pool_vars(self.h, C.byref(n)))
        return n.value

    def copy_state(self, host: np.ndarray, to_device: bool) -> None:
        assert host.dtype == np.float64 and host.flags.c_contiguous
        check(lib().ath_batch_copy_state(self.h, dptr(host), 1 if to_device else 0))

    def profile(self, reps: int = 3) -> np.ndarray:
        ms = np.zeros(8)
        check(lib().ath_batch_profile(self.h, reps, dptr(ms)))
        return ms

    def stats(self) -> Stats:
        s = Stats()
        check(lib().ath_batch_stats(self.h, C.byref(s)))
        return s


class Server:
    """Continuous-batching request loop (ath_server_*): every admitted request
    is a device-resident batch on its own stream; admission by slots and by
    the context's device-memory budget; retirement on the device at the
    residual drop."""

    def __init__(self, ctx: Context, precision: int = PREC_FP64, drop: float = 1e-6,
                 max_iters: int = 100000, chunk: int = 50, max_active: int = 16):
        h = C.c_void_p()
        check(lib().ath_server_create(ctx.h, precision, drop, max_iters, chunk, max_active,
                                      C.byref(h)))
        self.h = h
        self.shapes = {}

    def submit(self, inp_path: str) -> int:
        i = C.c_int64()
        check(lib().ath_server_submit(self.h, inp_path.encode(), C.byref(i)))
        s = Setup(inp_path)
        self.shapes[i.value] = [(v.nk, v.nj, v.ni, v.nv) for v in
                                (s.block_view(b) for b in range(s.counts()[1]))]
        s.close()
        return i.value

    def step(self):
        a, q = C.c_int(), C.c_int()
        check(lib().ath_server_step(self.h, C.byref(a), C.byref(q)))
        return a.value, q.value

    def poll(self, max_n: int = 256):
        out = (RequestStatus * max_n)()
        n = C.c_int()
        check(lib().ath_server_poll(self.h, out, max_n, C.byref(n)))
        return [out[i] for i in range(n.value)]

    def fetch(self, rid: int, block: int = 0) -> np.ndarray:
        nk, nj, ni, nv = self.shapes[rid][block]
        out = np.empty(nk * nj * ni * nv)
        check(lib().ath_server_fetch(self.h, rid, block, dptr(out)))
        return out.reshape(nk, nj, ni, nv)

    def release(self, rid: int) -> None:
        check(lib().ath_server_release(self.h, rid))

    def close(self):
        if self.h:
            lib().ath_server_destroy(self.h)
            self.h = None
