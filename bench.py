#!/usr/bin/env python3
"""Throughput of the per-iteration structured-grid solver step on GB300.

Workload (default): the batched bump-channel configuration -- 64 independent
single-block channels with a sinusoidal lower-wall bump (height 4-10 % of
chord), sizes drawn uniformly between 32^3 and 96x64x48 cells, Mach
0.3-0.85, inviscid Euler, MUSCL + minmod, Roe flux, scalar LU-SGS, CFL 20
(seeded synthetic grids; no dataset).  One step = one nonlinear iteration of
every case of the batch.  Metric: cell-iterations/s.

Arms:
  default            this project's sm_103a path through the C ABI.  `value`
                     is the FP64 path with the fast faces (MUSCL and Roe in
                     FP64 rearranged to fewer divisions; equal to the
                     reference to roundoff, within the parity tolerances);
                     the bit-exact FP64 faces are timed beside it under
                     "fp64_exact" and the mixed FP32/FP64 path under
                     "mixed".
  --impl reference   the reference algorithm on the host cores.  The
                     reference's own build needs its source tree, which this
                     machine may not have; the CPU oracle (a plain-C
                     restatement of the reference, bit-exact against it) is
                     timed instead, with every host thread.

Multi-GPU: replicas only (independent batches per rank, no data-path
collective); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-iterations/s"


# ----------------------------------------------------------------- workload
def make_workload(tmp: str, ncases: int):
    from aither_gb300 import cases
    specs = cases.bump_batch_specs(ncases)
    inps = []
    for q, (ni, nj, nk, h, m) in enumerate(specs):
        inp, _ = cases.bump_channel(os.path.join(tmp, f"c{q:03d}"), ni, nj, nk, h, m,
                                    cfl=20.0, name=f"bump{q:03d}")
        inps.append(inp)
    return inps, specs


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples during the timed region (read-only queries)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------- roofline model
def algorithmic_bytes(nv: int = 5, d: int = 1, b: int = 8, viscous: bool = False,
                      block: bool = False, rans: bool = False) -> dict:
    """Compulsory traffic per cell-iteration of the four irreducible passes
    (values counted once per pass that needs them; ghosts and metadata
    excluded): residual (2nv+17+d), forward sweep (4nv+d+12), backward
    sweep (4nv+d+12), update+norms (4nv); b bytes per value.  Viscous
    solves add 24 values to the residual (centres, wall distance, velocity,
    temperature, density and pressure gradients, viscosity, temperature) and
    4 per sweep (centres, viscosity), 13 with block solves (the velocity
    gradient); SST adds 9 to the residual (k and omega gradients, eddy
    viscosity, F1, F2) and 2 per sweep (eddy viscosity, F1)."""
    res = 2 * nv + 17 + d + (24 if viscous else 0) + (9 if rans else 0)
    sw = 4 * nv + d + 12 + ((13 if block else 4) if viscous else 0) + (2 if rans else 0)
    return {"residual": res * b, "forward": sw * b, "backward": sw * b, "update": 4 * nv * b,
            "total": (res + 2 * sw + 4 * nv) * b}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return {**json.load(f), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


# ------------------------------------------------------------------- arms
def run_native(args, rank: int, world: int, device: int):
    from aither_gb300 import BATCH_FAST_FACES, PREC_FP64, PREC_MIXED, Batch, Context, Setup
    with tempfile.TemporaryDirectory() as tmp:
        inps, specs = make_workload(tmp, args.ncases)
        t0 = time.time()
        setup = Setup(inps)
        t_setup = time.time() - t0
    nsolves, nblocks, ncells = setup.counts()
    ctx = Context(device)
    out = {"fp64_peak_tflops": ctx.fp64_peak(5)}
    # the same setup with the cells' geometry and wall distance on the device
    with tempfile.TemporaryDirectory() as tmp:
        inps, _ = make_workload(tmp, args.ncases)
        t0 = time.time()
        Setup(inps, device=device).close()
        out["setup_device_s"] = time.time() - t0
    for prec_name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
        if args.precision not in ("both", prec_name):
            continue
        batch = Batch(ctx, setup, prec,
                      BATCH_FAST_FACES if (args.fast_faces and prec == PREC_FP64) else 0)
        if args.sweep_shape:
            sh = [int(x) for x in args.sweep_shape.split(",")] + [0]
            batch.set_sweep_shape(sh[0], sh[1], sh[2])
        for _ in range(args.warmup):
            batch.iterate(1)
        if args.sweep_shape:
            sweep_threads = sh[1]
        else:
            sweep_threads = batch.autotune(3)  # restores the state it ran on
        shape = batch.sweep_shape()
        _barrier(world)
        clocks = ClockSampler(device)
        clocks.start()
        t0 = time.time()
        norms = batch.iterate(args.steps)
        wall = time.time() - t0
        st = batch.stats()
        clk = clocks.stop()
        ms = st.device_ms
        ms = _max_over_ranks(ms, world)
        status_ok = all(n.status == 0 for n in norms)
        res = {"value": ncells * args.steps * world / (ms * 1e-3), "ms_per_step": ms / args.steps,
               "wall_s": wall, "gpu_launches": int(st.kernel_launches), "clocks": clk,
               "status_ok": status_ok, "sweep_threads": sweep_threads, "sweep_shape": shape}
        # per-kernel-class CUDA-event times (one iteration's worth each)
        prof = batch.profile(2)
        res["kernel_ms"] = dict(zip(["ghost", "face_i", "face_j", "face_k", "cell",
                                     "sweep_fwd", "sweep_bwd", "update"], prof.tolist()))
        # end to end through the C ABI with host buffers: every step uploads
        # the state from page-locked host memory, iterates, reads back the
        # norms and the state
        res["e2e"] = run_e2e(batch, ncells, args.steps, world)
        batch.close()
        out[prec_name] = res
        if prec == PREC_FP64 and args.fast_faces and args.exact_arm:
            # the bit-exact faces on the same workload, for comparison
            ex = Batch(ctx, setup, prec)
            for _ in range(args.warmup):
                ex.iterate(1)
            ex.autotune(2)
            ex.iterate(args.steps)
            st2 = ex.stats()
            pe = ex.profile(1)
            out["fp64_exact"] = {
                "value": ncells * args.steps * world / (st2.device_ms * 1e-3),
                "ms_per_step": st2.device_ms / args.steps,
                "kernel_ms": dict(zip(["ghost", "face_i", "face_j", "face_k", "cell",
                                       "sweep_fwd", "sweep_bwd", "update"], pe.tolist()))}
            ex.close()
    if args.converge_drop > 0 and args.precision == "both":
        out["converge"] = run_converge(args, ctx, setup, specs, world)
    if args.vortex_iters > 0:
        out["vortex"] = run_vortex(args, ctx, world)
    if args.mg_iters > 0 and args.converge_drop > 0:
        out["multigrid"] = run_mg(args, ctx, world)
    if args.long_iters_c2 > 0 or args.long_iters_c3 > 0:
        out["long"] = run_long(args, ctx, world)
    if args.sst_steps > 0:
        out["sst"] = run_sst(args, ctx, world)
    if args.plate_iters > 0:
        out["plate"] = run_plate(args, ctx, world)
    if args.served_n > 0:
        out["served"] = {"definition": "latency = submit to retirement (host clock), "
                                       "retirement at the residual drop; solves/s = "
                                       "converged requests / makespan",
                         "drop": args.served_drop, "slots": args.served_slots,
                         "max_cells": args.served_max_cells}
        for pname, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
            out["served"][pname] = [run_served(args, ctx, prec, r, 11 + rank)
                                    for r in args.served_rates]
    ctx.close()
    return out, ncells, nsolves, t_setup, specs


def run_served(args, ctx, precision, rate, seed):
    """The served configuration: a Poisson stream of `args.served_n` solve
    requests at `rate` per second (cells log-normal, clipped; bump and
    wedge channels; Mach 0.3-2.5; angle of attack -4..4 degrees; half laminar
    Navier-Stokes, half SST-2003 RANS by default), admitted by the server as slots and device
    memory free up, retired on the device at the residual drop.  Returns
    time-to-convergence percentiles (submit to retirement) and solves/s."""
    import numpy as np

    from aither_gb300 import Server, cases
    specs = cases.served_specs(args.served_n, seed=seed, max_cells=args.served_max_cells,
                               mix=args.served_mix)
    rng = np.random.default_rng(seed + 1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=len(specs)))
    with tempfile.TemporaryDirectory() as tmp:
        inps = []
        for q, sp in enumerate(specs):
            kw = dict(sp)
            vis = kw.pop("viscous")
            inp, _ = cases.wall_channel(os.path.join(tmp, f"s{q}"), viscous=vis,
                                        stretch=1.1 if vis else 1.0, name=f"s{q}", **kw)
            inps.append(inp)
        srv = Server(ctx, precision, drop=args.served_drop, max_iters=args.served_max_iters,
                     chunk=50, max_active=args.served_slots)
        t0 = time.time()
        nxt, done, max_active = 0, {}, 0
        while len(done) < len(specs):
            now = time.time() - t0
            while nxt < len(specs) and arrivals[nxt] <= now:
                srv.submit(inps[nxt])
                nxt += 1
            a, _ = srv.step()
            max_active = max(max_active, a)
            for st in srv.poll():
                done[st.id] = st
                srv.release(st.id)
            time.sleep(0.0002)
        makespan = time.time() - t0
        srv.close()
    st = list(done.values())
    conv = [x for x in st if x.converged == 1]
    lat = [x.latency_ms for x in conv]
    kinds = {"sst": [x.latency_ms for x, sp in zip(sorted(st, key=lambda x: x.id), specs)
                     if x.converged == 1 and sp.get("rans")],
             "laminar": [x.latency_ms for x, sp in zip(sorted(st, key=lambda x: x.id), specs)
                         if x.converged == 1 and not sp.get("rans")]}
    return {"rate_per_s": rate, "requests": len(specs), "converged": len(conv),
            "p50_ms_by_kind": {k: _pct(v, 50) for k, v in kinds.items()},
            "nonphysical": sum(1 for x in st if x.converged == -1),
            "iteration_cap": sum(1 for x in st if x.converged == 0),
            "makespan_s": makespan, "solves_per_s": len(conv) / makespan,
            "p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99),
            "queue_p50_ms": _pct([x.queue_ms for x in st], 50),
            "max_concurrent": max_active,
            "cells": int(sum(sp["ni"] * sp["nj"] * sp["nk"] for sp in specs))}


def run_vortex(args, ctx, world):
    """The plain-method configuration: the 64x32x8 periodic vortex box
    (inviscid Euler, MUSCL minmod, Roe, LU-SGS at CFL 10), `vortex_iters`
    iterations timed in FP64 (bit-exact faces, the reference's arithmetic),
    FP64 with the fast faces and mixed precision; the oracle on rank 0 for
    a bounded sample."""
    from aither_gb300 import BATCH_FAST_FACES, PREC_FP64, PREC_MIXED, Batch, Setup, cases
    with tempfile.TemporaryDirectory() as tmp:
        inp, st = cases.vortex_box(tmp)
        setup = Setup(inp)
        setup.set_state(0, st[0])
    _, _, ncells = setup.counts()
    out = {"workload": "periodic vortex box 64x32x8 cells, Euler, MUSCL minmod, Roe, LU-SGS, "
                       "CFL 10", "cells": ncells, "iterations": args.vortex_iters}
    for name, prec, flags in (("fp64", PREC_FP64, 0), ("fp64_fast", PREC_FP64, BATCH_FAST_FACES),
                              ("mixed", PREC_MIXED, 0)):
        b = Batch(ctx, setup, prec, flags)
        b.autotune(2)
        _barrier(world)
        norms = b.iterate(args.vortex_iters)
        st2 = b.stats()
        ms = _max_over_ranks(st2.device_ms, world)
        out[name] = {"cell_iterations_per_s": ncells * args.vortex_iters * world / (ms * 1e-3),
                     "ms_per_iteration": ms / args.vortex_iters,
                     "status_ok": all(x.status == 0 for x in norms),
                     "sweep_shape": b.sweep_shape()}
        b.close()
    if not args.no_cpu_baseline and int(os.environ.get("RANK", "0")) == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from pyoracle import Oracle
        orc = Oracle(setup, 1)
        orc.iterate(1)
        t0 = time.perf_counter()
        orc.iterate(20)
        dt = (time.perf_counter() - t0) / 20
        out["cpu_baseline"] = {"value": ncells / dt, "unit": METRIC, "cores": 1, "kind": "port",
                               "sample": "20 iterations after 1 warm-up; oracle, one block so "
                                         "one thread"}
        orc.close()
    return out


def run_sst(args, ctx, world):
    """Turbulent flat plate (SST-2003 k-omega RANS, seven equations): one
    256x192x4 block, Re_L 5e6, Mach 0.2, first cell at y+ = 1, WENO, AUSM,
    block LU-SGS, CFL 10.  Cell-iterations/s of the FP64 and mixed paths over
    `args.sst_steps` iterations after warm-up, per-pass kernel times, the
    HBM roofline of the dominant FP64 pass and, on rank 0, the oracle's time
    for a bounded sample of the same case."""
    from aither_gb300 import PREC_FP64, PREC_MIXED, Batch, Setup, cases
    with tempfile.TemporaryDirectory() as tmp:
        inp, _ = cases.sst_plate(tmp, ni=args.sst_ni, nj=args.sst_nj, nk=args.sst_nk, cfl=10.0)
        setup = Setup(inp)
    _, _, ncells = setup.counts()
    out = {"workload": f"SST-2003 turbulent flat plate {args.sst_ni}x{args.sst_nj}x"
                       f"{args.sst_nk} cells, Re 5e6, Mach 0.2, y+ 1, WENO, AUSM, block "
                       "LU-SGS, CFL 10", "cells": ncells, "steps": args.sst_steps}
    for name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
        b = Batch(ctx, setup, prec)
        for _ in range(max(args.warmup, 3)):
            b.iterate(1)
        tuned = b.autotune(2)
        shape = b.sweep_shape()
        _barrier(world)
        clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
        clocks.start()
        norms = b.iterate(args.sst_steps)
        st = b.stats()
        clk = clocks.stop()
        ms = _max_over_ranks(st.device_ms, world)
        prof = b.profile(2)
        out[name] = {"value": ncells * args.sst_steps * world / (ms * 1e-3),
                     "unit": METRIC, "ms_per_step": ms / args.sst_steps,
                     "gpu_launches": int(st.kernel_launches), "sweep_threads": tuned,
                     "sweep_shape": shape,
                     "status_ok": all(n.status == 0 for n in norms), "clocks": clk,
                     "kernel_ms": dict(zip(["ghost", "face_i", "face_j", "face_k",
                                            "viscous+cell", "sweep_fwd", "sweep_bwd",
                                            "update"], prof.tolist()))}
        b.close()
    out["mixed"]["speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    km = out["fp64"]["kernel_ms"]
    ab = algorithmic_bytes(nv=7, d=29, b=8, viscous=True, block=True, rans=True)
    pass_ms = {"residual": km["face_i"] + km["face_j"] + km["face_k"] + km["viscous+cell"],
               "forward": km["sweep_fwd"], "backward": km["sweep_bwd"], "update": km["update"]}
    dom = max(pass_ms, key=pass_ms.get)
    peaks = measured_peaks()
    achieved = ab[dom] * ncells / (pass_ms[dom] * 1e-3) / 1e9
    out["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": achieved,
                       "peak": peaks["hbm_gbs"], "unit": "GB/s",
                       "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                       "bytes_per_cell": ab}
    if not args.no_cpu_baseline and int(os.environ.get("RANK", "0")) == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from pyoracle import Oracle
        threads = os.cpu_count() or 1
        orc = Oracle(setup, threads)
        orc.iterate(1)
        t0 = time.perf_counter()
        orc.iterate(1)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": ncells / dt, "unit": METRIC, "cores": 1, "kind": "port",
                               "sample": "1 iteration of the full case after 1 warm-up "
                                         "iteration; oracle (C restatement of the "
                                         "reference), one block so one thread"}
        orc.close()
    return out


def run_plate(args, ctx, world):
    """Laminar flat plate, two 128x64x2 blocks joined by an interblock
    connection (first cell 1e-5, growth 1.08, Mach 0.3, Re_L 1e5, van
    Albada, Roe, block LU-SGS with 4 sweeps; with one sweep the reference
    itself turns nonphysical at CFL 100): `plate_iters` iterations in FP64
    and in mixed precision after autotuning.  The case's residual stalls
    near a 0.3 drop (a limit cycle, the same in the reference), so the
    section reports time per iteration rather than time to a drop, the
    mixed state's deviation from FP64 after the run and, on rank 0, the
    oracle's time per iteration."""
    import numpy as np

    from aither_gb300 import PREC_FP64, PREC_MIXED, Batch, Setup, cases
    with tempfile.TemporaryDirectory() as tmp:
        inp, _ = cases.flat_plate(tmp, matrix_solver="blusgs", sweeps=4, name="plate")
        setup = Setup(inp)
    _, _, ncells = setup.counts()
    out = {"workload": "laminar flat plate, two 128x64x2 blocks, interblock, block LU-SGS "
                       "with 4 sweeps, CFL 100", "cells": ncells, "iterations": args.plate_iters}
    states = {}
    for name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
        b = Batch(ctx, setup, prec)
        tuned = b.autotune(2)
        _barrier(world)
        norms = b.iterate(args.plate_iters)
        st = b.stats()
        states[name] = [b.field(k, "STATE") for k in range(2)]
        l2 = np.array([[x.l2[v] for v in range(5)] for x in norms])
        tot = np.sqrt((l2 ** 2).sum(axis=1))
        ms = _max_over_ranks(st.device_ms, world)
        out[name] = {"ms_per_iteration": ms / args.plate_iters,
                     "cell_iterations_per_s": ncells * args.plate_iters * world / (ms * 1e-3),
                     "drop": float(tot[-1] / tot[:5].max()),
                     "status_ok": all(x.status == 0 for x in norms),
                     "sweep_threads": tuned, "sweep_shape": b.sweep_shape()}
        b.close()
    out["mixed_speedup"] = out["fp64"]["ms_per_iteration"] / out["mixed"]["ms_per_iteration"]
    out["mixed_vs_fp64_state_max_rel_err"] = max(
        float(np.abs(a - b).max() / np.abs(b).max())
        for a, b in zip(states["mixed"], states["fp64"]))
    if not args.no_cpu_baseline and int(os.environ.get("RANK", "0")) == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from pyoracle import Oracle
        threads = os.cpu_count() or 1
        orc = Oracle(setup, threads)
        orc.iterate(1)
        t0 = time.perf_counter()
        orc.iterate(10)
        dt = (time.perf_counter() - t0) / 10
        out["cpu_baseline"] = {"value": ncells / dt, "unit": METRIC, "cores": min(2, threads),
                               "kind": "port", "ms_per_iteration": dt * 1e3,
                               "sample": "10 iterations after 1 warm-up; oracle, OpenMP over "
                                         "the two blocks"}
        orc.close()
    return out


def run_long(args, ctx, world):
    """The single-case configurations run to convergence rather than timed
    for a fixed count: c2 (the laminar two-block plate with block LU-SGS
    and 4 sweeps, here with wall-normal growth 1.15 capped at 0.05 L so the
    domain clears the boundary layer; to a 1e-8 drop) and c3 (the SST plate
    with a CFL ramp from 1 by 0.009 per iteration to 10; 5000 iterations).
    Per path: iterations run, the drop reached, device time, and whether the
    state stayed physical."""
    import numpy as np

    from aither_gb300 import PREC_FP64, PREC_MIXED, Batch, Setup, cases
    out = {}
    specs = [("c2", lambda d: cases.flat_plate(d, matrix_solver="blusgs", sweeps=4, ratio=1.15,
                                               dy_max=0.05, name="plate"), 1e-8,
              args.long_iters_c2,
              "laminar flat plate, two 128x64x2 blocks, first cell 1e-5, growth 1.15 capped "
              "at 0.05 L, Mach 0.3, Re_L 1e5, block LU-SGS 4 sweeps, CFL 100"),
             ("c3", lambda d: cases.sst_plate(d, cfl=10.0, cfl_start=1.0, cfl_step=0.009),
              1e-12, args.long_iters_c3,
              "SST-2003 flat plate 256x192x4, Re 5e6, Mach 0.2, y+ 1, WENO, AUSM, block "
              "LU-SGS, CFL 1 ramped by 0.009 per iteration to 10")]
    for key, gen, drop, iters, desc in specs:
        if iters <= 0:
            continue
        with tempfile.TemporaryDirectory() as tmp:
            inp, _ = gen(tmp)
            setup = Setup(inp)
        _, _, ncells = setup.counts()
        res = {"workload": desc, "cells": ncells, "drop": drop, "max_iterations": iters}
        states = {}
        for name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
            b = Batch(ctx, setup, prec)
            b.autotune(2)
            _barrier(world)
            info = b.converge(iters, drop, check_every=100)
            st = b.stats()
            states[name] = [b.field(k, "STATE") for k in range(b.nblocks)]
            b.close()
            x = info[0]
            res[name] = {"iterations": int(x.iterations), "drop_reached": x.drop,
                         "status": {1: "converged", 0: "iteration_cap", -1: "nonphysical"}.get(
                             int(x.converged), int(x.converged)),
                         "device_s": _max_over_ranks(st.device_ms * 1e-3, world),
                         "ms_per_iteration": st.device_ms / max(int(x.iterations), 1)}
        if all(np.isfinite(a).all() for a in states["fp64"] + states["mixed"]):
            res["mixed_vs_fp64_state_max_rel_err"] = max(
                float(np.abs(a - b).max() / np.abs(b).max())
                for a, b in zip(states["mixed"], states["fp64"]))
        out[key] = res
    return out


def _pct(x, q):
    import numpy as np
    return float(np.percentile(np.asarray(x, dtype=float), q)) if len(x) else None


def _converge_once(ctx, setup, prec, args, world):
    """Runs every solve of `setup` to the residual drop; per-solve times are
    device-clock intervals from the end of the solve's first iteration to
    its retirement (all solves start together)."""
    from aither_gb300 import Batch
    b = Batch(ctx, setup, prec)
    tuned = b.autotune(3)
    _barrier(world)
    t0 = time.time()
    info = b.converge(args.converge_max, args.converge_drop, check_every=100)
    wall = time.time() - t0
    st = b.stats()
    states = [b.field(s, "STATE") for s in range(b.nsolves)]
    b.close()
    ms = [x.ms for x in info]
    its = [int(x.iterations) for x in info]
    conv = [x.converged == 1 for x in info]
    dev_s = _max_over_ranks(st.device_ms * 1e-3, world)
    return {"solves": len(info), "converged": int(sum(conv)), "device_s": dev_s, "wall_s": wall,
            "solves_per_s": sum(conv) * world / dev_s, "p50_ms": _pct(ms, 50),
            "p99_ms": _pct(ms, 99), "iterations_p50": _pct(its, 50),
            "iterations_max": max(its) if its else None, "sweep_threads": tuned}, states, \
        (its, conv)


def run_converge(args, ctx, setup, specs, world):
    """Solves/s and time-to-convergence: the mixed path on the whole batch
    (the batched configuration runs mixed precision to a 1e-6 drop), and the
    FP64 and mixed paths on the smallest cases, whose converged states give
    the mixed path's error against FP64."""
    import numpy as np

    from aither_gb300 import PREC_FP64, PREC_MIXED, Setup
    out = {"drop": args.converge_drop, "max_iterations": args.converge_max,
           "definition": "per solve: total L2 over the equations relative to its first "
                         "iteration; a solve retires on the device in the iteration that "
                         "reaches the drop; p50/p99 over solves of the time from the end of "
                         "its first iteration to retirement (all solves start together)"}
    out["mixed"], _, _ = _converge_once(ctx, setup, PREC_MIXED, args, world)
    k = min(args.converge_fp64_cases, len(specs))
    if k > 0:
        order = sorted(range(len(specs)), key=lambda i: specs[i][0] * specs[i][1] * specs[i][2])
        pick = sorted(order[:k])
        with tempfile.TemporaryDirectory() as tmp:
            inps, _ = make_workload(tmp, args.ncases)
            sub = Setup([inps[i] for i in pick])
        f64, w64, (it64, cv64) = _converge_once(ctx, sub, PREC_FP64, args, world)
        mix, wmx, (itmx, cvmx) = _converge_once(ctx, sub, PREC_MIXED, args, world)
        # the converged solves' states (an unconverged one is anywhere on its
        # limit cycle)
        both = [q for q in range(len(w64)) if cv64[q] and cvmx[q]]
        err = max((float(np.abs(wmx[q] - w64[q]).max() / np.abs(w64[q]).max()) for q in both),
                  default=None)
        out["subset"] = {"cases": pick, "cells": int(sum(specs[i][0] * specs[i][1] * specs[i][2]
                                                         for i in pick)),
                         "fp64": f64, "mixed": mix,
                         "mixed_speedup": f64["device_s"] / mix["device_s"],
                         "mixed_vs_fp64_state_max_rel_err": err,
                         "state_err_over": "solves converged in both precisions",
                         "iterations_max_abs_diff": int(max(abs(a - b) for a, b in zip(itmx, it64)))}
    return out


def run_mg(args, ctx, world):
    """Multigrid against single-grid relaxation on one transonic bump channel
    with the scheme of the reference's multigrid case (testCases/
    transonicBump: Euler, upwind MUSCL with van Albada, DP-LUR with 4 sweeps,
    three levels, W cycle; here at CFL 1000): iterations and device time to
    the residual drop, FP64 and mixed."""
    from aither_gb300 import PREC_FP64, PREC_MIXED, Batch, Setup, cases
    ni, nj = args.mg_ni, args.mg_nj
    out = {"workload": f"transonic bump channel {ni}x{nj}x2 cells, Mach 0.7, bump 8 % of the "
                       "chord, Euler, upwind MUSCL with van Albada, Roe, DP-LUR 4 sweeps, "
                       "CFL 1000",
           "cells": ni * nj * 2, "drop": args.converge_drop, "max_iterations": args.mg_iters}
    for label, mg in (("multigrid_w3", (3, "W")), ("single_grid", None)):
        with tempfile.TemporaryDirectory() as tmp:
            inp, _ = cases.bump_channel(tmp, ni=ni, nj=nj, nk=2, height=0.08, mach=0.7,
                                        cfl=1000.0, matrix_solver="dplur", sweeps=4,
                                        recon="upwind", limiter="vanAlbada", multigrid=mg,
                                        name="tb")
            setup = Setup(inp)
        res = {}
        for pname, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
            b = Batch(ctx, setup, prec)
            _barrier(world)
            info = b.converge(args.mg_iters, args.converge_drop, check_every=50)
            st = b.stats()
            b.close()
            x = info[0]
            its = max(int(x.iterations), 1)
            dev_s = _max_over_ranks(st.device_ms * 1e-3, world)
            res[pname] = {"iterations": int(x.iterations),
                          "status": {1: "converged", 0: "iteration_cap",
                                     -1: "nonphysical"}.get(int(x.converged), int(x.converged)),
                          "drop_reached": x.drop, "device_s": dev_s,
                          "ms_per_iteration": dev_s * 1e3 / its,
                          "gpu_launches_per_iteration": int(st.kernel_launches) // its}
        out[label] = res
    return out


def run_e2e(batch, ncells: int, steps: int, world: int) -> dict:
    n = batch.pool_cells()
    host = _pinned(batch.pool_vars() * n)
    batch.copy_state(host, to_device=False)
    # one untimed round first: the iteration graph may need recapturing
    # after the per-kernel profile, and the host pages their first touch
    batch.copy_state(host, to_device=True)
    batch.iterate(1)
    batch.copy_state(host, to_device=False)
    t0 = time.perf_counter()
    for _ in range(steps):
        batch.copy_state(host, to_device=True)
        batch.iterate(1)
        batch.copy_state(host, to_device=False)
    dt = time.perf_counter() - t0
    dt = _max_over_ranks(dt * 1e3, world) * 1e-3
    from aither_gb300._lib import Norms
    import ctypes
    nb = host.size * 8
    return {"value": ncells * steps * world / dt, "unit": METRIC,
            "h2d_bytes_per_step": nb,
            "d2h_bytes_per_step": nb + ctypes.sizeof(Norms) * batch.nsolves}


def _pinned(count: int) -> np.ndarray:
    try:
        import torch
        if torch.cuda.is_available():
            t = torch.empty(count, dtype=torch.float64, pin_memory=True)
            a = t.numpy()
            a._keep = t  # noqa: SLF001 -- keep the pinned allocation alive
            return a
    except Exception:
        pass
    return np.empty(count, dtype=np.float64)


def cpu_baseline(sample_cases: int, iters: int, threads: int) -> dict:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from pyoracle import Oracle

    from aither_gb300 import Setup
    with tempfile.TemporaryDirectory() as tmp:
        inps, _ = make_workload(tmp, sample_cases)
        setup = Setup(inps)
    _, _, ncells = setup.counts()
    orc = Oracle(setup, threads)
    orc.iterate(1)
    t0 = time.perf_counter()
    orc.iterate(iters)
    dt = time.perf_counter() - t0
    return {"value": ncells * iters / dt, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"first {sample_cases} cases of the batched workload "
                      f"({ncells} cells), {iters} iterations, oracle "
                      f"(C restatement of the reference, bit-exact against it), "
                      f"OpenMP over blocks"}


# ------------------------------------------------------------- distributed
def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("BENCH_BACKEND", "") != "gloo" else "gloo"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
            else:
                torch.cuda.set_device(local)
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return rank, world, local


def _barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(x: float, world: int) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# -------------------------------------------------------------------- main
# One-off ncu captures of the FP64 batched path, per cell of the batch (a
# bump-channel batch's cells; the counts scale with cells):
#   * fast option -- `ncu --clock-control none --metrics dram__bytes_read.sum,
#     dram__bytes_write.sum,gpu__time_duration.sum,smsp__sass_thread_inst_
#     executed_op_{dfma,dadd,dmul}_pred_on.sum,... -s 1103 -c 355` (every
#     launch of the first timed iteration) on `python bench.py --ncases 8
#     --steps 1 --warmup 3 --no-cpu-baseline --converge-drop 0 --served-n 0
#     --sst-steps 0 --plate-iters 0 --vortex-iters 0 --mg-iters 0 --precision
#     fp64 --sweep-shape 2,32 --exact-arm 0` (the first 8 cases, 888,004
#     cells; GB300, 2026-12-04): residual-pass DRAM traffic 925.3 B per cell
#     (faces 133.3 + 140.4 + 143.9, cell kernel 507.7); executed FP64 FLOP
#     268.6 per face direction, 560.1 in the two sweeps, 165.0 cell, 73.2
#     update, 19.2 ghost fill;
#   * bit-exact path -- the same counters over one iteration of a 64x48x32
#     bump channel: 1026 FLOP per face direction, 1134 in the two sweeps,
#     502 cell, 188 update, 25 ghosts.
# FLOP = 2 x DFMA + DADD + DMUL (divisions and square roots run as FMA
# sequences and are counted in those).
NCU_PER_CELL = {
    "source": "ncu captures on GB300 of the batched bump-channel path (fast option: every "
              "launch of one iteration of the first 8 cases of the batched workload, "
              "888,004 cells; bit-exact path: one 64x48x32 case), 2026-12-04",
    "residual_traffic_bytes": {"fast": 925.3},
    "flop": {"fast": {"face_per_direction": 268.6, "sweeps": 560.1, "cell": 165.0,
                      "update": 73.2, "ghost": 19.2},
             "exact": {"face_per_direction": 1026.0, "sweeps": 1134.0, "cell": 502.0,
                       "update": 188.0, "ghost": 25.0}},
}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--ncases", type=int, default=64)
    ap.add_argument("--precision", default="both", choices=["both", "fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fast-faces", type=int, default=1,
                    help="1: FP64 batches use the fast MUSCL/Roe faces (roundoff-equal to "
                         "the reference instead of bit for bit)")
    ap.add_argument("--converge-drop", type=float, default=1e-6,
                    help="residual drop of the time-to-convergence runs (0: skip them)")
    ap.add_argument("--converge-max", type=int, default=8000)
    ap.add_argument("--served-n", type=int, default=6,
                    help="requests of the served configuration (0: skip it)")
    ap.add_argument("--served-rates", type=float, nargs="+", default=[2.0],
                    help="Poisson arrival rates (requests/s) to sweep")
    ap.add_argument("--served-max-cells", type=int, default=64_000,
                    help="upper clip of the request sizes (the configuration's is 4M)")
    ap.add_argument("--served-drop", type=float, default=1e-6)
    ap.add_argument("--served-slots", type=int, default=16)
    ap.add_argument("--served-mix", default="ns_sst", choices=["ns_sst", "euler_ns"],
                    help="half laminar / half SST-2003 requests, or half Euler / half laminar")
    ap.add_argument("--vortex-iters", type=int, default=200,
                    help="iterations of the 64x32x8 vortex box section (0 skips it)")
    ap.add_argument("--sst-steps", type=int, default=20,
                    help="iterations of the SST flat plate section (0 skips it)")
    ap.add_argument("--plate-iters", type=int, default=500,
                    help="iterations of the laminar plate section (0 skips it)")
    ap.add_argument("--sst-ni", type=int, default=256)
    ap.add_argument("--sst-nj", type=int, default=192)
    ap.add_argument("--sst-nk", type=int, default=4)
    ap.add_argument("--served-max-iters", type=int, default=6000)
    ap.add_argument("--long-iters-c2", type=int, default=0,
                    help="c2 to a 1e-8 drop with this iteration cap (0: skip)")
    ap.add_argument("--long-iters-c3", type=int, default=0,
                    help="c3 with a CFL ramp for this many iterations (0: skip)")
    ap.add_argument("--mg-iters", type=int, default=3000,
                    help="iteration cap of the multigrid section (0: skip it)")
    ap.add_argument("--mg-ni", type=int, default=256)
    ap.add_argument("--mg-nj", type=int, default=128)
    ap.add_argument("--sweep-shape", default=None,
                    help="mode,threads[,cluster]: a fixed LU-SGS sweep shape for the batched "
                         "arms instead of the autotuner's pick (mode 0: a thread per cell, 2: "
                         "lanes per neighbour term, 1: persistent clusters, 3: tile queue)")
    ap.add_argument("--exact-arm", type=int, default=1,
                    help="also time the bit-exact FP64 faces when --fast-faces is on")
    ap.add_argument("--converge-fp64-cases", type=int, default=8,
                    help="smallest cases also run to convergence in FP64 for the comparison")
    args = ap.parse_args()
    rank, world, local = _dist()
    config = {"workload": f"batched bump channels: {args.ncases} single-block cases, "
                          "32^3..96x64x48 cells, Mach 0.3-0.85, inviscid Euler, MUSCL minmod, "
                          "Roe, scalar LU-SGS, CFL 20",
              "ncases": args.ncases, "l2_flush": "inputs larger than L2 (GB-scale working set)",
              "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        threads = os.cpu_count() or 1
        base = cpu_baseline(args.ncases, 1, threads)  # one step = one iteration of the batch
        # warm-up and timed steps of the full workload
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from pyoracle import Oracle

        from aither_gb300 import Setup
        with tempfile.TemporaryDirectory() as tmp:
            inps, _ = make_workload(tmp, args.ncases)
            setup = Setup(inps)
        _, _, ncells = setup.counts()
        orc = Oracle(setup, threads)
        orc.iterate(args.warmup)
        t0 = time.perf_counter()
        orc.iterate(args.steps)
        dt = time.perf_counter() - t0
        v = ncells * args.steps / dt
        line = {"metric": METRIC, "value": v, "unit": METRIC, "impl": "reference",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config,
                "cpu_baseline": {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
                                 "sample": f"full batched workload ({ncells} cells), "
                                           f"{args.steps} iterations; the reference's own "
                                           "build is unavailable on this host (its sources "
                                           "are not shipped), so its C restatement is timed"},
                "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    res, ncells, nsolves, t_setup, specs = run_native(args, rank, world, local)
    if rank != 0:
        return
    fp = res.get("fp64") or res.get("mixed")
    km = fp["kernel_ms"]
    peaks = measured_peaks()
    ab = algorithmic_bytes()
    # per kernel class: algorithmic bytes of its pass over the batch
    pass_bytes = {"residual": ab["residual"] * ncells, "sweep_fwd": ab["forward"] * ncells,
                  "sweep_bwd": ab["backward"] * ncells, "update": ab["update"] * ncells}
    pass_ms = {"residual": km["face_i"] + km["face_j"] + km["face_k"] + km["cell"],
               "sweep_fwd": km["sweep_fwd"], "sweep_bwd": km["sweep_bwd"],
               "update": km["update"]}
    dom = max(pass_ms, key=pass_ms.get)
    achieved = pass_bytes[dom] / (pass_ms[dom] * 1e-3) / 1e9
    # FP64 bound: executed FP64 FLOP per cell-iteration (2 per DFMA, 1 per
    # DADD / DMUL, from the captures above; divisions and square roots run as
    # FMA sequences) against the FP64 issue peak measured on this GPU.  Only
    # for the FP64 arm of this workload (the physics the counts were taken on)
    roof_fp64 = None
    fp64_peak = res.get("fp64_peak_tflops") or 0.0
    if "fp64" in res and fp64_peak:
        mode = "fast" if args.fast_faces else "exact"
        fl = NCU_PER_CELL["flop"][mode]
        fpd = fl["face_per_direction"]
        face_ms = km["face_i"] + km["face_j"] + km["face_k"]
        face_tf = 3 * fpd * ncells / (face_ms * 1e-3) / 1e12
        path_flop = 3 * fpd + fl["sweeps"] + fl["cell"] + fl["update"] + fl["ghost"]
        path_tf = path_flop * fp["value"] / 1e12
        roof_fp64 = {"bound": "fp64", "kernel": "face (3 directions)", "achieved": face_tf,
                     "peak": fp64_peak, "unit": "TFLOP/s", "frac": face_tf / fp64_peak,
                     "peak_source": "measured on this GPU (ath_ctx_fp64_peak)",
                     "path_achieved": path_tf, "path_frac": path_tf / fp64_peak,
                     "faces": mode, "flop_per_cell_iteration": path_flop,
                     "flop_source": NCU_PER_CELL["source"]}
    traffic = None
    if "fp64" in res and args.fast_faces and dom == "residual":
        # DRAM bytes of one residual pass (3 face launches + the cell
        # launch), from the capture above scaled by the batch's cells
        traffic = NCU_PER_CELL["residual_traffic_bytes"]["fast"] * ncells
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
            "peak_source": peaks["source"], "traffic": traffic,
            "traffic_note": "DRAM bytes per residual pass from a one-off ncu capture of "
                            "the 8-case batch, scaled by cells; above the algorithmic "
                            "bytes because the face launches write per-face fluxes and "
                            "spectral radii that the cell launch reads back, and read "
                            "face areas, ghosts and neighbour states the per-cell count "
                            "leaves out",
            "bytes_per_cell": {k: v for k, v in ab.items()}}
    line = {"metric": METRIC, "value": fp["value"], "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": fp["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if "fp64" in res else "f32+f64",
            "data": "synthetic (seeded bump-channel grids)", "config": config,
            "cells": ncells, "solves": nsolves, "setup_s": t_setup,
            "setup_device_s": res.get("setup_device_s"),
            "gpu_launches": fp["gpu_launches"], "clocks": fp["clocks"],
            "e2e": fp["e2e"], "roofline": roof, "roofline_fp64": roof_fp64, "kernel_ms": km,
            "autotune": {"sweep_threads": fp["sweep_threads"], "sweep_shape": fp["sweep_shape"]}}
    if "mixed" in res and "fp64" in res:
        m = res["mixed"]
        line["mixed"] = {"value": m["value"], "ms_per_step": m["ms_per_step"],
                         "speedup_vs_fp64": m["value"] / fp["value"], "e2e": m["e2e"],
                         "kernel_ms": m["kernel_ms"], "gpu_launches": m["gpu_launches"],
                         "sweep_threads": m["sweep_threads"], "sweep_shape": m["sweep_shape"]}
    if "converge" in res:
        line["converge"] = res["converge"]
    if "served" in res:
        line["served"] = res["served"]
    if "sst" in res:
        line["sst"] = res["sst"]
    if "vortex" in res:
        line["vortex"] = res["vortex"]
    if "multigrid" in res:
        line["multigrid"] = res["multigrid"]
    if "long" in res:
        line["long"] = res["long"]
    if "fp64_exact" in res:
        line["fp64_exact"] = res["fp64_exact"]
    if "plate" in res:
        line["plate"] = res["plate"]
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        # at least as many cases as host threads (OpenMP over blocks)
        line["cpu_baseline"] = cpu_baseline(min(args.ncases, max(threads, 8)), 2, threads)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
