"""Seeded synthetic cases in the reference's file formats.

Each generator writes ``<name>.inp`` (the reference input format,
src/input.cpp:167-643) and ``<name>.xyz`` (binary multi-block Plot3D,
src/plot3d.cpp:363) into a directory and returns the input path plus the
analytic initial primitive state (nondimensional, per block, AoS over
physical cells with k slowest) when the case has one.

Workloads:
  vortex_box   -- single-block Cartesian box with an isentropic convecting
                  vortex, periodic in i and j, slip walls in k; inviscid
                  Euler, MUSCL (kappa=1/3) + minmod, Roe, LU-SGS.
                  Full size 64x32x8 cells on [0,10]x[0,5]x[0,1.25].
  bump_channel -- channel with a sinusoidal bump on the lower wall,
                  characteristic inflow/outflow, slip walls; inviscid Euler,
                  MUSCL minmod, Roe, LU-SGS, CFL 20.  Batches of these with
                  sizes drawn between 32^3 and 96x64x48 and Mach in
                  [0.3, 0.85] form the batched workload.
  block_pair   -- two blocks of a skewed box joined by an interblock
                  connection whose second block has its index axes in any
                  of the 24 right-handed signed permutations of the first's, so every
                  patch orientation (aligned, swapped, reversed; lower or
                  upper surfaces of any direction) can be exercised, with a
                  three-dimensional vortex crossing the connection.
"""
from __future__ import annotations

import math
import os
import struct
from dataclasses import dataclass

import numpy as np

GAS_N = 2.5
MOLAR_MASS = 28.97e-3
R_UNIV = 8.3144598
R_AIR = R_UNIV / MOLAR_MASS
GAMMA = (GAS_N + 1.0) / GAS_N


def write_plot3d(path: str, blocks: list[np.ndarray]) -> None:
    """blocks: arrays of shape (3, nk+1, nj+1, ni+1) (node coordinates)."""
    with open(path, "wb") as f:
        f.write(struct.pack("<i", len(blocks)))
        for b in blocks:
            _, nk1, nj1, ni1 = b.shape
            f.write(struct.pack("<iii", ni1, nj1, nk1))
        for b in blocks:
            for c in range(3):
                f.write(np.ascontiguousarray(b[c], dtype="<f8").tobytes())


def read_plot3d(path: str) -> list[np.ndarray]:
    with open(path, "rb") as f:
        (nb,) = struct.unpack("<i", f.read(4))
        dims = [struct.unpack("<iii", f.read(12)) for _ in range(nb)]
        out = []
        for ni1, nj1, nk1 in dims:
            n = ni1 * nj1 * nk1
            arr = np.frombuffer(f.read(3 * n * 8), dtype="<f8").reshape(3, nk1, nj1, ni1)
            out.append(arr.copy())
    return out


def box_nodes(ni, nj, nk, lx, ly, lz, x0=0.0, y0=0.0, z0=0.0) -> np.ndarray:
    x = x0 + lx * np.arange(ni + 1) / ni
    y = y0 + ly * np.arange(nj + 1) / nj
    z = z0 + lz * np.arange(nk + 1) / nk
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return np.stack([X, Y, Z])


def cell_centres(nodes: np.ndarray) -> np.ndarray:
    """Arithmetic mean of the 8 corner nodes, shape (3, nk, nj, ni)."""
    n = nodes
    return 0.125 * (n[:, :-1, :-1, :-1] + n[:, :-1, :-1, 1:] + n[:, :-1, 1:, :-1]
                    + n[:, :-1, 1:, 1:] + n[:, 1:, :-1, :-1] + n[:, 1:, :-1, 1:]
                    + n[:, 1:, 1:, :-1] + n[:, 1:, 1:, 1:])


@dataclass
class Refs:
    """Reference quantities as the reference derives them (src/input.cpp:617-621)."""

    t_ref: float
    r_ref: float

    @property
    def a_ref(self) -> float:
        return math.sqrt(0.0 + 1.0 * GAMMA * R_AIR * self.t_ref)


def _fmt(x: float) -> str:
    return repr(float(x))


def _bc_block(surfs: list[tuple]) -> str:
    """surfs: (name, i1, i2, j1, j2, k1, k2, tag) grouped i, j, k."""
    counts = [0, 0, 0]
    for s in surfs:
        _, i1, i2, j1, j2, k1, k2, _ = s
        d = 0 if i1 == i2 else (1 if j1 == j2 else 2)
        counts[d] += 1
    lines = [f"{counts[0]} {counts[1]} {counts[2]}"]
    surfs_sorted = sorted(surfs, key=lambda s: 0 if s[1] == s[2] else (1 if s[3] == s[4] else 2))
    for s in surfs_sorted:
        lines.append("   " + " ".join(str(x) for x in s))
    return "\n".join(lines)


def write_input(path: str, grid: str, scheme: dict, refs: Refs, ic: str,
                states: list[str], bcs: list[list[tuple]], iterations: int = 1) -> None:
    body = [
        "# generated by aither_gb300.cases",
        f"gridName: {grid}",
        f"equationSet: {scheme.get('equationSet', 'euler')}",
        f"turbulenceModel: {scheme.get('turbulenceModel', 'none')}",
        f"timeIntegration: {scheme.get('timeIntegration', 'implicitEuler')}",
        f"cflStart: {_fmt(scheme.get('cflStart', scheme['cfl']))}",
        f"cflStep: {_fmt(scheme.get('cflStep', 0.0))}",
        f"cflMax: {_fmt(scheme['cfl'])}",
        f"faceReconstruction: {scheme.get('faceReconstruction', 'thirdOrder')}",
        f"limiter: {scheme.get('limiter', 'minmod')}",
        f"inviscidFlux: {scheme.get('inviscidFlux', 'roe')}",
        f"iterations: {iterations}",
        f"outputFrequency: {max(iterations, 1)}",
        "outputVariables: <density, vel_x, vel_y, vel_z, pressure>",
        "fluids: <fluid(name=air; referenceMassFraction=1.0)>",
        f"referenceTemperature: {_fmt(refs.t_ref)}",
        f"referenceDensity: {_fmt(refs.r_ref)}",
        f"initialConditions: <{ic}>",
        f"matrixSolver: {scheme.get('matrixSolver', 'lusgs')}",
        f"matrixSweeps: {int(scheme.get('matrixSweeps', 1))}",
        "matrixRelaxation: 1.0",
    ]
    for key in ("multigridLevels", "multigridCycle"):
        if key in scheme:
            body.append(f"{key}: {scheme[key]}")
    for key in ("timeStep", "nonlinearIterations", "dualTimeCFL"):
        if key in scheme:
            body.append(f"{key}: {_fmt(scheme[key]) if isinstance(scheme[key], float) else scheme[key]}")
    if states:
        body.append("boundaryStates: <" + ",\n                 ".join(states) + ">")
    body.append(f"boundaryConditions: {len(bcs)}")
    for b in bcs:
        body.append(_bc_block(b))
    with open(path, "w") as f:
        f.write("\n".join(body) + "\n")


def isentropic_vortex(xc: np.ndarray, yc: np.ndarray, mach: float, p_inf: float,
                      t_inf: float, strength: float, radius: float, x0: float,
                      y0: float) -> tuple[np.ndarray, ...]:
    """Dimensional primitive state of an isentropic vortex in a uniform stream.

    Velocity perturbation (scaled by the freestream speed of sound)
      du = -b/(2 pi) (y-y0)/R exp((1-r^2)/2),  dv = b/(2 pi) (x-x0)/R exp((1-r^2)/2)
    temperature T = T_inf (1 - (g-1) b^2 / (8 g pi^2) exp(1-r^2)),
    density rho = rho_inf (T/T_inf)^(1/(g-1)), pressure p = rho R T,
    with r the distance from (x0, y0) divided by R.
    """
    a_inf = math.sqrt(GAMMA * R_AIR * t_inf)
    rho_inf = p_inf / (R_AIR * t_inf)
    dx = (xc - x0) / radius
    dy = (yc - y0) / radius
    r2 = dx * dx + dy * dy
    e = np.exp(0.5 * (1.0 - r2))
    u = mach * a_inf - a_inf * strength / (2 * math.pi) * dy * e
    v = a_inf * strength / (2 * math.pi) * dx * e
    w = np.zeros_like(u)
    tt = t_inf * (1.0 - (GAMMA - 1.0) * strength ** 2 / (8.0 * GAMMA * math.pi ** 2) * e * e)
    rho = rho_inf * (tt / t_inf) ** (1.0 / (GAMMA - 1.0))
    p = rho * R_AIR * tt
    return rho, u, v, w, p


def nondimensional_prim(rho, u, v, w, p, refs: Refs) -> np.ndarray:
    """Reference nondimensionalisation (src/inputStates.cpp:464-473)."""
    a = refs.a_ref
    return np.stack([rho / refs.r_ref, u / a, v / a, w / a, p / (refs.r_ref * a * a)], axis=-1)


def multigrid_keys(multigrid: tuple | None) -> dict:
    """multigridLevels / multigridCycle input keys from (levels, "V"|"W")."""
    if not multigrid:
        return {}
    return {"multigridLevels": int(multigrid[0]), "multigridCycle": multigrid[1]}


def time_keys(time: str = "implicitEuler", dt: float | None = None, nl: int = 1,
              dual_cfl: float | None = None) -> dict:
    """Input-file keys of the time integration: scheme (implicitEuler,
    crankNicholson, bdf2), global time step in seconds, nonlinear iterations
    per time step and dual-time CFL."""
    keys = {"timeIntegration": time, "nonlinearIterations": int(nl)}
    if dt is not None:
        keys["timeStep"] = float(dt)
    if dual_cfl is not None:
        keys["dualTimeCFL"] = float(dual_cfl)
    return keys


def vortex_box(outdir: str, ni: int = 64, nj: int = 32, nk: int = 8,
               lx: float = 10.0, ly: float = 5.0, lz: float = 1.25,
               cfl: float = 10.0, limiter: str = "minmod", name: str = "vortex_box",
               time: str = "implicitEuler", dt: float | None = None, nl: int = 1,
               dual_cfl: float | None = None):
    os.makedirs(outdir, exist_ok=True)
    nodes = box_nodes(ni, nj, nk, lx, ly, lz)
    write_plot3d(os.path.join(outdir, name + ".xyz"), [nodes])
    p_inf, t_inf, mach = 101325.0, 288.0, 0.5
    refs = Refs(t_ref=t_inf, r_ref=p_inf / (R_AIR * t_inf))
    a_inf = math.sqrt(GAMMA * R_AIR * t_inf)
    ic = (f"icState(tag=-1; pressure={_fmt(p_inf)}; density={_fmt(refs.r_ref)}; "
          f"velocity=[{_fmt(mach * a_inf)}, 0, 0])")
    states = [f"periodic(startTag=1; endTag=2; translation=[{_fmt(lx)}, 0, 0])",
              f"periodic(startTag=3; endTag=4; translation=[0, {_fmt(ly)}, 0])"]
    bcs = [[("periodic", 0, 0, 0, nj, 0, nk, 1),
            ("periodic", ni, ni, 0, nj, 0, nk, 2),
            ("periodic", 0, ni, 0, 0, 0, nk, 3),
            ("periodic", 0, ni, nj, nj, 0, nk, 4),
            ("slipWall", 0, ni, 0, nj, 0, 0, 5),
            ("slipWall", 0, ni, 0, nj, nk, nk, 6)]]
    inp = os.path.join(outdir, name + ".inp")
    write_input(inp, name, {"cfl": cfl, "limiter": limiter, **time_keys(time, dt, nl, dual_cfl)},
                refs, ic, states, bcs)
    cen = cell_centres(nodes)
    rho, u, v, w, p = isentropic_vortex(cen[0], cen[1], mach, p_inf, t_inf, 5.0, 1.0,
                                        lx / 2, ly / 2)
    prim = nondimensional_prim(rho, u, v, w, p, refs)  # (nk, nj, ni, 5)
    return inp, [np.ascontiguousarray(prim.reshape(-1))]


def bump_nodes(ni: int, nj: int, nk: int, height: float, length: float = 3.0,
               h_chan: float = 1.0, depth: float = 0.5) -> np.ndarray:
    """Channel [-1, length-1] x [0, h_chan] x [0, depth] with a sin^2 bump
    of the given height (fraction of the unit chord) on x in [0, 1]."""
    x = -1.0 + length * np.arange(ni + 1) / ni
    eta = np.arange(nj + 1) / nj
    z = depth * np.arange(nk + 1) / nk
    yb = np.where((x >= 0.0) & (x <= 1.0), height * np.sin(np.pi * x) ** 2, 0.0)
    X = np.broadcast_to(x[None, None, :], (nk + 1, nj + 1, ni + 1))
    Y = yb[None, None, :] + eta[None, :, None] * (h_chan - yb[None, None, :])
    Y = np.broadcast_to(Y, (nk + 1, nj + 1, ni + 1))
    Z = np.broadcast_to(z[:, None, None], (nk + 1, nj + 1, ni + 1))
    return np.ascontiguousarray(np.stack([X, Y, Z]))


def bump_channel(outdir: str, ni: int, nj: int, nk: int, height: float, mach: float,
                 cfl: float = 20.0, name: str = "bump", recon: str = "thirdOrder",
                 limiter: str = "minmod", flux: str = "roe", matrix_solver: str = "lusgs",
                 sweeps: int = 1, inflow: str = "characteristic",
                 outflow: str = "characteristic", back_pressure: float = 1.0,
                 nonreflecting: float | None = None, time: str = "implicitEuler",
                 dt: float | None = None, nl: int = 1, nr_outlet: float | None = None,
                 multigrid: tuple | None = None):
    """Inviscid channel over a sin^2 bump.  `multigrid` = (levels, cycle
    "V" or "W") adds the multigrid keys.  `nonreflecting` (a length in
    metres) makes the inlet nonreflecting with that lengthScale, `nr_outlet`
    the pressure outlet; time, dt and nl select the time integration.    Inflow at i = 0 and outflow at
    i = ni are characteristic far fields, or (inflow "stagnation") a
    stagnation inlet at the freestream's total pressure and temperature
    along +x, (inflow "inlet") the reference's inlet boundary with the
    freestream state, and (outflow "pressure") a pressure outlet at
    back_pressure times the freestream pressure."""
    os.makedirs(outdir, exist_ok=True)
    nodes = bump_nodes(ni, nj, nk, height)
    write_plot3d(os.path.join(outdir, name + ".xyz"), [nodes])
    p_inf, t_inf = 101325.0, 288.0
    refs = Refs(t_ref=t_inf, r_ref=p_inf / (R_AIR * t_inf))
    a_inf = math.sqrt(GAMMA * R_AIR * t_inf)
    vel = f"[{_fmt(mach * a_inf)}, 0, 0]"
    ic = f"icState(tag=-1; pressure={_fmt(p_inf)}; density={_fmt(refs.r_ref)}; velocity={vel})"
    states = [f"characteristic(tag=1; pressure={_fmt(p_inf)}; density={_fmt(refs.r_ref)}; "
              f"velocity={vel})"]
    in_bc, out_bc = ("characteristic", 0, 0, 0, nj, 0, nk, 1), ("characteristic", ni, ni, 0, nj,
                                                                  0, nk, 1)
    ratio = 1.0 + 0.5 * (GAMMA - 1.0) * mach * mach
    if inflow == "stagnation":
        p0, t0 = p_inf * ratio ** (GAMMA / (GAMMA - 1.0)), t_inf * ratio
        states.append(f"stagnationInlet(tag=3; p0={_fmt(p0)}; t0={_fmt(t0)}; "
                      "direction=[1, 0, 0])")
        in_bc = ("stagnationInlet", 0, 0, 0, nj, 0, nk, 3)
    elif inflow == "inlet":
        nr = (f"; nonreflecting=true; lengthScale={_fmt(nonreflecting)}"
              if nonreflecting else "")
        states.append(f"inlet(tag=3; pressure={_fmt(p_inf)}; density={_fmt(refs.r_ref)}; "
                      f"velocity={vel}{nr})")
        in_bc = ("inlet", 0, 0, 0, nj, 0, nk, 3)
    if outflow == "pressure":
        nro = (f"; nonreflecting=true; lengthScale={_fmt(nr_outlet)}" if nr_outlet else "")
        states.append(f"pressureOutlet(tag=4; pressure={_fmt(back_pressure * p_inf)}{nro})")
        out_bc = ("pressureOutlet", ni, ni, 0, nj, 0, nk, 4)
    bcs = [[in_bc, out_bc,
            ("slipWall", 0, ni, 0, 0, 0, nk, 2),
            ("slipWall", 0, ni, nj, nj, 0, nk, 2),
            ("slipWall", 0, ni, 0, nj, 0, 0, 2),
            ("slipWall", 0, ni, 0, nj, nk, nk, 2)]]
    inp = os.path.join(outdir, name + ".inp")
    write_input(inp, name, {"cfl": cfl, "limiter": limiter, "faceReconstruction": recon,
                            "inviscidFlux": flux, "matrixSolver": matrix_solver,
                            "matrixSweeps": sweeps, **time_keys(time, dt, nl),
                            **multigrid_keys(multigrid)},
                refs, ic, states, bcs)
    return inp, None


def wall_channel_nodes(ni: int, nj: int, nk: int, kind: str, param: float,
                       stretch: float = 1.0, length: float = 3.0, h_chan: float = 1.0,
                       depth: float = 0.5) -> np.ndarray:
    """Channel [-1, length-1] x [0, h_chan] x [0, depth] whose lower wall is
    a sin^2 bump of height `param` on x in [0, 1] (kind "bump") or a
    compression ramp of angle `param` degrees starting at x = 0 (kind
    "wedge"); wall-normal spacing grows geometrically by `stretch`."""
    x = -1.0 + length * np.arange(ni + 1) / ni
    if stretch == 1.0:
        eta = np.arange(nj + 1) / nj
    else:
        eta = (stretch ** np.arange(nj + 1) - 1.0) / (stretch ** nj - 1.0)
    z = depth * np.arange(nk + 1) / nk
    if kind == "bump":
        yb = np.where((x >= 0.0) & (x <= 1.0), param * np.sin(np.pi * x) ** 2, 0.0)
    else:
        yb = np.where(x > 0.0, x * math.tan(math.radians(param)), 0.0)
        yb = np.minimum(yb, 0.15 * h_chan)
    X = np.broadcast_to(x[None, None, :], (nk + 1, nj + 1, ni + 1))
    Y = yb[None, None, :] + eta[None, :, None] * (h_chan - yb[None, None, :])
    Y = np.broadcast_to(Y, (nk + 1, nj + 1, ni + 1))
    Z = np.broadcast_to(z[:, None, None], (nk + 1, nj + 1, ni + 1))
    return np.ascontiguousarray(np.stack([X, Y, Z]))


def wall_channel(outdir: str, ni: int, nj: int, nk: int, kind: str, param: float,
                 mach: float, alpha: float = 0.0, viscous: bool = False,
                 reynolds: float = 1e5, stretch: float = 1.0, cfl: float = 20.0,
                 name: str = "chan", precision_note: str = "", rans: bool = False,
                 tint: float = 0.001, vratio: float = 10.0, inflow: str = "characteristic",
                 outflow: str = "characteristic", back_pressure: float = 1.0,
                 nr_outlet: float | None = None):
    """Bump or wedge channel with free-stream Mach `mach` at angle of attack
    `alpha` (degrees, in the x-y plane); characteristic in- and outflow
    (or a stagnation inlet at the free stream's total state and a pressure
    outlet at back_pressure times its pressure),
    slip upper and side walls; the lower wall is a slip wall (Euler) or an
    adiabatic viscous wall (laminar Navier-Stokes, or SST-2003 RANS with
    `rans`; density from Re based on the unit chord and Sutherland's
    viscosity)."""
    viscous = viscous or rans
    os.makedirs(outdir, exist_ok=True)
    nodes = wall_channel_nodes(ni, nj, nk, kind, param, stretch)
    write_plot3d(os.path.join(outdir, name + ".xyz"), [nodes])
    t_inf = 288.0
    a_inf = math.sqrt(GAMMA * R_AIR * t_inf)
    u_inf = mach * a_inf
    if viscous:
        rho_inf = reynolds * sutherland_mu(t_inf) / u_inf
    else:
        rho_inf = 101325.0 / (R_AIR * t_inf)
    p_inf = rho_inf * R_AIR * t_inf
    refs = Refs(t_ref=t_inf, r_ref=rho_inf)
    ca, sa = math.cos(math.radians(alpha)), math.sin(math.radians(alpha))
    vel = f"[{_fmt(u_inf * ca)}, {_fmt(u_inf * sa)}, 0]"
    turb = f"; turbulenceIntensity={_fmt(tint)}; eddyViscosityRatio={_fmt(vratio)}" if rans else ""
    ic = (f"icState(tag=-1; pressure={_fmt(p_inf)}; density={_fmt(rho_inf)}; velocity={vel}"
          f"{turb})")
    states = [f"characteristic(tag=1; pressure={_fmt(p_inf)}; density={_fmt(rho_inf)}; "
              f"velocity={vel}{turb})"]
    lower = ("slipWall", 0, ni, 0, 0, 0, nk, 2)
    if viscous:
        states.append("viscousWall(tag=3)")
        lower = ("viscousWall", 0, ni, 0, 0, 0, nk, 3)
    in_bc, out_bc = ("characteristic", 0, 0, 0, nj, 0, nk, 1), ("characteristic", ni, ni, 0, nj,
                                                                  0, nk, 1)
    ratio = 1.0 + 0.5 * (GAMMA - 1.0) * mach * mach
    if inflow == "stagnation":
        p0, t0 = p_inf * ratio ** (GAMMA / (GAMMA - 1.0)), t_inf * ratio
        states.append(f"stagnationInlet(tag=5; p0={_fmt(p0)}; t0={_fmt(t0)}; "
                      f"direction=[{_fmt(ca)}, {_fmt(sa)}, 0]{turb})")
        in_bc = ("stagnationInlet", 0, 0, 0, nj, 0, nk, 5)
    if outflow == "pressure":
        nro = (f"; nonreflecting=true; lengthScale={_fmt(nr_outlet)}" if nr_outlet else "")
        states.append(f"pressureOutlet(tag=6; pressure={_fmt(back_pressure * p_inf)}{nro})")
        out_bc = ("pressureOutlet", ni, ni, 0, nj, 0, nk, 6)
    bcs = [[in_bc, out_bc,
            lower,
            ("slipWall", 0, ni, nj, nj, 0, nk, 2),
            ("slipWall", 0, ni, 0, nj, 0, 0, 2),
            ("slipWall", 0, ni, 0, nj, nk, nk, 2)]]
    inp = os.path.join(outdir, name + ".inp")
    scheme = {"cfl": cfl, "cflStart": 1.0, "cflStep": 1.0,
              "limiter": "vanAlbada" if viscous else "minmod",
              "equationSet": "rans" if rans else ("navierStokes" if viscous else "euler"),
              "turbulenceModel": "sst2003" if rans else "none"}
    write_input(inp, name, scheme, refs, ic, states, bcs)
    return inp, None


def served_specs(n: int, seed: int = 7, min_cells: int = 16_000, max_cells: int = 4_000_000,
                 log_mean: float = math.log(150_000.0), log_sigma: float = 1.2,
                 mix: str = "ns_sst"):
    """Request stream of the served workload: cell counts log-normal, clipped
    to [min_cells, max_cells], shaped ni : nj : nk = 4 : 2 : 1; bump or wedge
    lower wall; Mach U[0.3, 2.5]; angle of attack U[-4, 4] degrees.  mix
    "ns_sst": every second request SST-2003 RANS, the others laminar
    Navier-Stokes, both with a stretched wall-normal grid; "euler_ns": every
    second request laminar Navier-Stokes, the others Euler."""
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        cells = float(np.clip(math.exp(rng.normal(log_mean, log_sigma)), min_cells, max_cells))
        nk = max(2, int(round((cells / 8.0) ** (1.0 / 3.0))))
        nj = 2 * nk
        ni = max(8, int(round(cells / (nj * nk))))
        kind = "bump" if rng.uniform() < 0.5 else "wedge"
        param = float(rng.uniform(0.04, 0.10)) if kind == "bump" else float(rng.uniform(4, 10))
        out.append({"ni": ni, "nj": nj, "nk": nk, "kind": kind, "param": param,
                    "mach": float(rng.uniform(0.3, 2.5)), "alpha": float(rng.uniform(-4, 4)),
                    "viscous": mix == "ns_sst" or q % 2 == 1,
                    "rans": mix == "ns_sst" and q % 2 == 1,
                    # SST requests ramp to CFL 5: at 20 the supersonic ones
                    # turn nonphysical
                    "cfl": 5.0 if (mix == "ns_sst" and q % 2 == 1) else 20.0})
    return out


def bump_batch_specs(n: int = 64, seed: int = 2024, lo=(32, 32, 32), hi=(96, 64, 48)):
    """Sizes, bump heights and Mach numbers of the batched workload."""
    rng = np.random.default_rng(seed)
    specs = []
    for c in range(n):
        ni = int(rng.integers(lo[0], hi[0] + 1))
        nj = int(rng.integers(lo[1], hi[1] + 1))
        nk = int(rng.integers(lo[2], hi[2] + 1))
        h = float(rng.uniform(0.04, 0.10))
        m = float(rng.uniform(0.3, 0.85))
        specs.append((ni, nj, nk, h, m))
    return specs


def sutherland_mu(t: float, c1: float = 1.458e-6, s: float = 110.4) -> float:
    return c1 * t ** 1.5 / (t + s)


def plate_nodes(x0: float, x1: float, ni: int, nj: int, nk: int, dy0: float, ratio: float,
                dz: float, dy_max: float | None = None) -> np.ndarray:
    """Block on [x0, x1] in x, geometric wall-normal spacing from y=0
    (held at dy_max once it reaches it)."""
    x = x0 + (x1 - x0) * np.arange(ni + 1) / ni
    dy = dy0 * ratio ** np.arange(nj)
    if dy_max is not None:
        dy = np.minimum(dy, dy_max)
    y = np.concatenate([[0.0], np.cumsum(dy)])
    z = dz * np.arange(nk + 1)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return np.stack([X, Y, Z])


def flat_plate(outdir: str, ni: int = 128, nj: int = 64, nk: int = 2, dy0: float = 1e-5,
               ratio: float = 1.08, length: float = 1.0, mach: float = 0.3,
               reynolds: float = 1e5, t_inf: float = 288.0, cfl: float = 100.0,
               wall_t: float | None = None, limiter: str = "vanAlbada",
               name: str = "plate", matrix_solver: str = "lusgs", recon: str = "thirdOrder",
               sweeps: int = 1, rans: bool = False, tint: float = 0.001, vratio: float = 10.0,
               flux: str = "roe", nblocks: int = 2, dy_max: float | None = None,
               lead: float = 0.0, cfl_start: float | None = None, cfl_step: float = 0.0,
               wall_q: float | None = None, time: str = "implicitEuler",
               dt: float | None = None, nl: int = 1, dual_cfl: float | None = None,
               multigrid: tuple | None = None, turb_model: str = "sst2003"):
    """Laminar flat plate as two blocks of ni x nj x nk cells joined by an
    interblock connection at x = length/2; viscous wall at y = 0 (adiabatic,
    or isothermal at wall_t), characteristic far field on the other sides of
    the x-y plane, slip walls in z.  Freestream density from Re_L with
    Sutherland's law at t_inf; a wall heat flux wall_q (W/m^2) instead of an
    adiabatic or isothermal wall.  One block (nblocks=1) may start `lead` ahead
    of the leading edge, with a slip wall (symmetry plane) on y = 0 there.
    The CFL ramps from cfl_start by cfl_step per iteration up to cfl."""
    os.makedirs(outdir, exist_ok=True)
    dz = 0.02 * length
    b0 = plate_nodes(0.0, 0.5 * length, ni, nj, nk, dy0, ratio, dz, dy_max)
    b1 = plate_nodes(0.5 * length, length, ni, nj, nk, dy0, ratio, dz, dy_max)
    write_plot3d(os.path.join(outdir, name + ".xyz"), [b0, b1])
    a_inf = math.sqrt(GAMMA * R_AIR * t_inf)
    u_inf = mach * a_inf
    rho_inf = reynolds * sutherland_mu(t_inf) / (u_inf * length)
    p_inf = rho_inf * R_AIR * t_inf
    refs = Refs(t_ref=t_inf, r_ref=rho_inf)
    vel = f"[{_fmt(u_inf)}, 0, 0]"
    turb = f"; turbulenceIntensity={_fmt(tint)}; eddyViscosityRatio={_fmt(vratio)}" if rans else ""
    ic = (f"icState(tag=-1; pressure={_fmt(p_inf)}; density={_fmt(rho_inf)}; velocity={vel}"
          f"{turb})")
    wall = ("viscousWall(tag=2)" if wall_t is None and wall_q is None
            else f"viscousWall(tag=2; temperature={_fmt(wall_t)})" if wall_t is not None
            else f"viscousWall(tag=2; heatFlux={_fmt(wall_q)})")
    states = [f"characteristic(tag=1; pressure={_fmt(p_inf)}; density={_fmt(rho_inf)}; "
              f"velocity={vel}{turb})", wall]
    blk0 = [("characteristic", 0, 0, 0, nj, 0, nk, 1),
            ("interblock", ni, ni, 0, nj, 0, nk, 1001),
            ("viscousWall", 0, ni, 0, 0, 0, nk, 2),
            ("characteristic", 0, ni, nj, nj, 0, nk, 1),
            ("slipWall", 0, ni, 0, nj, 0, 0, 4),
            ("slipWall", 0, ni, 0, nj, nk, nk, 4)]
    blk1 = [("interblock", 0, 0, 0, nj, 0, nk, 2000),
            ("characteristic", ni, ni, 0, nj, 0, nk, 1),
            ("viscousWall", 0, ni, 0, 0, 0, nk, 2),
            ("characteristic", 0, ni, nj, nj, 0, nk, 1),
            ("slipWall", 0, ni, 0, nj, 0, 0, 4),
            ("slipWall", 0, ni, 0, nj, nk, nk, 4)]
    inp = os.path.join(outdir, name + ".inp")
    scheme = {"cfl": cfl, "cflStart": cfl if cfl_start is None else cfl_start,
              "cflStep": cfl_step,
              "limiter": limiter, "equationSet": "rans" if rans else "navierStokes",
              "turbulenceModel": turb_model if rans else "none", "inviscidFlux": flux,
              "matrixSolver": matrix_solver, "faceReconstruction": recon, "matrixSweeps": sweeps,
              **time_keys(time, dt, nl, dual_cfl), **multigrid_keys(multigrid)}
    if nblocks == 1:
        nodes = plate_nodes(-lead, length, ni, nj, nk, dy0, ratio, dz, dy_max)
        write_plot3d(os.path.join(outdir, name + ".xyz"), [nodes])
        # first node at or behind x = 0 starts the viscous wall
        i_le = int(np.searchsorted(nodes[0, 0, 0, :], -1e-12 * length)) if lead > 0 else 0
        bottom = [("viscousWall", i_le, ni, 0, 0, 0, nk, 2)]
        if i_le > 0:
            bottom.insert(0, ("slipWall", 0, i_le, 0, 0, 0, nk, 4))
        blk = [("characteristic", 0, 0, 0, nj, 0, nk, 1),
               ("characteristic", ni, ni, 0, nj, 0, nk, 1),
               *bottom,
               ("characteristic", 0, ni, nj, nj, 0, nk, 1),
               ("slipWall", 0, ni, 0, nj, 0, 0, 4),
               ("slipWall", 0, ni, 0, nj, nk, nk, 4)]
        write_input(inp, name, scheme, refs, ic, states, [blk])
    else:
        write_input(inp, name, scheme, refs, ic, states, [blk0, blk1])
    return inp, None


def turbulent_plate_dy0(reynolds: float, yplus: float = 1.0, length: float = 1.0) -> float:
    """Wall spacing for a target y+ at the end of a turbulent flat plate:
    skin friction from the 1/7-power correlation Cf = 0.026 Re^(-1/7),
    u_tau = U sqrt(Cf/2), y = y+ nu / u_tau."""
    cf = 0.026 * reynolds ** (-1.0 / 7.0)
    return yplus * length / (reynolds * math.sqrt(0.5 * cf))


def sst_plate(outdir: str, ni: int = 256, nj: int = 192, nk: int = 4, name: str = "sstplate",
              cfl: float = 50.0, **kw):
    """SST-2003 turbulent flat plate: one block of ni x nj x nk cells,
    Re_L = 5e6, Mach 0.2, turbulence intensity 0.1 %, eddy viscosity ratio
    10, first cell at y+ = 1, growth 1.1 up to 0.05 L, WENO, AUSM, block
    LU-SGS."""
    re = kw.pop("reynolds", 5e6)
    args = dict(ni=ni, nj=nj, nk=nk, dy0=turbulent_plate_dy0(re), ratio=1.1, mach=0.2,
                reynolds=re, cfl=cfl, name=name, matrix_solver="blusgs", recon="weno",
                limiter="none", flux="ausm", rans=True, tint=0.001, vratio=10.0, nblocks=1,
                dy_max=0.05)
    args.update(kw)
    return flat_plate(outdir, **args)


def set_output_keys(inp: str, iterations: int, variables: list | None = None,
                    output_freq: int | None = None, restart_freq: int = 0) -> None:
    """Rewrites the output controls of an input file written by this module:
    iterations, outputFrequency, restartFrequency and outputVariables."""
    with open(inp) as f:
        lines = f.read().split("\n")
    out = []
    for ln in lines:
        key = ln.split(":", 1)[0].strip()
        if key in ("iterations", "outputFrequency", "restartFrequency", "outputVariables"):
            continue
        out.append(ln)
    at = next(i for i, ln in enumerate(out) if ln.startswith("gridName:")) + 1
    extra = [f"iterations: {iterations}",
             f"outputFrequency: {output_freq if output_freq else iterations}"]
    if restart_freq:
        extra.append(f"restartFrequency: {restart_freq}")
    if variables:
        extra.append("outputVariables: <" + ", ".join(variables) + ">")
    out[at:at] = extra
    with open(inp, "w") as f:
        f.write("\n".join(out))


# ---------------------------------------------------------------------------
# two-block connections in every orientation

def _signed_perms():
    """The 24 right-handed signed permutations (ax, sg): index axis t of the
    second block runs along physical axis ax[t] (0 x, 1 y, 2 z) in direction
    sg[t] (a left-handed index system has negative cell volumes, which the
    reference rejects)."""
    import itertools
    out = []
    for ax in itertools.permutations(range(3)):
        parity = 1 if sum(1 for a in range(3) for b in range(a + 1, 3) if ax[a] > ax[b]) % 2 == 0 \
            else -1
        for sg in itertools.product((1, -1), repeat=3):
            if parity * sg[0] * sg[1] * sg[2] > 0:
                out.append((tuple(ax), tuple(sg)))
    return out


def patch_orientation(ax, sg) -> tuple:
    """In-plane orientation of the second block's connection patch relative
    to the first block's i-upper patch (in-plane axes j, k): whether the
    first in-plane axes are swapped, and the directions along which y and z
    run on the second block.  The 8 combinations are the reference's 8
    patch orientations (connection::Orientation)."""
    t_n = ax.index(0)
    d1 = (t_n + 1) % 3
    t_y, t_z = ax.index(1), ax.index(2)
    return (t_y != d1, sg[t_y], sg[t_z])


def orientation_set():
    """One signed permutation per in-plane orientation (8), cycling the
    second block's connecting direction through i, j, k and alternating its
    lower and upper surface, so that normal directions and surface sides
    vary too."""
    seen, picks = set(), []
    perms = _signed_perms()
    want_n = 0
    for _ in range(len(perms)):
        for ax, sg in perms:
            o = patch_orientation(ax, sg)
            t_n = ax.index(0)
            if o in seen or t_n != want_n % 3:
                continue
            if (sg[t_n] > 0) != (want_n % 2 == 0):
                continue
            seen.add(o)
            picks.append((ax, sg))
            want_n += 1
            break
        else:
            want_n += 1
        if len(picks) == 8:
            break
    return picks


def block_pair(outdir: str, orient: int = 0, na: int = 5, nb: int = 6, nc: int = 4,
               physics: str = "euler", cfl: float = 10.0, name: str = "pair", sweeps: int = 1):
    """Skewed box [0, 2] x [0, 1] x [0, 0.6] split at x = 1 into two blocks
    of na x nb x nc cells.  The first block's index axes are x, y, z; the
    second block's are the signed permutation orientation_set()[orient]
    of them, so its connecting surface may be any of its six surfaces and
    the patch may be swapped and reversed in plane.  Characteristic far
    field at x = 0 and x = 2, slip walls elsewhere.  Initial state: a
    free stream at Mach 0.4 along x with a vortex about an axis along z
    centred on the connection, a z-dependent cross-flow and a density
    perturbation (the field differs along every axis, so an index mapping
    error across the connection changes the result).

    physics: "euler" (MUSCL minmod, Roe, LU-SGS), "ns" (laminar
    Navier-Stokes, MUSCL van Albada, Roe, block LU-SGS with 2 sweeps) or
    "sst" (SST-2003 RANS, as "ns")."""
    os.makedirs(outdir, exist_ok=True)
    ax, sg = orientation_set()[orient]
    # global node array, 2 na cells along x; smooth stretching and a skew so
    # that face areas and widths vary
    xi = np.arange(2 * na + 1) / (2 * na)
    eta = np.arange(nb + 1) / nb
    zeta = np.arange(nc + 1) / nc
    Z, Y, X = np.meshgrid(zeta, eta, xi, indexing="ij")
    x = 2.0 * X
    y = Y + 0.08 * np.sin(np.pi * Y) * (X - 0.5)
    z = 0.6 * Z
    x = x + 0.06 * Y * Z + 0.04 * np.sin(np.pi * Z) * Y
    G = np.ascontiguousarray(np.stack([x, y, z]))
    A = np.ascontiguousarray(G[:, :, :, : na + 1])
    Bg = G[:, :, :, na:]
    arr_of = {0: 3, 1: 2, 2: 1}  # physical axis -> array axis of (c, z, y, x)
    B = np.transpose(Bg, (0, arr_of[ax[2]], arr_of[ax[1]], arr_of[ax[0]]))
    for t in range(3):
        if sg[t] < 0:
            B = np.flip(B, axis=3 - t)
    B = np.ascontiguousarray(B)
    write_plot3d(os.path.join(outdir, name + ".xyz"), [A, B])

    viscous = physics in ("ns", "sst")
    rans = physics == "sst"
    t_inf, mach = 288.0, 0.4
    a_inf = math.sqrt(GAMMA * R_AIR * t_inf)
    u_inf = mach * a_inf
    rho_inf = 2.0e4 * sutherland_mu(t_inf) / u_inf if viscous else 101325.0 / (R_AIR * t_inf)
    p_inf = rho_inf * R_AIR * t_inf
    refs = Refs(t_ref=t_inf, r_ref=rho_inf)
    vel = f"[{_fmt(u_inf)}, 0, 0]"
    turb = "; turbulenceIntensity=0.01; eddyViscosityRatio=10.0" if rans else ""
    ic = (f"icState(tag=-1; pressure={_fmt(p_inf)}; density={_fmt(rho_inf)}; velocity={vel}"
          f"{turb})")
    states = [f"characteristic(tag=1; pressure={_fmt(p_inf)}; density={_fmt(rho_inf)}; "
              f"velocity={vel}{turb})"]
    # surfaces: first block's i-upper joins the second block's surface that
    # lies on x = 1
    t_n = ax.index(0)
    surf_b = 2 * t_n + (1 if sg[t_n] > 0 else 2)
    dims_b = [B.shape[3] - 1, B.shape[2] - 1, B.shape[1] - 1]

    def surfaces(dims, conn_surf, conn_tag, far_surf):
        out = []
        for t in range(3):
            for upper in (0, 1):
                sid = 2 * t + 1 + upper
                r = [[0, dims[0]], [0, dims[1]], [0, dims[2]]]
                r[t] = [dims[t], dims[t]] if upper else [0, 0]
                if sid == conn_surf:
                    kind, tag = "interblock", conn_tag
                elif sid == far_surf:
                    kind, tag = "characteristic", 1
                else:
                    kind, tag = "slipWall", 2
                out.append((kind, r[0][0], r[0][1], r[1][0], r[1][1], r[2][0], r[2][1], tag))
        return out

    far_b = 2 * t_n + (2 if sg[t_n] > 0 else 1)
    bc_a = surfaces([na, nb, nc], 2, surf_b * 1000 + 1, 1)
    bc_b = surfaces(dims_b, surf_b, 2 * 1000 + 0, far_b)
    scheme = {"cfl": cfl, "limiter": "vanAlbada" if viscous else "minmod",
              "equationSet": "rans" if rans else ("navierStokes" if viscous else "euler"),
              "turbulenceModel": "sst2003" if rans else "none",
              "matrixSolver": "blusgs" if viscous else "lusgs",
              "matrixSweeps": 2 if viscous else sweeps}
    inp = os.path.join(outdir, name + ".inp")
    write_input(inp, name, scheme, refs, ic, states, [bc_a, bc_b])

    prims = []
    for nodes in (A, B):
        cen = cell_centres(nodes)
        xc, yc, zc = cen[0], cen[1], cen[2]
        rho, u, v, w, p = isentropic_vortex(xc, yc, mach, p_inf, t_inf, 1.5, 0.3, 1.0, 0.45)
        w = w + 0.05 * a_inf * np.sin(2.0 * np.pi * zc / 0.6) * np.exp(-((xc - 1.0) / 0.4) ** 2)
        rho = rho * (1.0 + 0.02 * zc / 0.6 + 0.01 * yc)
        prim = nondimensional_prim(rho, u, v, w, p, refs)
        if rans:
            kw = _farfield_turbulence(inp)
            prim = np.concatenate([prim, np.broadcast_to(kw, prim.shape[:3] + (2,))], axis=-1)
        prims.append(np.ascontiguousarray(prim.reshape(-1)))
    return inp, prims


def _farfield_turbulence(inp: str) -> np.ndarray:
    """Nondimensional (k, omega) of a solve's initial condition, as its
    setup forms them from the input's turbulence intensity and eddy
    viscosity ratio."""
    from ._lib import Setup
    s = Setup(inp)
    v = s.block_view(0)
    c = v.ng + (v.ni + 2 * v.ng) * (v.ng + (v.nj + 2 * v.ng) * v.ng)
    kw = np.array([v.state0[c * v.nv + 5], v.state0[c * v.nv + 6]])
    s.close()
    return kw
