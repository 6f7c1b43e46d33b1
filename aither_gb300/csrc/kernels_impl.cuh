// Kernel bodies (see kernels.cuh).  Included by one translation unit per
// arithmetic type so each is compiled with its own contraction setting.
#pragma once

#include "kernels.cuh"

namespace ath {

// ---------------------------------------------------------------------------
// ghost cells (FP64 state)

// ExtrapolateHoldMixture (src/ghostStates.cpp:693) for one species.
__device__ __forceinline__ Prim<double> ExtrapHold(const Prim<double> &bnd,
                                                   double factor,
                                                   const Prim<double> &in) {
  const double ghostRho = factor * bnd.rho - in.rho;
  if (ghostRho <= 0.0) return bnd;
  Prim<double> g;
  g.rho = fmax(ghostRho * (bnd.rho / bnd.rho), 0.0);
  g.u = factor * bnd.u - in.u;
  g.v = factor * bnd.v - in.v;
  g.w = factor * bnd.w - in.w;
  g.p = factor * bnd.p - in.p;
  return g;
}

template <typename T>
__global__ void k_ghost(Pools<T> P, const GhostOpDev *ops, int nops,
                        const int32_t *op_solve) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nops) return;
  const GhostOpDev op = ops[t];
  const int64_t n = P.ncell;
  Prim<double> in = LoadW<double>(P.W, n, op.src);
  Prim<double> g = in;
  if (op.type == ATH_BC_PERIODIC || op.type == ATH_BC_INTERBLOCK) {
    // plain copy of the partner's interior cell
  } else {
    const SolveDev sv = P.solves[op_solve[t]];
    const Gas<double> gas = GasOf<double>(sv);
    const double *fa = P.fa[op.dir];
    const double sgn = op.lower ? -1.0 : 1.0;
    const double nx = sgn * fa[op.face], ny = sgn * fa[n + op.face],
                 nz = sgn * fa[2 * n + op.face];
    if (op.type == ATH_BC_SLIP_WALL) {
      // reflect the interior velocity across the boundary face
      // (src/ghostStates.cpp:109-124)
      const double vn = Dot(in.u, in.v, in.w, nx, ny, nz);
      g.u = in.u - 2.0 * nx * vn;
      g.v = in.v - 2.0 * ny * vn;
      g.w = in.w - 2.0 * nz * vn;
    } else if (op.type == ATH_BC_CHARACTERISTIC) {
      // src/ghostStates.cpp:287-392
      const ath_bc_state bs = P.states[sv.state0 + op.state];
      Prim<double> fr;
      fr.rho = bs.rho;
      fr.u = bs.u;
      fr.v = bs.v;
      fr.w = bs.w;
      fr.p = bs.p;
      const double velIntNorm = Dot(in.u, in.v, in.w, nx, ny, nz);
      const double sosInt = SoS(in, gas);
      const double machInt = fabs(velIntNorm) / sosInt;
      if (machInt >= 1.0 && velIntNorm < 0.0) {
        g = fr;
      } else if (machInt >= 1.0 && velIntNorm >= 0.0) {
        // all characteristics leave: interior values
      } else if (machInt < 1.0 && velIntNorm < 0.0) {
        const double rhoSoSInt = in.rho * sosInt;
        const double dvx = fr.u - in.u, dvy = fr.v - in.v, dvz = fr.w - in.w;
        g.p = 0.5 * (fr.p + in.p - rhoSoSInt * Dot(nx, ny, nz, dvx, dvy, dvz));
        const double deltaPressure = fr.p - g.p;
        const double rho = fr.rho - deltaPressure / (sosInt * sosInt);
        g.rho = rho * (fr.rho / fr.rho);
        g.u = fr.u - nx * deltaPressure / rhoSoSInt;
        g.v = fr.v - ny * deltaPressure / rhoSoSInt;
        g.w = fr.w - nz * deltaPressure / rhoSoSInt;
      } else {
        const double rhoSoSInt = in.rho * sosInt;
        const double deltaPressure = in.p - fr.p;
        const double rho = in.rho - deltaPressure / (sosInt * sosInt);
        g.rho = rho * (in.rho / in.rho);
        g.u = in.u + nx * deltaPressure / rhoSoSInt;
        g.v = in.v + ny * deltaPressure / rhoSoSInt;
        g.w = in.w + nz * deltaPressure / rhoSoSInt;
        g.p = fr.p;
      }
      g = ExtrapHold(g, 2.0, in);
      if (op.layer > 1) g = ExtrapHold(g, (double)op.layer, in);
    } else if (op.type == ATH_BC_SUPERSONIC_INFLOW) {
      const ath_bc_state bs = P.states[sv.state0 + op.state];
      g.rho = bs.rho;
      g.u = bs.u;
      g.v = bs.v;
      g.w = bs.w;
      g.p = bs.p;
    } else if (op.type == ATH_BC_SUPERSONIC_OUTFLOW) {
      if (op.layer > 1) {
        const double f = (double)op.layer;
        g.rho = f * in.rho - in.rho;
        g.u = f * in.u - in.u;
        g.v = f * in.v - in.v;
        g.w = f * in.w - in.w;
        g.p = f * in.p - in.p;
      }
    }
  }
  P.W[op.dst] = g.rho;
  P.W[n + op.dst] = g.u;
  P.W[2 * n + op.dst] = g.v;
  P.W[3 * n + op.dst] = g.w;
  P.W[4 * n + op.dst] = g.p;
}

// ---------------------------------------------------------------------------
// face fluxes
template <typename T, int D>
__global__ void __launch_bounds__(kCta) k_face(Pools<T> P, const int32_t *list,
                                               const int32_t *cta_block) {
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  if (c < 0) return;
  const BlockDev b = P.blocks[cta_block[blockIdx.x]];
  const SolveDev sv = P.solves[b.solve];
  const Gas<T> g = GasOf<T>(sv);
  const int64_t n = P.ncell;
  const int64_t s = StrideOf(b, D);
  const double *wd = P.width[D];
  const Prim<T> wm1 = LoadW<T>(P.W, n, c - s);
  const Prim<T> w0 = LoadW<T>(P.W, n, c);
  Prim<T> L, R;
  if (sv.recon == ATH_RECON_CONSTANT) {
    L = wm1;
    R = w0;
  } else if (sv.recon == ATH_RECON_MUSCL) {
    const Prim<T> wm2 = LoadW<T>(P.W, n, c - 2 * s);
    const Prim<T> wp1 = LoadW<T>(P.W, n, c + s);
    const T xm2 = (T)wd[c - 2 * s], xm1 = (T)wd[c - s], x0 = (T)wd[c], xp1 = (T)wd[c + s];
    const T kappa = (T)sv.kappa;
    // lower side: upwind2 = c-2, upwind1 = c-1, downwind = c
    L = Muscl(wm2, wm1, w0, xm2, xm1, x0, kappa, sv.limiter);
    // upper side: upwind2 = c+1, upwind1 = c, downwind = c-1
    R = Muscl(wp1, w0, wm1, xp1, x0, xm1, kappa, sv.limiter);
  } else {
    const Prim<T> wm3 = LoadW<T>(P.W, n, c - 3 * s);
    const Prim<T> wm2 = LoadW<T>(P.W, n, c - 2 * s);
    const Prim<T> wp1 = LoadW<T>(P.W, n, c + s);
    const Prim<T> wp2 = LoadW<T>(P.W, n, c + 2 * s);
    const bool z = sv.recon == ATH_RECON_WENOZ;
    const T wl[5] = {(T)wd[c - 3 * s], (T)wd[c - 2 * s], (T)wd[c - s], (T)wd[c],
                     (T)wd[c + s]};
    const T wu[5] = {(T)wd[c + 2 * s], (T)wd[c + s], (T)wd[c], (T)wd[c - s],
                     (T)wd[c - 2 * s]};
    L = Weno(wm3, wm2, wm1, w0, wp1, wl, z);
    R = Weno(wp2, wp1, w0, wm1, wm2, wu, z);
  }
  const double *fa = P.fa[D];
  const T nx = (T)fa[c], ny = (T)fa[n + c], nz = (T)fa[2 * n + c],
          mag = (T)fa[3 * n + c];
  T f[5];
  if (sv.flux == ATH_FLUX_AUSM)
    AusmFlux(L, R, g, nx, ny, nz, f);
  else
    RoeFlux(L, R, g, nx, ny, nz, f);
  T *out = P.flux[D];
#pragma unroll
  for (int v = 0; v < 5; ++v) out[v * n + c] = f[v] * mag;
}

// ---------------------------------------------------------------------------
// residual assembly + spectral radius + dt + diagonal
template <typename T>
__global__ void __launch_bounds__(kCta) k_cell(Pools<T> P, const int32_t *list,
                                               const int32_t *cta_block) {
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  if (c < 0) return;
  const BlockDev b = P.blocks[cta_block[blockIdx.x]];
  const SolveDev sv = P.solves[b.solve];
  const int64_t n = P.ncell;
  const int64_t st[3] = {1, (int64_t)b.NI, (int64_t)b.NI * b.NJ};
  // R = 0 - Fi(lo) + Fi(hi) - Fj(lo) + Fj(hi) - Fk(lo) + Fk(hi), each face
  // term rounded in this order (src/procBlock.cpp:447-463)
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double r = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const T *F = P.flux[d] + v * n;
      r = r - (double)F[c];
      r = r + (double)F[c + st[d]];
    }
    P.R[v * n + c] = r;
  }
  // inviscid cell spectral radius, summed i, j, k
  const Gas<T> g = GasOf<T>(sv);
  const Prim<T> w = LoadW<T>(P.W, n, c);
  double lam = 0.0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double *fa = P.fa[d];
    const int64_t u = c + st[d];
    lam = lam + (double)InvCellSpecRad(w, g, (T)fa[c], (T)fa[n + c], (T)fa[2 * n + c],
                                       (T)fa[3 * n + c], (T)fa[u], (T)fa[n + u],
                                       (T)fa[2 * n + u], (T)fa[3 * n + u]);
  }
  P.lam[c] = lam;
  // local time step and diagonal: A = lam*relax + V(1+zeta)/(dt theta)
  const double cfl = P.cfl[b.solve];
  const double vol = P.vol[c];
  const double dt = cfl * (vol / lam);
  P.dt[c] = dt;
  const double a = lam * sv.relax + (vol * (1.0 + sv.zeta)) / (dt * sv.theta);
  // hyperplane-ordered copies for the sweeps
  const int64_t q = P.qpos[c];
  const int64_t nq = P.nq;
  P.Ainvq[q] = (T)(1.0 / a);
  P.Aq[q] = (T)a;
  P.Wq[q] = w.rho;
  P.Wq[nq + q] = w.u;
  P.Wq[2 * nq + q] = w.v;
  P.Wq[3 * nq + q] = w.w;
  P.Wq[4 * nq + q] = w.p;
#pragma unroll
  for (int v = 0; v < 5; ++v) P.Rq[v * nq + q] = (T)P.R[v * n + c];
}

// ---------------------------------------------------------------------------
// Off-diagonal sum of one cell: lower neighbours with the "positive" sign
// (procBlock::ImplicitLower) or upper neighbours with the negative sign
// (ImplicitUpper), accumulated i, j, k from zero.
template <typename T>
__device__ __forceinline__ void OffDiagSum(const Pools<T> &P, const Gas<T> &g, int64_t q,
                                           bool lower, T acc[5]) {
  const int64_t nq = P.nq, ng = P.nghost, n = P.ncell;
  const T *face = lower ? P.face_lo : P.face_hi;
  const int32_t *nbq = P.nbq + (lower ? 0 : 3 * nq);
#pragma unroll
  for (int v = 0; v < 5; ++v) acc[v] = T(0);
#pragma unroll 1
  for (int d = 0; d < 3; ++d) {
    const int32_t nb = nbq[d * nq + q];
    if (nb == -1) continue;
    Prim<T> s;
    T du[5];
    if (nb >= 0) {
      s.rho = P.Wq[nb];
      s.u = P.Wq[nq + nb];
      s.v = P.Wq[2 * nq + nb];
      s.w = P.Wq[3 * nq + nb];
      s.p = P.Wq[4 * nq + nb];
#pragma unroll
      for (int v = 0; v < 5; ++v) du[v] = P.dUq[v * nq + nb];
    } else {
      const int64_t slot = -(int64_t)nb - 2;
      s = LoadW<T>(P.W, n, P.ghost_cell[slot]);
#pragma unroll
      for (int v = 0; v < 5; ++v) du[v] = P.dUg[v * ng + slot];
    }
    const T *f = face + (int64_t)d * 4 * nq;
    T o[5];
    ScalarOffDiag(s, du, g, f[q], f[nq + q], f[2 * nq + q], f[3 * nq + q], lower, o);
#pragma unroll
    for (int v = 0; v < 5; ++v) acc[v] = acc[v] + o[v];
  }
}

// ---------------------------------------------------------------------------
// LU-SGS hyperplane sweep on the q-ordered working set
template <typename T>
__global__ void __launch_bounds__(128) k_sweep(Pools<T> P, const int2 *items, int n_items,
                                               int forward) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_items) return;
  const int2 it = items[t];
  const int64_t q = it.x;
  const BlockDev b = P.blocks[it.y];
  const SolveDev sv = P.solves[b.solve];
  const Gas<T> g = GasOf<T>(sv);
  const int64_t nq = P.nq;
  T acc[5];
  OffDiagSum(P, g, q, forward != 0, acc);
  const T ainv = P.Ainvq[q];
  if (forward) {
    const T thetaInv = (T)(1.0 / sv.theta);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const T bv = -thetaInv * P.Rq[v * nq + q];
      P.dUq[v * nq + q] = (bv + acc[v]) * ainv;
    }
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const T xold = P.dUq[v * nq + q];
      P.dUq[v * nq + q] = xold - acc[v] * ainv;
    }
  }
}

template <typename T>
__global__ void k_conn_du(Pools<T> P) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P.nghost) return;
  const int64_t src = P.ghost_src[t];
#pragma unroll
  for (int v = 0; v < 5; ++v) P.dUg[v * P.nghost + t] = P.dUq[v * P.nq + src];
}

// ---------------------------------------------------------------------------
// conserved update and partial norms
template <typename T>
__global__ void __launch_bounds__(kCta) k_update(Pools<T> P, const int32_t *list,
                                                 const int32_t *cta_block,
                                                 const int32_t *cta_pos0,
                                                 NormPartial *partials) {
  __shared__ double s_l2[kCta / 32][kNv];
  __shared__ double s_max[kCta / 32];
  __shared__ int64_t s_pos[kCta / 32];
  __shared__ int32_t s_bad[kCta / 32];
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  const int64_t n = P.ncell;
  double l2[kNv] = {0, 0, 0, 0, 0};
  double mx = 0.0;
  int64_t mpos = INT64_MAX;
  int bad = 0;
  if (c >= 0) {
    const BlockDev b = P.blocks[cta_block[blockIdx.x]];
    const SolveDev sv = P.solves[b.solve];
    const Gas<double> g = GasOf<double>(sv);
    const Prim<double> w = LoadW<double>(P.W, n, c);
    double du[5];
    const int64_t q = P.qpos[c];
#pragma unroll
    for (int v = 0; v < 5; ++v) du[v] = (double)P.dUq[v * P.nq + q];
    const Prim<double> u = UpdateWithCons(w, g, du);
    if (!(u.rho > 0.0) || !(u.p > 0.0) || !isfinite(u.u) || !isfinite(u.v) ||
        !isfinite(u.w))
      bad = 1;
    P.W[c] = u.rho;
    P.W[n + c] = u.u;
    P.W[2 * n + c] = u.v;
    P.W[3 * n + c] = u.w;
    P.W[4 * n + c] = u.p;
    const int64_t pos0 = (int64_t)cta_pos0[blockIdx.x] + threadIdx.x;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double r = P.R[v * n + c];
      l2[v] = r * r;
      // L-infinity follows the reference's signed comparison
      // (procBlock::UpdateBlock): a new maximum replaces the old one only
      // when strictly larger; ties keep the first in loop order
      if (r > mx) {
        mx = r;
        mpos = pos0 * kNv + v;
      }
    }
  }
  // warp reduction; the sum order is fixed, so results are reproducible
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int v = 0; v < kNv; ++v) l2[v] += __shfl_down_sync(0xffffffffu, l2[v], off);
    const double om = __shfl_down_sync(0xffffffffu, mx, off);
    const int64_t op = __shfl_down_sync(0xffffffffu, mpos, off);
    if (om > mx || (om == mx && op < mpos)) {
      mx = om;
      mpos = op;
    }
    bad |= __shfl_down_sync(0xffffffffu, bad, off);
  }
  if (lane == 0) {
#pragma unroll
    for (int v = 0; v < kNv; ++v) s_l2[warp][v] = l2[v];
    s_max[warp] = mx;
    s_pos[warp] = mpos;
    s_bad[warp] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    NormPartial p;
    for (int v = 0; v < kNv; ++v) p.l2[v] = 0.0;
    p.linf = 0.0;
    p.linf_pos = INT64_MAX;
    p.bad = 0;
    for (int w = 0; w < kCta / 32; ++w) {
      for (int v = 0; v < kNv; ++v) p.l2[v] += s_l2[w][v];
      if (s_max[w] > p.linf || (s_max[w] == p.linf && s_pos[w] < p.linf_pos)) {
        p.linf = s_max[w];
        p.linf_pos = s_pos[w];
      }
      p.bad |= s_bad[w];
    }
    p.linf_cell = 0;
    p.linf_eqn = 0;
    p.pad = 0;
    partials[blockIdx.x] = p;
  }
}

// ---------------------------------------------------------------------------
// logged matrix residual
template <typename T>
__global__ void __launch_bounds__(kCta) k_matres(Pools<T> P, const int32_t *list,
                                                 const int32_t *cta_block,
                                                 double *mres_partials) {
  __shared__ double s_sum[kCta / 32];
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  double sum = 0.0;
  if (c >= 0) {
    const BlockDev b = P.blocks[cta_block[blockIdx.x]];
    const SolveDev sv = P.solves[b.solve];
    const Gas<T> g = GasOf<T>(sv);
    const int64_t q = P.qpos[c], nq = P.nq;
    T L[5], U[5];
    OffDiagSum(P, g, q, true, L);
    OffDiagSum(P, g, q, false, U);
    const T thetaInv = (T)(1.0 / sv.theta);
    const T a = P.Aq[q];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const T off = L[v] - U[v];
      const T bv = -thetaInv * P.Rq[v * nq + q];
      const T axmb = P.dUq[v * nq + q] * a - off - bv;
      const double r = 0.0 - (double)axmb;
      sum += r * r;
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, off);
  if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kCta / 32; ++w) t += s_sum[w];
    mres_partials[blockIdx.x] = t;
  }
}

// ---------------------------------------------------------------------------
template <typename T>
void Launch<T>::MatRes(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                       double *mres_partials, int ncta, cudaStream_t s) {
  if (ncta > 0) k_matres<T><<<ncta, kCta, 0, s>>>(P, list, cta_block, mres_partials);
}
template <typename T>
void Launch<T>::Ghost(const Pools<T> &P, const GhostOpDev *ops, int nops,
                      const int32_t *op_solve, cudaStream_t s) {
  if (nops > 0) k_ghost<T><<<(nops + 127) / 128, 128, 0, s>>>(P, ops, nops, op_solve);
}
template <typename T>
void Launch<T>::Face(int d, const Pools<T> &P, const int32_t *list,
                     const int32_t *cta_block, int ncta, cudaStream_t s) {
  if (ncta <= 0) return;
  if (d == 0) k_face<T, 0><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  else if (d == 1) k_face<T, 1><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  else k_face<T, 2><<<ncta, kCta, 0, s>>>(P, list, cta_block);
}
template <typename T>
void Launch<T>::Cell(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                     int ncta, cudaStream_t s) {
  if (ncta > 0) k_cell<T><<<ncta, kCta, 0, s>>>(P, list, cta_block);
}
template <typename T>
void Launch<T>::Sweep(const Pools<T> &P, const int2 *items, int n, int forward,
                      cudaStream_t s) {
  if (n > 0) k_sweep<T><<<(n + 127) / 128, 128, 0, s>>>(P, items, n, forward);
}
template <typename T>
void Launch<T>::ConnDu(const Pools<T> &P, cudaStream_t s) {
  if (P.nghost > 0) k_conn_du<T><<<(unsigned)((P.nghost + 127) / 128), 128, 0, s>>>(P);
}
template <typename T>
void Launch<T>::Update(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                       const int32_t *cta_pos0, NormPartial *partials, int ncta,
                       cudaStream_t s) {
  if (ncta > 0) k_update<T><<<ncta, kCta, 0, s>>>(P, list, cta_block, cta_pos0, partials);
}

}  // namespace ath
