// Kernel bodies (see kernels.cuh).  Included by one translation unit per
// arithmetic type so each is compiled with its own contraction setting.
#pragma once

#include <cfloat>
#include <cooperative_groups.h>
#include <type_traits>

#include "block.cuh"
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

// SST-2003 constants (turbKWSst, include/turbulence.hpp:489-501) and the
// turbulence floors (turbModel::TkeMin / OmegaMin, :63-64)
constexpr double kSstBetaStar = 0.09, kSstSigmaK1 = 0.85, kSstSigmaK2 = 1.0;
constexpr double kSstSigmaW1 = 0.5, kSstSigmaW2 = 0.856, kSstBeta1 = 0.075;
constexpr double kSstBeta2 = 0.0828, kSstGamma2 = 0.44, kSstA1 = 0.31;
constexpr double kSstProd2Dest = 10.0, kTurbMin = 1.0e-20;
__device__ __forceinline__ double SstGamma1() { return 5.0 / 9.0; }
// std::max / std::min
template <typename T>
__device__ __forceinline__ T CMax(T a, T b) { return (a < b) ? b : a; }
template <typename T>
__device__ __forceinline__ T CMin(T a, T b) { return (b < a) ? b : a; }
// turbKWSst::BlendedCoeff (src/turbulence.cpp:598)
template <typename T>
__device__ __forceinline__ T Blended(T c1, T c2, T f1) { return f1 * c1 + (T(1) - f1) * c2; }

// tensor DoubleDotTrans (include/tensor.hpp:353)
__device__ __forceinline__ double DDot(const double *a, const double *b) {
  double s = 0.0;
#pragma unroll
  for (int e = 0; e < 9; ++e) s += a[e] * b[e];
  return s;
}

// turbKWSst::EddyViscAndBlending (src/turbulence.cpp:668) with Alpha1-3,
// CDkw, F1, F2 and EddyVisc (:573-634, include/turbulence.hpp:529); T is
// double on the FP64 path, float for the mixed path's viscous faces
template <typename T>
__device__ __forceinline__ void SstEddyVisc(const Prim<T> &w, const T kw[2], const T vg[9],
                                            const T kg[3], const T wg[3], T mu, T wd, T scale,
                                            T &mut, T &f1, T &f2) {
  const T k = kw[0], om = kw[1], rho = w.rho;
  const T a1 = scale * sqrt(k) / (T(kSstBetaStar) * om * (wd + T(1.0e-30)));
  const T a2 = scale * scale * T(500.0) * mu / ((wd + T(1.0e-30)) * (wd + T(1.0e-30)) * rho * om);
  const T cd = CMax(T(2.0) * rho * T(kSstSigmaW2) / om * Dot(kg[0], kg[1], kg[2], wg[0], wg[1],
                                                              wg[2]),
                    T(1.0e-10));
  const T a3 = T(4.0) * rho * T(kSstSigmaW2) * k / (cd * (wd + T(1.0e-30)) * (wd + T(1.0e-30)));
  f1 = tanh(pow(CMin(CMax(a1, a2), a3), T(4.0)));
  const T arg2 = CMax(T(2.0) * a1, a2);
  f2 = tanh(arg2 * arg2);
  T S[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int q = 0; q < 3; ++q) S[r * 3 + q] = T(0.5) * (vg[r * 3 + q] + vg[q * 3 + r]);
  T ss = T(0);
#pragma unroll
  for (int e = 0; e < 9; ++e) ss += S[e] * S[e];
  const T msr = sqrt(T(2.0) * ss);
  mut = rho * T(kSstA1) * k / CMax(T(kSstA1) * om, scale * msr * f2);
}

// turbKWSst::CalcTurbSrc (src/turbulence.cpp:637) with the Boussinesq
// Reynolds stress (turbModel::ReynoldsStressDDotVelGrad, :53); returns the
// blended beta of the source Jacobian
__device__ __forceinline__ double SstSource(const Prim<double> &w, const double kw[2],
                                            const double vg[9], const double kg[3],
                                            const double wg[3], double mut, double f1,
                                            double scale, double src[2]) {
  const double k = kw[0], om = kw[1], rho = w.rho;
  const double inv = 1.0 / scale;
  const double cd = CMax(2.0 * rho * kSstSigmaW2 / om * Dot(kg[0], kg[1], kg[2], wg[0], wg[1],
                                                            wg[2]),
                         1.0e-10);
  const double gamma = Blended(SstGamma1(), kSstGamma2, f1);
  const double beta = Blended(kSstBeta1, kSstBeta2, f1);
  const double tkeDest = inv * kSstBetaStar * (rho * k * om * 1.0);
  const double omgDest = inv * beta * (rho * om * om);
  const double lambda = 0.0 - (2.0 / 3.0) * mut;
  const double tr = vg[0] + vg[4] + vg[8];
  const double c23 = 2.0 / 3.0 * rho * k;
  double tau[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const double I = (r == q) ? 1.0 : 0.0;
      tau[r * 3 + q] = (I * (lambda * tr) + (vg[r * 3 + q] + vg[q * 3 + r]) * mut) - I * c23;
    }
  double tkeProd = CMin(scale * DDot(tau, vg), kSstProd2Dest * tkeDest);
  tkeProd = CMax(tkeProd, 0.0);
  double omgProd = gamma * rho / mut * tkeProd;
  omgProd = CMax(omgProd, 0.0);
  const double omgCd = scale * (1.0 - f1) * cd;
  src[0] = tkeProd - tkeDest;
  src[1] = omgProd - omgDest + omgCd;
  return beta;
}

// x^3 rounded once: x^2 and x^2 x as exact two-term products (FMA error-free
// transformation, Dekker's TwoProduct), summed with the error terms; the
// host's pow(x, 3.0) in the reference rounds the exact cube once too
__device__ __forceinline__ double Cube(double x) {
  const double h = x * x;
  const double l = fma(x, x, -h);
  const double c = h * x;
  const double e = fma(h, x, -c);
  return c + fma(l, x, e);
}

// Wilcox k-omega 2006 constants (turbKWWilcox, include/turbulence.hpp:391-398)
constexpr double kWkGamma = 0.52, kWkBetaStar = 0.09, kWkSigma = 0.5, kWkSigmaStar = 0.6;
constexpr double kWkSigmaD0 = 0.125, kWkBeta0 = 0.0708, kWkClim = 0.875;
// turbModel::TurbPrandtlNumber of the solve's model
__device__ __forceinline__ double PrtOf(const SolveDev &sv) { return sv.wilcox ? 8.0 / 9.0 : 0.9; }

// turbKWWilcox::EddyVisc with OmegaTilda (src/turbulence.cpp:270,339): rho k
// over omega limited below by clim sqrt(2 S^:S^ / beta*), S^ the traceless
// strain rate of the face velocity gradient
__device__ __forceinline__ double WkEddyVisc(const Prim<double> &w, const double kw[2],
                                             const double vg[9], double scale) {
  const double tr = (vg[0] + vg[4]) + vg[8];
  const double c = 1.0 / 3.0 * tr;
  double sh[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int q = 0; q < 3; ++q)
      sh[r * 3 + q] = 0.5 * (vg[r * 3 + q] + vg[q * 3 + r]) - c * (r == q ? 1.0 : 0.0);
  const double omt = CMax(kw[1], scale * kWkClim * sqrt(2.0 * DDot(sh, sh) / kWkBetaStar));
  return w.rho * kw[0] / omt;
}

// turbKWWilcox::CalcTurbSrc (src/turbulence.cpp:359) with Beta / FBeta / Xw
// / StrainKI / SigmaD (:283-337): production (not limited by destruction),
// destruction with the vortex-stretching beta, and cross diffusion where
// grad k . grad omega > 0; returns beta for the source Jacobian
__device__ __forceinline__ double WkSource(const Prim<double> &w, const double kw[2],
                                           const double vg[9], const double kg[3],
                                           const double wg[3], double mut, double scale,
                                           double src[2]) {
  const double k = kw[0], om = kw[1], rho = w.rho;
  const double inv = 1.0 / scale;
  const double tkeDest = inv * kWkBetaStar * (rho * k * om * 1.0);
  const double tr = (vg[0] + vg[4]) + vg[8];
  double vo[9], skI[9], vv[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      vo[r * 3 + q] = 0.5 * (vg[r * 3 + q] - vg[q * 3 + r]);
      skI[r * 3 + q] = 0.5 * ((vg[r * 3 + q] + vg[q * 3 + r]) - tr * (r == q ? 1.0 : 0.0));
    }
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      double t = 0.0;
#pragma unroll
      for (int m = 0; m < 3; ++m) t += vo[r * 3 + m] * vo[m * 3 + q];
      vv[r * 3 + q] = t;
    }
  const double xw = fabs(DDot(vv, skI) / Cube(kWkBetaStar * om)) * Cube(scale);
  const double beta = kWkBeta0 * ((1.0 + 85.0 * xw) / (1.0 + 100.0 * xw));
  const double omgDest = inv * beta * (rho * om * om);
  const double lambda = 0.0 - (2.0 / 3.0) * mut;
  const double c23 = 2.0 / 3.0 * rho * k;
  double tau[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const double I = (r == q) ? 1.0 : 0.0;
      tau[r * 3 + q] = (I * (lambda * tr) + (vg[r * 3 + q] + vg[q * 3 + r]) * mut) - I * c23;
    }
  double tkeProd = scale * DDot(tau, vg);
  tkeProd = CMax(tkeProd, 0.0);
  double omgProd = kWkGamma * om / k * tkeProd;
  omgProd = CMax(omgProd, 0.0);
  const double kdw = ((0.0 + kg[0] * wg[0]) + kg[1] * wg[1]) + kg[2] * wg[2];
  const double sigd = kdw <= 0.0 ? 0.0 : kWkSigmaD0;
  const double omgCd = scale * sigd * (rho / om * kdw);
  src[0] = tkeProd - tkeDest;
  src[1] = omgProd - omgDest + omgCd;
  return beta;
}

// primitive::ApplyFarfieldTurbBC (src/primitive.cpp:83) + LimitTurb
__device__ __forceinline__ void FarfieldTurb(const Prim<double> &g, double vx, double vy,
                                             double vz, double tint, double ratio,
                                             const SolveDev &sv, const Gas<double> &gas,
                                             double kw[2]) {
  const double vmag = sqrt(vx * vx + vy * vy + vz * vz);
  kw[0] = 1.5 * pow(tint * vmag, 2.0);
  const double mu = SutherlandRatio(Temperature(g, gas), sv.t_ref, sv.mu_c1, sv.mu_s, sv.mu_ref);
  kw[1] = g.rho * kw[0] / (ratio * mu);
  kw[0] = CMax(kw[0], kTurbMin);
  kw[1] = CMax(kw[1], kTurbMin);
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
  // turbulence (RANS solves): copied unless the boundary sets it
  const bool rans = P.Wt != nullptr && P.solves[op_solve[t]].rans;
  double tin[2] = {0.0, 0.0}, gt[2] = {0.0, 0.0};
  if (rans) {
    tin[0] = P.Wt[op.src];
    tin[1] = P.Wt[n + op.src];
    gt[0] = tin[0];
    gt[1] = tin[1];
  }
  if (op.type == ATH_BC_PERIODIC || op.type == ATH_BC_INTERBLOCK || op.type == ATH_EDGE_COPY) {
    // plain copy of the partner's interior cell / of the adjacent ghost
  } else if (op.type == ATH_EDGE_AVG) {
    const Prim<double> o = LoadW<double>(P.W, n, op.src2);
    g.rho = 0.5 * (in.rho + o.rho);
    g.u = 0.5 * (in.u + o.u);
    g.v = 0.5 * (in.v + o.v);
    g.w = 0.5 * (in.w + o.w);
    g.p = 0.5 * (in.p + o.p);
    if (rans) {
      gt[0] = 0.5 * (tin[0] + P.Wt[op.src2]);
      gt[1] = 0.5 * (tin[1] + P.Wt[n + op.src2]);
    }
  } else if (op.type == ATH_EDGE_SLIP) {
    // slip-wall reflection of the adjacent ghost across a ghost-layer face
    const double *fa = P.fa[op.dir];
    const double sgn = op.lower ? -1.0 : 1.0;
    const double nx = sgn * fa[op.face], ny = sgn * fa[n + op.face],
                 nz = sgn * fa[2 * n + op.face];
    const double vn = Dot(in.u, in.v, in.w, nx, ny, nz);
    g.u = in.u - 2.0 * nx * vn;
    g.v = in.v - 2.0 * ny * vn;
    g.w = in.w - 2.0 * nz * vn;
  } else if (op.type == ATH_BC_VISCOUS_WALL) {
    // viscousWall, low-Re treatment (src/ghostStates.cpp:130-200): velocity
    // 2 u_wall - u; isothermal walls set the density from 2 T_wall - T
    const SolveDev sv = P.solves[op_solve[t]];
    const ath_bc_state bs = P.states[sv.state0 + op.state];
    g.u = 2.0 * bs.wall_u - in.u;
    g.v = 2.0 * bs.wall_v - in.v;
    g.w = 2.0 * bs.wall_w - in.w;
    if (bs.isothermal) {
      const Gas<double> gas = GasOf<double>(sv);
      const double tGhost = 2.0 * bs.wall_t - Temperature(in, gas);
      const double rho = g.p / ((0.0 + 1.0 * gas.r) * tGhost);
      g.rho = rho * (in.rho / in.rho);
    } else if (bs.heat_flux) {
      // constant heat flux, low-Re (src/ghostStates.cpp:230-241): the
      // temperature gradient q / kappa over twice the wall distance of the
      // wall-adjacent cell; kappa = EffectiveConductivity of the interior
      const Gas<double> gas = GasOf<double>(sv);
      const double t = Temperature(in, gas);
      const double kappa =
          SutherlandRatio(t, sv.t_ref, sv.k_c1, sv.k_s, sv.k_ref) * sv.visc_scale;
      const double tGhost = Temperature(in, gas) - bs.wall_q / kappa * 2.0 * P.wd[op.src2];
      const double rho = g.p / ((0.0 + 1.0 * gas.r) * tGhost);
      g.rho = rho * (in.rho / in.rho);
    }
    if (rans) {
      // low-Re wall (src/ghostStates.cpp:262-275): k = 0 and omega =
      // 60 nu / (beta1 d^2) at the face; nu and d of the wall-adjacent cell,
      // nu from the previous auxiliary update
      const int64_t a = op.src2;
      const double nuW = P.mu[a] / P.W[a];
      const double s = sv.visc_scale;
      // turbModel::WallBeta: SST beta1, Wilcox 2006 beta0
      const double wWall =
          s * s * 60.0 * nuW / (P.wd[a] * P.wd[a] * (sv.wilcox ? kWkBeta0 : kSstBeta1));
      gt[0] = -1.0 * tin[0];
      gt[1] = 2.0 * wWall - tin[1];
      if (op.layer > 1) gt[1] = (double)op.layer * gt[1] - wWall;
    }
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
        if (rans)
          FarfieldTurb(g, bs.u, bs.v, bs.w, bs.turb_intensity, bs.eddy_visc_ratio, sv, gas, gt);
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
        if (rans)
          FarfieldTurb(g, bs.u, bs.v, bs.w, bs.turb_intensity, bs.eddy_visc_ratio, sv, gas, gt);
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
      // ExtrapolateHoldMixture over every variable: the turbulence follows
      // the flow's density test
      auto hold = [&](double f) {
        const bool applies = f * g.rho - in.rho > 0.0;
        g = ExtrapHold(g, f, in);
        if (rans && applies) {
          gt[0] = f * gt[0] - tin[0];
          gt[1] = f * gt[1] - tin[1];
        }
      };
      hold(2.0);
      if (op.layer > 1) {
        hold((double)op.layer);
        if (rans)
          FarfieldTurb(g, bs.u, bs.v, bs.w, bs.turb_intensity, bs.eddy_visc_ratio, sv, gas, gt);
      }
    } else if (op.type == ATH_BC_PRESSURE_OUTLET) {
      // src/ghostStates.cpp:605-672, reflecting form: the boundary pressure
      // with the outgoing characteristics of the interior; the interior
      // state where the ghost's normal Mach number reaches 1; then linear
      // extrapolation of every variable
      const ath_bc_state bs = P.states[sv.state0 + op.state];
      const double sosInt = SoS(in, gas);
      const double rhoSoSInt = in.rho * sosInt;
      g.p = bs.p_out;
      if (bs.nonreflecting) {
        // LODI relaxation of the boundary pressure towards the specified
        // one with the transverse terms (src/ghostStates.cpp:612-638): the
        // time-n state, previous time step and previous residual's velocity
        // and pressure gradients of the boundary-adjacent cell, and the
        // surface's average and largest normal Mach number
        double cn[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) cn[v] = P.Un[v * n + op.src];
        const Prim<double> sN = ConsToPrim(cn, gas);
        const double dt = P.dt[op.src];
        const double avgMach = P.nr_mach[2 * op.src2], maxMach = P.nr_mach[2 * op.src2 + 1];
        double vg[9], pgr[3];
#pragma unroll
        for (int e = 0; e < 9; ++e) vg[e] = P.nrg[e * n + op.src];
#pragma unroll
        for (int e = 0; e < 3; ++e) pgr[e] = P.nrg[(9 + e) * n + op.src];
        const double deltaVel = Dot(in.u - sN.u, in.v - sN.v, in.w - sN.w, nx, ny, nz);
        const double sigma = 0.25;
        const double rhoN = sN.rho;
        const double sosN = SoS(sN, gas);
        const double rhoSoSN = rhoN * sosN;
        const double k = sigma * sosN * (1.0 - maxMach * maxMach) / bs.length_scale;
        const double beta = avgMach;
        const double pgn = Dot(pgr[0], pgr[1], pgr[2], nx, ny, nz);
        const double pgT[3] = {pgr[0] - pgn * nx, pgr[1] - pgn * ny, pgr[2] - pgn * nz};
        const double vnN = Dot(sN.u, sN.v, sN.w, nx, ny, nz);
        const double velT[3] = {sN.u - vnN * nx, sN.v - vnN * ny, sN.w - vnN * nz};
        // velocity gradient without its normal component, row by row
        // (tensor::RemoveComponent), then the rows' normal-weighted sum
        // (LinearCombination) and the sum of all entries (Sum)
        double gT[9];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          const double rn = Dot(vg[r * 3], vg[r * 3 + 1], vg[r * 3 + 2], nx, ny, nz);
          gT[r * 3] = vg[r * 3] - rn * nx;
          gT[r * 3 + 1] = vg[r * 3 + 1] - rn * ny;
          gT[r * 3 + 2] = vg[r * 3 + 2] - rn * nz;
        }
        double dVn[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          dVn[q] = gT[q] * nx;
          dVn[q] += gT[3 + q] * ny;
          dVn[q] += gT[6 + q] * nz;
        }
        double gsum = 0.0;
#pragma unroll
        for (int e = 0; e < 9; ++e) gsum += gT[e];
        const double dVelT = gsum - (((0.0 + dVn[0]) + dVn[1]) + dVn[2]);
        const double gamma = gas.Gamma();
        const double tr =
            -0.5 * (Dot(velT[0], velT[1], velT[2], pgT[0] - rhoSoSN * dVn[0],
                        pgT[1] - rhoSoSN * dVn[1], pgT[2] - rhoSoSN * dVn[2]) +
                    gamma * sN.p * dVelT);
        g.p = (sN.p + rhoSoSN * deltaVel + dt * k * bs.p_out - dt * beta * tr) / (1.0 + dt * k);
      }
      const double deltaPressure = in.p - g.p;
      const double rho = in.rho - deltaPressure / (sosInt * sosInt);
      g.rho = rho * (in.rho / in.rho);
      g.u = in.u + nx * deltaPressure / rhoSoSInt;
      g.v = in.v + ny * deltaPressure / rhoSoSInt;
      g.w = in.w + nz * deltaPressure / rhoSoSInt;
      if (Dot(g.u, g.v, g.w, nx, ny, nz) / SoS(g, gas) >= 1.0) g = in;
      auto extrap = [&](double f) {
        g.rho = f * g.rho - in.rho;
        g.u = f * g.u - in.u;
        g.v = f * g.v - in.v;
        g.w = f * g.w - in.w;
        g.p = f * g.p - in.p;
        if (rans) {
          gt[0] = f * gt[0] - tin[0];
          gt[1] = f * gt[1] - tin[1];
        }
      };
      extrap(2.0);
      if (op.layer > 1) extrap((double)op.layer);
    } else if (op.type == ATH_BC_STAGNATION_INLET) {
      // src/ghostStates.cpp:535-604: the outgoing Riemann invariant and the
      // inflow angle give the boundary speed of sound; temperature,
      // pressure and speed follow from the stagnation values (isentropic),
      // along the prescribed direction; extrapolated with the hold rule
      const ath_bc_state bs = P.states[sv.state0 + op.state];
      const double gm1 = gas.Gamma() - 1.0;
      const double vn = Dot(in.u, in.v, in.w, nx, ny, nz);
      const double sosInt = SoS(in, gas);
      const double rNeg = vn - 2.0 * sosInt / gm1;
      const double cosTheta = -1.0 * vn / VelMag(in);
      const double stagSoSsq = sosInt * sosInt + 0.5 * gm1 * Dot(in.u, in.v, in.w, in.u, in.v, in.w);
      const double sosB = -1.0 * rNeg * gm1 / (gm1 * cosTheta * cosTheta + 2.0) *
                          (1.0 + cosTheta * sqrt((gm1 * cosTheta * cosTheta + 2.0) * stagSoSsq /
                                                     (gm1 * rNeg * rNeg) -
                                                 0.5 * gm1));
      const double tb = bs.t0 * (sosB * sosB / stagSoSsq);
      const double pb = bs.p0 * pow(sosB * sosB / stagSoSsq, gas.Gamma() / gm1);
      const double vbMag = sqrt(2.0 / gm1 * (bs.t0 - tb));
      const double rhoGhost = pb / ((0.0 + 1.0 * gas.r) * tb);
      g.rho = rhoGhost * 1.0;
      g.u = vbMag * bs.dir[0];
      g.v = vbMag * bs.dir[1];
      g.w = vbMag * bs.dir[2];
      g.p = pb;
      if (rans)
        FarfieldTurb(g, g.u, g.v, g.w, bs.turb_intensity, bs.eddy_visc_ratio, sv, gas, gt);
      auto hold = [&](double f) {
        const bool applies = f * g.rho - in.rho > 0.0;
        g = ExtrapHold(g, f, in);
        if (rans && applies) {
          gt[0] = f * gt[0] - tin[0];
          gt[1] = f * gt[1] - tin[1];
        }
      };
      hold(2.0);
      if (op.layer > 1) {
        hold((double)op.layer);
        if (rans)
          FarfieldTurb(g, g.u, g.v, g.w, bs.turb_intensity, bs.eddy_visc_ratio, sv, gas, gt);
      }
    } else if (op.type == ATH_BC_INLET) {
      // src/ghostStates.cpp:392-493, reflecting form: the freestream state
      // when the interior's normal Mach number reaches 1, else the incoming
      // characteristics of the freestream and the outgoing one of the
      // interior, extrapolated with the hold rule
      const ath_bc_state bs = P.states[sv.state0 + op.state];
      const Prim<double> fr{bs.rho, bs.u, bs.v, bs.w, bs.p};
      const double velIntNorm = Dot(in.u, in.v, in.w, nx, ny, nz);
      const double sosInt = SoS(in, gas);
      const double machInt = fabs(velIntNorm) / sosInt;
      if (machInt >= 1.0) {
        g = fr;
        if (rans)
          FarfieldTurb(g, bs.u, bs.v, bs.w, bs.turb_intensity, bs.eddy_visc_ratio, sv, gas, gt);
      } else {
        const double rhoSoSInt = in.rho * sosInt;
        const double dvx = fr.u - in.u, dvy = fr.v - in.v, dvz = fr.w - in.w;
        g.p = 0.5 * (fr.p + in.p - rhoSoSInt * Dot(nx, ny, nz, dvx, dvy, dvz));
        if (bs.nonreflecting) {
          // LODI relaxation of the incoming characteristic towards the
          // specified state (src/ghostStates.cpp:433-461): the time-n state
          // of the boundary-adjacent cell, its time step of the previous
          // iteration and the surface's largest normal Mach number
          const double *un = P.Un;
          double cn[5];
#pragma unroll
          for (int v = 0; v < 5; ++v) cn[v] = un[v * n + op.src];
          const Prim<double> sN = ConsToPrim(cn, gas);
          const double dt = P.dt[op.src];
          const double maxMach = P.nr_mach[2 * op.src2 + 1];
          const double sigma = 0.25;
          const double rhoN = sN.rho;
          const double sosN = SoS(sN, gas);
          const double rhoSoSN = rhoN * sosN;
          const double deltaPressure = g.p - sN.p;
          const double alpha = sigma * sosN / bs.length_scale;
          const double rhoNp1 =
              (rhoN + dt * alpha * fr.rho + deltaPressure / (sosN * sosN)) / (1.0 + dt * alpha);
          g.rho = rhoNp1 * (fr.rho / fr.rho);
          const double k = alpha * (1.0 - maxMach * maxMach);
          g.u = (sN.u + dt * k * fr.u - nx * deltaPressure / rhoSoSN) / (1.0 + dt * k);
          g.v = (sN.v + dt * k * fr.v - ny * deltaPressure / rhoSoSN) / (1.0 + dt * k);
          g.w = (sN.w + dt * k * fr.w - nz * deltaPressure / rhoSoSN) / (1.0 + dt * k);
        } else {
          const double deltaPressure = fr.p - g.p;
          const double rho = fr.rho - deltaPressure / (sosInt * sosInt);
          g.rho = rho * (fr.rho / fr.rho);
          g.u = fr.u - nx * deltaPressure / rhoSoSInt;
          g.v = fr.v - ny * deltaPressure / rhoSoSInt;
          g.w = fr.w - nz * deltaPressure / rhoSoSInt;
        }
        if (rans)
          FarfieldTurb(g, bs.u, bs.v, bs.w, bs.turb_intensity, bs.eddy_visc_ratio, sv, gas, gt);
        auto hold = [&](double f) {
          const bool applies = f * g.rho - in.rho > 0.0;
          g = ExtrapHold(g, f, in);
          if (rans && applies) {
            gt[0] = f * gt[0] - tin[0];
            gt[1] = f * gt[1] - tin[1];
          }
        };
        hold(2.0);
        if (op.layer > 1) hold((double)op.layer);
      }
    } else if (op.type == ATH_BC_SUPERSONIC_INFLOW) {
      const ath_bc_state bs = P.states[sv.state0 + op.state];
      g.rho = bs.rho;
      g.u = bs.u;
      g.v = bs.v;
      g.w = bs.w;
      g.p = bs.p;
      if (rans)
        FarfieldTurb(g, bs.u, bs.v, bs.w, bs.turb_intensity, bs.eddy_visc_ratio, sv, gas, gt);
    } else if (op.type == ATH_BC_SUPERSONIC_OUTFLOW) {
      if (op.layer > 1) {
        const double f = (double)op.layer;
        g.rho = f * in.rho - in.rho;
        g.u = f * in.u - in.u;
        g.v = f * in.v - in.v;
        g.w = f * in.w - in.w;
        g.p = f * in.p - in.p;
        if (rans) {
          gt[0] = f * tin[0] - tin[0];
          gt[1] = f * tin[1] - tin[1];
        }
      }
    }
  }
  if (rans) {
    P.Wt[op.dst] = gt[0];
    P.Wt[n + op.dst] = gt[1];
  }
  P.W[op.dst] = g.rho;
  P.W[n + op.dst] = g.u;
  P.W[2 * n + op.dst] = g.v;
  P.W[3 * n + op.dst] = g.w;
  P.W[4 * n + op.dst] = g.p;
}

// ---------------------------------------------------------------------------
// face fluxes

// Reconstruction and inviscid flux of face c (direction D) in arithmetic U:
// f is the flux per unit area, L and R the reconstructed face states.
// FAST (FP64 batches with the fast-face option): MUSCL and the Roe flux in
// their fast forms (MusclFastPair, RoeFluxFast), equal to the reference to
// roundoff instead of bit for bit, and f is the flux times the face's area.
// MR: the solve reconstructs with MUSCL and takes the Roe flux, and
// nothing else is built in (FP64 faces; the mixed faces' FaceFluxMixed is
// unchanged, k_face's MR only raises their occupancy).
template <typename U, int D, typename PT, bool FAST = false, bool MR = false>
__device__ __forceinline__ void FaceFlux(const Pools<PT> &P, const SolveDev &sv, int64_t c,
                                         int64_t s, U f[5], Prim<U> &L, Prim<U> &R,
                                         U ft[2] = nullptr) {
  const Gas<U> g = GasOf<U>(sv);
  const int64_t n = P.ncell;
  if constexpr (FAST && MR && std::is_same<U, double>::value) {
    const Prim<U> wm2 = LoadW<U>(P.W, n, c - 2 * s), wm1 = LoadW<U>(P.W, n, c - s),
                  w0 = LoadW<U>(P.W, n, c), wp1 = LoadW<U>(P.W, n, c + s);
    const double *fg = P.fgeo[D];
    MusclFastPair(wm2, wm1, w0, wp1, fg[c], fg[n + c], fg[2 * n + c], fg[3 * n + c],
                  (U)sv.kappa, sv.limiter, L, R);
    const double *fa = P.fa[D];
    RoeFluxFast(L, R, g, fa[c], fa[n + c], fa[2 * n + c], fa[3 * n + c], f);
    return;
  } else if constexpr (!FAST && MR && std::is_same<U, double>::value) {
    // bit-exact MUSCL-Roe: Muscl with the batch's ratio table, RoeFlux
    const Prim<U> wm2 = LoadW<U>(P.W, n, c - 2 * s), wm1 = LoadW<U>(P.W, n, c - s),
                  w0 = LoadW<U>(P.W, n, c), wp1 = LoadW<U>(P.W, n, c + s);
    const double *fg = P.fgeo[D];
    const U kappa = (U)sv.kappa;
    L = MusclR(wm2, wm1, w0, (U)fg[c], (U)fg[n + c], kappa, sv.limiter);
    R = MusclR(wp1, w0, wm1, (U)fg[2 * n + c], (U)fg[3 * n + c], kappa, sv.limiter);
    const double *fa = P.fa[D];
    RoeFlux(L, R, g, (U)fa[c], (U)fa[n + c], (U)fa[2 * n + c], f);
    return;
  }
  const double *wd = P.width[D];
  const Prim<U> wm1 = LoadW<U>(P.W, n, c - s);
  const Prim<U> w0 = LoadW<U>(P.W, n, c);
  if (sv.recon == ATH_RECON_CONSTANT) {
    L = wm1;
    R = w0;
  } else if (sv.recon == ATH_RECON_MUSCL) {
    const Prim<U> wm2 = LoadW<U>(P.W, n, c - 2 * s);
    const Prim<U> wp1 = LoadW<U>(P.W, n, c + s);
    const U kappa = (U)sv.kappa;
    if constexpr (FAST) {
      // the width ratios formed once from the geometry (Pools::fgeo)
      const double *fg = P.fgeo[D];
      const U dpL = (U)fg[c], dmL = (U)fg[n + c], dpR = (U)fg[2 * n + c], dmR = (U)fg[3 * n + c];
      MusclFastPair(wm2, wm1, w0, wp1, dpL, dmL, dpR, dmR, kappa, sv.limiter, L, R);
    } else if (P.fgeo[D] && !P.fast_fp64) {
      // bit-exact FP64 batches: the same ratios, formed once per batch with
      // Muscl's expressions (Pools::fgeo)
      const double *fg = P.fgeo[D];
      L = MusclR(wm2, wm1, w0, (U)fg[c], (U)fg[n + c], kappa, sv.limiter);
      R = MusclR(wp1, w0, wm1, (U)fg[2 * n + c], (U)fg[3 * n + c], kappa, sv.limiter);
    } else {
      const U xm2 = (U)wd[c - 2 * s], xm1 = (U)wd[c - s], x0 = (U)wd[c], xp1 = (U)wd[c + s];
      // lower side: upwind2 = c-2, upwind1 = c-1, downwind = c
      L = Muscl(wm2, wm1, w0, xm2, xm1, x0, kappa, sv.limiter);
      // upper side: upwind2 = c+1, upwind1 = c, downwind = c-1
      R = Muscl(wp1, w0, wm1, xp1, x0, xm1, kappa, sv.limiter);
    }
  } else {
    const Prim<U> wm3 = LoadW<U>(P.W, n, c - 3 * s);
    const Prim<U> wm2 = LoadW<U>(P.W, n, c - 2 * s);
    const Prim<U> wp1 = LoadW<U>(P.W, n, c + s);
    const Prim<U> wp2 = LoadW<U>(P.W, n, c + 2 * s);
    const bool z = sv.recon == ATH_RECON_WENOZ;
    const U wl[5] = {(U)wd[c - 3 * s], (U)wd[c - 2 * s], (U)wd[c - s], (U)wd[c],
                     (U)wd[c + s]};
    const U wu[5] = {(U)wd[c + 2 * s], (U)wd[c + s], (U)wd[c], (U)wd[c - s],
                     (U)wd[c - 2 * s]};
    // the interpolation weights depend on the widths only: one set per side
    // serves the flow variables and k, omega
    const WenoCoeffs<U> kl = MakeWeno(wl), ku = MakeWeno(wu);
    L = Weno(kl, wm3, wm2, wm1, w0, wp1, wl, z);
    R = Weno(ku, wp2, wp1, w0, wm1, wm2, wu, z);
    if (ft) {
      // k and omega with the same weights, then their fluxes
      const double *Wt = P.Wt;
      auto kt = [&](int64_t x, int q) { return (U)Wt[q * n + x]; };
      U Lt[2], Rt[2];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        Lt[q] = Weno1(kl, wl, kt(c - 3 * s, q), kt(c - 2 * s, q), kt(c - s, q), kt(c, q),
                      kt(c + s, q), z);
        Rt[q] = Weno1(ku, wu, kt(c + 2 * s, q), kt(c + s, q), kt(c, q), kt(c - s, q),
                      kt(c - 2 * s, q), z);
      }
      const double *fa = P.fa[D];
      const U nx = (U)fa[c], ny = (U)fa[n + c], nz = (U)fa[2 * n + c];
      U vlr[2];
      if (sv.flux == ATH_FLUX_AUSM) {
        AusmFlux(L, R, g, nx, ny, nz, f, vlr);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          ft[q] = L.rho * vlr[0] * Lt[q];
          ft[q] += R.rho * vlr[1] * Rt[q];
        }
      } else {
        RoeFlux(L, R, g, nx, ny, nz, f);
        RoeTurbFlux(L, R, Lt, Rt, g, nx, ny, nz, ft);
      }
      return;
    }
  }
  const double *fa = P.fa[D];
  const U nx = (U)fa[c], ny = (U)fa[n + c], nz = (U)fa[2 * n + c];
  U vlr[2];
  if (sv.flux == ATH_FLUX_AUSM) {
    AusmFlux(L, R, g, nx, ny, nz, f, vlr);
    if constexpr (FAST) {
      const U mag = (U)fa[3 * n + c];
#pragma unroll
      for (int v = 0; v < 5; ++v) f[v] = f[v] * mag;
    }
  } else if constexpr (FAST && std::is_same<U, double>::value) {
    RoeFluxFast(L, R, g, nx, ny, nz, (U)fa[3 * n + c], f);
  } else {
    RoeFlux(L, R, g, nx, ny, nz, f);
  }
  if (ft) {
    // k and omega reconstructed like the flow variables, then their fluxes
    const double *Wt = P.Wt;
    auto kt = [&](int64_t x, int q) { return (U)Wt[q * n + x]; };
    U Lt[2], Rt[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (sv.recon == ATH_RECON_CONSTANT) {
        Lt[q] = kt(c - s, q);
        Rt[q] = kt(c, q);
      } else if (sv.recon == ATH_RECON_MUSCL) {
        const U kappa = (U)sv.kappa;
        U dpL, dmL, dpR, dmR;
        if (P.fgeo[D] && !P.fast_fp64) {
          const double *fg = P.fgeo[D];
          dpL = (U)fg[c];
          dmL = (U)fg[n + c];
          dpR = (U)fg[2 * n + c];
          dmR = (U)fg[3 * n + c];
        } else {
          const U xm2 = (U)wd[c - 2 * s], xm1 = (U)wd[c - s], x0 = (U)wd[c],
                  xp1 = (U)wd[c + s];
          MusclRatios(xm2, xm1, x0, dpL, dmL);
          MusclRatios(xp1, x0, xm1, dpR, dmR);
        }
        Lt[q] = Muscl1(kt(c - 2 * s, q), kt(c - s, q), kt(c, q), dpL, dmL, kappa, sv.limiter);
        Rt[q] = Muscl1(kt(c + s, q), kt(c, q), kt(c - s, q), dpR, dmR, kappa, sv.limiter);
      } else {
        const bool z = sv.recon == ATH_RECON_WENOZ;
        const U wl[5] = {(U)wd[c - 3 * s], (U)wd[c - 2 * s], (U)wd[c - s], (U)wd[c],
                         (U)wd[c + s]};
        const U wu[5] = {(U)wd[c + 2 * s], (U)wd[c + s], (U)wd[c], (U)wd[c - s],
                         (U)wd[c - 2 * s]};
        const WenoCoeffs<U> kl = MakeWeno(wl), ku = MakeWeno(wu);
        Lt[q] = Weno1(kl, wl, kt(c - 3 * s, q), kt(c - 2 * s, q), kt(c - s, q), kt(c, q),
                      kt(c + s, q), z);
        Rt[q] = Weno1(ku, wu, kt(c + 2 * s, q), kt(c + s, q), kt(c, q), kt(c - s, q),
                      kt(c - 2 * s, q), z);
      }
    }
    if (sv.flux == ATH_FLUX_AUSM) {
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        ft[q] = L.rho * vlr[0] * Lt[q];
        ft[q] += R.rho * vlr[1] * Rt[q];
      }
    } else {
      RoeTurbFlux(L, R, Lt, Rt, g, nx, ny, nz, ft);
    }
  }
}

// Mixed-precision Roe/MUSCL face: the face states are the FP64 upwind cell
// values plus MUSCL increments computed in FP32 from differences formed in
// FP64; the central part 0.5 (F(L) + F(R)) is FP64 and only the Roe
// dissipation is FP32, evaluated from the jumps R - L formed in FP64.  The
// flux's rounding error is then relative to the increments and to the
// dissipation, not to the flux itself, so the iteration converges to the
// FP64 fixed point to within that error.
template <int D, typename PT>
__device__ __forceinline__ void FaceFluxMixedRoe(const Pools<PT> &P, const SolveDev &sv,
                                                 int64_t c, int64_t s, double f[5],
                                                 Prim<double> &L, Prim<double> &R) {
  const int64_t n = P.ncell;
  const double *wd = P.width[D];
  const Prim<double> wm1 = LoadW<double>(P.W, n, c - s);
  const Prim<double> w0 = LoadW<double>(P.W, n, c);
  L = wm1;
  R = w0;
  if (sv.recon == ATH_RECON_MUSCL) {
    const Prim<double> wm2 = LoadW<double>(P.W, n, c - 2 * s);
    const Prim<double> wp1 = LoadW<double>(P.W, n, c + s);
    const float xm2 = (float)wd[c - 2 * s], xm1 = (float)wd[c - s], x0 = (float)wd[c],
                xp1 = (float)wd[c + s];
    const float kappa = (float)sv.kappa;
    const float dpL = (xm1 + xm1) / (xm1 + x0), dmL = (xm1 + xm1) / (xm1 + xm2);
    const float dpR = (x0 + x0) / (x0 + xm1), dmR = (x0 + x0) / (x0 + xp1);
    const double am[5] = {wm2.rho, wm2.u, wm2.v, wm2.w, wm2.p};
    const double a1[5] = {wm1.rho, wm1.u, wm1.v, wm1.w, wm1.p};
    const double a0[5] = {w0.rho, w0.u, w0.v, w0.w, w0.p};
    const double ap[5] = {wp1.rho, wp1.u, wp1.v, wp1.w, wp1.p};
    double l[5], r[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      // the difference across the face serves both sides: a1 - a0 is
      // -(a0 - a1) exactly, before and after rounding to FP32
      const float d0 = (float)(a0[v] - a1[v]);
      const float dl = MusclDelta1((float)(a1[v] - am[v]), d0, dpL, dmL, kappa, sv.limiter);
      const float dr = MusclDelta1((float)(a0[v] - ap[v]), -d0, dpR, dmR, kappa, sv.limiter);
      l[v] = a1[v] + (double)dl;
      r[v] = a0[v] + (double)dr;
    }
    L = Prim<double>{l[0], l[1], l[2], l[3], l[4]};
    R = Prim<double>{r[0], r[1], r[2], r[3], r[4]};
  }
  const double *fa = P.fa[D];
  const double nx = fa[c], ny = fa[n + c], nz = fa[2 * n + c];
  const float dq[5] = {(float)(R.rho - L.rho), (float)(R.u - L.u), (float)(R.v - L.v),
                       (float)(R.w - L.w), (float)(R.p - L.p)};
  const Prim<float> Lf{(float)L.rho, (float)L.u, (float)L.v, (float)L.w, (float)L.p};
  const Prim<float> Rf{(float)R.rho, (float)R.u, (float)R.v, (float)R.w, (float)R.p};
  float d[5];
  RoeDissipation(Lf, Rf, dq, GasOf<float>(sv), (float)nx, (float)ny, (float)nz, d);
  const Gas<double> g = GasOf<double>(sv);
  // FP64 central part FL + FR summed term by term, the two pressures once
  const double vnL = L.u * nx + L.v * ny + L.w * nz, vnR = R.u * nx + R.v * ny + R.w * nz;
  const double mL = L.rho * vnL, mR = R.rho * vnR;
  const double np1 = g.n + 1.0;
  const double rhoHL = L.rho * (g.hf + 0.5 * (L.u * L.u + L.v * L.v + L.w * L.w)) + np1 * L.p;
  const double rhoHR = R.rho * (g.hf + 0.5 * (R.u * R.u + R.v * R.v + R.w * R.w)) + np1 * R.p;
  const double pLR = L.p + R.p;
  f[0] = ((mL + mR) - (double)d[0]) * 0.5;
  f[1] = ((mL * L.u + (mR * R.u + pLR * nx)) - (double)d[1]) * 0.5;
  f[2] = ((mL * L.v + (mR * R.v + pLR * ny)) - (double)d[2]) * 0.5;
  f[3] = ((mL * L.w + (mR * R.w + pLR * nz)) - (double)d[3]) * 0.5;
  f[4] = ((vnL * rhoHL + vnR * rhoHR) - (double)d[4]) * 0.5;
}

// WENO increment over the upwind cell value in FP32, from differences to
// it formed in FP64: each stencil's interpolation weights sum to one and
// the smoothness indicators use differences only, so shifting the five
// values by the upwind one yields the increment itself.
__device__ __forceinline__ float WenoDelta1(const WenoCoeffs<float> &k, const float w[5],
                                            double y3, double y2, double y1, double d1,
                                            double d2, bool z) {
  return Weno1<float>(k, w, (float)(y3 - y1), (float)(y2 - y1), 0.0f, (float)(d1 - y1),
                      (float)(d2 - y1), z);
}

// Mixed-precision face of any reconstruction and flux: FP64 face states are
// the FP64 upwind cell values plus increments computed in FP32 (MUSCL or
// WENO, k and omega too), so their rounding is relative to the increments;
// Roe faces then take the FP64 central flux and FP32 dissipation
// (FaceFluxMixedRoe), AUSMPW+ faces and the turbulence fluxes are evaluated
// in FP64 from the FP64 face states (their pressure splitting is not a
// small correction to a central flux, so FP32 would put its rounding on the
// flux itself).
template <int D, typename PT>
__device__ __forceinline__ void FaceFluxMixed(const Pools<PT> &P, const SolveDev &sv, int64_t c,
                                              int64_t s, double f[5], Prim<double> &L,
                                              Prim<double> &R, double ft[2] = nullptr) {
  if (!ft && sv.flux == ATH_FLUX_ROE &&
      (sv.recon == ATH_RECON_MUSCL || sv.recon == ATH_RECON_CONSTANT)) {
    FaceFluxMixedRoe<D>(P, sv, c, s, f, L, R);
    return;
  }
  const int64_t n = P.ncell;
  const double *wd = P.width[D];
  const double *W = P.W;
  auto val = [&](int v, int64_t x) { return W[v * n + x]; };
  double l[5], r[5], lt[2] = {0, 0}, rt[2] = {0, 0};
  const double *Wt = P.Wt;
  if (sv.recon == ATH_RECON_CONSTANT) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      l[v] = val(v, c - s);
      r[v] = val(v, c);
    }
    if (ft)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        lt[q] = Wt[q * n + c - s];
        rt[q] = Wt[q * n + c];
      }
  } else if (sv.recon == ATH_RECON_MUSCL) {
    const float xm2 = (float)wd[c - 2 * s], xm1 = (float)wd[c - s], x0 = (float)wd[c],
                xp1 = (float)wd[c + s];
    const float kappa = (float)sv.kappa;
    const float dpL = (xm1 + xm1) / (xm1 + x0), dmL = (xm1 + xm1) / (xm1 + xm2);
    const float dpR = (x0 + x0) / (x0 + xm1), dmR = (x0 + x0) / (x0 + xp1);
    auto muscl = [&](double am, double a1, double a0, double ap, double &lo, double &hi) {
      const float dl = MusclDelta1((float)(a1 - am), (float)(a0 - a1), dpL, dmL, kappa,
                                   sv.limiter);
      const float dr = MusclDelta1((float)(a0 - ap), (float)(a1 - a0), dpR, dmR, kappa,
                                   sv.limiter);
      lo = a1 + (double)dl;
      hi = a0 + (double)dr;
    };
#pragma unroll
    for (int v = 0; v < 5; ++v)
      muscl(val(v, c - 2 * s), val(v, c - s), val(v, c), val(v, c + s), l[v], r[v]);
    if (ft)
#pragma unroll
      for (int q = 0; q < 2; ++q)
        muscl(Wt[q * n + c - 2 * s], Wt[q * n + c - s], Wt[q * n + c], Wt[q * n + c + s],
              lt[q], rt[q]);
  } else {
    const bool z = sv.recon == ATH_RECON_WENOZ;
    const float wl[5] = {(float)wd[c - 3 * s], (float)wd[c - 2 * s], (float)wd[c - s],
                         (float)wd[c], (float)wd[c + s]};
    const float wu[5] = {(float)wd[c + 2 * s], (float)wd[c + s], (float)wd[c],
                         (float)wd[c - s], (float)wd[c - 2 * s]};
    const WenoCoeffs<float> kl = MakeWeno(wl), ku = MakeWeno(wu);
    auto weno = [&](const double *a, double &lo, double &hi) {
      const double ym3 = a[c - 3 * s], ym2 = a[c - 2 * s], ym1 = a[c - s], y0 = a[c],
                   yp1 = a[c + s], yp2 = a[c + 2 * s];
      lo = ym1 + (double)WenoDelta1(kl, wl, ym3, ym2, ym1, y0, yp1, z);
      hi = y0 + (double)WenoDelta1(ku, wu, yp2, yp1, y0, ym1, ym2, z);
    };
#pragma unroll
    for (int v = 0; v < 5; ++v) weno(W + v * n, l[v], r[v]);
    if (ft)
#pragma unroll
      for (int q = 0; q < 2; ++q) weno(Wt + q * n, lt[q], rt[q]);
  }
  L = Prim<double>{l[0], l[1], l[2], l[3], l[4]};
  R = Prim<double>{r[0], r[1], r[2], r[3], r[4]};
  const double *fa = P.fa[D];
  const double nx = fa[c], ny = fa[n + c], nz = fa[2 * n + c];
  const Gas<double> g = GasOf<double>(sv);
  if (sv.flux == ATH_FLUX_AUSM) {
    double vlr[2];
    AusmFlux(L, R, g, nx, ny, nz, f, vlr);
    if (ft)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        ft[q] = L.rho * vlr[0] * lt[q];
        ft[q] += R.rho * vlr[1] * rt[q];
      }
    return;
  }
  // Roe: FP64 central flux, FP32 dissipation from FP64-formed jumps
  const float dq[5] = {(float)(R.rho - L.rho), (float)(R.u - L.u), (float)(R.v - L.v),
                       (float)(R.w - L.w), (float)(R.p - L.p)};
  const Prim<float> Lf{(float)L.rho, (float)L.u, (float)L.v, (float)L.w, (float)L.p};
  const Prim<float> Rf{(float)R.rho, (float)R.u, (float)R.v, (float)R.w, (float)R.p};
  float d[5];
  RoeDissipation(Lf, Rf, dq, GasOf<float>(sv), (float)nx, (float)ny, (float)nz, d);
  double fl[5], fr[5];
  InvFluxCentral(L, g, nx, ny, nz, fl);
  InvFluxCentral(R, g, nx, ny, nz, fr);
#pragma unroll
  for (int v = 0; v < 5; ++v) f[v] = (fl[v] + (fr[v] - (double)d[v])) * 0.5;
  if (ft) RoeTurbFlux(L, R, lt, rt, g, nx, ny, nz, ft);
}

template <typename T, int D, bool RANS, bool FAST = false, bool MR = false>
__global__ void __launch_bounds__(kCta, (MR || FAST) ? 2 : 1) k_face(Pools<T> P, const int32_t *list,
                                               const int32_t *cta_block) {
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  if (c < 0) return;
  const BlockDev b = P.blocks[cta_block[blockIdx.x]];
  const SolveDev sv = P.solves[b.solve];
  if (!sv.active || (sv.rans != 0) != RANS) return;
  const int64_t n = P.ncell;
  const int64_t s = StrideOf(b, D);
  double *out = P.flux[D];
  const double mag = P.fa[D][3 * n + c];
  T lr[10];
  if constexpr (std::is_same<T, float>::value) {
    double f[5];
    Prim<double> L, R;
    double ft[2];
    FaceFluxMixed<D>(P, sv, c, s, f, L, R, RANS ? ft : nullptr);
    if (RANS)
#pragma unroll
      for (int q = 0; q < 2; ++q) P.fluxt[D][q * n + c] = ft[q] * mag;
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v * n + c] = f[v] * mag;
    const double q[10] = {L.rho, L.u, L.v, L.w, L.p, R.rho, R.u, R.v, R.w, R.p};
#pragma unroll
    for (int v = 0; v < 10; ++v) lr[v] = (T)q[v];
  } else {
    T f[5], ft[2];
    Prim<T> L, R;
    FaceFlux<T, D, T, FAST, MR>(P, sv, c, s, f, L, R, RANS ? ft : nullptr);
    const T magT = (T)mag;
    // (the fast faces return F.|A| already)
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v * n + c] = FAST ? f[v] : f[v] * magT;
    if (RANS)
#pragma unroll
      for (int q = 0; q < 2; ++q) P.fluxt[D][q * n + c] = ft[q] * magT;
    const T q[10] = {L.rho, L.u, L.v, L.w, L.p, R.rho, R.u, R.v, R.w, R.p};
#pragma unroll
    for (int v = 0; v < 10; ++v) lr[v] = q[v];
  }
  if (sv.block) {
    // face states for the block diagonal's Rusanov Jacobians
    T *fs = P.fst[D];
#pragma unroll
    for (int v = 0; v < 10; ++v) fs[v * n + c] = lr[v];
  }
}

// ---------------------------------------------------------------------------
// residual assembly + spectral radius + dt + diagonal.  BLOCK: the 5x5
// diagonal of block solves (scalar solves are served by the other
// instantiation; a CTA never mixes the two).  RANS solves add the k and
// omega residuals, turbulence radii, SST sources (from cell averages of the
// six faces' gradients, eddy viscosity and blending) and the turbulence
// diagonal (scalar, or 2x2 for block solves).
template <typename T, bool BLOCK, bool RANS>
__global__ void __launch_bounds__(kCta, (!BLOCK && !RANS) ? 3 : 1) k_cell(Pools<T> P,
                                                                         const int32_t *list,
                                               const int32_t *cta_block) {
  const BlockDev b = P.blocks[cta_block[blockIdx.x]];
  const SolveDev sv = P.solves[b.solve];
  if ((sv.block != 0) != BLOCK || !sv.active) return;
  // fast FP64 option and mixed precision (roundoff-equal by construction),
  // with a local time step: the solve's 1 / CFL formed once per CTA (the
  // CTA lies in one block) for the diagonal
  __shared__ double s_cfl_inv;
  const bool fastdt =
      (std::is_same<T, float>::value || P.fast_fp64) && sv.dt_global <= 0.0;
  if (fastdt) {
    if (threadIdx.x == 0) s_cfl_inv = 1.0 / P.cfl[b.solve];
    __syncthreads();
  }
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  if (c < 0) return;
  const int64_t n = P.ncell;
  const int64_t st[3] = {1, (int64_t)b.NI, (int64_t)b.NI * b.NJ};
  if ((sv.rans != 0) != RANS) return;
  constexpr bool rans = RANS;
  // R = 0 - Fi(lo) + Fi(hi) - Fj(lo) + Fj(hi) - Fk(lo) + Fk(hi), each face
  // term rounded in this order (src/procBlock.cpp:447-463); viscous faces
  // follow with + Fv(lo) - Fv(hi) per direction (:1392-1429)
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double r = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double *F = P.flux[d] + v * n;
      r = r - F[c];
      r = r + F[c + st[d]];
    }
    if (sv.viscous) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const T *F = P.vflux[d] + v * n;
        r = r + (double)F[c];
        r = r - (double)F[c + st[d]];
      }
    }
    P.R[v * n + c] = r;
  }
  double rt[2] = {0.0, 0.0};
  if (rans) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const double *F = P.fluxt[d] + q * n;
        rt[q] = rt[q] - F[c];
        rt[q] = rt[q] + F[c + st[d]];
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const T *F = P.vfluxt[d] + q * n;
        rt[q] = rt[q] + (double)F[c];
        rt[q] = rt[q] - (double)F[c + st[d]];
      }
    }
  }
  // inviscid cell spectral radius, summed i, j, k
  const Gas<T> g = GasOf<T>(sv);
  const Prim<T> w = LoadW<T>(P.W, n, c);
  double lam = 0.0, lamt = 0.0;
  const int64_t q = P.qpos[c];
  // scalar main diagonal: accumulates like the radius, from zero or (a
  // multigrid level visited again in this iteration) from its previous value
  double adiag = (!BLOCK && P.mg_accum) ? (double)P.Aq[q] : 0.0;
  // the sound speed once per cell; fast FP64 option: p / rho once (also for
  // the enthalpy), the radius's geometry from Pools::cgeo
  // (one sound speed per cell either way, chosen by a branch: both forms
  // are divisions and square roots the other path must not execute)
  const bool fastc = std::is_same<T, double>::value && P.fast_fp64;
  T porc = T(0), sosc;
  if (fastc) {
    porc = w.p / w.rho;
    sosc = sqrt(g.Gamma() * porc);
  } else {
    sosc = SoS(w, g);
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double *fa = P.fa[d];
    const int64_t u = c + st[d];
    double lcd;
    if (fastc) {
      // normalised normal and average area formed once (Pools::cgeo)
      const double *cg = P.cgeo[d];
      const T vn = fabs(Dot(w.u, w.v, w.w, (T)cg[c], (T)cg[n + c], (T)cg[2 * n + c]));
      lcd = (double)((vn + sosc) * (T)cg[3 * n + c]);
    } else if (std::is_same<T, double>::value && P.cgeo[d]) {
      // bit-exact FP64 batches: InvCellSpecRad with its geometry formed once
      // per batch by the same expressions (Pools::cgeo)
      const double *cg = P.cgeo[d];
      lcd = (double)((fabs(Dot(w.u, w.v, w.w, (T)cg[c], (T)cg[n + c], (T)cg[2 * n + c])) +
                      sosc) *
                     (T)cg[3 * n + c]);
    } else {
      // InvCellSpecRad with the cell's sound speed formed above
      T ax, ay, az, fMag;
      CellAvgNormal((T)fa[c], (T)fa[n + c], (T)fa[2 * n + c], (T)fa[3 * n + c], (T)fa[u],
                    (T)fa[n + u], (T)fa[2 * n + u], (T)fa[3 * n + u], ax, ay, az, fMag);
      lcd = (double)((fabs(Dot(w.u, w.v, w.w, ax, ay, az)) + sosc) * fMag);
    }
    lam = lam + lcd;
    adiag = adiag + lcd;
    if (rans) {
      // turbModel::InviscidCellSpectralRadius (src/turbulence.cpp:94): |v.n_avg| |A|
      const Prim<double> wd = LoadW<double>(P.W, n, c);
      double ax, ay, az, fm;
      if (P.cgeo[d] && !P.fast_fp64) {
        const double *cg = P.cgeo[d];
        ax = cg[c];
        ay = cg[n + c];
        az = cg[2 * n + c];
        fm = cg[3 * n + c];
      } else {
        CellAvgNormal(fa[c], fa[n + c], fa[2 * n + c], fa[3 * n + c], fa[u], fa[n + u],
                      fa[2 * n + u], fa[3 * n + u], ax, ay, az, fm);
      }
      lamt = lamt + fabs(Dot(wd.u, wd.v, wd.w, ax, ay, az)) * fm;
    }
  }
  double adiagt = lamt;  // the scalar diagonal's turbulence part
  const double vol = P.vol[c];
  if (sv.viscous) {
    // viscous cell spectral radii (ViscCellSpectralRadius): the time-step
    // radius takes them times the viscous CFL coefficient, the diagonal
    // twice (CalcViscFluxI/J/K); with RANS the eddy viscosity and F1 of the
    // cell's lower face enter them
    const T mu = (T)P.mu[c];
    const T vmax = ViscMaxTerm(w, g);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const T mutf = rans ? P.rst[d][15 * n + c] : T(0);
      const T vt = vmax * ViscTerm2(mu, mutf, (T)sv.visc_scale, g, (T)PrtOf(sv));
      const T fMag = T(0.5) * ((T)P.fa[d][3 * n + c] + (T)P.fa[d][3 * n + c + st[d]]);
      const T lv = vt * fMag * fMag / (T)vol;
      lam = lam + (double)(lv * (T)sv.visc_coeff);
      adiag = adiag + (double)(T(2) * lv);
      if (rans) {
        // ViscousCellSpectralRadius (turbKWSst src/turbulence.cpp:785,
        // turbKWWilcox :511): the face's mut and F1, or the cell's rho k / omega
        const double f1f = P.rst[d][16 * n + c];
        const double fm = 0.5 * (P.fa[d][3 * n + c] + P.fa[d][3 * n + c + st[d]]);
        const double length = fm * fm / vol;
        const double nutc = sv.wilcox ? P.W[c] * P.Wt[c] / P.Wt[n + c] : 0.0;
        const TurbDiff<double> df =
            TurbDiffOf<double>(sv.wilcox, (double)P.mu[c], (double)mutf, f1f, nutc);
        const double lvt = sv.visc_scale * length / (double)P.W[c] * df.k;
        lamt = lamt + lvt * sv.visc_coeff;
        adiagt = adiagt + 2.0 * lvt;
      }
    }
    P.muq[q] = mu;
  }
  double srcJ[2] = {0.0, 0.0};
  if (rans) {
    // cell averages of the six faces (one sixth each, i lo, i hi, j lo, ...)
    const double sixth = 1.0 / 6.0;
    double vg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, kg[3] = {0, 0, 0}, wg[3] = {0, 0, 0};
    double mutc = 0.0, f1c = 0.0, f2c = 0.0;
#pragma unroll 1
    for (int d = 0; d < 3; ++d)
#pragma unroll 1
      for (int side = 0; side < 2; ++side) {
        const int64_t f = side ? c + st[d] : c;
        const T *rs = P.rst[d];
#pragma unroll
        for (int e = 0; e < 9; ++e) vg[e] += sixth * (double)rs[e * n + f];
#pragma unroll
        for (int e = 0; e < 3; ++e) {
          kg[e] += sixth * (double)rs[(9 + e) * n + f];
          wg[e] += sixth * (double)rs[(12 + e) * n + f];
        }
        mutc += sixth * (double)rs[15 * n + f];
        f1c += sixth * (double)rs[16 * n + f];
        f2c += sixth * (double)rs[17 * n + f];
      }
    const Prim<double> wd = LoadW<double>(P.W, n, c);
    const double kw[2] = {P.Wt[c], P.Wt[n + c]};
    double src[2];
    const double beta = sv.wilcox ? WkSource(wd, kw, vg, kg, wg, mutc, sv.visc_scale, src)
                                  : SstSource(wd, kw, vg, kg, wg, mutc, f1c, sv.visc_scale, src);
    if (P.nutq) P.nutq[q] = (T)(wd.rho * kw[0] / kw[1]);
    const double inv = 1.0 / sv.visc_scale;
    const double srcSR = -2.0 * kSstBetaStar * kw[1] * vol * inv;
    lamt = lamt - srcSR;
    adiagt = adiagt - srcSR;
    srcJ[0] = -2.0 * kSstBetaStar * kw[1] * 1.0 * vol * inv;
    srcJ[1] = -2.0 * beta * kw[1] * vol * inv;
#pragma unroll
    for (int qq = 0; qq < 2; ++qq) {
      rt[qq] = rt[qq] - src[qq] * vol;
      P.Rt[qq * n + c] = rt[qq];
    }
    const int64_t nq = P.nq;
    P.mutq[q] = (T)mutc;
    P.f1q[q] = (T)f1c;
    P.f2q[q] = (T)f2c;
    P.Rtq[q] = (T)rt[0];
    P.Rtq[nq + q] = (T)rt[1];
#pragma unroll
    for (int e = 0; e < 9; ++e) P.vgq[e * nq + q] = (T)vg[e];
  }
  P.lam[c] = lam;
  if (rans) P.lamt[c] = lamt;
  // time step (global when given, else local from the CFL) and the diagonal
  // A = A*relax + V(1+zeta)/(dt theta) [+ max radius / dual-time CFL]
  // (CalcBlockTimeStep src/procBlock.cpp:798, AddDiagonalTerms
  // src/linearSolver.cpp:146)
  const double cfl = P.cfl[b.solve];
  const double lmax = rans ? CMax(lam, lamt) : lam;
  double dt, diagVolTimeD;
  if (fastdt) {
    // dt = CFL V / lambda and V (1 + zeta) / (dt theta) = (1 + zeta) lambda /
    // (CFL theta): one reciprocal of lambda
    const double il = 1.0 / lmax;
    dt = cfl * (vol * il);
    diagVolTimeD = ((1.0 + sv.zeta) * sv.theta_inv * s_cfl_inv) * lmax;
  } else {
    dt = sv.dt_global > 0.0 ? sv.dt_global : cfl * (vol / lmax);
    diagVolTimeD = (vol * (1.0 + sv.zeta)) / (dt * sv.theta);
  }
  P.dt[c] = dt;
  const int64_t nq = P.nq;
  if (sv.dual_cfl > 0.0) diagVolTimeD += (rans ? lmax : CMax(lam, 0.0)) / sv.dual_cfl;
  if (sv.unsteady) {
    // b = -R/theta + SolDeltaNm1 - SolDeltaMmN (procBlock::SolDeltaMmN /
    // SolDeltaNm1, src/procBlock.cpp:1015-1034) in FP64
    const Gas<double> gd = GasOf<double>(sv);
    const Prim<double> wd = LoadW<double>(P.W, n, c);
    double cn[7];
    PrimToCons(wd, gd, cn);
    cn[5] = rans ? wd.rho * P.Wt[c] : 0.0;
    cn[6] = rans ? wd.rho * P.Wt[n + c] : 0.0;
    const double thetaInvD = sv.theta_inv;
    const double coeffN = (vol * (1.0 + sv.zeta)) / (dt * sv.theta);
    const double coeffNm1 = (vol * sv.zeta) / (dt * sv.theta);
    const int nvs = rans ? 7 : 5;
    for (int v = 0; v < nvs; ++v) {
      const double un = P.Un[v * n + c];
      const double dMmN = coeffN * (cn[v] - un);
      const double dNm1 = sv.multilevel ? coeffNm1 * (un - P.Unm1[v * n + c]) : 0.0;
      const double r = v < 5 ? P.R[v * n + c] : P.Rt[(v - 5) * n + c];
      const double bb = -thetaInvD * r + dNm1 - dMmN;
      if (v < 5) P.Bq[v * nq + q] = (T)bb;
      else P.Btq[(v - 5) * nq + q] = (T)bb;
    }
  }
  if constexpr (BLOCK) {
    // 5x5 diagonal (CalcInvFluxI/J/K, CalcViscFluxI/J/K block branches,
    // src/procBlock.cpp:452-484,1417-1474): per direction, minus the
    // Rusanov Jacobian of the upper-side state of the lower face, plus the
    // one of the lower-side state of the upper face; then per direction the
    // thin-shear-layer Jacobians, plus at the lower face, minus at the
    // upper face; the 2x2 turbulence block alongside
    T A[kJac], At[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
    for (int e = 0; e < kJac; ++e) A[e] = P.mg_accum ? P.Aq[e * nq + q] : T(0);
#pragma unroll 1
    for (int d = 0; d < 3; ++d) {
      const double *fa = P.fa[d];
      const T *fs = P.fst[d];
      T J[kJac], Jt[4];
      const int64_t u = c + st[d];
      const Prim<T> sR{fs[5 * n + c], fs[6 * n + c], fs[7 * n + c], fs[8 * n + c],
                       fs[9 * n + c]};
      RusanovJac(sR, g, (T)fa[c], (T)fa[n + c], (T)fa[2 * n + c], (T)fa[3 * n + c], false, J);
#pragma unroll
      for (int e = 0; e < kJac; ++e) A[e] = A[e] - J[e];
      if (rans) {
        TurbRusanovJac(sR, (T)fa[c], (T)fa[n + c], (T)fa[2 * n + c], (T)fa[3 * n + c], false, Jt);
#pragma unroll
        for (int e = 0; e < 4; ++e) At[e] = At[e] - Jt[e];
      }
      const Prim<T> sL{fs[u], fs[n + u], fs[2 * n + u], fs[3 * n + u], fs[4 * n + u]};
      RusanovJac(sL, g, (T)fa[u], (T)fa[n + u], (T)fa[2 * n + u], (T)fa[3 * n + u], true, J);
#pragma unroll
      for (int e = 0; e < kJac; ++e) A[e] = A[e] + J[e];
      if (rans) {
        TurbRusanovJac(sL, (T)fa[u], (T)fa[n + u], (T)fa[2 * n + u], (T)fa[3 * n + u], true, Jt);
#pragma unroll
        for (int e = 0; e < 4; ++e) At[e] = At[e] + Jt[e];
      }
    }
    if (sv.viscous) {
      const TslCoeffs<T> tk{(T)sv.visc_scale, (T)sv.t_ref, (T)sv.k_c1, (T)sv.k_s,
                            (T)sv.k_ref, (T)PrtOf(sv)};
      T vg[9];
#pragma unroll
      for (int e = 0; e < 9; ++e) vg[e] = T(0);
      const T sixth = T(1) / T(6);
#pragma unroll 1
      for (int d = 0; d < 3; ++d) {
        const double *fa = P.fa[d];
        const T *vs = P.vst[d];
#pragma unroll 1
        for (int side = 0; side < 2; ++side) {
          const int64_t f = side ? c + st[d] : c;
          const Prim<T> fsx{vs[f], vs[n + f], vs[2 * n + f], vs[3 * n + f], vs[4 * n + f]};
          T gr[9];
#pragma unroll
          for (int e = 0; e < 9; ++e) {
            gr[e] = vs[(6 + e) * n + f];
            vg[e] = vg[e] + sixth * gr[e];
          }
          const T dist = side ? P.dist_hi[d * nq + q] : P.dist_lo[d * nq + q];
          const T mutf = rans ? P.rst[d][15 * n + f] : T(0);
          TslJacAccum(fsx, vs[5 * n + f], mutf, g, tk, (T)fa[f], (T)fa[n + f], (T)fa[2 * n + f],
                      (T)fa[3 * n + f], dist, side != 0, gr, side != 0, A);
          if (rans) {
            T Jt[4];
            const TurbDiff<T> df = TurbDiffOf<T>(sv.wilcox, vs[5 * n + f], mutf,
                                                 P.rst[d][16 * n + f], P.rst[d][18 * n + f]);
            TurbViscJac(fsx.rho, (T)fa[3 * n + f], df, dist, (T)sv.visc_scale,
                        side ? T(-1) : T(1), Jt);
#pragma unroll
            for (int e = 0; e < 4; ++e) At[e] = side ? At[e] - Jt[e] : At[e] + Jt[e];
          }
        }
      }
      if (!rans)
#pragma unroll
        for (int e = 0; e < 9; ++e) P.vgq[e * nq + q] = vg[e];
    }
    if (rans) {
      At[0] = At[0] - (T)srcJ[0];
      At[1] = At[1] - T(0);
      At[2] = At[2] - T(0);
      At[3] = At[3] - (T)srcJ[1];
    }
    const T diagVolTime = (T)diagVolTimeD;
#pragma unroll
    for (int r = 0; r < 5; ++r) A[r * 6] *= (T)sv.relax;
#pragma unroll
    for (int r = 0; r < 5; ++r) A[r * 6] += diagVolTime;
#pragma unroll
    for (int e = 0; e < kJac; ++e) P.Aq[e * nq + q] = A[e];
    Inverse5(A);
#pragma unroll
    for (int e = 0; e < kJac; ++e) P.Ainvq[e * nq + q] = A[e];
    if (rans) {
      At[0] *= (T)sv.relax;
      At[3] *= (T)sv.relax;
      At[0] += diagVolTime;
      At[3] += diagVolTime;
#pragma unroll
      for (int e = 0; e < 4; ++e) P.Atq[e * nq + q] = At[e];
      Inverse2(At);
#pragma unroll
      for (int e = 0; e < 4; ++e) P.Ainvtq[e * nq + q] = At[e];
    }
  } else {
    const double a = adiag * sv.relax + diagVolTimeD;
    // mixed precision: the FP32 operator's inverse diagonal divides in FP32
    P.Ainvq[q] = std::is_same<T, float>::value ? (T)(T(1) / (T)a) : (T)(1.0 / a);
    P.Aq[q] = (T)a;
    if (rans) {
      const double at = adiagt * sv.relax + diagVolTimeD;
      P.Ainvtq[q] = std::is_same<T, float>::value ? (T)(T(1) / (T)at) : (T)(1.0 / at);
      P.Atq[q] = (T)at;
    }
  }
  // hyperplane-ordered copies for the sweeps
  P.Wq[q] = w.rho;
  P.Wq[nq + q] = w.u;
  P.Wq[2 * nq + q] = w.v;
  P.Wq[3 * nq + q] = w.w;
  P.Wq[4 * nq + q] = w.p;
#pragma unroll
  for (int v = 0; v < 5; ++v) P.Rq[v * nq + q] = (T)P.R[v * n + c];
  // the cell's state terms of the off-diagonal contributions it makes as a
  // neighbour in the scalar sweeps (FP64 batches)
  if constexpr (!BLOCK) {
    if (P.Npre) {
      const Gas<T> gq = GasOf<T>(sv);
      T cc[5];
      PrimToCons(w, gq, cc);
#pragma unroll
      for (int v = 0; v < 5; ++v) P.Npre[v * nq + q] = cc[v];
      if (fastc) {
        // h = hf + cp T + |v|^2 / 2 with cp T = (n + 1) p / rho
        P.Npre[5 * nq + q] = (gq.hf + (gq.n + T(1)) * porc) +
                             T(0.5) * Dot(w.u, w.v, w.w, w.u, w.v, w.w);
        P.Npre[6 * nq + q] = sosc;
      } else {
        P.Npre[5 * nq + q] = Enthalpy(w, gq);
        P.Npre[6 * nq + q] = sosc;  // SoS(w, gq), formed above
      }
      if (sv.viscous) {
        P.Npre[7 * nq + q] = ViscMaxTerm(w, gq);
        P.Npre[8 * nq + q] =
            ViscTerm2(P.muq[q], rans ? P.mutq[q] : T(0), (T)sv.visc_scale, gq, (T)PrtOf(sv));
      }
    }
  }
}

// Right-hand side b of the linear system for equation v (flow 0-4, k and
// omega 5-6) of q-ordered cell q: -R / theta, or for time-accurate solves
// the value k_cell formed with the time-level terms
// (src/linearSolver.cpp:350-352)
template <typename T>
__device__ __forceinline__ T RhsB0(const Pools<T> &P, const SolveDev &sv, T thetaInv, int v,
                                   int64_t q) {
  const int64_t nq = P.nq;
  if (sv.unsteady) return v < 5 ? P.Bq[v * nq + q] : P.Btq[(v - 5) * nq + q];
  return -thetaInv * (v < 5 ? P.Rq[v * nq + q] : P.Rtq[(v - 5) * nq + q]);
}
// ... with the multigrid forcing of a coarse level added, as the sweeps
// read it (-R/theta + f, src/linearSolver.cpp:350,407,483; multigrid
// levels are steady, so the time-level terms are zero)
template <typename T>
__device__ __forceinline__ T RhsB(const Pools<T> &P, const SolveDev &sv, T thetaInv, int v,
                                  int64_t q) {
  const T b0 = RhsB0(P, sv, thetaInv, v, q);
  return (P.Fq && v < 5) ? b0 + P.Fq[v * P.nq + q] : b0;
}

// Neighbour data of an off-diagonal term: the state, laminar viscosity and
// update of the neighbour across face d of q-ordered cell q, and, for RANS
// solves, its eddy viscosity, F1 and turbulence update.  Connection ghosts
// (nb <= -2) carry the partner cell's data (SwapImplicitUpdate,
// SwapEddyViscAndGradients, SwapTurbVars; src/gridLevel.cpp:321,343).
template <typename T>
struct Nbr {
  Prim<T> s;
  T du[5], dut[2];
  T mu, mut, f1;
  T nut;       // rho k / omega (Wilcox k-omega 2006 solves)
  int64_t vq;  // q index whose cell-averaged gradient the neighbour carries
  bool has_pre;    // pre holds the neighbour's precomputed state terms
  NbrPre<T> pre;
};
// The part of a neighbour's data that depends on the neighbour alone and
// that the sweeps do not change: its state and, for q-ordered neighbours,
// the precomputed state terms; for connection ghosts the partner cell's
// state, and the q index of the cell whose turbulence data applies (vq)
template <typename T>
__device__ __forceinline__ void LoadNbrCell(const Pools<T> &P, int32_t nb, Nbr<T> &o) {
  const int64_t nq = P.nq, n = P.ncell;
  o.mu = o.mut = o.f1 = o.nut = T(0);
  o.dut[0] = o.dut[1] = T(0);
  if (nb >= 0) {
    o.s.rho = P.Wq[nb];
    o.s.u = P.Wq[nq + nb];
    o.s.v = P.Wq[2 * nq + nb];
    o.s.w = P.Wq[3 * nq + nb];
    o.s.p = P.Wq[4 * nq + nb];
    o.has_pre = P.Npre != nullptr;
    if (o.has_pre) {
#pragma unroll
      for (int v = 0; v < 5; ++v) o.pre.c[v] = P.Npre[v * nq + nb];
      o.pre.h = P.Npre[5 * nq + nb];
      o.pre.sos = P.Npre[6 * nq + nb];
    }
    o.vq = nb;
  } else {
    o.has_pre = false;
    const int64_t slot = -(int64_t)nb - 2;
    o.s = LoadW<T>(P.W, n, P.ghost_cell[slot]);
    o.vq = P.ghost_src[slot];
  }
}
// ... its flow update (a connection ghost's: the partner cell's)
template <typename T>
__device__ __forceinline__ void LoadNbrDu(const Pools<T> &P, int32_t nb, Nbr<T> &o) {
  if (nb >= 0) {
#pragma unroll
    for (int v = 0; v < 5; ++v) o.du[v] = P.dUq[v * P.nq + nb];
  } else {
    const int64_t slot = -(int64_t)nb - 2;
#pragma unroll
    for (int v = 0; v < 5; ++v) o.du[v] = P.dUg[v * P.nghost + slot];
  }
}
// ... and the part that depends on the solve's equations: laminar
// viscosity and the precomputed viscous terms (viscous solves), the
// turbulence update, eddy viscosity, F1 and rho k / omega (RANS solves)
template <typename T>
__device__ __forceinline__ void LoadNbrSolve(const Pools<T> &P, const SolveDev &sv, int32_t nb,
                                             Nbr<T> &o) {
  const int64_t nq = P.nq, ng = P.nghost;
  if (nb >= 0) {
    if (sv.viscous) o.mu = P.muq[nb];
    if (sv.rans) {
      o.dut[0] = P.dUtq[nb];
      o.dut[1] = P.dUtq[nq + nb];
    }
    if (o.has_pre && sv.viscous) {
      o.pre.vmax = P.Npre[7 * nq + nb];
      o.pre.vt2 = P.Npre[8 * nq + nb];
    }
  } else {
    const int64_t slot = -(int64_t)nb - 2;
    if (sv.viscous) o.mu = (T)P.mu[P.ghost_cell[slot]];
    if (sv.rans) {
      o.dut[0] = P.dUtg[slot];
      o.dut[1] = P.dUtg[ng + slot];
    }
  }
  if (sv.rans) {
    o.mut = P.mutq[o.vq];
    o.f1 = P.f1q[o.vq];
    if (sv.wilcox) o.nut = P.nutq[o.vq];
  }
}
template <typename T>
__device__ __forceinline__ void LoadNbr(const Pools<T> &P, const SolveDev &sv, int32_t nb,
                                        Nbr<T> &o) {
  LoadNbrCell(P, nb, o);
  LoadNbrDu(P, nb, o);
  LoadNbrSolve(P, sv, nb, o);
}

// Off-diagonal sum of one cell: lower neighbours with the "positive" sign
// (procBlock::ImplicitLower) or upper neighbours with the negative sign
// (ImplicitUpper), accumulated i, j, k from zero.  RANS solves add the
// turbulence rows: the neighbour's turbulence face radius times its update
// (turbModel::FaceSpectralRadius, include/spectralRadius.hpp).
// WAIT: the neighbours' updates are read after GridDependencyWait (a
// hyperplane kernel launched programmatically after the previous plane's)
template <typename T, bool WAIT = false>
__device__ __forceinline__ void OffDiagSum(const Pools<T> &P, const Gas<T> &g,
                                           const SolveDev &sv, int64_t q, bool lower,
                                           T acc[5], T acct[2]) {
  const int64_t nq = P.nq;
  const T *face = lower ? P.face_lo : P.face_hi;
  const T *dist = lower ? P.dist_lo : P.dist_hi;
  const int32_t *nbq = P.nbq + (lower ? 0 : 3 * nq);
#pragma unroll
  for (int v = 0; v < 5; ++v) acc[v] = T(0);
  acct[0] = acct[1] = T(0);
  // neighbour indices and records first, so their dependent loads overlap;
  // the sum keeps the i, j, k order
  int32_t nbs[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) nbs[d] = nbq[d * nq + q];
  Nbr<T> os[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (nbs[d] != -1) LoadNbrCell(P, nbs[d], os[d]);
  if constexpr (WAIT) {
    GridDependencyWait();
    GridDependentsLaunch();
  }
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (nbs[d] != -1) {
      LoadNbrDu(P, nbs[d], os[d]);
      LoadNbrSolve(P, sv, nbs[d], os[d]);
    }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (nbs[d] == -1) continue;
    const Nbr<T> &o = os[d];
    const T *f = face + (int64_t)d * 4 * nq;
    const T mag = f[3 * nq + q];
    // ViscFaceSpectralRadius (include/spectralRadius.hpp:126) across this
    // face, ProjC2CDist as the length
    const T vsr = !sv.viscous ? T(0)
                  : o.has_pre ? mag / dist[d * nq + q] * o.pre.vmax * o.pre.vt2
                              : mag / dist[d * nq + q] * ViscMaxTerm(o.s, g) *
                                    ViscTerm2(o.mu, o.mut, (T)sv.visc_scale, g, (T)PrtOf(sv));
    T r[5];
    if (o.has_pre && P.fast_fp64)
      ScalarOffDiagPreFast(o.s, o.pre, o.du, g, f[q], f[nq + q], f[2 * nq + q], mag, lower,
                           sv.viscous != 0, vsr, r);
    else if (o.has_pre)
      ScalarOffDiagPre(o.s, o.pre, o.du, g, f[q], f[nq + q], f[2 * nq + q], mag, lower, vsr, r);
    else
      ScalarOffDiag(o.s, o.du, g, f[q], f[nq + q], f[2 * nq + q], mag, lower, vsr, r);
#pragma unroll
    for (int v = 0; v < 5; ++v) acc[v] = acc[v] + r[v];
    if (sv.rans) {
      const T vn = Dot(o.s.u, o.s.v, o.s.w, f[q], f[nq + q], f[2 * nq + q]);
      T sr = lower ? T(0.5) * mag * fabs(vn + fabs(vn)) : T(0.5) * mag * fabs(vn - fabs(vn));
      if (sv.viscous) {
        const T length = mag / dist[d * nq + q];
        sr += (T)sv.visc_scale * length / o.s.rho *
              TurbDiffOf<T>(sv.wilcox, o.mu, o.mut, o.f1, o.nut).k;
      }
#pragma unroll
      for (int k = 0; k < 2; ++k) acct[k] = acct[k] + (lower ? o.dut[k] * sr : -(o.dut[k] * sr));
    }
  }
}

// The term of one neighbour (face d) of OffDiagSum, for the grouped sweep
// that gives each neighbour its own lane: r (flow) and rt (turbulence) as
// OffDiagSum adds them, from the neighbour's loaded data o and the face's
// normal (fx, fy, fz) and area mag
template <typename T>
__device__ __forceinline__ void NbrTermFrom(const Pools<T> &P, const Gas<T> &g,
                                            const SolveDev &sv, int64_t q, bool lower, int d,
                                            const Nbr<T> &o, T fx, T fy, T fz, T mag, T r[5],
                                            T rt[2]) {
  const int64_t nq = P.nq;
  const T *dist = lower ? P.dist_lo : P.dist_hi;
  const T vsr = !sv.viscous ? T(0)
                : o.has_pre ? mag / dist[d * nq + q] * o.pre.vmax * o.pre.vt2
                            : mag / dist[d * nq + q] * ViscMaxTerm(o.s, g) *
                                  ViscTerm2(o.mu, o.mut, (T)sv.visc_scale, g, (T)PrtOf(sv));
  if (o.has_pre && P.fast_fp64)
    ScalarOffDiagPreFast(o.s, o.pre, o.du, g, fx, fy, fz, mag, lower, sv.viscous != 0, vsr, r);
  else if (o.has_pre)
    ScalarOffDiagPre(o.s, o.pre, o.du, g, fx, fy, fz, mag, lower, vsr, r);
  else
    ScalarOffDiag(o.s, o.du, g, fx, fy, fz, mag, lower, vsr, r);
  rt[0] = rt[1] = T(0);
  if (sv.rans) {
    const T vn = Dot(o.s.u, o.s.v, o.s.w, fx, fy, fz);
    T sr = lower ? T(0.5) * mag * fabs(vn + fabs(vn)) : T(0.5) * mag * fabs(vn - fabs(vn));
    if (sv.viscous) {
      const T length = mag / dist[d * nq + q];
      sr += (T)sv.visc_scale * length / o.s.rho *
            TurbDiffOf<T>(sv.wilcox, o.mu, o.mut, o.f1, o.nut).k;
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) rt[k] = lower ? o.dut[k] * sr : -(o.dut[k] * sr);
  }
}

// Off-diagonal Jacobians of one neighbour of a block solve's cell
// (RusanovBlockOffDiagonal, src/fluxJacobian.cpp:164): the Rusanov Jacobian
// of the neighbour's state minus (lower) or plus (upper) its thin-shear-
// layer Jacobian with its viscosity and cell-averaged gradient; the 2x2
// turbulence block likewise from the Rusanov and viscous Jacobians
// (turbKWSst::ViscJac, src/turbulence.cpp:764).  They depend on nothing the
// sweeps change, so k_offjac evaluates them once per iteration.
template <typename T>
__device__ __forceinline__ void BlockOffJac(const Pools<T> &P, const Gas<T> &g,
                                            const SolveDev &sv, const TslCoeffs<T> &tk,
                                            int64_t q, bool lower, int d, int32_t nb,
                                            T J[kJac], T Jt[4]) {
  const int64_t nq = P.nq;
  const T *face = lower ? P.face_lo : P.face_hi;
  const T *dist = lower ? P.dist_lo : P.dist_hi;
  Nbr<T> o;
  LoadNbr(P, sv, nb, o);
  const T *f = face + (int64_t)d * 4 * nq;
  const T fx = f[q], fy = f[nq + q], fz = f[2 * nq + q], mag = f[3 * nq + q];
  RusanovJac(o.s, g, fx, fy, fz, mag, lower, J);
  if (sv.viscous) {
    T vg[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) vg[e] = P.vgq[e * nq + o.vq];
    TslJacAccum(o.s, o.mu, o.mut, g, tk, fx, fy, fz, mag, dist[d * nq + q], lower, vg, lower,
                J);
  }
  if (sv.rans) {
    TurbRusanovJac(o.s, fx, fy, fz, mag, lower, Jt);
    if (sv.viscous) {
      T Tv[4];
      TurbViscJac(o.s.rho, mag, TurbDiffOf<T>(sv.wilcox, o.mu, o.mut, o.f1, o.nut),
                  dist[d * nq + q], (T)sv.visc_scale, lower ? T(-1) : T(1), Tv);
#pragma unroll
      for (int e = 0; e < 4; ++e) Jt[e] = lower ? Jt[e] - Tv[e] : Jt[e] + Tv[e];
    }
  }
}

// Stored off-diagonal blocks: Joff[(side*3 + d)*25 + e][nq] (side 0 =
// lower neighbours), Jtoff[(side*3 + d)*4 + e][nq]
template <typename T>
__global__ void __launch_bounds__(128) k_offjac(Pools<T> P, const int2 *items, int n_items) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_items) return;
  const int2 it = items[t];
  const int64_t q = it.x, nq = P.nq;
  const SolveDev sv = P.solves[P.blocks[it.y].solve];
  if (!sv.block || !sv.active) return;
  const Gas<T> g = GasOf<T>(sv);
  const TslCoeffs<T> tk{(T)sv.visc_scale, (T)sv.t_ref, (T)sv.k_c1, (T)sv.k_s, (T)sv.k_ref,
                        (T)PrtOf(sv)};
#pragma unroll 1
  for (int side = 0; side < 2; ++side) {
    const int32_t *nbq = P.nbq + (side == 0 ? 0 : 3 * nq);
#pragma unroll 1
    for (int d = 0; d < 3; ++d) {
      const int32_t nb = nbq[d * nq + q];
      if (nb == -1) continue;
      T J[kJac], Jt[4];
      BlockOffJac(P, g, sv, tk, q, side == 0, d, nb, J, Jt);
      T *out = P.Joff + (int64_t)(side * 3 + d) * kJac * nq + q;
#pragma unroll
      for (int e = 0; e < kJac; ++e) out[e * nq] = J[e];
      if (sv.rans) {
        T *ot = P.Jtoff + (int64_t)(side * 3 + d) * 4 * nq + q;
#pragma unroll
        for (int e = 0; e < 4; ++e) ot[e * nq] = Jt[e];
      }
    }
  }
}

// Update of the neighbour across face d (flow and turbulence)
template <typename T>
__device__ __forceinline__ void LoadNbrDu(const Pools<T> &P, const SolveDev &sv, int32_t nb,
                                          T du[5], T dut[2]) {
  const int64_t nq = P.nq, ng = P.nghost;
  dut[0] = dut[1] = T(0);
  if (nb >= 0) {
#pragma unroll
    for (int v = 0; v < 5; ++v) du[v] = P.dUq[v * nq + nb];
    if (sv.rans) {
      dut[0] = P.dUtq[nb];
      dut[1] = P.dUtq[nq + nb];
    }
  } else {
    const int64_t slot = -(int64_t)nb - 2;
#pragma unroll
    for (int v = 0; v < 5; ++v) du[v] = P.dUg[v * ng + slot];
    if (sv.rans) {
      dut[0] = P.dUtg[slot];
      dut[1] = P.dUtg[ng + slot];
    }
  }
}

// Off-diagonal sum of one cell of a block solve: the stored Jacobian of each
// neighbour times its update (ArrayMultiplication), accumulated i, j, k.
template <typename T>
__device__ __forceinline__ void OffDiagSumBlock(const Pools<T> &P, const SolveDev &sv,
                                                int64_t q, bool lower, T acc[5], T acct[2]) {
  const int64_t nq = P.nq;
  const int32_t *nbq = P.nbq + (lower ? 0 : 3 * nq);
  const int side = lower ? 0 : 1;
  // the three neighbour indices, then their updates, are requested before
  // any product so the dependent loads of the neighbours overlap; the sum
  // keeps the i, j, k order
  int32_t nb[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) nb[d] = nbq[d * nq + q];
  T du[3][5], dut[3][2];
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (nb[d] != -1) LoadNbrDu(P, sv, nb[d], du[d], dut[d]);
#pragma unroll
  for (int v = 0; v < 5; ++v) acc[v] = T(0);
  acct[0] = acct[1] = T(0);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (nb[d] == -1) continue;
    T J[kJac], r[5];
    const T *Jp = P.Joff + (int64_t)(side * 3 + d) * kJac * nq + q;
#pragma unroll
    for (int e = 0; e < kJac; ++e) J[e] = Jp[e * nq];
    MatVec5(J, du[d], r);
#pragma unroll
    for (int v = 0; v < 5; ++v) acc[v] = acc[v] + r[v];
    if (sv.rans) {
      T Jt[4], rt[2];
      const T *Jtp = P.Jtoff + (int64_t)(side * 3 + d) * 4 * nq + q;
#pragma unroll
      for (int e = 0; e < 4; ++e) Jt[e] = Jtp[e * nq];
      MatVec2(Jt, dut[d], rt);
      acct[0] = acct[0] + rt[0];
      acct[1] = acct[1] + rt[1];
    }
  }
}

// ---------------------------------------------------------------------------
// LU-SGS hyperplane sweep on the q-ordered working set.  A pass uses one
// triangle (sweep 0 of a one-sweep solve: forward x = A^-1 (b + L x),
// backward x -= A^-1 U x) or both (x = A^-1 (b + L x - U x)).
// New update of one cell of a scalar LU-SGS pass from its off-diagonal
// sums: acc over the pass's triangle, other over the opposite one (used
// from the second sweep on, or with several sweeps)
template <typename T, bool FULL>
__device__ __forceinline__ void ScalarFinish(const Pools<T> &P, const SolveDev &sv, int64_t q,
                                             int forward, bool both, const T acc[5],
                                             const T acct[2], const T other[5],
                                             const T othert[2]) {
  const int64_t nq = P.nq;
  const T ainv = P.Ainvq[q];
  const T thetaInv = (T)sv.theta_inv;
  if constexpr (FULL) {
    if (both) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const T bv = RhsB(P, sv, thetaInv, v, q);
        const T in = forward ? bv + (acc[v] - other[v]) : (bv + other[v]) - acc[v];
        P.dUq[v * nq + q] = in * ainv;
      }
      if (sv.rans) {
        const T ainvt = P.Ainvtq[q];
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          const T bv = RhsB(P, sv, thetaInv, 5 + v, q);
          const T in = forward ? bv + (acct[v] - othert[v]) : (bv + othert[v]) - acct[v];
          P.dUtq[v * nq + q] = in * ainvt;
        }
      }
      return;
    }
  }
  if (forward) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const T bv = RhsB(P, sv, thetaInv, v, q);
      P.dUq[v * nq + q] = (bv + acc[v]) * ainv;
    }
    if (sv.rans) {
      const T ainvt = P.Ainvtq[q];
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const T bv = RhsB(P, sv, thetaInv, 5 + v, q);
        P.dUtq[v * nq + q] = (bv + acct[v]) * ainvt;
      }
    }
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const T xold = P.dUq[v * nq + q];
      P.dUq[v * nq + q] = xold - acc[v] * ainv;
    }
    if (sv.rans) {
      const T ainvt = P.Ainvtq[q];
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const T xold = P.dUtq[v * nq + q];
        P.dUtq[v * nq + q] = xold - acct[v] * ainvt;
      }
    }
  }
}

template <typename T, bool FULL, bool WAIT = false>
__device__ __forceinline__ void SweepScalarQ(const Pools<T> &P, const SolveDev &sv, int64_t q,
                                             int forward, int sweep) {
  const Gas<T> g = GasOf<T>(sv);
  T acc[5], acct[2], other[5], othert[2];
  OffDiagSum<T, WAIT>(P, g, sv, q, forward != 0, acc, acct);
  bool both = false;
  if constexpr (FULL) {
    if (sweep >= sv.sweeps) return;
    both = sweep > 0 || sv.sweeps > 1;
    if (both) OffDiagSum(P, g, sv, q, forward == 0, other, othert);
  }
  ScalarFinish<T, FULL>(P, sv, q, forward, both, acc, acct, other, othert);
}

// one plane of every scalar solve, one thread per cell
// TURB = false: the batch has no solves with turbulence equations, and the
// kernel is built without their rows (fewer registers)
template <typename T, bool FULL, bool TURB>
__global__ void __launch_bounds__(256) k_sweep(Pools<T> P, const int2 *items, int n_items,
                                               int forward, int sweep) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_items) return;
  const int2 it = items[t];
  SolveDev sv = P.solves[P.blocks[it.y].solve];
  if (sv.block || sv.jacobi || !sv.active) return;
  if constexpr (!TURB) {
    sv.rans = 0;
    sv.wilcox = 0;
  }
  // programmatic launches (chained planes) wait inside before reading the
  // previous plane's updates; threads that stop above read none
  SweepScalarQ<T, FULL, true>(P, sv, it.x, forward, sweep);
}

// Scalar pass with a group of lanes per cell: lane d (0-2) evaluates the
// term of neighbour d of the pass's triangle and, when both triangles
// enter (FULL sweeps after the first, or several sweeps), lane 3 + d that
// of the opposite one -- SweepScalarQ's arithmetic with the three (six)
// independent neighbour terms in parallel, so a plane keeps three (six)
// times as many warps busy: the faster form where a plane has too few
// cells to fill the SMs (the autotuner chooses).  A warp holds 10 (5)
// groups; its last 2 lanes idle.
//
// The group's lanes then share the cell's equations: lane li finishes
// equations e = li + L m (flow 0-4, then k and omega).  In rotation j of
// a round m every lane sends the term its lane (li - j) mod L needs and
// receives from lane (li + j) mod L, so the L shuffles of a round move a
// different term to every lane; each lane then sums its equations' terms
// from zero in the reference's i, j, k order (a neighbour the cell lacks
// gives +0, which leaves the sum's bits as skipping it does) and updates
// them.  The neighbour's index, state and update and the face geometry
// depend on the cell alone and are requested before the solve's flags.
// Every lane of the warp calls it (the shuffles span the warp); c is the
// cell's position in items, valid for c < n_items.
template <typename T, bool FULL, bool TURB = true>
__device__ __forceinline__ void SweepGroupItem(const Pools<T> &P, const int2 *items, int c,
                                               int n_items, int forward, int sweep) {
  constexpr int L = FULL ? 6 : 3, CPW = 32 / L;
  constexpr int NE = TURB ? 7 : 5;         // equations of a cell
  constexpr int M = (NE + L - 1) / L;      // equations per lane
  const int lane = (int)(threadIdx.x & 31);
  const int li = lane % L;
  const bool grouped = lane < CPW * L;
  bool valid = grouped && c < n_items;
  const int2 it = valid ? items[c] : make_int2(0, 0);
  const int64_t nq = P.nq, q = it.x;
  const int side = li / 3, d = li % 3;
  const bool lower = side == 0 ? forward != 0 : forward == 0;
  const int32_t nb = P.nbq[(lower ? 0 : 3 * nq) + d * nq + q];
  Nbr<T> o;
  if (nb != -1) LoadNbrCell(P, nb, o);
  const T *f = (lower ? P.face_lo : P.face_hi) + (int64_t)d * 4 * nq;
  const T fx = f[q], fy = f[nq + q], fz = f[2 * nq + q], mag = f[3 * nq + q];
  SolveDev sv = P.solves[P.blocks[it.y].solve];
  if constexpr (!TURB) {
    sv.rans = 0;
    sv.wilcox = 0;
  }
  valid = valid && !sv.block && !sv.jacobi && sv.active;
  bool both = false;
  if constexpr (FULL) {
    valid = valid && sweep < sv.sweeps;
    both = sweep > 0 || sv.sweeps > 1;
  }
  const Gas<T> g = GasOf<T>(sv);
  const bool term = valid && (side == 0 || both) && nb != -1;
  // FP64 batches, inviscid solves: the neighbour's own part of the term is
  // formed before the wait (it does not depend on the updates), in the fast
  // option's form or the bit-exact one
  const bool early = term && o.has_pre && !sv.viscous && !sv.rans;
  FastOld<T> fo{};
  ExactOld<T> eo{};
  if (early) {
    if (P.fast_fp64) fo = ScalarOffDiagFastOld(o.s, o.pre, fx, fy, fz, mag);
    else eo = ScalarOffDiagExactOld(o.s, o.pre, fx, fy, fz, mag);
  }
  // the previous plane's updates are read from here on: with a programmatic
  // launch after that plane's kernel, wait for it (a no-op otherwise), and
  // let the next plane's kernel start its own loads of this kind
  GridDependencyWait();
  GridDependentsLaunch();
  T r[7] = {T(0), T(0), T(0), T(0), T(0), T(0), T(0)};
  if (term) {
    LoadNbrDu(P, nb, o);
    if (early && P.fast_fp64) {
      ScalarOffDiagFastNew(fo, o.pre, o.du, g, fx, fy, fz, lower, r);
    } else if (early) {
      ScalarOffDiagExactNew(eo, o.pre, o.du, g, fx, fy, fz, lower, r);
    } else {
      LoadNbrSolve(P, sv, nb, o);
      NbrTermFrom(P, g, sv, q, lower, d, o, fx, fy, fz, mag, r, r + 5);
    }
  }
  const int gbase = lane - li;
  T xs[M][L];
#pragma unroll
  for (int m = 0; m < M; ++m) {
#pragma unroll
    for (int j = 0; j < L; ++j) {
      const int e = (li - j + L) % L + L * m;  // equation the receiving lane finishes
      T send = T(0);
#pragma unroll
      for (int ee = 0; ee < NE; ++ee)
        if (ee == e) send = r[ee];
      const int src = grouped ? gbase + (li + j) % L : lane;
      xs[m][j] = __shfl_sync(0xffffffffu, send, src);
    }
  }
  if (!valid) return;
  const T thetaInv = (T)sv.theta_inv;
#pragma unroll
  for (int m = 0; m < M; ++m) {
    const int e = li + L * m;
    if (e >= NE || (e >= 5 && !sv.rans)) continue;
    // the term of group lane k arrived in rotation (k - li) mod L
    T t[L];
#pragma unroll
    for (int k = 0; k < L; ++k) {
      const int jk = (k - li + L) % L;
      t[k] = xs[m][0];
#pragma unroll
      for (int j = 1; j < L; ++j)
        if (j == jk) t[k] = xs[m][j];
    }
    T acc = T(0), other = T(0);
#pragma unroll
    for (int k = 0; k < 3; ++k) acc = acc + t[k];
    if constexpr (FULL) {
#pragma unroll
      for (int k = 3; k < L; ++k) other = other + t[k];
    }
    const bool turb = e >= 5;
    const int64_t at = turb ? (int64_t)(e - 5) * nq + q : (int64_t)e * nq + q;
    T *x = turb ? P.dUtq : P.dUq;
    const T ainv = turb ? P.Ainvtq[q] : P.Ainvq[q];
    if (FULL && both) {
      const T bv = RhsB(P, sv, thetaInv, e, q);
      const T in = forward ? bv + (acc - other) : (bv + other) - acc;
      x[at] = in * ainv;
    } else if (forward) {
      const T bv = RhsB(P, sv, thetaInv, e, q);
      x[at] = (bv + acc) * ainv;
    } else {
      const T xold = x[at];
      x[at] = xold - acc * ainv;
    }
  }
}

template <typename T, bool FULL, int MINB, bool TURB>
__global__ void __launch_bounds__(256, MINB) k_sweepg(Pools<T> P, const int2 *items, int n_items,
                                                int forward, int sweep) {
  constexpr int L = FULL ? 6 : 3, CPW = 32 / L;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = (int)(threadIdx.x & 31);
  SweepGroupItem<T, FULL, TURB>(P, items, (t >> 5) * CPW + lane / L, n_items, forward, sweep);
}

// One hyperplane of the thread-per-cell scalar sweep (k_sweep), chained
// launches as LaunchSweepGroup's
template <typename T>
void LaunchSweepCell(const Pools<T> &P, const int2 *items, int n, int forward, int sweep,
                     bool full, int threads, bool chained, cudaStream_t s) {
  const unsigned grid = (unsigned)((n + threads - 1) / threads);
  const bool turb = (P.fkinds & 2) != 0;
  void (*kern)(Pools<T>, const int2 *, int, int, int) =
      full ? (turb ? k_sweep<T, true, true> : k_sweep<T, true, false>)
           : (turb ? k_sweep<T, false, true> : k_sweep<T, false, false>);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = chained ? 1 : 0;
  // a failed launch leaves its error for the caller's cudaGetLastError
  (void)cudaLaunchKernelEx(&cfg, kern, P, items, n, forward, sweep);
}

// One hyperplane of the grouped scalar sweep over n items with CTAs of
// `threads`; chained launches carry the programmatic-serialization
// attribute (k_sweepg waits for the previous plane before reading its
// updates)
template <typename T>
void LaunchSweepGroup(const Pools<T> &P, const int2 *items, int n, int forward, int sweep,
                      bool full, int threads, bool chained, cudaStream_t s) {
  const int cpw = full ? 32 / 6 : 32 / 3;  // cells per warp
  const unsigned grid = (unsigned)(((int64_t)(n + cpw - 1) / cpw * 32 + threads - 1) / threads);
  const bool turb = (P.fkinds & 2) != 0;
  void (*kern)(Pools<T>, const int2 *, int, int, int) =
      full ? (turb ? k_sweepg<T, true, 1, true> : k_sweepg<T, true, 1, false>)
           : (turb ? k_sweepg<T, false, 1, true> : k_sweepg<T, false, 1, false>);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = chained ? 1 : 0;
  // a failed launch leaves its error for the caller's cudaGetLastError
  (void)cudaLaunchKernelEx(&cfg, kern, P, items, n, forward, sweep);
}

// Loads of one row of a block sweep that depend on the cell alone: the
// neighbour indices and the stored Jacobian row of each neighbour of one
// triangle.  They are issued before the solve's flags are read, so the
// cell's chain of dependent loads (neighbour index, then its update) does
// not wait behind the solve lookup.  Rows 5-6 read the turbulence
// Jacobians only in batches that hold them.
template <typename T>
struct BlockRowPre {
  int32_t nb[3];
  T j[3][5];
};
template <typename T>
__device__ __forceinline__ void PreloadBlockRow(const Pools<T> &P, int64_t q, bool lower,
                                                int row, BlockRowPre<T> &o) {
  const int64_t nq = P.nq;
  const int32_t *nbq = P.nbq + (lower ? 0 : 3 * nq);
  const int side = lower ? 0 : 1;
  const bool turb = row >= 5;
  const int r = turb ? row - 5 : row;
#pragma unroll
  for (int d = 0; d < 3; ++d) o.nb[d] = nbq[d * nq + q];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int c = 0; c < 5; ++c) o.j[d][c] = T(0);
    if (turb) {
      if (P.Jtoff) {
        const T *Jt = P.Jtoff + ((int64_t)(side * 3 + d) * 4 + r * 2) * nq + q;
        o.j[d][0] = Jt[0];
        o.j[d][1] = Jt[nq];
      }
    } else {
      const T *J = P.Joff + ((int64_t)(side * 3 + d) * kJac + r * 5) * nq + q;
#pragma unroll
      for (int c = 0; c < 5; ++c) o.j[d][c] = J[c * nq];
    }
  }
}

// Block version, one 8-lane group per cell: lanes 0-4 own the flow rows,
// lanes 5-6 the k and omega rows of SST solves.  Each lane forms its row of
// the off-diagonal products (stored Jacobian row times the neighbour's
// update, neighbours i, j, k) and of b + L - U, the group exchanges those by
// warp shuffles, and each lane forms its row of A^-1 (...) -- the sums of
// MatVec5/MatVec2 row by row, so the result is that of the whole-cell form.
// A plane's cells spread over five times as many threads, and SMs, which is
// what the FP64 rate of small planes needs.  Every lane of the warp must
// call this (the shuffles name the whole warp); `valid` marks lanes of a
// group that owns a cell of this solve and pass.
template <typename T>
__device__ __forceinline__ T BlockRowOffDiag(const Pools<T> &P, const BlockRowPre<T> &pre,
                                             bool turb) {
  const int64_t nq = P.nq, ng = P.nghost;
  const int nv = turb ? 2 : 5;
  T du[3][5];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int32_t nb = pre.nb[d];
    if (nb == -1) continue;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      if (v >= nv) break;
      if (nb >= 0)
        du[d][v] = turb ? P.dUtq[v * nq + nb] : P.dUq[v * nq + nb];
      else {
        const int64_t slot = -(int64_t)nb - 2;
        du[d][v] = turb ? P.dUtg[v * ng + slot] : P.dUg[v * ng + slot];
      }
    }
  }
  T acc = T(0);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (pre.nb[d] == -1) continue;
    T s = T(0);
    if (turb) {
      s = s + pre.j[d][0] * du[d][0];
      s = s + pre.j[d][1] * du[d][1];
    } else {
#pragma unroll
      for (int c = 0; c < 5; ++c) s = s + pre.j[d][c] * du[d][c];
    }
    acc = acc + s;
  }
  return acc;
}

// Row `row` of one cell of a block pass.  `sv` may still be in flight:
// everything read before its flags depends on the cell alone.  item: the
// lane's group has a cell (q valid); valid: its solve takes part in this
// pass.  full_any: some solve of the launch runs both triangles (preload
// the other one too).
template <typename T>
__device__ __forceinline__ void SweepBlockRow(const Pools<T> &P, const SolveDev &sv, int64_t q,
                                              bool item, bool valid, int row, int forward,
                                              int sweep, bool full_any) {
  const int64_t nq = P.nq;
  const int lane = (int)(threadIdx.x & 31), g0 = lane & ~7;
  const bool turb = row == 5 || row == 6;
  const int r = turb ? row - 5 : row;
  BlockRowPre<T> pre, pre_o;
  T ainv[5] = {T(0), T(0), T(0), T(0), T(0)};
  if (item && row < 7) {
    PreloadBlockRow(P, q, forward != 0, row, pre);
    if (full_any) PreloadBlockRow(P, q, forward == 0, row, pre_o);
    if (turb) {
      if (P.Ainvtq) {
        ainv[0] = P.Ainvtq[(r * 2) * nq + q];
        ainv[1] = P.Ainvtq[(r * 2 + 1) * nq + q];
      }
    } else {
#pragma unroll
      for (int c = 0; c < 5; ++c) ainv[c] = P.Ainvq[(row * 5 + c) * nq + q];
    }
  }
  const bool full = sweep > 0 || sv.sweeps > 1;
  const T thetaInv = (T)sv.theta_inv;
  const bool mine = valid && (row < 5 || (turb && sv.rans));
  T in = T(0);
  if (mine) {
    const T acc = BlockRowOffDiag(P, pre, turb);
    const T bv = RhsB(P, sv, thetaInv, row, q);
    if (full) {
      if (!full_any) PreloadBlockRow(P, q, forward == 0, row, pre_o);
      const T other = BlockRowOffDiag(P, pre_o, turb);
      in = forward ? bv + (acc - other) : (bv + other) - acc;
    } else {
      in = forward ? bv + acc : acc;
    }
  }
  T v5[5], v2[2];
#pragma unroll
  for (int c = 0; c < 5; ++c) v5[c] = __shfl_sync(0xffffffffu, in, g0 + c);
#pragma unroll
  for (int c = 0; c < 2; ++c) v2[c] = __shfl_sync(0xffffffffu, in, g0 + 5 + c);
  if (!mine) return;
  T x = T(0);
  if (turb) {
    x = x + ainv[0] * v2[0];
    x = x + ainv[1] * v2[1];
    T *dst = P.dUtq + r * nq + q;
    *dst = (full || forward) ? x : *dst - x;
  } else {
#pragma unroll
    for (int c = 0; c < 5; ++c) x = x + ainv[c] * v5[c];
    T *dst = P.dUq + row * nq + q;
    *dst = (full || forward) ? x : *dst - x;
  }
}

// one plane of every block solve: thread 8 c + r handles row r of item c
template <typename T>
__global__ void __launch_bounds__(256) k_sweepb(Pools<T> P, const int2 *items, int n_items,
                                                int forward, int sweep, int full_any) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = t >> 3, row = t & 7;
  const bool item = c < n_items;
  int2 it = make_int2(0, 0);
  if (item) it = items[c];
  const SolveDev sv = P.solves[P.blocks[it.y].solve];
  const bool valid = item && sv.block && !sv.jacobi && sv.active && sweep < sv.sweeps;
  SweepBlockRow<T>(P, sv, it.x, item, valid, row, forward, sweep, full_any != 0);
}

// Persistent sweep: one thread-block cluster per solve walks the solve's
// hyperplanes in order (forward or backward), the cluster's threads sharing
// each plane, with a cluster barrier (release/acquire at cluster scope, so
// a plane's updates are visible to the next plane's readers) between
// planes.  One launch per pass for every solve of the batch instead of one
// launch per hyperplane; each cell runs the same arithmetic as k_sweepg /
// k_sweepb.  Every exit condition depends on the solve alone, so either all
// CTAs of a cluster leave before the first barrier or none does.
template <typename T, bool FULL, bool BLOCK>
__global__ void __launch_bounds__(256) k_sweep_cl(Pools<T> P, const int2 *items,
                                                  const int32_t *step_off,
                                                  const int32_t *solve_step0,
                                                  const int32_t *solve_nsteps, int forward,
                                                  int sweep) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int csize = (int)cluster.num_blocks();
  const int s = (int)(blockIdx.x / csize);
  const SolveDev sv = P.solves[s];
  if (!sv.active || sv.jacobi || (sv.block != 0) != BLOCK || sweep >= sv.sweeps) return;
  const int nst = solve_nsteps[s], base = solve_step0[s];
  const int tid = (int)cluster.block_rank() * (int)blockDim.x + (int)threadIdx.x;
  const int nthr = csize * (int)blockDim.x;
  for (int k = 0; k < nst; ++k) {
    const int p = forward ? k : nst - 1 - k;
    const int a = step_off[base + p], b = step_off[base + p + 1];
    if constexpr (BLOCK) {
      // 8-lane groups; every lane runs the same number of rounds
      for (int i0 = a; i0 < b; i0 += nthr >> 3) {
        const int i = i0 + (tid >> 3);
        SweepBlockRow<T>(P, sv, i < b ? items[i].x : 0, i < b, i < b, tid & 7, forward, sweep,
                         FULL);
      }
    } else {
      for (int i = a + tid; i < b; i += nthr) SweepScalarQ<T, FULL>(P, sv, items[i].x, forward, sweep);
    }
    cluster.sync();
  }
}

// ---------------------------------------------------------------------------
// Persistent LU-SGS sweep over a (solve, hyperplane) tile work queue.
//
// A tile is a run of one solve's cells on one hyperplane (at most the
// queue's tile size).  Tiles are numbered in the pass's step order (plane
// order, ascending forward, descending backward, solves in turn), and each
// lists the tiles of the previous step that hold its cells' neighbours on
// the swept side.  CTAs claim tiles from an atomic ticket; a tile waits
// until the tiles it lists are done.  Every tile it waits on has a smaller
// ticket, so it was claimed earlier by a worker (a warp) that is running,
// and the smallest unfinished tile never waits: the queue cannot deadlock
// whatever the number of resident warps.  Neighbour pairs are the only dependencies
// between cells of a pass (both the read of an updated neighbour and the
// read of a not-yet-updated one), so a tile that waits for the tiles
// holding its swept-side neighbours runs in an order the per-plane launches
// also allow, and the result is bit for bit theirs.  Waits are bounded:
// after `spin_limit` polls the warp records ATH_ERR_TIMEOUT in *status and
// returns; a warp whose wait finds *status set returns at once.
// CTAs of two warp workers: the register-bound occupancy is filled in
// steps of two warps rather than eight
constexpr int kTqThreads = 64;
__device__ __forceinline__ int LoadAcquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void StoreRelease(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void FenceAcqRelGpu() {
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

template <typename T, bool FULL, bool BLOCK>
__global__ void __launch_bounds__(kTqThreads) k_sweep_tq(Pools<T> P, TileQueueDev Q,
                                                         int forward, int sweep) {
  // each warp is a worker: it claims a tile, its lane 0 waits for the tiles
  // the tile lists, the warp sweeps the tile's cells, lane 0 marks it done
  const int lane = (int)(threadIdx.x & 31);
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(Q.ticket, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= Q.ntiles) return;
    const int4 tl = Q.tiles[t];  // items [x, y), deps [z, z + w)
    int ok = 1;
    if (lane == 0) {
      for (int e = 0; e < tl.w && ok; ++e) {
        const int *flag = Q.wait_never ? Q.done + Q.ntiles : Q.done + Q.deps[tl.z + e];
        long long polls = 0;
        while (LoadAcquire(flag) == 0) {
          if (++polls > Q.spin_limit || LoadAcquire(Q.status) != 0) {
            atomicCAS(Q.status, 0, ATH_ERR_TIMEOUT);
            ok = 0;
            break;
          }
          __nanosleep(20);
        }
      }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) return;
    __syncwarp();
    if constexpr (BLOCK) {
      // 8-lane groups, one cell each (4 per round).  A retired solve, or one
      // past its sweep count, skips the work but still marks its tiles done
      const SolveDev sv = P.solves[P.blocks[Q.items[tl.x].y].solve];
      if (sv.active && !sv.jacobi && sweep < sv.sweeps) {
        for (int i0 = tl.x; i0 < tl.y; i0 += 4) {
          const int i = i0 + (lane >> 3);
          SweepBlockRow<T>(P, sv, i < tl.y ? Q.items[i].x : 0, i < tl.y, i < tl.y, lane & 7,
                           forward, sweep, FULL);
        }
      }
    } else {
      constexpr int L = FULL ? 6 : 3, CPW = 32 / L;
      for (int c0 = tl.x; c0 < tl.y; c0 += CPW)
        SweepGroupItem<T, FULL>(P, Q.items, c0 + lane / L, tl.y, forward, sweep);
    }
    __syncwarp();
    if (lane == 0) {
      FenceAcqRelGpu();
      StoreRelease(Q.done + t, 1);
    }
  }
}

// x = A^-1 b before the first sweep of multi-sweep and DP-LUR solves
// (InitializeMatrixUpdate, src/linearSolver.cpp:111), 0 otherwise; `jacobi`
// selects the DP-LUR solves or the LU-SGS ones
template <typename T>
__global__ void __launch_bounds__(128) k_init(Pools<T> P, const int2 *items, int n_items,
                                              int jacobi) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_items) return;
  const int2 it = items[t];
  const int64_t q = it.x, nq = P.nq;
  const SolveDev sv = P.solves[P.blocks[it.y].solve];
  if (!sv.active || (sv.jacobi != 0) != (jacobi != 0)) return;
  T x[5], xt[2] = {T(0), T(0)};
  if (sv.sweeps <= 1 && !sv.jacobi) {
#pragma unroll
    for (int v = 0; v < 5; ++v) x[v] = T(0);
  } else {
    const T thetaInv = (T)sv.theta_inv;
    T in[5], int_[2];
#pragma unroll
    for (int v = 0; v < 5; ++v) in[v] = RhsB(P, sv, thetaInv, v, q);
    if (sv.rans)
#pragma unroll
      for (int v = 0; v < 2; ++v) int_[v] = RhsB(P, sv, thetaInv, 5 + v, q);
    if (sv.block) {
      T Ai[kJac];
#pragma unroll
      for (int e = 0; e < kJac; ++e) Ai[e] = P.Ainvq[e * nq + q];
      MatVec5(Ai, in, x);
      if (sv.rans) {
        T Ait[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) Ait[e] = P.Ainvtq[e * nq + q];
        MatVec2(Ait, int_, xt);
      }
    } else {
      const T ainv = P.Ainvq[q];
#pragma unroll
      for (int v = 0; v < 5; ++v) x[v] = in[v] * ainv;
      if (sv.rans) {
        const T ainvt = P.Ainvtq[q];
        xt[0] = int_[0] * ainvt;
        xt[1] = int_[1] * ainvt;
      }
    }
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) P.dUq[v * nq + q] = x[v];
  if (sv.rans) {
    P.dUtq[q] = xt[0];
    P.dUtq[nq + q] = xt[1];
  }
}

// One DP-LUR sweep (dplur::DPLUR, src/linearSolver.cpp:473): from the
// previous iterate P.dUq (and its connection ghosts), x = A^-1 (b + L(x) -
// U(x)) into dst; every cell is independent
template <typename T, bool BLOCK>
__global__ void __launch_bounds__(128) k_jacobi(Pools<T> P, T *dst, T *dstt, const int2 *items,
                                                int n_items, int sweep) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_items) return;
  const int2 it = items[t];
  const int64_t q = it.x, nq = P.nq;
  const SolveDev sv = P.solves[P.blocks[it.y].solve];
  if (!sv.jacobi || !sv.active || (sv.block != 0) != BLOCK) return;
  if (sweep >= sv.sweeps) {
#pragma unroll
    for (int v = 0; v < 5; ++v) dst[v * nq + q] = P.dUq[v * nq + q];
    if (sv.rans) {
      dstt[q] = P.dUtq[q];
      dstt[nq + q] = P.dUtq[nq + q];
    }
    return;
  }
  const T thetaInv = (T)sv.theta_inv;
  T L[5], U[5], Lt[2], Ut[2], in[5], x[5];
  if constexpr (BLOCK) {
    OffDiagSumBlock(P, sv, q, true, L, Lt);
    OffDiagSumBlock(P, sv, q, false, U, Ut);
  } else {
    const Gas<T> g = GasOf<T>(sv);
    OffDiagSum(P, g, sv, q, true, L, Lt);
    OffDiagSum(P, g, sv, q, false, U, Ut);
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const T bv = RhsB(P, sv, thetaInv, v, q);
    in[v] = bv + (L[v] - U[v]);
  }
  if constexpr (BLOCK) {
    T Ai[kJac];
#pragma unroll
    for (int e = 0; e < kJac; ++e) Ai[e] = P.Ainvq[e * nq + q];
    MatVec5(Ai, in, x);
  } else {
    const T ainv = P.Ainvq[q];
#pragma unroll
    for (int v = 0; v < 5; ++v) x[v] = in[v] * ainv;
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) dst[v * nq + q] = x[v];
  if (sv.rans) {
    T int_[2], xt[2];
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const T bv = RhsB(P, sv, thetaInv, 5 + v, q);
      int_[v] = bv + (Lt[v] - Ut[v]);
    }
    if constexpr (BLOCK) {
      T Ait[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) Ait[e] = P.Ainvtq[e * nq + q];
      MatVec2(Ait, int_, xt);
    } else {
      const T ainvt = P.Ainvtq[q];
      xt[0] = int_[0] * ainvt;
      xt[1] = int_[1] * ainvt;
    }
    dstt[q] = xt[0];
    dstt[nq + q] = xt[1];
  }
}

template <typename T>
__global__ void __launch_bounds__(128) k_jacobi_copy(Pools<T> P, const T *src, const T *srct,
                                                     const int2 *items, int n_items) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_items) return;
  const int2 it = items[t];
  const int64_t q = it.x, nq = P.nq;
  const SolveDev sv = P.solves[P.blocks[it.y].solve];
  if (!sv.jacobi || !sv.active) return;
#pragma unroll
  for (int v = 0; v < 5; ++v) P.dUq[v * nq + q] = src[v * nq + q];
  if (sv.rans) {
    P.dUtq[q] = srct[q];
    P.dUtq[nq + q] = srct[nq + q];
  }
}

template <typename T>
__global__ void k_conn_du(Pools<T> P) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P.nghost) return;
  const int64_t src = P.ghost_src[t];
#pragma unroll
  for (int v = 0; v < 5; ++v) P.dUg[v * P.nghost + t] = P.dUq[v * P.nq + src];
  if (P.dUtg != nullptr) {
    P.dUtg[t] = P.dUtq[src];
    P.dUtg[P.nghost + t] = P.dUtq[P.nq + src];
  }
}

// Average and largest outward normal Mach number of each nonreflecting
// surface over its boundary-adjacent cells (procBlock::GetGhostStates,
// src/procBlock.cpp:6235-6260): one thread per surface sums in the
// surface's k, j, i order, as the reference does
template <typename T>
__global__ void k_nr_mach(Pools<T> P, const NrDev *nr, const int32_t *off, int nsurf) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsurf) return;
  const int64_t n = P.ncell;
  const int a = off[s], b = off[s + 1];
  double avg = 0.0, mx = -1.0 * DBL_MAX;
  for (int i = a; i < b; ++i) {
    const NrDev x = nr[i];
    const Prim<double> w = LoadW<double>(P.W, n, x.cell);
    const double *fa = P.fa[x.dir];
    const double ax = x.lower ? -1.0 * fa[x.face] : fa[x.face];
    const double ay = x.lower ? -1.0 * fa[n + x.face] : fa[n + x.face];
    const double az = x.lower ? -1.0 * fa[2 * n + x.face] : fa[2 * n + x.face];
    const double sos = SoS(w, GasOf<double>(P.solves[x.solve]));
    const double mach = Dot(w.u, w.v, w.w, ax, ay, az) / sos;
    mx = mx < mach ? mach : mx;
    avg += mach;
  }
  avg /= (double)(b - a);
  P.nr_mach[2 * s] = avg;
  P.nr_mach[2 * s + 1] = mx;
}

// StoreOldSolution (src/mgSolution.cpp:103) for the time-accurate solves:
// at a time step's first nonlinear iteration the conserved state of time
// n, and at the first step of a bdf2 solve that of time n-1 as well unless
// the host set it (a restart).  block >= 0: only that block, both levels,
// whatever the iteration (AssignSolToTimeN + AssignSolToTimeNm1 of a
// one-level restart, src/output.cpp:892)
template <typename T>
__global__ void __launch_bounds__(kCta) k_store_n(Pools<T> P, const int32_t *list,
                                                  const int32_t *cta_block,
                                                  const SolveState *sstate, int block) {
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  if (c < 0) return;
  const int bk = cta_block[blockIdx.x];
  if (block >= 0 && bk != block) return;
  const int s = P.blocks[bk].solve;
  const SolveDev sv = P.solves[s];
  if (!sv.store_n) return;
  const int64_t it = sstate[s].iter;
  const bool forced = block >= 0;
  if (!forced && (!sv.active || it % sv.nl_iters != 0)) return;
  const bool nm1 = sv.multilevel && (forced || (it == 0 && !sstate[s].nm1_given));
  const int64_t n = P.ncell;
  const Gas<double> g = GasOf<double>(sv);
  const Prim<double> w = LoadW<double>(P.W, n, c);
  double cn[7];
  PrimToCons(w, g, cn);
  cn[5] = sv.rans ? w.rho * P.Wt[c] : 0.0;
  cn[6] = sv.rans ? w.rho * P.Wt[n + c] : 0.0;
#pragma unroll
  for (int v = 0; v < 7; ++v) {
    P.Un[v * n + c] = cn[v];
    if (nm1) P.Unm1[v * n + c] = cn[v];
  }
}

// ---------------------------------------------------------------------------
// conserved update and partial norms
template <typename T>
__global__ void __launch_bounds__(kCta) k_update(Pools<T> P, const int32_t *list,
                                                 const int32_t *cta_block,
                                                 const int32_t *cta_pos0,
                                                 NormPartial *partials,
                                                 const SolveState *sstate) {
  __shared__ double s_l2[kCta / 32][kNvMax];
  __shared__ double s_max[kCta / 32];
  __shared__ int64_t s_pos[kCta / 32];
  __shared__ int32_t s_bad[kCta / 32];
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  const int64_t n = P.ncell;
  double l2[kNvMax] = {0, 0, 0, 0, 0, 0, 0};
  double mx = 0.0;
  int64_t mpos = INT64_MAX;
  int bad = 0;
  const BlockDev b = P.blocks[cta_block[blockIdx.x]];
  const SolveDev sv = P.solves[b.solve];
  if (c >= 0 && sv.active) {
    const Gas<double> g = GasOf<double>(sv);
    const Prim<double> w = LoadW<double>(P.W, n, c);
    double du[5];
    const int64_t q = P.qpos[c], qpos = q;
#pragma unroll
    for (int v = 0; v < 5; ++v) du[v] = (double)P.dUq[v * P.nq + q];
    Prim<double> u;
    if (P.fast_fp64 || std::is_same<T, float>::value) {
      // fast FP64 option, and mixed precision (whose results are roundoff-
      // equal to FP64's by construction): rho E = rho hf + n p + rho |v|^2 / 2
      // (cv T rho = n p), then the updated state with one reciprocal of the
      // density
      // the conserved state: the cell kernel's q-ordered copy (FP64 scalar
      // solves; W has not changed since), else formed here
      double k0, k1, k2, k3, k4;
      if (std::is_same<T, double>::value && P.Npre && !sv.block) {
        const int64_t nq = P.nq;
        k0 = (double)P.Npre[q];
        k1 = (double)P.Npre[nq + q];
        k2 = (double)P.Npre[2 * nq + q];
        k3 = (double)P.Npre[3 * nq + q];
        k4 = (double)P.Npre[4 * nq + q];
      } else {
        k0 = w.rho;
        k1 = w.rho * w.u;
        k2 = w.rho * w.v;
        k3 = w.rho * w.w;
        k4 = w.rho * g.hf + g.n * w.p + 0.5 * w.rho * Dot(w.u, w.v, w.w, w.u, w.v, w.w);
      }
      const double rho1 = k0 + du[0];
      const double c1 = k1 + du[1], c2 = k2 + du[2], c3 = k3 + du[3];
      const double rE = k4 + du[4];
      const double ir = 1.0 / rho1;
      u.rho = rho1;
      u.u = c1 * ir;
      u.v = c2 * ir;
      u.w = c3 * ir;
      u.p = (g.Gamma() - 1.0) *
            (rE - rho1 * (g.hf + 0.5 * Dot(u.u, u.v, u.w, u.u, u.v, u.w)));
    } else {
      u = UpdateWithCons(w, g, du);
    }
    if (!PositiveBits(u.rho) || !PositiveBits(u.p) || !FiniteBits(u.u) || !FiniteBits(u.v) ||
        !FiniteBits(u.w))
      bad = 1;
    P.W[c] = u.rho;
    P.W[n + c] = u.u;
    P.W[2 * n + c] = u.v;
    P.W[3 * n + c] = u.w;
    P.W[4 * n + c] = u.p;
    // gridLevel::UpdateBlocks (src/gridLevel.cpp:418): time n becomes n-1
    // after the last nonlinear iteration of a bdf2 time step
    if (sv.multilevel && sstate[b.solve].iter % sv.nl_iters == sv.nl_iters - 1)
#pragma unroll
      for (int v = 0; v < 7; ++v) P.Unm1[v * n + c] = P.Un[v * n + c];
    double rv[kNvMax];
#pragma unroll
    for (int v = 0; v < 5; ++v) rv[v] = P.R[v * n + c];
    rv[5] = rv[6] = 0.0;
    if (sv.rans) {
      // conserved rho k, rho omega updated, divided by the new density and
      // held above the floors (primitive(conserved), primitive::LimitTurb)
      const double rho1 = w.rho + du[0];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const double cq = w.rho * P.Wt[q * n + c] + (double)P.dUtq[q * P.nq + qpos];
        const double t = cq / rho1;
        P.Wt[q * n + c] = (t < 1.0e-20) ? 1.0e-20 : t;
        rv[5 + q] = P.Rt[q * n + c];
      }
    }
    const int nv = sv.rans ? kNvMax : kNv;
    const int64_t pos0 = (int64_t)cta_pos0[blockIdx.x] + threadIdx.x;
    for (int v = 0; v < nv; ++v) {
      const double r = rv[v];
      l2[v] = r * r;
      // L-infinity follows the reference's signed comparison
      // (procBlock::UpdateBlock): a new maximum replaces the old one only
      // when strictly larger; ties keep the first in loop order
      if (GreaterNonNeg(r, mx)) {
        mx = r;
        mpos = pos0 * kNvMax + v;
      }
    }
  }
  // warp reduction over the solve's equations (the CTA lies in one block,
  // so the turbulence rows are uniform over it; without them their sums
  // stay zero); the sum order is fixed, so results are reproducible
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int v = 0; v < kNv; ++v) l2[v] += __shfl_down_sync(0xffffffffu, l2[v], off);
    if (sv.rans) {
#pragma unroll
      for (int v = kNv; v < kNvMax; ++v) l2[v] += __shfl_down_sync(0xffffffffu, l2[v], off);
    }
    const double om = __shfl_down_sync(0xffffffffu, mx, off);
    const int64_t op = __shfl_down_sync(0xffffffffu, mpos, off);
    // maxima are +0 or positive, so their bits order them
    if (Bits(om) > Bits(mx) || (Bits(om) == Bits(mx) && op < mpos)) {
      mx = om;
      mpos = op;
    }
    bad |= __shfl_down_sync(0xffffffffu, bad, off);
  }
  if (lane == 0) {
#pragma unroll
    for (int v = 0; v < kNvMax; ++v) s_l2[warp][v] = l2[v];
    s_max[warp] = mx;
    s_pos[warp] = mpos;
    s_bad[warp] = bad;
  }
  __syncthreads();
  if (warp != 0) return;
  // lane v of the first warp sums equation v over the warps in warp order
  double sum = 0.0;
  if (lane < (sv.rans ? kNvMax : kNv))
    for (int w = 0; w < kCta / 32; ++w) sum += s_l2[w][lane];
  double l2s[kNvMax];
#pragma unroll
  for (int v = 0; v < kNvMax; ++v) l2s[v] = __shfl_sync(0xffffffffu, sum, v);
  if (lane == 0) {
    NormPartial p;
    for (int v = 0; v < kNvMax; ++v) p.l2[v] = l2s[v];
    p.linf = 0.0;
    p.linf_pos = INT64_MAX;
    p.bad = 0;
    for (int w = 0; w < kCta / 32; ++w) {
      if (Bits(s_max[w]) > Bits(p.linf) ||
          (Bits(s_max[w]) == Bits(p.linf) && s_pos[w] < p.linf_pos)) {
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
// laminar viscosity of every listed cell (UpdateAuxillaryVariables,
// src/procBlock.cpp:6171); temperature is recomputed from W where needed
template <typename T>
__global__ void k_aux(Pools<T> P, const int32_t *cells, const int32_t *cell_block, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t c = cells[t];
  const SolveDev sv = P.solves[P.blocks[cell_block[t]].solve];
  if (!sv.active) return;
  const Gas<double> g = GasOf<double>(sv);
  const Prim<double> w = LoadW<double>(P.W, P.ncell, c);
  const double temp = Temperature(w, g);
  P.mu[c] = SutherlandRatio(temp, sv.t_ref, sv.mu_c1, sv.mu_s, sv.mu_ref);
  if (P.Taux) P.Taux[c] = temp;
}

// viscous flux on faces of direction D (procBlock::CalcViscFluxI/J/K,
// src/procBlock.cpp:1233,1556,1879): Green-Gauss gradients on the dual
// cell around the face (CalcGradsI/J/K :5173-5955, VectorGradGG/ScalarGradGG
// src/utility.cpp:59,138), central face state and viscosity, laminar
// viscousFlux::CalcFlux (src/viscousFlux.cpp:58) with TauNormal
// (src/utility.cpp:426)
// Face gradients of velocity and temperature on the dual cell around face c
// of direction D, central face state and face viscosity.
template <typename T, int D, typename PT>
__device__ __forceinline__ void ViscFaceGather(const Pools<PT> &P, const BlockDev &b,
                                               const Gas<T> &g, int64_t c, T grad[3][3],
                                               T tg[3], Prim<T> &fs, T &muf) {
  const int64_t n = P.ncell;
  const int64_t st[3] = {1, (int64_t)b.NI, (int64_t)b.NI * b.NJ};
  const int64_t cu = c, cl = c - st[D];
  const Prim<T> Wl = LoadW<T>(P.W, n, cl), Wu = LoadW<T>(P.W, n, cu);
  const T Tl = Temperature(Wl, g), Tu = Temperature(Wu, g);
  auto area = [&](int e, int64_t x, T a[3]) {
    const double *fa = P.fa[e];
    const T m = (T)fa[3 * n + x];
    a[0] = (T)fa[x] * m;
    a[1] = (T)fa[n + x] * m;
    a[2] = (T)fa[2 * n + x] * m;
  };
  T vlo[3][3], vhi[3][3], tlo[3], thi[3], alo[3][3], ahi[3][3];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    if (e == D) {
      vlo[e][0] = Wl.u; vlo[e][1] = Wl.v; vlo[e][2] = Wl.w;
      vhi[e][0] = Wu.u; vhi[e][1] = Wu.v; vhi[e][2] = Wu.w;
      tlo[e] = Tl;
      thi[e] = Tu;
      T A0[3], A1[3], A2[3];
      area(D, cu, A0);
      area(D, cu + st[D], A1);
      area(D, cl, A2);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        ahi[e][r] = T(0.5) * (A0[r] + A1[r]);
        alo[e][r] = T(0.5) * (A0[r] + A2[r]);
      }
    } else {
      const Prim<T> Wup = LoadW<T>(P.W, n, cu + st[e]), Wlp = LoadW<T>(P.W, n, cl + st[e]);
      const Prim<T> Wum = LoadW<T>(P.W, n, cu - st[e]), Wlm = LoadW<T>(P.W, n, cl - st[e]);
      vhi[e][0] = T(0.25) * (((Wl.u + Wu.u) + Wup.u) + Wlp.u);
      vhi[e][1] = T(0.25) * (((Wl.v + Wu.v) + Wup.v) + Wlp.v);
      vhi[e][2] = T(0.25) * (((Wl.w + Wu.w) + Wup.w) + Wlp.w);
      vlo[e][0] = T(0.25) * (((Wl.u + Wu.u) + Wum.u) + Wlm.u);
      vlo[e][1] = T(0.25) * (((Wl.v + Wu.v) + Wum.v) + Wlm.v);
      vlo[e][2] = T(0.25) * (((Wl.w + Wu.w) + Wum.w) + Wlm.w);
      thi[e] = T(0.25) * (((Tl + Tu) + Temperature(Wup, g)) + Temperature(Wlp, g));
      tlo[e] = T(0.25) * (((Tl + Tu) + Temperature(Wum, g)) + Temperature(Wlm, g));
      T Au[3], Al[3], Aup[3], Alp[3];
      area(e, cu, Au);
      area(e, cl, Al);
      area(e, cu + st[e], Aup);
      area(e, cl + st[e], Alp);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        ahi[e][r] = T(0.5) * (Aup[r] + Alp[r]);
        alo[e][r] = T(0.5) * (Au[r] + Al[r]);
      }
    }
  }
  const T vol = T(0.5) * ((T)P.vol[cl] + (T)P.vol[cu]);
  const T invVol = T(1) / vol;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int qv = 0; qv < 3; ++qv) {
      grad[r][qv] = vhi[0][qv] * ahi[0][r] - vlo[0][qv] * alo[0][r] +
                    vhi[1][qv] * ahi[1][r] - vlo[1][qv] * alo[1][r] +
                    vhi[2][qv] * ahi[2][r] - vlo[2][qv] * alo[2][r];
      grad[r][qv] *= invVol;
    }
    tg[r] = thi[0] * ahi[0][r] - tlo[0] * alo[0][r] + thi[1] * ahi[1][r] -
            tlo[1] * alo[1][r] + thi[2] * ahi[2][r] - tlo[2] * alo[2][r];
    tg[r] *= invVol;
  }
  // central face state and viscosity
  const double *wd = P.width[D];
  T cd, cw;
  CentralCoeffs((T)wd[cl], (T)wd[cu], cd, cw);
  fs.rho = cd * Wu.rho + cw * Wl.rho;
  fs.u = cd * Wu.u + cw * Wl.u;
  fs.v = cd * Wu.v + cw * Wl.v;
  fs.w = cd * Wu.w + cw * Wl.w;
  fs.p = cd * Wu.p + cw * Wl.p;
  muf = cd * (T)P.mu[cu] + cw * (T)P.mu[cl];
}

// Dual-cell Green-Gauss gradients of velocity and pressure at face c of
// direction D (procBlock::CalcGradsI/J/K, src/procBlock.cpp:5173: the
// velocity part of VectorGradGG and ScalarGradGG of the pressure), in the
// order of ViscFaceGather.
template <int D, typename PT>
__device__ __forceinline__ void FaceGradVP(const Pools<PT> &P, const BlockDev &b, int64_t c,
                                           double grad[3][3], double pg[3]) {
  const int64_t n = P.ncell;
  const int64_t st[3] = {1, (int64_t)b.NI, (int64_t)b.NI * b.NJ};
  const int64_t cu = c, cl = c - st[D];
  const Prim<double> Wl = LoadW<double>(P.W, n, cl), Wu = LoadW<double>(P.W, n, cu);
  auto area = [&](int e, int64_t x, double a[3]) {
    const double *fa = P.fa[e];
    const double m = fa[3 * n + x];
    a[0] = fa[x] * m;
    a[1] = fa[n + x] * m;
    a[2] = fa[2 * n + x] * m;
  };
  double vlo[3][3], vhi[3][3], plo[3], phi[3], alo[3][3], ahi[3][3];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    if (e == D) {
      vlo[e][0] = Wl.u; vlo[e][1] = Wl.v; vlo[e][2] = Wl.w;
      vhi[e][0] = Wu.u; vhi[e][1] = Wu.v; vhi[e][2] = Wu.w;
      plo[e] = Wl.p;
      phi[e] = Wu.p;
      double A0[3], A1[3], A2[3];
      area(D, cu, A0);
      area(D, cu + st[D], A1);
      area(D, cl, A2);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        ahi[e][r] = 0.5 * (A0[r] + A1[r]);
        alo[e][r] = 0.5 * (A0[r] + A2[r]);
      }
    } else {
      const Prim<double> Wup = LoadW<double>(P.W, n, cu + st[e]),
                         Wlp = LoadW<double>(P.W, n, cl + st[e]);
      const Prim<double> Wum = LoadW<double>(P.W, n, cu - st[e]),
                         Wlm = LoadW<double>(P.W, n, cl - st[e]);
      vhi[e][0] = 0.25 * (((Wl.u + Wu.u) + Wup.u) + Wlp.u);
      vhi[e][1] = 0.25 * (((Wl.v + Wu.v) + Wup.v) + Wlp.v);
      vhi[e][2] = 0.25 * (((Wl.w + Wu.w) + Wup.w) + Wlp.w);
      vlo[e][0] = 0.25 * (((Wl.u + Wu.u) + Wum.u) + Wlm.u);
      vlo[e][1] = 0.25 * (((Wl.v + Wu.v) + Wum.v) + Wlm.v);
      vlo[e][2] = 0.25 * (((Wl.w + Wu.w) + Wum.w) + Wlm.w);
      phi[e] = 0.25 * (((Wl.p + Wu.p) + Wup.p) + Wlp.p);
      plo[e] = 0.25 * (((Wl.p + Wu.p) + Wum.p) + Wlm.p);
      double Au[3], Al[3], Aup[3], Alp[3];
      area(e, cu, Au);
      area(e, cl, Al);
      area(e, cu + st[e], Aup);
      area(e, cl + st[e], Alp);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        ahi[e][r] = 0.5 * (Aup[r] + Alp[r]);
        alo[e][r] = 0.5 * (Au[r] + Al[r]);
      }
    }
  }
  const double vol = 0.5 * (P.vol[cl] + P.vol[cu]);
  const double invVol = 1.0 / vol;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int qv = 0; qv < 3; ++qv) {
      grad[r][qv] = vhi[0][qv] * ahi[0][r] - vlo[0][qv] * alo[0][r] +
                    vhi[1][qv] * ahi[1][r] - vlo[1][qv] * alo[1][r] +
                    vhi[2][qv] * ahi[2][r] - vlo[2][qv] * alo[2][r];
      grad[r][qv] *= invVol;
    }
    pg[r] = phi[0] * ahi[0][r] - plo[0] * alo[0][r] + phi[1] * ahi[1][r] -
            plo[1] * alo[1][r] + phi[2] * ahi[2][r] - plo[2] * alo[2][r];
    pg[r] *= invVol;
  }
}

// Cell-averaged velocity and pressure gradients (one sixth of each face's,
// faces in the order i low, i high, j low, ..., as procBlock::CalcGradsI/J/K
// and CalcViscFluxI/J/K accumulate them, src/procBlock.cpp:5790) of the
// cells whose ghosts a nonreflecting pressure outlet fills; they are read
// at the next iteration's ghost fill, as the reference reads the previous
// residual's gradients.
template <typename T>
__global__ void k_nr_grads(Pools<T> P, const int32_t *cells, const int32_t *cell_block, int ncl) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncl) return;
  const int64_t c = cells[t];
  const BlockDev b = P.blocks[cell_block[t]];
  if (!P.solves[b.solve].active) return;
  const int64_t n = P.ncell;
  const int64_t st[3] = {1, (int64_t)b.NI, (int64_t)b.NI * b.NJ};
  const double sixth = 1.0 / 6.0;
  double vg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, pg[3] = {0, 0, 0};
  auto add = [&](const double grad[3][3], const double p[3]) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int q = 0; q < 3; ++q) vg[r * 3 + q] += sixth * grad[r][q];
      pg[r] += sixth * p[r];
    }
  };
  double grad[3][3], p[3];
  FaceGradVP<0>(P, b, c, grad, p);
  add(grad, p);
  FaceGradVP<0>(P, b, c + st[0], grad, p);
  add(grad, p);
  FaceGradVP<1>(P, b, c, grad, p);
  add(grad, p);
  FaceGradVP<1>(P, b, c + st[1], grad, p);
  add(grad, p);
  FaceGradVP<2>(P, b, c, grad, p);
  add(grad, p);
  FaceGradVP<2>(P, b, c + st[2], grad, p);
  add(grad, p);
#pragma unroll
  for (int e = 0; e < 9; ++e) P.nrg[e * n + c] = vg[e];
#pragma unroll
  for (int e = 0; e < 3; ++e) P.nrg[(9 + e) * n + c] = pg[e];
}

// Green-Gauss gradients at a face of direction D (upper cell c) of the NS
// cell scalars u, v, w, T, rho, p and, for RANS, k, omega over the dual
// cell (procBlock::CalcGradsI/J/K, src/procBlock.cpp:5173-5790): the
// scalars at the dual cell's lower and upper faces of the other directions
// are four-cell averages summed in the reference's order; temperature from
// the state, p / (rho R) (src/eos.cpp:100).
template <int D, int NS, typename PT>
__device__ __forceinline__ void FaceGradAll(const Pools<PT> &P, const BlockDev &b,
                                            const SolveDev &sv, int64_t c, double grad[NS][3]) {
  const int64_t n = P.ncell;
  const int64_t st[3] = {1, (int64_t)b.NI, (int64_t)b.NI * b.NJ};
  const int64_t cu = c, cl = c - st[D];
  auto load = [&](int64_t x, double s[NS]) {
    s[0] = P.W[n + x];
    s[1] = P.W[2 * n + x];
    s[2] = P.W[3 * n + x];
    const double rho = P.W[x], p = P.W[4 * n + x];
    s[3] = p / (0.0 + rho * sv.gas_r);
    s[4] = rho;
    s[5] = p;
    if constexpr (NS > 6) {
      s[6] = P.Wt[x];
      s[7] = P.Wt[n + x];
    }
  };
  auto area = [&](int e, int64_t x, double a[3]) {
    const double *fa = P.fa[e];
    const double m = fa[3 * n + x];
    a[0] = fa[x] * m;
    a[1] = fa[n + x] * m;
    a[2] = fa[2 * n + x] * m;
  };
  double sl[NS], su[NS];
  load(cl, sl);
  load(cu, su);
  double lo[3][NS], hi[3][NS], alo[3][3], ahi[3][3];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    if (e == D) {
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        lo[e][k] = sl[k];
        hi[e][k] = su[k];
      }
      double A0[3], A1[3], A2[3];
      area(D, cu, A0);
      area(D, cu + st[D], A1);
      area(D, cl, A2);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        ahi[e][r] = 0.5 * (A0[r] + A1[r]);
        alo[e][r] = 0.5 * (A0[r] + A2[r]);
      }
    } else {
      double sup[NS], slp[NS], sum[NS], slm[NS];
      load(cu + st[e], sup);
      load(cl + st[e], slp);
      load(cu - st[e], sum);
      load(cl - st[e], slm);
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        hi[e][k] = 0.25 * (((sl[k] + su[k]) + sup[k]) + slp[k]);
        lo[e][k] = 0.25 * (((sl[k] + su[k]) + sum[k]) + slm[k]);
      }
      double Au[3], Al[3], Aup[3], Alp[3];
      area(e, cu, Au);
      area(e, cl, Al);
      area(e, cu + st[e], Aup);
      area(e, cl + st[e], Alp);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        ahi[e][r] = 0.5 * (Aup[r] + Alp[r]);
        alo[e][r] = 0.5 * (Au[r] + Al[r]);
      }
    }
  }
  const double vol = 0.5 * (P.vol[cl] + P.vol[cu]);
  const double invVol = 1.0 / vol;
#pragma unroll
  for (int k = 0; k < NS; ++k)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double g = hi[0][k] * ahi[0][r] - lo[0][k] * alo[0][r] + hi[1][k] * ahi[1][r] -
                 lo[1][k] * alo[1][r] + hi[2][k] * ahi[2][r] - lo[2][k] * alo[2][r];
      grad[k][r] = g * invVol;
    }
}

// Cell-averaged gradients of the last residual kept for output (the
// reference's velocityGrad_, temperatureGrad_, densityGrad_, pressureGrad_,
// tkeGrad_, omegaGrad_: one sixth of each face's, faces i low, i high, j
// low, ...; written by WriteFunFile, src/output.cpp:309-395) of every
// physical cell: P.ogr [24][ncell] = velocity gradient (9, row = derivative
// axis), T, rho, p, k, omega gradients (3 each; k, omega zero without RANS).
template <typename T, bool RANS>
__global__ void __launch_bounds__(kCta) k_out_grads(Pools<T> P, const int32_t *list,
                                                    const int32_t *cta_block) {
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  if (c < 0) return;
  const BlockDev b = P.blocks[cta_block[blockIdx.x]];
  const SolveDev sv = P.solves[b.solve];
  if (!sv.active || (sv.rans != 0) != RANS) return;
  constexpr int NS = RANS ? 8 : 6;
  const int64_t n = P.ncell;
  const int64_t st[3] = {1, (int64_t)b.NI, (int64_t)b.NI * b.NJ};
  const double sixth = 1.0 / 6.0;
  double acc[8][3];  // k, omega stay zero without RANS
#pragma unroll
  for (int k = 0; k < 8; ++k) acc[k][0] = acc[k][1] = acc[k][2] = 0.0;
  double g[NS][3];
  auto add = [&]() {
#pragma unroll
    for (int k = 0; k < NS; ++k)
#pragma unroll
      for (int r = 0; r < 3; ++r) acc[k][r] += sixth * g[k][r];
  };
  FaceGradAll<0, NS>(P, b, sv, c, g);
  add();
  FaceGradAll<0, NS>(P, b, sv, c + st[0], g);
  add();
  FaceGradAll<1, NS>(P, b, sv, c, g);
  add();
  FaceGradAll<1, NS>(P, b, sv, c + st[1], g);
  add();
  FaceGradAll<2, NS>(P, b, sv, c, g);
  add();
  FaceGradAll<2, NS>(P, b, sv, c + st[2], g);
  add();
  double *o = P.ogr;
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int q = 0; q < 3; ++q) o[(r * 3 + q) * n + c] = acc[q][r];
#pragma unroll
  for (int k = 3; k < 8; ++k)
#pragma unroll
    for (int r = 0; r < 3; ++r) o[(9 + (k - 3) * 3 + r) * n + c] = acc[k][r];
}

// Mixed-precision version of ViscFaceGather: velocities and temperatures
// enter the dual-cell sums as offsets from the upper cell's values, formed
// in FP64 (the temperature offset as (p rho_u - p_u rho) / (rho rho_u R)),
// so that the FP32 sums carry rounding relative to the differences across
// the dual cell rather than to the values; the dual cell is closed, so the
// offsets leave the gradients unchanged.  Face state and viscosity in FP32.
template <int D, typename PT>
__device__ __forceinline__ void ViscFaceGatherMixed(const Pools<PT> &P, const BlockDev &b,
                                                    const SolveDev &sv, int64_t c,
                                                    float grad[3][3], float tg[3],
                                                    Prim<float> &fs, float &muf) {
  const int64_t n = P.ncell;
  const int64_t st[3] = {1, (int64_t)b.NI, (int64_t)b.NI * b.NJ};
  const int64_t cu = c, cl = c - st[D];
  const Prim<double> Wu = LoadW<double>(P.W, n, cu), Wl = LoadW<double>(P.W, n, cl);
  const float rgas = (float)sv.gas_r;
  auto rel = [&](const Prim<double> &w, float o[4]) {
    o[0] = (float)(w.u - Wu.u);
    o[1] = (float)(w.v - Wu.v);
    o[2] = (float)(w.w - Wu.w);
    o[3] = (float)(w.p * Wu.rho - Wu.p * w.rho) / ((float)w.rho * (float)Wu.rho * rgas);
  };
  auto area = [&](int e, int64_t x, float a[3]) {
    const double *fa = P.fa[e];
    const float m = (float)fa[3 * n + x];
    a[0] = (float)fa[x] * m;
    a[1] = (float)fa[n + x] * m;
    a[2] = (float)fa[2 * n + x] * m;
  };
  float ol[4], ou[4] = {0.f, 0.f, 0.f, 0.f};
  rel(Wl, ol);
  float vlo[3][4], vhi[3][4], alo[3][3], ahi[3][3];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    if (e == D) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        vlo[e][k] = ol[k];
        vhi[e][k] = ou[k];
      }
      float A0[3], A1[3], A2[3];
      area(D, cu, A0);
      area(D, cu + st[D], A1);
      area(D, cl, A2);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        ahi[e][r] = 0.5f * (A0[r] + A1[r]);
        alo[e][r] = 0.5f * (A0[r] + A2[r]);
      }
    } else {
      float oup[4], olp[4], oum[4], olm[4];
      rel(LoadW<double>(P.W, n, cu + st[e]), oup);
      rel(LoadW<double>(P.W, n, cl + st[e]), olp);
      rel(LoadW<double>(P.W, n, cu - st[e]), oum);
      rel(LoadW<double>(P.W, n, cl - st[e]), olm);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        vhi[e][k] = 0.25f * (((ol[k] + ou[k]) + oup[k]) + olp[k]);
        vlo[e][k] = 0.25f * (((ol[k] + ou[k]) + oum[k]) + olm[k]);
      }
      float Au[3], Al[3], Aup[3], Alp[3];
      area(e, cu, Au);
      area(e, cl, Al);
      area(e, cu + st[e], Aup);
      area(e, cl + st[e], Alp);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        ahi[e][r] = 0.5f * (Aup[r] + Alp[r]);
        alo[e][r] = 0.5f * (Au[r] + Al[r]);
      }
    }
  }
  const float invVol = 1.f / (0.5f * ((float)P.vol[cl] + (float)P.vol[cu]));
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int qv = 0; qv < 3; ++qv)
      grad[r][qv] = (vhi[0][qv] * ahi[0][r] - vlo[0][qv] * alo[0][r] +
                     vhi[1][qv] * ahi[1][r] - vlo[1][qv] * alo[1][r] +
                     vhi[2][qv] * ahi[2][r] - vlo[2][qv] * alo[2][r]) *
                    invVol;
    tg[r] = (vhi[0][3] * ahi[0][r] - vlo[0][3] * alo[0][r] + vhi[1][3] * ahi[1][r] -
             vlo[1][3] * alo[1][r] + vhi[2][3] * ahi[2][r] - vlo[2][3] * alo[2][r]) *
            invVol;
  }
  const double *wd = P.width[D];
  float cd, cw;
  CentralCoeffs((float)wd[cl], (float)wd[cu], cd, cw);
  fs.rho = cd * (float)Wu.rho + cw * (float)Wl.rho;
  fs.u = cd * (float)Wu.u + cw * (float)Wl.u;
  fs.v = cd * (float)Wu.v + cw * (float)Wl.v;
  fs.w = cd * (float)Wu.w + cw * (float)Wl.w;
  fs.p = cd * (float)Wu.p + cw * (float)Wl.p;
  muf = cd * (float)P.mu[cu] + cw * (float)P.mu[cl];
}

// Dual-cell Green-Gauss gradients of k and omega at face c of direction D
// (ScalarGradGG, src/utility.cpp:138): values on the dual faces are the
// cells themselves along D and 4-cell averages across
template <int D, typename PT>
__device__ __forceinline__ void TurbFaceGrads(const Pools<PT> &P, const BlockDev &b, int64_t c,
                                              double kg[3], double wg[3]) {
  const int64_t n = P.ncell;
  const int64_t st[3] = {1, (int64_t)b.NI, (int64_t)b.NI * b.NJ};
  const int64_t cu = c, cl = c - st[D];
  auto area = [&](int e, int64_t x, double a[3]) {
    const double *fa = P.fa[e];
    const double m = fa[3 * n + x];
    a[0] = fa[x] * m;
    a[1] = fa[n + x] * m;
    a[2] = fa[2 * n + x] * m;
  };
  double lo[3][2], hi[3][2], alo[3][3], ahi[3][3];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const double *T_ = P.Wt + q * n;
      if (e == D) {
        lo[e][q] = T_[cl];
        hi[e][q] = T_[cu];
      } else {
        hi[e][q] = 0.25 * (((T_[cl] + T_[cu]) + T_[cu + st[e]]) + T_[cl + st[e]]);
        lo[e][q] = 0.25 * (((T_[cl] + T_[cu]) + T_[cu - st[e]]) + T_[cl - st[e]]);
      }
    }
    if (e == D) {
      double A0[3], A1[3], A2[3];
      area(D, cu, A0);
      area(D, cu + st[D], A1);
      area(D, cl, A2);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        ahi[e][r] = 0.5 * (A0[r] + A1[r]);
        alo[e][r] = 0.5 * (A0[r] + A2[r]);
      }
    } else {
      double Au[3], Al[3], Aup[3], Alp[3];
      area(e, cu, Au);
      area(e, cl, Al);
      area(e, cu + st[e], Aup);
      area(e, cl + st[e], Alp);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        ahi[e][r] = 0.5 * (Aup[r] + Alp[r]);
        alo[e][r] = 0.5 * (Au[r] + Al[r]);
      }
    }
  }
  const double invVol = 1.0 / (0.5 * (P.vol[cl] + P.vol[cu]));
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    kg[r] = hi[0][0] * ahi[0][r] - lo[0][0] * alo[0][r] + hi[1][0] * ahi[1][r] -
            lo[1][0] * alo[1][r] + hi[2][0] * ahi[2][r] - lo[2][0] * alo[2][r];
    kg[r] *= invVol;
    wg[r] = hi[0][1] * ahi[0][r] - lo[0][1] * alo[0][r] + hi[1][1] * ahi[1][r] -
            lo[1][1] * alo[1][r] + hi[2][1] * ahi[2][r] - lo[2][1] * alo[2][r];
    wg[r] *= invVol;
  }
}

// Viscous face of a RANS solve (CalcViscFluxI/J/K with SST, in FP64): eddy viscosity and blending from the central face
// state (turbulence floors applied), the face gradients and the central
// wall distance (clipped to 0 within WALL_DIST_NEG_TOL); flow flux with
// mu + mut and the turbulent conductivity, k and omega diffusion fluxes.
// Stores the flux, the per-face SST data and (block solves) the face state.
template <typename T, int D>
__device__ __forceinline__ void RansViscFace(Pools<T> &P, const BlockDev &b, const SolveDev &sv,
                                             int64_t c) {
  const Gas<double> g = GasOf<double>(sv);
  const int64_t n = P.ncell;
  double grad[3][3], tg[3], muf;
  Prim<double> fs;
  ViscFaceGather<double, D>(P, b, g, c, grad, tg, fs, muf);
  double kg[3], wg[3];
  TurbFaceGrads<D>(P, b, c, kg, wg);
  const int64_t cu = c, cl = c - StrideOf(b, D);
  const double *wd = P.width[D];
  double cd, cw;
  CentralCoeffs(wd[cl], wd[cu], cd, cw);
  double fst[2];
#pragma unroll
  for (int q = 0; q < 2; ++q)
    fst[q] = CMax(cd * P.Wt[q * n + cu] + cw * P.Wt[q * n + cl], kTurbMin);
  double wdf = cd * P.wd[cu] + cw * P.wd[cl];
  if (wdf < 0.0 && wdf > -1.0e-10) wdf = 0.0;
  const double scale = sv.visc_scale;
  const double vg[9] = {grad[0][0], grad[0][1], grad[0][2], grad[1][0], grad[1][1],
                        grad[1][2], grad[2][0], grad[2][1], grad[2][2]};
  double mutf, f1f, f2f;
  if (sv.wilcox) {
    // turbKWWilcox::EddyViscAndBlending (src/turbulence.cpp:412)
    mutf = WkEddyVisc(fs, fst, vg, scale);
    f1f = 1.0;
    f2f = 0.0;
  } else {
    SstEddyVisc<double>(fs, fst, vg, kg, wg, muf, wdf, scale, mutf, f1f, f2f);
  }
  // the face state's unlimited eddy viscosity (Wilcox: turbulence diffusion
  // and the 2x2 viscous Jacobian)
  const double nutf = sv.wilcox ? fs.rho * fst[0] / fst[1] : 0.0;
  const double *fa = P.fa[D];
  const double nx = fa[c], ny = fa[n + c], nz = fa[2 * n + c], mag = fa[3 * n + c];
  const double mus = scale * muf, muts = scale * mutf;
  double tau[3];
  TauNormal(vg, nx, ny, nz, mus, muts, tau);
  const double kf = SutherlandRatio(Temperature(fs, g), sv.t_ref, sv.k_c1, sv.k_s, sv.k_ref) *
                    scale;
  const double kt = muts * g.Cp() / PrtOf(sv);
  double F[5];
  F[0] = 0.0;
  F[1] = tau[0];
  F[2] = tau[1];
  F[3] = tau[2];
  F[4] = Dot(tau[0], tau[1], tau[2], fs.u, fs.v, fs.w) +
         (kf + kt) * Dot(tg[0], tg[1], tg[2], nx, ny, nz) + 0.0;
  // viscousFlux::CalcFlux (src/viscousFlux.cpp:118-133): Wilcox 2006 takes
  // the unlimited eddy viscosity in the turbulence diffusion
  const double mutt = sv.wilcox ? scale * nutf : muts;
  const double sk = sv.wilcox ? kWkSigmaStar : Blended(kSstSigmaK1, kSstSigmaK2, f1f);
  const double sw = sv.wilcox ? kWkSigma : Blended(kSstSigmaW1, kSstSigmaW2, f1f);
  const double Ft0 = (mus + sk * mutt) * Dot(kg[0], kg[1], kg[2], nx, ny, nz);
  const double Ft1 = (mus + sw * mutt) * Dot(wg[0], wg[1], wg[2], nx, ny, nz);
  T *out = P.vflux[D];
#pragma unroll
  for (int v = 0; v < 5; ++v) out[v * n + c] = (T)(F[v] * mag);
  P.vfluxt[D][c] = (T)(Ft0 * mag);
  P.vfluxt[D][n + c] = (T)(Ft1 * mag);
  T *rs = P.rst[D];
#pragma unroll
  for (int e = 0; e < 9; ++e) rs[e * n + c] = (T)vg[e];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    rs[(9 + e) * n + c] = (T)kg[e];
    rs[(12 + e) * n + c] = (T)wg[e];
  }
  rs[15 * n + c] = (T)mutf;
  rs[16 * n + c] = (T)f1f;
  rs[18 * n + c] = (T)nutf;
  rs[17 * n + c] = (T)f2f;
  if (sv.block) {
    T *vs = P.vst[D];
    vs[0 * n + c] = (T)fs.rho;
    vs[1 * n + c] = (T)fs.u;
    vs[2 * n + c] = (T)fs.v;
    vs[3 * n + c] = (T)fs.w;
    vs[4 * n + c] = (T)fs.p;
    vs[5 * n + c] = (T)muf;
#pragma unroll
    for (int e = 0; e < 9; ++e) vs[(6 + e) * n + c] = (T)vg[e];
  }
}

template <typename T, int D, bool RANS>
__global__ void __launch_bounds__(kCta) k_vface(Pools<T> P, const int32_t *list,
                                                const int32_t *cta_block) {
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  if (c < 0) return;
  const BlockDev b = P.blocks[cta_block[blockIdx.x]];
  const SolveDev sv = P.solves[b.solve];
  if (!sv.viscous || !sv.active || (sv.rans != 0) != RANS) return;
  if constexpr (RANS) {
    // in FP64 for both precisions: near walls the k and omega diffusion
    // fluxes of a cell's two faces are large and nearly cancel, so FP32
    // rounding of the flux itself moves the converged k and omega by ~1e-4
    // (measured against FP64 on an SST bump channel)
    RansViscFace<T, D>(P, b, sv, c);
    return;
  }
  const Gas<T> g = GasOf<T>(sv);
  const int64_t n = P.ncell;
  T grad[3][3], tg[3];
  Prim<T> fs;
  T muf;
  if constexpr (std::is_same<T, float>::value)
    ViscFaceGatherMixed<D>(P, b, sv, c, grad, tg, fs, muf);
  else
    ViscFaceGather<T, D>(P, b, g, c, grad, tg, fs, muf);
  const double *fa = P.fa[D];
  const T nx = (T)fa[c], ny = (T)fa[n + c], nz = (T)fa[2 * n + c], mag = (T)fa[3 * n + c];
  const T nrm[3] = {nx, ny, nz};
  const T scale = (T)sv.visc_scale;
  const T mus = scale * muf, muts = scale * T(0);
  const T lambda = T(0) - (T(2) / T(3)) * (mus + muts);
  const T trace = grad[0][0] + grad[1][1] + grad[2][2];
  T tau[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const T sn = (grad[r][0] + grad[0][r]) * nrm[0] + (grad[r][1] + grad[1][r]) * nrm[1] +
                 (grad[r][2] + grad[2][r]) * nrm[2];
    tau[r] = lambda * trace * nrm[r] + (mus + muts) * sn;
  }
  const T tf = Temperature(fs, g);
  const T kf = SutherlandRatio(tf, (T)sv.t_ref, (T)sv.k_c1, (T)sv.k_s, (T)sv.k_ref) * scale;
  const T kt = muts * g.Cp() / T(0.9);
  T F[5];
  F[0] = T(0);
  F[1] = tau[0];
  F[2] = tau[1];
  F[3] = tau[2];
  F[4] = Dot(tau[0], tau[1], tau[2], fs.u, fs.v, fs.w) +
         (kf + kt) * Dot(tg[0], tg[1], tg[2], nx, ny, nz) + T(0);
  T *out = P.vflux[D];
#pragma unroll
  for (int v = 0; v < 5; ++v) out[v * n + c] = F[v] * mag;
  if (sv.block) {
    // face state, viscosity and gradient for the block diagonal's
    // thin-shear-layer Jacobians and the cell-averaged gradients
    T *vs = P.vst[D];
    vs[0 * n + c] = fs.rho;
    vs[1 * n + c] = fs.u;
    vs[2 * n + c] = fs.v;
    vs[3 * n + c] = fs.w;
    vs[4 * n + c] = fs.p;
    vs[5 * n + c] = muf;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int qv = 0; qv < 3; ++qv) vs[(6 + r * 3 + qv) * n + c] = grad[r][qv];
  }
}

// ---------------------------------------------------------------------------
// Wall data of the viscous-wall faces (viscousFlux::CalcWallFlux,
// src/viscousFlux.cpp:137; wallData::WallPressure src/wallData.cpp:140),
// always in FP64: per face p_w A (area vector) and tau_w |A|.
template <typename T>
__global__ void k_wall(Pools<T> P, const WallFaceDev *faces, int nfaces, double *wbuf) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nfaces) return;
  const WallFaceDev wf = faces[t];
  const BlockDev b = P.blocks[wf.block];
  const SolveDev sv = P.solves[b.solve];
  const Gas<double> g = GasOf<double>(sv);
  const int64_t n = P.ncell, c = wf.face;
  double grad[3][3], tg[3], muf;
  Prim<double> fs;
  if (wf.dir == 0) ViscFaceGather<double, 0>(P, b, g, c, grad, tg, fs, muf);
  else if (wf.dir == 1) ViscFaceGather<double, 1>(P, b, g, c, grad, tg, fs, muf);
  else ViscFaceGather<double, 2>(P, b, g, c, grad, tg, fs, muf);
  const double *fa = P.fa[wf.dir];
  const double nx = fa[c], ny = fa[n + c], nz = fa[2 * n + c], mag = fa[3 * n + c];
  // RANS: the face eddy viscosity of the viscous flux kernel
  const double mutf = sv.rans ? (double)P.rst[wf.dir][15 * n + c] : 0.0;
  const double mus = sv.visc_scale * muf, muts = sv.visc_scale * mutf;
  const double vg[9] = {grad[0][0], grad[0][1], grad[0][2], grad[1][0], grad[1][1],
                        grad[1][2], grad[2][0], grad[2][1], grad[2][2]};
  double tau[3];
  TauNormal(vg, nx, ny, nz, mus, muts, tau);
  const double pw = fs.rho * g.r * Temperature(fs, g);
  wbuf[0 * (int64_t)nfaces + t] = pw * nx * mag;
  wbuf[1 * (int64_t)nfaces + t] = pw * ny * mag;
  wbuf[2 * (int64_t)nfaces + t] = pw * nz * mag;
  wbuf[3 * (int64_t)nfaces + t] = tau[0] * mag;
  wbuf[4 * (int64_t)nfaces + t] = tau[1] * mag;
  wbuf[5 * (int64_t)nfaces + t] = tau[2] * mag;
}

// ---------------------------------------------------------------------------
// logged matrix residual
template <typename T, bool BLOCK>
__global__ void __launch_bounds__(kCta) k_matres(Pools<T> P, const int32_t *list,
                                                 const int32_t *cta_block,
                                                 double *mres_partials, int forcing) {
  __shared__ double s_sum[kCta / 32];
  const BlockDev b = P.blocks[cta_block[blockIdx.x]];
  const SolveDev sv = P.solves[b.solve];
  if ((sv.block != 0) != BLOCK) return;
  const int32_t c = list[blockIdx.x * kCta + threadIdx.x];
  double sum = 0.0;
  if (c >= 0) {
    const Gas<T> g = GasOf<T>(sv);
    const int64_t q = P.qpos[c], nq = P.nq;
    const int nv = sv.rans ? 7 : 5;
    T L[7], U[7], Ax[7], x[7], bt[7];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      x[v] = P.dUq[v * nq + q];
      bt[v] = P.Rq[v * nq + q];
    }
    x[5] = x[6] = bt[5] = bt[6] = T(0);
    if (sv.rans)
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        x[5 + v] = P.dUtq[v * nq + q];
        bt[5 + v] = P.Rtq[v * nq + q];
      }
    if constexpr (BLOCK) {
      OffDiagSumBlock(P, sv, q, true, L, L + 5);
      OffDiagSumBlock(P, sv, q, false, U, U + 5);
      T A[kJac];
#pragma unroll
      for (int e = 0; e < kJac; ++e) A[e] = P.Aq[e * nq + q];
      MatVec5(A, x, Ax);
      if (sv.rans) {
        T At[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) At[e] = P.Atq[e * nq + q];
        MatVec2(At, x + 5, Ax + 5);
      }
    } else {
      OffDiagSum(P, g, sv, q, true, L, L + 5);
      OffDiagSum(P, g, sv, q, false, U, U + 5);
      const T a = P.Aq[q];
#pragma unroll
      for (int v = 0; v < 5; ++v) Ax[v] = x[v] * a;
      if (sv.rans) {
        const T at = P.Atq[q];
        Ax[5] = x[5] * at;
        Ax[6] = x[6] * at;
      }
    }
    const T thetaInv = (T)sv.theta_inv;
#pragma unroll
    for (int v = 0; v < 7; ++v) {
      if (v >= nv) break;
      const T off = L[v] - U[v];
      const T bv = RhsB0(P, sv, thetaInv, v, q);
      const T axmb = Ax[v] - off - bv;
      if (forcing) {
        // a coarse level's forcing: A x - b of the restricted update plus
        // the restricted fine matrix residual already in Fq
        // (gridLevel::Restriction src/gridLevel.cpp:571-589)
        if (v < 5) P.Fq[v * nq + q] = axmb + P.Fq[v * nq + q];
        continue;
      }
      // linearSolver::Residual (src/linearSolver.cpp:92): f - (A x - b)
      const T f = (P.Fq && v < 5) ? P.Fq[v * nq + q] : T(0);
      const T rt = f - axmb;
      if (P.MRq && v < 5) P.MRq[v * nq + q] = rt;
      const double r = (double)rt;
      sum += r * r;
    }
  }
  if (forcing) return;
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
                       double *mres_partials, int ncta, int kinds, cudaStream_t s) {
  if (ncta <= 0) return;
  if (kinds & 1) k_matres<T, false><<<ncta, kCta, 0, s>>>(P, list, cta_block, mres_partials, 0);
  if (kinds & 2) k_matres<T, true><<<ncta, kCta, 0, s>>>(P, list, cta_block, mres_partials, 0);
}
template <typename T>
void Launch<T>::MgForcing(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                          int ncta, int kinds, cudaStream_t s) {
  if (ncta <= 0) return;
  if (kinds & 1) k_matres<T, false><<<ncta, kCta, 0, s>>>(P, list, cta_block, nullptr, 1);
  if (kinds & 2) k_matres<T, true><<<ncta, kCta, 0, s>>>(P, list, cta_block, nullptr, 1);
}

// ---------------------------------------------------------------------------
// Multigrid transfers (gridLevel::Restriction / Prolongation,
// src/gridLevel.cpp:538-611; BlockRestriction include/procBlock.hpp:637-690;
// BlockProlongation include/gridLevel.hpp:160).  Every coarse value is a sum
// from zero over its fine cells in the fine k, j, i order, as the
// reference's loop adds them.
template <typename U, bool WEIGHTED>
__global__ void k_mg_gather(MgLinkDev k, const U *src, int64_t src_n, bool src_pool, U *dst,
                            int64_t dst_n, bool dst_pool) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k.ncoarse) return;
  const int e0 = k.off[c], e1 = k.off[c + 1];
  const int64_t dc = dst_pool ? k.c_pool[c] : k.c_q[c];
#pragma unroll 1
  for (int v = 0; v < 5; ++v) {
    U acc = U(0);
    for (int e = e0; e < e1; ++e) {
      const int64_t sc = src_pool ? k.f_pool[e] : k.f_q[e];
      const U x = src[v * src_n + sc];
      const U t = WEIGHTED ? (U)k.f_w[e] * x : x;
      acc = acc + t;
    }
    dst[v * dst_n + dc] = acc;
  }
}

template <typename T>
__global__ void k_mg_sub(T *x, const T *x0, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = x[i] - x0[i];
}

// ConvertCellToNode without ghosts (include/utility.hpp:187): each node the
// sum of its cells, times 1 (block corners), 1/2 (block edges) or 1/8
template <typename T>
__global__ void k_mg_nodes(MgLinkDev k, const T *du, int64_t nq, T *nodes) {
  const int nd = blockIdx.x * blockDim.x + threadIdx.x;
  if (nd >= k.nnode) return;
  const int32_t *cl = k.node_cells + 8 * (int64_t)nd;
  const T f = (T)k.node_fac[nd];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    T acc = T(0);
#pragma unroll
    for (int e = 0; e < 8; ++e)
      if (cl[e] >= 0) acc = acc + du[v * nq + cl[e]];
    nodes[v * (int64_t)k.nnode + nd] = acc * f;
  }
}

// TrilinearInterp (include/utility.hpp:357) of the coarse correction at the
// fine cell centre, added to the fine update (linearSolver::AddToUpdate)
template <typename T>
__device__ __forceinline__ T MgLin(T d0, T d1, T c) { return (T(1) - c) * d0 + c * d1; }
template <typename T>
__global__ void k_mg_prolong(MgLinkDev k, const T *nodes, T *du, int64_t nq) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= k.nfine) return;
  const int64_t n0 = k.p_node0[e], sx = k.p_sx[e], sxy = k.p_sxy[e];
  const int64_t id[8] = {n0,           n0 + 1,           n0 + sx,       n0 + sx + 1,
                         n0 + sxy,     n0 + sxy + 1,     n0 + sxy + sx, n0 + sxy + sx + 1};
  T co[7];
#pragma unroll
  for (int a = 0; a < 7; ++a) co[a] = (T)k.p_coef[a * (int64_t)k.nfine + e];
  const int64_t fq = k.p_q[e];
  const int64_t nn = k.nnode;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const T *nv = nodes + v * nn;
    const T d04 = MgLin(nv[id[0]], nv[id[4]], co[0]);
    const T d15 = MgLin(nv[id[1]], nv[id[5]], co[1]);
    const T d26 = MgLin(nv[id[2]], nv[id[6]], co[2]);
    const T d37 = MgLin(nv[id[3]], nv[id[7]], co[3]);
    const T d0415 = MgLin(d04, d15, co[4]);
    const T d2637 = MgLin(d26, d37, co[5]);
    du[v * nq + fq] = du[v * nq + fq] + MgLin(d0415, d2637, co[6]);
  }
}

template <typename T>
void Launch<T>::MgRestrictState(const MgLinkDev &k, const double *fineW, int64_t fine_n,
                                double *coarseW, int64_t coarse_n, cudaStream_t s) {
  if (k.ncoarse <= 0) return;
  k_mg_gather<double, true><<<(k.ncoarse + 127) / 128, 128, 0, s>>>(k, fineW, fine_n, true,
                                                                    coarseW, coarse_n, true);
}
template <typename T>
void Launch<T>::MgRestrictQ(const MgLinkDev &k, const T *fine, int64_t fine_nq, T *coarse,
                            int64_t coarse_nq, bool weighted, cudaStream_t s) {
  if (k.ncoarse <= 0) return;
  if (weighted)
    k_mg_gather<T, true><<<(k.ncoarse + 127) / 128, 128, 0, s>>>(k, fine, fine_nq, false,
                                                                 coarse, coarse_nq, false);
  else
    k_mg_gather<T, false><<<(k.ncoarse + 127) / 128, 128, 0, s>>>(k, fine, fine_nq, false,
                                                                  coarse, coarse_nq, false);
}
template <typename T>
void Launch<T>::MgSubtract(T *x, const T *x0, int64_t nq, cudaStream_t s) {
  const int64_t n = 5 * nq;
  if (n > 0) k_mg_sub<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, x0, n);
}
template <typename T>
void Launch<T>::MgProlong(const MgLinkDev &k, const T *coarse_du, int64_t coarse_nq, T *nodes,
                          T *fine_du, int64_t fine_nq, cudaStream_t s) {
  if (k.nnode > 0)
    k_mg_nodes<T><<<(k.nnode + 127) / 128, 128, 0, s>>>(k, coarse_du, coarse_nq, nodes);
  if (k.nfine > 0)
    k_mg_prolong<T><<<(k.nfine + 127) / 128, 128, 0, s>>>(k, nodes, fine_du, fine_nq);
}
template <typename T>
void Launch<T>::Wall(const Pools<T> &P, const WallFaceDev *faces, int n, double *wbuf,
                     cudaStream_t s) {
  if (n > 0) k_wall<T><<<(n + 127) / 128, 128, 0, s>>>(P, faces, n, wbuf);
}
template <typename T>
void Launch<T>::Ghost(const Pools<T> &P, const GhostOpDev *ops, int nops,
                      const int32_t *op_solve, cudaStream_t s) {
  if (nops > 0) k_ghost<T><<<(nops + 127) / 128, 128, 0, s>>>(P, ops, nops, op_solve);
}
template <typename T>
void Launch<T>::Aux(const Pools<T> &P, const int32_t *cells, const int32_t *cell_block,
                    int n, cudaStream_t s) {
  if (n > 0) k_aux<T><<<(n + 127) / 128, 128, 0, s>>>(P, cells, cell_block, n);
}
template <typename T, int D>
static void LaunchVFace(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                        int ncta, int rkinds, cudaStream_t s) {
  if (rkinds & 1) k_vface<T, D, false><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  if (rkinds & 2) k_vface<T, D, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
}
template <typename T>
void Launch<T>::ViscFace(int d, const Pools<T> &P, const int32_t *list,
                         const int32_t *cta_block, int ncta, int rkinds, cudaStream_t s) {
  if (ncta <= 0) return;
  if (d == 0) LaunchVFace<T, 0>(P, list, cta_block, ncta, rkinds, s);
  else if (d == 1) LaunchVFace<T, 1>(P, list, cta_block, ncta, rkinds, s);
  else LaunchVFace<T, 2>(P, list, cta_block, ncta, rkinds, s);
}
template <typename T, int D>
static void LaunchFace(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                       int ncta, int rkinds, cudaStream_t s) {
  // rkinds bit 2: the fast-face option of FP64 batches (non-RANS solves),
  // compiled in its own unit with contracted multiply-adds; bit 3: every
  // solve without turbulence equations is MUSCL-Roe
  bool fast = false;
  if constexpr (std::is_same<T, double>::value) {
    if ((rkinds & 1) && (rkinds & 4)) {
      LaunchFastFaceFp64(D, P, list, cta_block, ncta, (rkinds & 8) != 0, s);
      fast = true;
    }
  }
  if ((rkinds & 1) && !fast) {
    // batches whose solves are all MUSCL-Roe run the kernel built for that
    // alone (bit-exact FP64: the MUSCL-Roe path only; mixed: the same
    // FaceFluxMixed, at two CTAs per SM)
    if (rkinds & 8)
      k_face<T, D, false, false, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
    else
      k_face<T, D, false><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  }
  if (rkinds & 2) k_face<T, D, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
}
template <typename T>
void Launch<T>::Face(int d, const Pools<T> &P, const int32_t *list,
                     const int32_t *cta_block, int ncta, int rkinds, cudaStream_t s) {
  if (ncta <= 0) return;
  if (d == 0) LaunchFace<T, 0>(P, list, cta_block, ncta, rkinds, s);
  else if (d == 1) LaunchFace<T, 1>(P, list, cta_block, ncta, rkinds, s);
  else LaunchFace<T, 2>(P, list, cta_block, ncta, rkinds, s);
}
template <typename T>
void Launch<T>::Cell(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                     int ncta, int kinds, cudaStream_t s) {
  if (ncta <= 0) return;
  if constexpr (std::is_same<T, double>::value) {
    if (P.fast_fp64) {
      LaunchFastCellFp64(P, list, cta_block, ncta, kinds, s);
      return;
    }
  }
  // one kernel per solve kind (block / scalar, with / without turbulence
  // equations), so the laminar ones keep their register budget
  if ((kinds & 1) && (P.fkinds & 1)) k_cell<T, false, false><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  if ((kinds & 1) && (P.fkinds & 2)) k_cell<T, false, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  if ((kinds & 2) && (P.fkinds & 1)) k_cell<T, true, false><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  if ((kinds & 2) && (P.fkinds & 2)) k_cell<T, true, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
}
template <typename T>
void Launch<T>::Sweep(const Pools<T> &P, const int2 *items, int n, int forward, int sweep,
                      bool full, int kinds, int threads, bool group, bool chained,
                      cudaStream_t s) {
  if (n <= 0) return;
  bool fast = false;
  if constexpr (std::is_same<T, double>::value) {
    if (P.fast_fp64 && (kinds & 1)) {
      LaunchFastSweepFp64(P, items, n, forward, sweep, full, threads, group, chained, s);
      fast = true;
    }
  }
  if (fast) {
  } else if ((kinds & 1) && group) {
    LaunchSweepGroup<T>(P, items, n, forward, sweep, full, threads, chained, s);
  } else if (kinds & 1) {
    LaunchSweepCell<T>(P, items, n, forward, sweep, full, threads, chained, s);
  }
  if (kinds & 2) {
    const unsigned gridb = (unsigned)(((int64_t)n * 8 + threads - 1) / threads);
    k_sweepb<T><<<gridb, threads, 0, s>>>(P, items, n, forward, sweep, full ? 1 : 0);
  }
}
template <typename T, bool FULL, bool BLOCK>
static void LaunchSweepCl(const Pools<T> &P, const SweepLists &L, int forward, int sweep,
                          int threads, int cluster, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(L.nsolves * cluster));
  cfg.blockDim = dim3((unsigned)threads);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_sweep_cl<T, FULL, BLOCK>, P, L.items, L.step_off, L.solve_step0,
                     L.solve_nsteps, forward, sweep);
}
template <typename T>
void Launch<T>::SweepCl(const Pools<T> &P, const SweepLists &L, int forward, int sweep,
                        bool full, int kinds, int threads, int cluster, cudaStream_t s) {
  if (L.nsolves <= 0) return;
  if (kinds & 1) {
    if (full) LaunchSweepCl<T, true, false>(P, L, forward, sweep, threads, cluster, s);
    else LaunchSweepCl<T, false, false>(P, L, forward, sweep, threads, cluster, s);
  }
  if (kinds & 2) LaunchSweepCl<T, true, true>(P, L, forward, sweep, threads, cluster, s);
}
template <typename T>
void Launch<T>::NrGrads(const Pools<T> &P, const int32_t *cells, const int32_t *cell_block,
                        int n, cudaStream_t s) {
  if (n > 0) k_nr_grads<T><<<(n + 127) / 128, 128, 0, s>>>(P, cells, cell_block, n);
}
template <typename T>
void Launch<T>::OutGrads(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                         int ncta, int fkinds, cudaStream_t s) {
  if (ncta <= 0) return;
  if (fkinds & 1) k_out_grads<T, false><<<ncta, kCta, 0, s>>>(P, list, cta_block);
  if (fkinds & 2) k_out_grads<T, true><<<ncta, kCta, 0, s>>>(P, list, cta_block);
}
template <typename T>
void Launch<T>::SweepTq(const Pools<T> &P, const TileQueueDev &Q, int forward, int sweep,
                        bool full, bool block, int ctas, cudaStream_t s) {
  if (Q.ntiles <= 0) return;
  const unsigned grid = (unsigned)std::max(1, std::min(ctas, Q.ntiles));
  if (block)
    k_sweep_tq<T, true, true><<<grid, kTqThreads, 0, s>>>(P, Q, forward, sweep);
  else if (full)
    k_sweep_tq<T, true, false><<<grid, kTqThreads, 0, s>>>(P, Q, forward, sweep);
  else
    k_sweep_tq<T, false, false><<<grid, kTqThreads, 0, s>>>(P, Q, forward, sweep);
}
template <typename T>
int Launch<T>::TqOccupancy(bool full, bool block) {
  int n = 0;
  cudaError_t e;
  if (block)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_tq<T, true, true>,
                                                      kTqThreads, 0);
  else if (full)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_tq<T, true, false>,
                                                      kTqThreads, 0);
  else
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_tq<T, false, false>,
                                                      kTqThreads, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}
template <typename T>
int Launch<T>::MaxClusters(int kinds, int threads, int cluster) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cluster);
  cfg.blockDim = dim3((unsigned)threads);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int best = 1 << 30, n = 0;
  if (kinds & 1) {
    if (cudaOccupancyMaxActiveClusters(&n, k_sweep_cl<T, true, false>, &cfg) != cudaSuccess)
      n = 0;
    best = std::min(best, n);
    if (cudaOccupancyMaxActiveClusters(&n, k_sweep_cl<T, false, false>, &cfg) != cudaSuccess)
      n = 0;
    best = std::min(best, n);
  }
  if (kinds & 2) {
    if (cudaOccupancyMaxActiveClusters(&n, k_sweep_cl<T, true, true>, &cfg) != cudaSuccess)
      n = 0;
    best = std::min(best, n);
  }
  cudaGetLastError();  // a refused query leaves no sticky error
  return best == (1 << 30) ? 0 : best;
}
template <typename T>
void Launch<T>::OffJac(const Pools<T> &P, const int2 *items, int n, cudaStream_t s) {
  if (n > 0) k_offjac<T><<<(n + 127) / 128, 128, 0, s>>>(P, items, n);
}
template <typename T>
void Launch<T>::Init(const Pools<T> &P, const int2 *items, int n, int jacobi, cudaStream_t s) {
  if (n > 0) k_init<T><<<(n + 127) / 128, 128, 0, s>>>(P, items, n, jacobi);
}
template <typename T>
void Launch<T>::Jacobi(const Pools<T> &P, T *dst, T *dstt, const int2 *items, int n, int sweep,
                       int kinds, cudaStream_t s) {
  if (n <= 0) return;
  const unsigned grid = (unsigned)((n + 127) / 128);
  if (kinds & 1) k_jacobi<T, false><<<grid, 128, 0, s>>>(P, dst, dstt, items, n, sweep);
  if (kinds & 2) k_jacobi<T, true><<<grid, 128, 0, s>>>(P, dst, dstt, items, n, sweep);
}
template <typename T>
void Launch<T>::JacobiCopy(const Pools<T> &P, const T *src, const T *srct, const int2 *items,
                           int n, cudaStream_t s) {
  if (n > 0) k_jacobi_copy<T><<<(n + 127) / 128, 128, 0, s>>>(P, src, srct, items, n);
}
template <typename T>
void Launch<T>::ConnDu(const Pools<T> &P, cudaStream_t s) {
  if (P.nghost > 0) k_conn_du<T><<<(unsigned)((P.nghost + 127) / 128), 128, 0, s>>>(P);
}
template <typename T>
void Launch<T>::Update(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                       const int32_t *cta_pos0, NormPartial *partials, int ncta,
                       const SolveState *ss, cudaStream_t s) {
  if constexpr (std::is_same<T, double>::value) {
    if (P.fast_fp64) {
      LaunchFastUpdateFp64(P, list, cta_block, cta_pos0, partials, ncta, ss, s);
      return;
    }
  }
  if (ncta > 0) k_update<T><<<ncta, kCta, 0, s>>>(P, list, cta_block, cta_pos0, partials, ss);
}
template <typename T>
void Launch<T>::NrMach(const Pools<T> &P, const NrDev *nr, const int32_t *off, int nsurf,
                       cudaStream_t s) {
  if (nsurf > 0) k_nr_mach<T><<<(nsurf + 127) / 128, 128, 0, s>>>(P, nr, off, nsurf);
}
template <typename T>
void Launch<T>::StoreN(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                       int ncta, const SolveState *ss, int block, cudaStream_t s) {
  if (ncta > 0) k_store_n<T><<<ncta, kCta, 0, s>>>(P, list, cta_block, ss, block);
}

}  // namespace ath
