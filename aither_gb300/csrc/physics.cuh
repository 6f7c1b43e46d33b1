// Point physics of the per-iteration path, as device functions templated
// on the arithmetic type T (double for the FP64 path, float for the FP32
// parts of the mixed path).  Calorically perfect single-species ideal gas,
// primitive variables W = (rho, u, v, w, p).
//
// Each function states the reference function it restates.  The operation
// order follows the reference expression by expression (it matters for
// last-bit agreement with the reference CPU build when the translation
// unit is compiled with --fmad=false).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

namespace ath {

template <typename T>
struct Gas {
  T r;   // nondimensional gas constant
  T n;   // cv / R
  T hf;  // nondimensional heat of formation
  // caloricallyPerfect::SpeciesCv / SpeciesCp (include/thermodynamic.hpp:110-115)
  // and thermodynamic::Gamma (include/thermodynamic.hpp:58), formed once by
  // Set() with the reference's expressions: cv = R n, cp = R (n + 1),
  // gamma = cp / cv
  T cv, cp, gam;
  __host__ __device__ __forceinline__ void Set(T r_, T n_, T hf_) {
    r = r_;
    n = n_;
    hf = hf_;
    cv = r * n;
    cp = r * (n + T(1));
    gam = cp / cv;
  }
  __device__ __forceinline__ T Cv() const { return cv; }
  __device__ __forceinline__ T Cp() const { return cp; }
  __device__ __forceinline__ T Gamma() const { return gam; }
};

// Tests of doubles on the integer pipe (FP64 comparisons issue on GB300's
// narrow FP64 pipe).  An IEEE double's sign is its top bit, and
// non-negative values order as their bit patterns do as signed integers.
__device__ __forceinline__ long long Bits(double x) { return __double_as_longlong(x); }
// x > 0 (x = +inf included, NaN not)
__device__ __forceinline__ bool PositiveBits(double x) {
  const long long b = Bits(x);
  return b > 0 && b <= 0x7ff0000000000000LL;
}
// x neither infinite nor NaN
__device__ __forceinline__ bool FiniteBits(double x) {
  return (Bits(x) & 0x7fffffffffffffffLL) < 0x7ff0000000000000LL;
}
// x > m for m = +0 or positive and not NaN (x NaN: false)
__device__ __forceinline__ bool GreaterNonNeg(double x, double m) {
  const long long b = Bits(x);
  return b > Bits(m) && b <= 0x7ff0000000000000LL;
}

template <typename T>
struct Prim {
  T rho, u, v, w, p;
};

template <typename T>
struct Vec3 {
  T x, y, z;
};

// vector3d::DotProd via inner_product (include/vector3d.hpp:303)
template <typename T>
__device__ __forceinline__ T Dot(T ax, T ay, T az, T bx, T by, T bz) {
  return ax * bx + ay * by + az * bz;
}

// idealGas::Temperature (src/eos.cpp:100)
template <typename T>
__device__ __forceinline__ T Temperature(const Prim<T> &s, const Gas<T> &g) {
  return s.p / (s.rho * g.r);
}

// SpeedOfSound (include/arrayView.hpp:384)
template <typename T>
__device__ __forceinline__ T SoS(const Prim<T> &s, const Gas<T> &g) {
  return sqrt(g.Gamma() * s.p / s.rho);
}

template <typename T>
__device__ __forceinline__ T VelMag(const Prim<T> &s) {
  return sqrt(Dot(s.u, s.v, s.w, s.u, s.v, s.w));
}

// EnthalpyFunc -> idealGas::Enthalpy (include/arrayView.hpp:401,
// src/eos.cpp:64): hf + cp T + 0.5 |v| |v|
template <typename T>
__device__ __forceinline__ T Enthalpy(const Prim<T> &s, const Gas<T> &g) {
  const T t = Temperature(s, g);
  const T vm = VelMag(s);
  return (g.hf + g.Cp() * t) + T(0.5) * vm * vm;
}

// InternalEnergy -> idealGas::Energy (include/arrayView.hpp:436,
// src/eos.cpp:58): hf + cv T + 0.5 |v| |v|
template <typename T>
__device__ __forceinline__ T Energy(const Prim<T> &s, const Gas<T> &g) {
  const T t = Temperature(s, g);
  const T vm = VelMag(s);
  return (g.hf + g.Cv() * t) + T(0.5) * vm * vm;
}

// PrimToCons (include/primitive.hpp:183)
template <typename T>
__device__ __forceinline__ void PrimToCons(const Prim<T> &s, const Gas<T> &g,
                                           T c[5]) {
  c[0] = s.rho;
  c[1] = s.rho * s.u;
  c[2] = s.rho * s.v;
  c[3] = s.rho * s.w;
  c[4] = s.rho * Energy(s, g);
}

// primitive(conserved) constructor (include/primitive.hpp:137) with
// idealGas::PressFromEnergy (src/eos.cpp:40) and
// caloricallyPerfect::TemperatureFromSpecEnergy (src/thermodynamic.cpp:107)
template <typename T>
__device__ __forceinline__ Prim<T> ConsToPrim(const T c[5], const Gas<T> &g) {
  Prim<T> s;
  s.rho = c[0];
  const T rho = c[0];
  s.u = c[1] / rho;
  s.v = c[2] / rho;
  s.w = c[3] / rho;
  const T energy = c[4] / rho;
  const T vel = VelMag(s);
  const T spec = energy - T(0.5) * vel * vel;
  const T t = (spec - g.hf) / g.Cv();
  s.p = rho * g.r * t;
  return s;
}

// UpdatePrimWithCons (include/primitive.hpp:206): W <- prim(cons(W) + dU).
// The mass-fraction renormalisation is the identity for one species.
template <typename T>
__device__ __forceinline__ Prim<T> UpdateWithCons(const Prim<T> &s,
                                                  const Gas<T> &g,
                                                  const T du[5]) {
  T c[5];
  PrimToCons(s, g, c);
#pragma unroll
  for (int v = 0; v < 5; ++v) c[v] = c[v] + du[v];
  return ConsToPrim(c, g);
}

// inviscidFlux::ConstructFromPrim (include/inviscidFlux.hpp:129)
template <typename T>
__device__ __forceinline__ void InvFlux(const Prim<T> &s, const Gas<T> &g,
                                        T nx, T ny, T nz, T f[5]) {
  const T vn = Dot(s.u, s.v, s.w, nx, ny, nz);
  f[0] = s.rho * vn;
  f[1] = s.rho * vn * s.u + s.p * nx;
  f[2] = s.rho * vn * s.v + s.p * ny;
  f[3] = s.rho * vn * s.w + s.p * nz;
  f[4] = s.rho * vn * Enthalpy(s, g);
}

// Limiters (src/limiter.cpp:24,36)
template <typename T>
__device__ __forceinline__ T LimMinmod(T r) {
  return fmax(T(0), fmin(T(1), r));
}
template <typename T>
__device__ __forceinline__ T LimVanAlbada(T r) {
  const T r2 = r * r;
  return fmax(T(0), (r + r2) / (T(1) + r2));
}

// FaceReconMUSCL (include/reconstruction.hpp:110), one variable.
// limiter: 0 none, 1 minmod, 2 van Albada.
template <typename T>
__device__ __forceinline__ T Muscl1(T up2, T up1, T dw1, T dplus, T dminus,
                                    T kappa, int limiter) {
  const T eps = T(1.0e-30);
  const T r = (eps + (dw1 - up1) * dplus) / (eps + (up1 - up2) * dminus);
  T lim, ilim;
  if (limiter == 1) {
    lim = LimMinmod(r);
    ilim = LimMinmod(T(1) / r);
  } else if (limiter == 2) {
    lim = LimVanAlbada(r);
    ilim = LimVanAlbada(T(1) / r);
  } else {
    lim = T(1);
    ilim = T(1);
  }
  return up1 + T(0.25) * ((up1 - up2) * dminus) *
                   ((T(1) - kappa) * lim + (T(1) + kappa) * r * ilim);
}

// Delta form of Muscl1 for the mixed path: the increment over the upwind
// cell value, from the upwind difference a = up1 - up2 and the downwind
// difference b = dw1 - up1 (formed in FP64 before rounding).
template <typename T>
__device__ __forceinline__ T MusclDelta1(T a, T b, T dplus, T dminus, T kappa,
                                         int limiter) {
  const T eps = T(1.0e-30);
  const T r = (eps + b * dplus) / (eps + a * dminus);
  T lim, ilim;
  if (limiter == 1) {
    lim = LimMinmod(r);
    ilim = LimMinmod(T(1) / r);
  } else if (limiter == 2) {
    lim = LimVanAlbada(r);
    ilim = LimVanAlbada(T(1) / r);
  } else {
    lim = T(1);
    ilim = T(1);
  }
  return T(0.25) * (a * dminus) * ((T(1) - kappa) * lim + (T(1) + kappa) * r * ilim);
}

// MUSCL's width ratios of one side: dplus = 2 uw / (uw + dw), dminus =
// 2 uw / (uw + uw2) (FaceReconMUSCL, include/reconstruction.hpp:110)
template <typename T>
__device__ __forceinline__ void MusclRatios(T uw2, T uw, T dw, T &dplus, T &dminus) {
  dplus = (uw + uw) / (uw + dw);
  dminus = (uw + uw) / (uw + uw2);
}
// ... and the face state from given ratios
template <typename T>
__device__ __forceinline__ Prim<T> MusclR(const Prim<T> &up2, const Prim<T> &up1,
                                          const Prim<T> &dw1, T dplus, T dminus, T kappa,
                                          int limiter) {
  Prim<T> o;
  o.rho = Muscl1(up2.rho, up1.rho, dw1.rho, dplus, dminus, kappa, limiter);
  o.u = Muscl1(up2.u, up1.u, dw1.u, dplus, dminus, kappa, limiter);
  o.v = Muscl1(up2.v, up1.v, dw1.v, dplus, dminus, kappa, limiter);
  o.w = Muscl1(up2.w, up1.w, dw1.w, dplus, dminus, kappa, limiter);
  o.p = Muscl1(up2.p, up1.p, dw1.p, dplus, dminus, kappa, limiter);
  return o;
}
template <typename T>
__device__ __forceinline__ Prim<T> Muscl(const Prim<T> &up2, const Prim<T> &up1,
                                         const Prim<T> &dw1, T uw2, T uw, T dw,
                                         T kappa, int limiter) {
  T dplus, dminus;
  MusclRatios(uw2, uw, dw, dplus, dminus);
  Prim<T> o;
  o.rho = Muscl1(up2.rho, up1.rho, dw1.rho, dplus, dminus, kappa, limiter);
  o.u = Muscl1(up2.u, up1.u, dw1.u, dplus, dminus, kappa, limiter);
  o.v = Muscl1(up2.v, up1.v, dw1.v, dplus, dminus, kappa, limiter);
  o.w = Muscl1(up2.w, up1.w, dw1.w, dplus, dminus, kappa, limiter);
  o.p = Muscl1(up2.p, up1.p, dw1.p, dplus, dminus, kappa, limiter);
  return o;
}

// ---------------------------------------------------------------------------
// Fast forms of the FP64 faces (a batch option): the reference's arithmetic
// rearranged to need fewer divisions and square roots, the slow operations
// of GB300's FP64 pipe.  They agree with the reference to roundoff, not bit
// for bit.
//
// MUSCL with the reference's ratio r = (eps + y) / (eps + x), x = (up1 -
// up2) dminus, y = (dw1 - up1) dplus.  For minmod phi(r) = r phi(1/r) =
// min(max(r, 0), 1): both limiter terms are equal, kappa cancels, and the
// increment is x / 2 when r >= 1, y / 2 when 0 < r < 1 (to within eps =
// 1e-30) and 0 otherwise -- no division.  In FP64 the tests r > 0 (A =
// eps + x and B = eps + y nonzero with one sign) and |B| < |A| read the
// bit patterns on the integer pipe: for IEEE doubles the sign is the top
// bit and magnitudes order as the remaining bits do.  van Albada takes one
// quotient q = (r + 1) / (r^2 + 1) for both phi(r) = r q and phi(1/r) = q.
template <typename T>
__device__ __forceinline__ T MusclFast1(T up2, T up1, T dw1, T dplus, T dminus, T kappa,
                                        int limiter) {
  const T eps = T(1.0e-30);
  const T x = (up1 - up2) * dminus, y = (dw1 - up1) * dplus;
  if (limiter == 1) {
    const T A = eps + x, B = eps + y;
    if constexpr (std::is_same<T, double>::value) {
      const long long ia = __double_as_longlong(A), ib = __double_as_longlong(B);
      const long long ma = ia & 0x7fffffffffffffffLL, mb = ib & 0x7fffffffffffffffLL;
      if ((ia ^ ib) < 0 || ma == 0 || mb == 0) return up1;
      return up1 + T(0.5) * (mb < ma ? y : x);
    } else {
      if (!(A * B > T(0))) return up1;
      return up1 + T(0.5) * (fabs(B) < fabs(A) ? y : x);
    }
  }
  const T r = (eps + y) / (eps + x);
  T lim = T(1), rilim = r;
  if (limiter == 2) {
    const T q = (r + T(1)) / (r * r + T(1));
    lim = fmax(T(0), r * q);
    rilim = r * fmax(T(0), q);
  }
  return up1 + T(0.25) * x * ((T(1) - kappa) * lim + (T(1) + kappa) * rilim);
}
// Both face states of the face between cells m1 and 0 in MusclFast1's form
// (lower side: upwind2 m2, upwind1 m1, downwind 0; upper side: upwind2 p1,
// upwind1 0, downwind m1), the difference across the face formed once:
// the upper side's y = (wm1 - w0) dplus is -(w0 - wm1) dplus exactly
template <typename T>
__device__ __forceinline__ void MusclFastPair1(T wm2, T wm1, T w0, T wp1, T dpL, T dmL, T dpR,
                                               T dmR, T kappa, int limiter, T &l, T &r) {
  if (limiter != 1) {
    l = MusclFast1(wm2, wm1, w0, dpL, dmL, kappa, limiter);
    r = MusclFast1(wp1, w0, wm1, dpR, dmR, kappa, limiter);
    return;
  }
  const T eps = T(1.0e-30);
  const T d0 = w0 - wm1;
  const T xs[2] = {(wm1 - wm2) * dmL, (w0 - wp1) * dmR};
  const T ys[2] = {d0 * dpL, (-d0) * dpR};
  const T up[2] = {wm1, w0};
  T o[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const T x = xs[k], y = ys[k];
    if constexpr (std::is_same<T, double>::value) {
      // in FP64 the tests read the slopes x and y themselves instead of
      // eps + x and eps + y: the increment changes only where a slope is
      // below about eps in magnitude, by less than eps
      const long long ia = __double_as_longlong(x), ib = __double_as_longlong(y);
      const long long ma = ia & 0x7fffffffffffffffLL, mb = ib & 0x7fffffffffffffffLL;
      o[k] = ((ia ^ ib) < 0 || ma == 0 || mb == 0) ? up[k]
                                                     : up[k] + T(0.5) * (mb < ma ? y : x);
    } else {
      const T A = eps + x, B = eps + y;
      o[k] = !(A * B > T(0)) ? up[k] : up[k] + T(0.5) * (fabs(B) < fabs(A) ? y : x);
    }
  }
  l = o[0];
  r = o[1];
}
template <typename T>
__device__ __forceinline__ void MusclFastPair(const Prim<T> &wm2, const Prim<T> &wm1,
                                              const Prim<T> &w0, const Prim<T> &wp1, T dpL,
                                              T dmL, T dpR, T dmR, T kappa, int limiter,
                                              Prim<T> &L, Prim<T> &R) {
  MusclFastPair1(wm2.rho, wm1.rho, w0.rho, wp1.rho, dpL, dmL, dpR, dmR, kappa, limiter, L.rho,
                 R.rho);
  MusclFastPair1(wm2.u, wm1.u, w0.u, wp1.u, dpL, dmL, dpR, dmR, kappa, limiter, L.u, R.u);
  MusclFastPair1(wm2.v, wm1.v, w0.v, wp1.v, dpL, dmL, dpR, dmR, kappa, limiter, L.v, R.v);
  MusclFastPair1(wm2.w, wm1.w, w0.w, wp1.w, dpL, dmL, dpR, dmR, kappa, limiter, L.w, R.w);
  MusclFastPair1(wm2.p, wm1.p, w0.p, wp1.p, dpL, dmL, dpR, dmR, kappa, limiter, L.p, R.p);
}
// The width ratios of both sides of the face between cells m1 and 0 (cell
// widths xm2, xm1 | x0, xp1 along the face normal): lower side dplus =
// 2 xm1 / (xm1 + x0), dminus = 2 xm1 / (xm1 + xm2); upper side dplus =
// 2 x0 / (x0 + xm1), dminus = 2 x0 / (x0 + xp1) -- with one reciprocal of
// the product of the three sums in place of four divisions
template <typename T>
__device__ __forceinline__ void MusclFastRatios(T xm2, T xm1, T x0, T xp1, T &dpL, T &dmL,
                                                T &dpR, T &dmR) {
  const T a = xm1 + x0, b = xm1 + xm2, c = x0 + xp1;
  const T ab = a * b;
  const T r = T(1) / (ab * c);
  const T ia = (b * c) * r, ib = (a * c) * r, ic = ab * r;
  const T tm1 = xm1 + xm1, t0 = x0 + x0;
  dpL = tm1 * ia;
  dmL = tm1 * ib;
  dpR = t0 * ia;
  dmR = t0 * ic;
}

// RoeFlux with Harten's entropy fix (include/inviscidFlux.hpp:260-382,
// src/inviscidFlux.cpp:27): F = 0.5 (FL + (FR - D)).
// Dissipation D of the Roe flux from the face states L, R and their jumps
// dq = R - L (rho, u, v, w, p).
template <typename T>
__device__ __forceinline__ void RoeDissipation(const Prim<T> &L, const Prim<T> &R,
                                               const T dq[5], const Gas<T> &g, T nx, T ny,
                                               T nz, T dout[5]) {
  // RoeAveragedState (include/primitive.hpp:245)
  const T denRatio = sqrt(R.rho / L.rho);
  Prim<T> roe;
  roe.rho = L.rho * denRatio;
  roe.u = (L.u + denRatio * R.u) / (T(1) + denRatio);
  roe.v = (L.v + denRatio * R.v) / (T(1) + denRatio);
  roe.w = (L.w + denRatio * R.w) / (T(1) + denRatio);
  roe.p = (L.p + denRatio * R.p) / (T(1) + denRatio);

  const T hR = Enthalpy(roe, g);
  const T aR = SoS(roe, g);
  const T rhoR = roe.rho;
  const T velNormR = Dot(roe.u, roe.v, roe.w, nx, ny, nz);
  const T mfR = roe.rho / rhoR;  // mass fraction of the single species
  const T dRho = dq[0], dU = dq[1], dV = dq[2], dW = dq[3], dP = dq[4];
  const T normVelDiff = Dot(dU, dV, dW, nx, ny, nz);
  const T entropyFix = T(0.1);

  T d0 = T(0), d1 = T(0), d2 = T(0), d3 = T(0), d4 = T(0);
  // left moving acoustic wave
  T waveSpeed = fabs(velNormR - aR);
  if (waveSpeed < entropyFix)
    waveSpeed = T(0.5) * (waveSpeed * waveSpeed / entropyFix + entropyFix);
  T waveStrength = (dP - rhoR * aR * normVelDiff) / (T(2) * aR * aR);
  T ws = waveSpeed * waveStrength;
  d0 += ws * mfR;
  d1 += ws * (roe.u - aR * nx);
  d2 += ws * (roe.v - aR * ny);
  d3 += ws * (roe.w - aR * nz);
  d4 += ws * (hR - aR * velNormR);
  // entropy wave
  waveSpeed = fabs(velNormR);
  waveStrength = -dP / (aR * aR);
  ws = waveSpeed * waveStrength;
  d0 += ws * mfR + waveSpeed * dRho;
  waveStrength = dRho - dP / (aR * aR);
  ws = waveSpeed * waveStrength;
  d1 += ws * roe.u;
  d2 += ws * roe.v;
  d3 += ws * roe.w;
  d4 += ws * T(0.5) * Dot(roe.u, roe.v, roe.w, roe.u, roe.v, roe.w);
  // shear waves
  waveStrength = rhoR;
  ws = waveSpeed * waveStrength;
  d1 += ws * (dU - normVelDiff * nx);
  d2 += ws * (dV - normVelDiff * ny);
  d3 += ws * (dW - normVelDiff * nz);
  d4 += ws * (Dot(roe.u, roe.v, roe.w, dU, dV, dW) - velNormR * normVelDiff);
  // right moving acoustic wave
  waveSpeed = fabs(velNormR + aR);
  if (waveSpeed < entropyFix)
    waveSpeed = T(0.5) * (waveSpeed * waveSpeed / entropyFix + entropyFix);
  waveStrength = (dP + rhoR * aR * normVelDiff) / (T(2) * aR * aR);
  ws = waveSpeed * waveStrength;
  d0 += ws * mfR;
  d1 += ws * (roe.u + aR * nx);
  d2 += ws * (roe.v + aR * ny);
  d3 += ws * (roe.w + aR * nz);
  d4 += ws * (hR + aR * velNormR);
  dout[0] = d0;
  dout[1] = d1;
  dout[2] = d2;
  dout[3] = d3;
  dout[4] = d4;
}

template <typename T>
__device__ __forceinline__ void RoeFlux(const Prim<T> &L, const Prim<T> &R,
                                        const Gas<T> &g, T nx, T ny, T nz,
                                        T f[5]) {
  const T dq[5] = {R.rho - L.rho, R.u - L.u, R.v - L.v, R.w - L.w, R.p - L.p};
  T d[5];
  RoeDissipation(L, R, dq, g, nx, ny, nz, d);
  T fl[5], fr[5];
  InvFlux(L, g, nx, ny, nz, fl);
  InvFlux(R, g, nx, ny, nz, fr);
#pragma unroll
  for (int v = 0; v < 5; ++v) f[v] = (fl[v] + (fr[v] - d[v])) * T(0.5);
}

// Convective flux for the mixed path's FP64 central part, free of
// divisions and square roots: rho H = rho hf + (n + 1) p + rho |v|^2 / 2
// (cp T rho = (n + 1) p for the calorically perfect gas, cv = n R).
__device__ __forceinline__ void InvFluxCentral(const Prim<double> &s, const Gas<double> &g,
                                               double nx, double ny, double nz,
                                               double f[5]) {
  const double vn = s.u * nx + s.v * ny + s.w * nz;
  const double m = s.rho * vn;
  const double rhoH = s.rho * (g.hf + 0.5 * (s.u * s.u + s.v * s.v + s.w * s.w)) +
                      (g.n + 1.0) * s.p;
  f[0] = m;
  f[1] = m * s.u + s.p * nx;
  f[2] = m * s.v + s.p * ny;
  f[3] = m * s.w + s.p * nz;
  f[4] = vn * rhoH;
}

// Roe flux of RoeFlux in the fast form: one reciprocal square root of
// rhoL rhoR gives the density ratio sqrt(rhoR / rhoL) and the reciprocal of
// the Roe density; one reciprocal of 1 + sqrt(rhoR / rhoL) for the Roe
// averages; p / rho of the Roe state formed once for its enthalpy (hf +
// (n + 1) p / rho + |v|^2 / 2, as cp T = (n + 1) p / rho for the
// calorically perfect gas) and sound speed; one reciprocal square root of
// a^2 gives a and 1 / a^2; the dissipation's four waves summed in closed
// form; and the division-free central flux.
// f is the flux times `scale` (the face's area: F.|A| directly)
__device__ __forceinline__ void RoeFluxFast(const Prim<double> &L, const Prim<double> &R,
                                            const Gas<double> &g, double nx, double ny,
                                            double nz, double scale, double f[5]) {
  const double dRho = R.rho - L.rho, dU = R.u - L.u, dV = R.v - L.v, dW = R.w - L.w,
               dP = R.p - L.p;
  // t = 1 / sqrt(rhoL rhoR): sqrt(rhoR / rhoL) = rhoR t, and t is the
  // reciprocal of the Roe density sqrt(rhoL rhoR)
  const double t = rsqrt(R.rho * L.rho);
  const double denRatio = R.rho * t;
  const double inv = 1.0 / (1.0 + denRatio);
  const double ru = (L.u + denRatio * R.u) * inv, rv = (L.v + denRatio * R.v) * inv,
               rw = (L.w + denRatio * R.w) * inv, rp = (L.p + denRatio * R.p) * inv;
  const double rhoR = L.rho * denRatio;
  const double por = rp * t;
  const double q2h = 0.5 * (ru * ru + rv * rv + rw * rw);
  const double hR = (g.hf + (g.n + 1.0) * por) + q2h;
  const double a2 = g.gam * por;
  // s = 1 / a: a = a^2 s, 1 / a^2 = s^2
  const double sa = rsqrt(a2);
  const double aR = a2 * sa;
  const double ia2 = sa * sa;
  const double velNormR = ru * nx + rv * ny + rw * nz;
  const double normVelDiff = dU * nx + dV * ny + dW * nz;
  const double entropyFix = 0.1;
  // wave speeds; Harten's fix on the acoustic ones (the tests compare
  // non-negative speeds by their bits)
  const long long fixBits = Bits(entropyFix);
  double lamL = fabs(velNormR - aR), lamR = fabs(velNormR + aR);
  if (Bits(lamL) < fixBits) lamL = 0.5 * (lamL * lamL / entropyFix + entropyFix);
  if (Bits(lamR) < fixBits) lamR = 0.5 * (lamR * lamR / entropyFix + entropyFix);
  const double lamE = fabs(velNormR);
  // wave strengths: acoustic aL, aR5, entropy aE, shear beta (times the
  // velocity jump's tangential part)
  const double rc = rhoR * aR, hia2 = 0.5 * ia2;
  const double aL = lamL * ((dP - rc * normVelDiff) * hia2);
  const double aR5 = lamR * ((dP + rc * normVelDiff) * hia2);
  const double aE = lamE * (dRho - dP * ia2);
  const double beta = lamE * rhoR;
  // the four waves' eigenvectors summed in closed form: with sA = aL + aR5
  // and tA = a (aR5 - aL), D = (sA + aE) [1, u, v, w] + (tA - beta dVn) n
  // + beta dv in the momenta, and H sA + Vn tA + aE |v|^2 / 2 + beta (v .
  // dv - Vn dVn) in the energy -- the reference's wave-by-wave sum
  // regrouped, equal to it to roundoff
  const double sA = aL + aR5, tA = aR * (aR5 - aL);
  const double gn = tA - beta * normVelDiff;
  const double d0 = sA + aE;
  const double d1 = d0 * ru + (nx * gn + beta * dU);
  const double d2 = d0 * rv + (ny * gn + beta * dV);
  const double d3 = d0 * rw + (nz * gn + beta * dW);
  const double d4 = (hR * sA + velNormR * tA) + aE * q2h +
                    beta * ((ru * dU + rv * dV + rw * dW) - velNormR * normVelDiff);
  // central part FL + FR summed term by term, the two pressures once
  const double vnL = L.u * nx + L.v * ny + L.w * nz, vnR = R.u * nx + R.v * ny + R.w * nz;
  const double mL = L.rho * vnL, mR = R.rho * vnR;
  const double np1 = g.n + 1.0;
  const double rhoHL = L.rho * (g.hf + 0.5 * (L.u * L.u + L.v * L.v + L.w * L.w)) + np1 * L.p;
  const double rhoHR = R.rho * (g.hf + 0.5 * (R.u * R.u + R.v * R.v + R.w * R.w)) + np1 * R.p;
  const double pLR = L.p + R.p;
  const double hs = 0.5 * scale;
  f[0] = ((mL + mR) - d0) * hs;
  f[1] = ((mL * L.u + (mR * R.u + pLR * nx)) - d1) * hs;
  f[2] = ((mL * L.v + (mR * R.v + pLR * ny)) - d2) * hs;
  f[3] = ((mL * L.w + (mR * R.w + pLR * nz)) - d3) * hs;
  f[4] = ((vnL * rhoHL + vnR * rhoHR) - d4) * hs;
}

// ---------------------------------------------------------------------------
// WENO5 / WENO-Z on non-uniform cell widths (FaceReconWENO,
// include/reconstruction.hpp:244)

// StencilWidth (include/utility.hpp:104)
template <typename T>
__device__ __forceinline__ T StencilWidth(const T w[5], int start, int end) {
  T width = T(0);
  if (end > start) {
    for (int q = start; q < end; ++q) width += w[q];
  } else if (start > end) {
    T a = T(0);
    for (int q = end; q < start; ++q) a += w[q];
    width = T(-1) * a;
  }
  return width;
}

// LagrangeCoeff (src/utility.cpp:449)
template <typename T, int DEG>
__device__ __forceinline__ void LagrangeCoeff(const T w[5], int rr, int ii, T coeffs[DEG + 1]) {
#pragma unroll
  for (int jj = 0; jj <= DEG; ++jj) {
    coeffs[jj] = T(0);
    for (int mm = jj + 1; mm <= DEG + 1; ++mm) {
      T numer = T(0), denom = T(1);
      for (int ll = 0; ll <= DEG + 1; ++ll) {
        if (ll != mm) {
          T numProd = T(1);
          for (int qq = 0; qq <= DEG + 1; ++qq)
            if (qq != mm && qq != ll) numProd *= StencilWidth(w, ii - rr + qq, ii + 1);
          numer += numProd;
          denom *= StencilWidth(w, ii - rr + ll, ii - rr + mm);
        }
      }
      coeffs[jj] += numer / denom;
    }
    coeffs[jj] *= w[ii - rr + jj];
  }
}

// Derivative2nd (include/utility.hpp:117)
template <typename T>
__device__ __forceinline__ T Deriv2nd(T x0, T x1, T x2, T y0, T y1, T y2) {
  const T fwd = (y2 - y1) / (T(0.5) * (x2 + x1));
  const T bck = (y1 - y0) / (T(0.5) * (x1 + x0));
  return (fwd - bck) / (T(0.25) * (x2 + x0) + T(0.5) * x1);
}

// BetaIntegral (include/reconstruction.hpp:157,171).  The reference's
// pow(x, 3) is a cube here: CUDA's FP64 pow costs ~100 FP64 instructions and
// twelve of them per variable and side made WENO faces pow-bound; the
// product differs from a correctly rounded cube by at most an ulp, as
// CUDA's pow itself may.
template <typename T>
__device__ __forceinline__ T Cube(T x) {
  return x * x * x;
}
template <typename T>
__device__ __forceinline__ T BetaInt(T d1, T d2, T dx, T x) {
  return (d1 * d1 * x + d1 * d2 * x * x + d2 * d2 * Cube(x) / T(3)) * dx +
         d2 * d2 * x * Cube(dx);
}
template <typename T>
__device__ __forceinline__ T BetaInt2(T d1, T d2, T dx) {
  return BetaInt(d1, d2, dx, T(0.5) * dx) - BetaInt(d1, d2, dx, T(-0.5) * dx);
}

// per-face WENO weights, shared by the five variables
template <typename T>
struct WenoCoeffs {
  T c0[3], c1[3], c2[3], lw0, lw1, lw2;
};
template <typename T>
__device__ __forceinline__ WenoCoeffs<T> MakeWeno(const T w[5]) {
  WenoCoeffs<T> k;
  T full[5];
  LagrangeCoeff<T, 2>(w, 2, 2, k.c0);
  LagrangeCoeff<T, 2>(w, 1, 2, k.c1);
  LagrangeCoeff<T, 2>(w, 0, 2, k.c2);
  LagrangeCoeff<T, 4>(w, 2, 2, full);
  k.lw0 = full[0] / k.c0[0];
  k.lw1 = full[4] / k.c2[2];
  k.lw2 = T(1) - k.lw0 - k.lw1;
  return k;
}
// one variable: y = (upwind3, upwind2, upwind1, downwind1, downwind2)
template <typename T>
__device__ __forceinline__ T Weno1(const WenoCoeffs<T> &k, const T w[5], T y3, T y2, T y1,
                                   T d1, T d2, bool wenoz) {
  const T st0 = k.c0[0] * y3 + k.c0[1] * y2 + k.c0[2] * y1;
  const T st1 = k.c1[0] * y2 + k.c1[1] * y1 + k.c1[2] * d1;
  const T st2 = k.c2[0] * y1 + k.c2[1] * d1 + k.c2[2] * d2;
  // Beta0/Beta1/Beta2 (include/reconstruction.hpp:186-240)
  T dd = Deriv2nd(w[0], w[1], w[2], y3, y2, y1);
  T d = (y1 - y2) / (T(0.5) * (w[2] + w[1])) + T(0.5) * w[2] * dd;
  const T b0 = BetaInt2(d, dd, w[2]);
  dd = Deriv2nd(w[1], w[2], w[3], y2, y1, d1);
  d = (d1 - y1) / (T(0.5) * (w[3] + w[2])) - T(0.5) * w[2] * dd;
  const T b1 = BetaInt2(d, dd, w[2]);
  dd = Deriv2nd(w[2], w[3], w[4], y1, d1, d2);
  d = (d1 - y1) / (T(0.5) * (w[3] + w[2])) - T(0.5) * w[2] * dd;
  const T b2 = BetaInt2(d, dd, w[2]);
  T n0, n1, n2;
  if (wenoz) {
    const T eps = T(1.0e-40);
    const T tau5 = fabs(b0 - b2);
    const T t0 = tau5 / (eps + b0), t1 = tau5 / (eps + b1), t2 = tau5 / (eps + b2);
    n0 = k.lw0 * (T(1) + t0 * t0);
    n1 = k.lw1 * (T(1) + t1 * t1);
    n2 = k.lw2 * (T(1) + t2 * t2);
  } else {
    const T eps = T(1.0e-6);
    n0 = k.lw0 / ((eps + b0) * (eps + b0));
    n1 = k.lw1 / ((eps + b1) * (eps + b1));
    n2 = k.lw2 / ((eps + b2) * (eps + b2));
  }
  const T sum = n0 + n1 + n2;
  n0 /= sum;
  n1 /= sum;
  n2 /= sum;
  return n0 * st0 + n1 * st1 + n2 * st2;
}
template <typename T>
__device__ __forceinline__ Prim<T> Weno(const WenoCoeffs<T> &k, const Prim<T> &u3,
                                        const Prim<T> &u2, const Prim<T> &u1,
                                        const Prim<T> &d1, const Prim<T> &d2, const T w[5],
                                        bool wenoz) {
  Prim<T> o;
  o.rho = Weno1(k, w, u3.rho, u2.rho, u1.rho, d1.rho, d2.rho, wenoz);
  o.u = Weno1(k, w, u3.u, u2.u, u1.u, d1.u, d2.u, wenoz);
  o.v = Weno1(k, w, u3.v, u2.v, u1.v, d1.v, d2.v, wenoz);
  o.w = Weno1(k, w, u3.w, u2.w, u1.w, d1.w, d2.w, wenoz);
  o.p = Weno1(k, w, u3.p, u2.p, u1.p, d1.p, d2.p, wenoz);
  return o;
}

// ---------------------------------------------------------------------------
// AUSMPW+ (Kim, Kim & Rho 1998) with c* = sqrt(cL cR) (AUSMFlux,
// include/inviscidFlux.hpp:396; inviscidFlux::AUSMFlux :162)
template <typename T>
__device__ __forceinline__ T SignOf(T x) {
  return (T)((T(0) < x) - (x < T(0)));
}
template <typename T>
__device__ __forceinline__ void AusmFlux(const Prim<T> &L, const Prim<T> &R, const Gas<T> &g,
                                         T nx, T ny, T nz, T f[5], T *vlr = nullptr) {
  const T vnL = Dot(L.u, L.v, L.w, nx, ny, nz);
  const T vnR = Dot(R.u, R.v, R.w, nx, ny, nz);
  const T sosStar = sqrt(SoS(L, g) * SoS(R, g));
  const T vel = T(0.5) * (vnL + vnR);
  T sos = sosStar;
  if (vel < T(0)) {
    sos = sosStar * sosStar / ((vnR < sosStar) ? sosStar : vnR);
  } else if (vel > T(0)) {
    sos = sosStar * sosStar / ((vnL < sosStar) ? sosStar : vnL);
  }
  const T ml = vnL / sos, mr = vnR / sos;
  const T mlp = ml + T(1), mrm = mr - T(1);
  const T mPlusL = fabs(ml) <= T(1) ? T(0.25) * (mlp * mlp) : T(0.5) * (ml + fabs(ml));
  const T mMinusR = fabs(mr) <= T(1) ? T(-0.25) * (mrm * mrm) : T(0.5) * (mr - fabs(mr));
  const T pPlus = fabs(ml) <= T(1) ? T(0.25) * (mlp * mlp) * (T(2) - ml)
                                   : T(0.5) * (T(1) + SignOf(ml));
  const T pMinus = fabs(mr) <= T(1) ? T(0.25) * (mrm * mrm) * (T(2) + mr)
                                    : T(0.5) * (T(1) - SignOf(mr));
  const T ps = pPlus * L.p + pMinus * R.p;
  const T ra = L.p / R.p, rb = R.p / L.p;
  const T w = T(1) - Cube((rb < ra) ? rb : ra);
  const T fl = fabs(ml) < T(1) ? L.p / ps - T(1) : T(0);
  const T fr = fabs(mr) < T(1) ? R.p / ps - T(1) : T(0);
  const T mavg = mPlusL + mMinusR;
  const T mPlusLBar = mavg >= T(0) ? mPlusL + mMinusR * ((T(1) - w) * (T(1) + fr) - fl)
                                   : mPlusL * w * (T(1) + fl);
  const T mMinusRBar = mavg >= T(0) ? mMinusR * w * (T(1) + fr)
                                    : mMinusR + mPlusL * ((T(1) - w) * (T(1) + fl) - fr);
  const T vl = mPlusLBar * sos;
  f[0] = L.rho * vl;
  f[1] = L.rho * vl * L.u + pPlus * L.p * nx;
  f[2] = L.rho * vl * L.v + pPlus * L.p * ny;
  f[3] = L.rho * vl * L.w + pPlus * L.p * nz;
  f[4] = L.rho * vl * Enthalpy(L, g);
  const T vr = mMinusRBar * sos;
  f[0] += R.rho * vr;
  f[1] += R.rho * vr * R.u + pMinus * R.p * nx;
  f[2] += R.rho * vr * R.v + pMinus * R.p * ny;
  f[3] += R.rho * vr * R.w + pMinus * R.p * nz;
  f[4] += R.rho * vr * Enthalpy(R, g);
  if (vlr) {
    vlr[0] = vl;
    vlr[1] = vr;
  }
}

// Turbulence components of the Roe flux (include/inviscidFlux.hpp:311-368):
// both acoustic waves carry the Roe-averaged k and omega, plus the
// turbulence waves; F = 0.5 (FL + (FR - D)) with F = rho vn k.
template <typename T>
__device__ __forceinline__ void RoeTurbFlux(const Prim<T> &L, const Prim<T> &R, const T Lt[2],
                                            const T Rt[2], const Gas<T> &g, T nx, T ny, T nz,
                                            T ft[2]) {
  const T denRatio = sqrt(R.rho / L.rho);
  Prim<T> roe;
  roe.rho = L.rho * denRatio;
  roe.u = (L.u + denRatio * R.u) / (T(1) + denRatio);
  roe.v = (L.v + denRatio * R.v) / (T(1) + denRatio);
  roe.w = (L.w + denRatio * R.w) / (T(1) + denRatio);
  roe.p = (L.p + denRatio * R.p) / (T(1) + denRatio);
  const T aR = SoS(roe, g);
  const T rhoR = roe.rho;
  const T velNormR = Dot(roe.u, roe.v, roe.w, nx, ny, nz);
  const T dRho = R.rho - L.rho, dP = R.p - L.p;
  const T normVelDiff = Dot(R.u - L.u, R.v - L.v, R.w - L.w, nx, ny, nz);
  const T entropyFix = T(0.1);
  T ws = fabs(velNormR - aR);
  if (ws < entropyFix) ws = T(0.5) * (ws * ws / entropyFix + entropyFix);
  const T wssL = ws * ((dP - rhoR * aR * normVelDiff) / (T(2) * aR * aR));
  ws = fabs(velNormR + aR);
  if (ws < entropyFix) ws = T(0.5) * (ws * ws / entropyFix + entropyFix);
  const T wssR = ws * ((dP + rhoR * aR * normVelDiff) / (T(2) * aR * aR));
  const T wsT = fabs(velNormR);
  const T vnL = Dot(L.u, L.v, L.w, nx, ny, nz), vnR = Dot(R.u, R.v, R.w, nx, ny, nz);
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const T rt = (Lt[q] + denRatio * Rt[q]) / (T(1) + denRatio);
    T d = T(0);
    d += wssL * rt;
    d += wssR * rt;
    d += wsT * (rhoR * (Rt[q] - Lt[q]) + rt * dRho - dP * rt / (aR * aR)) * T(1);
    const T fl = L.rho * vnL * Lt[q], fr = R.rho * vnR * Rt[q];
    ft[q] = (fl + (fr - d)) * T(0.5);
  }
}

// ---------------------------------------------------------------------------
// laminar viscous terms

// thermodynamic::Prandtl (include/thermodynamic.hpp:61)
template <typename T>
__device__ __forceinline__ T Prandtl(const Gas<T> &g) {
  const T gamma = g.Gamma();
  return (T(4) * gamma) / (T(9) * gamma - T(5));
}
// max(4/(3 rho), gamma/rho) of ViscCell/ViscFaceSpectralRadius
// (include/spectralRadius.hpp:94,126)
template <typename T>
__device__ __forceinline__ T ViscMaxTerm(const Prim<T> &s, const Gas<T> &g) {
  const T a = T(4) / (T(3) * s.rho), b = g.Gamma() / s.rho;
  return (a < b) ? b : a;
}
// NondimScaling * (mu/Pr + mut/Prt), laminar (mut = 0, Prt = 0.9)
template <typename T>
__device__ __forceinline__ T ViscTerm(T mu, T scale, const Gas<T> &g) {
  return scale * (mu / Prandtl(g) + T(0) / T(0.9));
}
// the same with the eddy viscosity mut (turbulent Prandtl number 0.9)
template <typename T>
__device__ __forceinline__ T ViscTerm2(T mu, T mut, T scale, const Gas<T> &g, T prt = T(0.9)) {
  return scale * (mu / Prandtl(g) + mut / prt);
}
// sutherland::SpeciesViscosity / SpeciesConductivity (src/transport.cpp:100,108)
template <typename T>
__device__ __forceinline__ T SutherlandRatio(T t, T tref, T c1, T s, T ref) {
  const T temp = t * tref;
  const T v = (c1 * pow(temp, T(1.5))) / (temp + s);
  return v / ref;
}
// FaceReconCentral (include/reconstruction.hpp:315) weights of the upper
// (downwind) and lower (upwind) cell: LagrangeCoeff of a 2-cell stencil
template <typename T>
__device__ __forceinline__ void CentralCoeffs(T wl, T wu, T &cdown, T &cup) {
  const T w[5] = {wl, wu, T(0), T(0), T(0)};
  T c[2];
  LagrangeCoeff<T, 1>(w, 0, 0, c);
  cdown = c[0];
  cup = c[1];
}

// InvCellSpectralRadius (include/spectralRadius.hpp:44)
// the radius's geometry of one direction: the average of the cell's two
// face normals, normalised, and their average area
template <typename T>
__device__ __forceinline__ void CellAvgNormal(T lx, T ly, T lz, T lm, T ux, T uy, T uz, T um,
                                              T &ax, T &ay, T &az, T &fMag) {
  ax = T(0.5) * (lx + ux);
  ay = T(0.5) * (ly + uy);
  az = T(0.5) * (lz + uz);
  const T am = sqrt(Dot(ax, ay, az, ax, ay, az));
  ax = ax / am;
  ay = ay / am;
  az = az / am;
  fMag = T(0.5) * (lm + um);
}
template <typename T>
__device__ __forceinline__ T InvCellSpecRad(const Prim<T> &s, const Gas<T> &g,
                                            T lx, T ly, T lz, T lm, T ux,
                                            T uy, T uz, T um) {
  T ax, ay, az, fMag;
  CellAvgNormal(lx, ly, lz, lm, ux, uy, uz, um, ax, ay, az, fMag);
  return (fabs(Dot(s.u, s.v, s.w, ax, ay, az)) + SoS(s, g)) * fMag;
}

// InvFaceSpectralRadius (include/spectralRadius.hpp:67)
template <typename T>
__device__ __forceinline__ T InvFaceSpecRad(const Prim<T> &s, const Gas<T> &g,
                                            T nx, T ny, T nz, T mag) {
  return T(0.5) * mag * (fabs(Dot(s.u, s.v, s.w, nx, ny, nz)) + SoS(s, g));
}

// Terms of a neighbour's off-diagonal contribution that depend on its state
// alone, formed once per cell and iteration for the FP64 scalar sweeps
// (each cell is the neighbour of up to six off-diagonal terms): conserved
// state, enthalpy, speed of sound; viscous solves also ViscMaxTerm and
// ViscTerm2.  Each is the value the term itself would form.
template <typename T>
struct NbrPre {
  T c[5], h, sos, vmax, vt2;
};

// F(W') - F(W) with W' = prim(cons(W) + dU) (ConvectiveFluxUpdate,
// include/inviscidFlux.hpp:544) rewritten exactly in terms of the
// increments, for the FP32 sweeps: every term carries a factor of dU, so the
// rounding error is relative to the update instead of to the flux (the
// reference form subtracts two O(|F|) fluxes).
template <typename T>
__device__ __forceinline__ void ConvFluxDelta(const Prim<T> &s, const T du[5],
                                              const Gas<T> &g, T nx, T ny, T nz, T out[5]) {
  const T rho1 = s.rho + du[0];
  const T ir1 = T(1) / rho1;
  const T dux = (du[1] - s.u * du[0]) * ir1;
  const T duy = (du[2] - s.v * du[0]) * ir1;
  const T duz = (du[3] - s.w * du[0]) * ir1;
  const T t = s.p / (s.rho * g.r);
  const T ke = T(0.5) * (s.u * s.u + s.v * s.v + s.w * s.w);
  const T E = (g.hf + g.Cv() * t) + ke;  // specific total energy
  const T dE = (du[4] - E * du[0]) * ir1;
  const T dke = T(0.5) * ((T(2) * s.u + dux) * dux + (T(2) * s.v + duy) * duy +
                          (T(2) * s.w + duz) * duz);
  const T dt = (dE - dke) / g.Cv();
  const T dp = g.r * (rho1 * dt + du[0] * t);
  const T vn = s.u * nx + s.v * ny + s.w * nz;
  const T dvn = dux * nx + duy * ny + duz * nz;
  const T rhoE = s.rho * E;
  const T m0 = rho1 * dvn + du[0] * vn;  // (rho vn)' - rho vn
  const T rvn = s.rho * vn;
  out[0] = m0;
  out[1] = m0 * (s.u + dux) + rvn * dux + dp * nx;
  out[2] = m0 * (s.v + duy) + rvn * duy + dp * ny;
  out[3] = m0 * (s.w + duz) + rvn * duz + dp * nz;
  out[4] = dvn * (rhoE + du[4] + s.p + dp) + vn * (du[4] + dp);
}

// RusanovScalarOffDiagonal (src/fluxJacobian.cpp:122) for an inviscid,
// non-turbulent case: 0.5|A| (F(W+dU) - F(W)) +/- lambda_face dU.
template <typename T>
__device__ __forceinline__ void ScalarOffDiag(const Prim<T> &s, const T du[5],
                                              const Gas<T> &g, T nx, T ny, T nz,
                                              T mag, bool positive, T visc_sr, T out[5]) {
  T df[5];
  if constexpr (sizeof(T) == sizeof(float)) {
    ConvFluxDelta(s, du, g, nx, ny, nz, df);
  } else {
    const Prim<T> su = UpdateWithCons(s, g, du);
    T fo[5], fn[5];
    InvFlux(s, g, nx, ny, nz, fo);
    InvFlux(su, g, nx, ny, nz, fn);
#pragma unroll
    for (int v = 0; v < 5; ++v) df[v] = fn[v] - fo[v];
  }
  const T half = T(0.5) * mag;
  T lam = InvFaceSpecRad(s, g, nx, ny, nz, mag);
  lam += visc_sr;  // FaceSpectralRadius (include/spectralRadius.hpp:182)
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const T fc = half * df[v];
    out[v] = positive ? fc + lam * du[v] : fc - lam * du[v];
  }
}

// ScalarOffDiag with the neighbour's precomputed state terms (FP64): the
// same operations, with cons(W), H(W) and a(W) read instead of re-formed
template <typename T>
__device__ __forceinline__ void ScalarOffDiagPre(const Prim<T> &s, const NbrPre<T> &pre,
                                                 const T du[5], const Gas<T> &g, T nx, T ny,
                                                 T nz, T mag, bool positive, T visc_sr,
                                                 T out[5]) {
  T c[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) c[v] = pre.c[v] + du[v];
  const Prim<T> su = ConsToPrim(c, g);
  T fo[5], fn[5];
  const T vn = Dot(s.u, s.v, s.w, nx, ny, nz);
  fo[0] = s.rho * vn;
  fo[1] = s.rho * vn * s.u + s.p * nx;
  fo[2] = s.rho * vn * s.v + s.p * ny;
  fo[3] = s.rho * vn * s.w + s.p * nz;
  fo[4] = s.rho * vn * pre.h;
  InvFlux(su, g, nx, ny, nz, fn);
  T df[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) df[v] = fn[v] - fo[v];
  const T half = T(0.5) * mag;
  T lam = T(0.5) * mag * (fabs(vn) + pre.sos);
  lam += visc_sr;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const T fc = half * df[v];
    out[v] = positive ? fc + lam * du[v] : fc - lam * du[v];
  }
}

// ScalarOffDiagPre in the same two parts for an inviscid neighbour term
// (visc_sr = 0), with its operations and their order unchanged
template <typename T>
struct ExactOld {
  T vn, fo[5], half, lam;
};
template <typename T>
__device__ __forceinline__ ExactOld<T> ScalarOffDiagExactOld(const Prim<T> &s,
                                                            const NbrPre<T> &pre, T nx, T ny,
                                                            T nz, T mag) {
  ExactOld<T> o;
  o.vn = Dot(s.u, s.v, s.w, nx, ny, nz);
  o.fo[0] = s.rho * o.vn;
  o.fo[1] = s.rho * o.vn * s.u + s.p * nx;
  o.fo[2] = s.rho * o.vn * s.v + s.p * ny;
  o.fo[3] = s.rho * o.vn * s.w + s.p * nz;
  o.fo[4] = s.rho * o.vn * pre.h;
  o.half = T(0.5) * mag;
  o.lam = T(0.5) * mag * (fabs(o.vn) + pre.sos);
  return o;
}
template <typename T>
__device__ __forceinline__ void ScalarOffDiagExactNew(const ExactOld<T> &eo,
                                                      const NbrPre<T> &pre, const T du[5],
                                                      const Gas<T> &g, T nx, T ny, T nz,
                                                      bool positive, T out[5]) {
  T c[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) c[v] = pre.c[v] + du[v];
  const Prim<T> su = ConsToPrim(c, g);
  T fn[5];
  InvFlux(su, g, nx, ny, nz, fn);
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const T fc = eo.half * (fn[v] - eo.fo[v]);
    out[v] = positive ? fc + eo.lam * du[v] : fc - eo.lam * du[v];
  }
}

// ScalarOffDiagPreFast in two parts for an inviscid neighbour term: the
// part of the neighbour's state alone (its normal velocity and mass flux,
// its flux F(W).n, half the face area and the term's radius), which a
// hyperplane kernel forms before it waits for the previous plane, and the
// part with the neighbour's update
template <typename T>
struct FastOld {
  T vn, mo, f1, f2, f3, f4, half, lam;
};
template <typename T>
__device__ __forceinline__ FastOld<T> ScalarOffDiagFastOld(const Prim<T> &s,
                                                          const NbrPre<T> &pre, T nx, T ny,
                                                          T nz, T mag) {
  FastOld<T> o;
  o.vn = Dot(s.u, s.v, s.w, nx, ny, nz);
  o.mo = s.rho * o.vn;
  o.f1 = o.mo * s.u + s.p * nx;
  o.f2 = o.mo * s.v + s.p * ny;
  o.f3 = o.mo * s.w + s.p * nz;
  o.f4 = o.mo * pre.h;
  o.half = T(0.5) * mag;
  o.lam = o.half * (fabs(o.vn) + pre.sos);
  return o;
}
template <typename T>
__device__ __forceinline__ void ScalarOffDiagFastNew(const FastOld<T> &fo,
                                                     const NbrPre<T> &pre, const T du[5],
                                                     const Gas<T> &g, T nx, T ny, T nz,
                                                     bool positive, T out[5]) {
  T c[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) c[v] = pre.c[v] + du[v];
  const T ir = T(1) / c[0];
  const T u = c[1] * ir, v = c[2] * ir, w = c[3] * ir;
  const T ke = T(0.5) * (u * u + v * v + w * w);
  const T p = (g.gam - T(1)) * (c[4] - c[0] * (g.hf + ke));
  const T vnn = u * nx + v * ny + w * nz;
  const T mn = c[0] * vnn;
  T df[5];
  df[0] = mn - fo.mo;
  df[1] = (mn * u + p * nx) - fo.f1;
  df[2] = (mn * v + p * ny) - fo.f2;
  df[3] = (mn * w + p * nz) - fo.f3;
  df[4] = vnn * (c[4] + p) - fo.f4;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const T fc = fo.half * df[k];
    out[k] = positive ? fc + fo.lam * du[k] : fc - fo.lam * du[k];
  }
}

// ScalarOffDiagPre in the fast-arithmetic form of FP64 batches with the
// fast option: the updated state with one reciprocal of the density and no
// square root, p = (gamma - 1) (rho E - rho (hf + |v|^2 / 2)) and
// rho H = rho E + p; equal to the reference's form to roundoff.
template <typename T>
__device__ __forceinline__ void ScalarOffDiagPreFast(const Prim<T> &s, const NbrPre<T> &pre,
                                                     const T du[5], const Gas<T> &g, T nx, T ny,
                                                     T nz, T mag, bool positive, bool viscous,
                                                     T visc_sr, T out[5]) {
  T c[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) c[v] = pre.c[v] + du[v];
  const T ir = T(1) / c[0];
  const T u = c[1] * ir, v = c[2] * ir, w = c[3] * ir;
  const T ke = T(0.5) * (u * u + v * v + w * w);
  const T p = (g.gam - T(1)) * (c[4] - c[0] * (g.hf + ke));
  const T vnn = u * nx + v * ny + w * nz;
  const T mn = c[0] * vnn;
  const T vn = Dot(s.u, s.v, s.w, nx, ny, nz);
  const T mo = s.rho * vn;
  T df[5];
  df[0] = mn - mo;
  df[1] = (mn * u + p * nx) - (mo * s.u + s.p * nx);
  df[2] = (mn * v + p * ny) - (mo * s.v + s.p * ny);
  df[3] = (mn * w + p * nz) - (mo * s.w + s.p * nz);
  df[4] = vnn * (c[4] + p) - mo * pre.h;
  const T half = T(0.5) * mag;
  T lam = half * (fabs(vn) + pre.sos);
  if (viscous) lam += visc_sr;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const T fc = half * df[k];
    out[k] = positive ? fc + lam * du[k] : fc - lam * du[k];
  }
}

}  // namespace ath
