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

namespace ath {

template <typename T>
struct Gas {
  T r;   // nondimensional gas constant
  T n;   // cv / R
  T hf;  // nondimensional heat of formation
  // caloricallyPerfect::SpeciesCv / SpeciesCp (include/thermodynamic.hpp:110-115)
  __device__ __forceinline__ T Cv() const { return r * n; }
  __device__ __forceinline__ T Cp() const { return r * (n + T(1)); }
  // thermodynamic::Gamma (include/thermodynamic.hpp:58)
  __device__ __forceinline__ T Gamma() const { return Cp() / Cv(); }
};

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

template <typename T>
__device__ __forceinline__ Prim<T> Muscl(const Prim<T> &up2, const Prim<T> &up1,
                                         const Prim<T> &dw1, T uw2, T uw, T dw,
                                         T kappa, int limiter) {
  const T dplus = (uw + uw) / (uw + dw);
  const T dminus = (uw + uw) / (uw + uw2);
  Prim<T> o;
  o.rho = Muscl1(up2.rho, up1.rho, dw1.rho, dplus, dminus, kappa, limiter);
  o.u = Muscl1(up2.u, up1.u, dw1.u, dplus, dminus, kappa, limiter);
  o.v = Muscl1(up2.v, up1.v, dw1.v, dplus, dminus, kappa, limiter);
  o.w = Muscl1(up2.w, up1.w, dw1.w, dplus, dminus, kappa, limiter);
  o.p = Muscl1(up2.p, up1.p, dw1.p, dplus, dminus, kappa, limiter);
  return o;
}

// RoeFlux with Harten's entropy fix (include/inviscidFlux.hpp:260-382,
// src/inviscidFlux.cpp:27): F = 0.5 (FL + (FR - D)).
template <typename T>
__device__ __forceinline__ void RoeFlux(const Prim<T> &L, const Prim<T> &R,
                                        const Gas<T> &g, T nx, T ny, T nz,
                                        T f[5]) {
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
  const T dRho = R.rho - L.rho, dU = R.u - L.u, dV = R.v - L.v,
          dW = R.w - L.w, dP = R.p - L.p;
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

  T fl[5], fr[5];
  InvFlux(L, g, nx, ny, nz, fl);
  InvFlux(R, g, nx, ny, nz, fr);
  const T d[5] = {d0, d1, d2, d3, d4};
#pragma unroll
  for (int v = 0; v < 5; ++v) f[v] = (fl[v] + (fr[v] - d[v])) * T(0.5);
}

// InvCellSpectralRadius (include/spectralRadius.hpp:44)
template <typename T>
__device__ __forceinline__ T InvCellSpecRad(const Prim<T> &s, const Gas<T> &g,
                                            T lx, T ly, T lz, T lm, T ux,
                                            T uy, T uz, T um) {
  T ax = T(0.5) * (lx + ux), ay = T(0.5) * (ly + uy), az = T(0.5) * (lz + uz);
  const T am = sqrt(Dot(ax, ay, az, ax, ay, az));
  ax = ax / am;
  ay = ay / am;
  az = az / am;
  const T fMag = T(0.5) * (lm + um);
  return (fabs(Dot(s.u, s.v, s.w, ax, ay, az)) + SoS(s, g)) * fMag;
}

// InvFaceSpectralRadius (include/spectralRadius.hpp:67)
template <typename T>
__device__ __forceinline__ T InvFaceSpecRad(const Prim<T> &s, const Gas<T> &g,
                                            T nx, T ny, T nz, T mag) {
  return T(0.5) * mag * (fabs(Dot(s.u, s.v, s.w, nx, ny, nz)) + SoS(s, g));
}

// RusanovScalarOffDiagonal (src/fluxJacobian.cpp:122) for an inviscid,
// non-turbulent case: 0.5|A| (F(W+dU) - F(W)) +/- lambda_face dU.
template <typename T>
__device__ __forceinline__ void ScalarOffDiag(const Prim<T> &s, const T du[5],
                                              const Gas<T> &g, T nx, T ny, T nz,
                                              T mag, bool positive, T out[5]) {
  const Prim<T> su = UpdateWithCons(s, g, du);
  T fo[5], fn[5];
  InvFlux(s, g, nx, ny, nz, fo);
  InvFlux(su, g, nx, ny, nz, fn);
  const T half = T(0.5) * mag;
  const T lam = InvFaceSpecRad(s, g, nx, ny, nz, mag);
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const T fc = half * (fn[v] - fo[v]);
    out[v] = positive ? fc + lam * du[v] : fc - lam * du[v];
  }
}

}  // namespace ath
