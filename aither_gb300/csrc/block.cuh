// 5x5 block implicit operator of the block LU-SGS (blusgs) path: flux
// Jacobians, the thin-shear-layer viscous Jacobian, matrix-vector products
// and the Gauss-Jordan inverse, as device functions templated on the
// arithmetic type.  Matrices are row-major m[r * 5 + c] in registers (the
// fluxJacobian flow block with one species and no turbulence equations,
// include/fluxJacobian.hpp:92).  Operation order follows the reference
// expression by expression, so the FP64 instantiation compiled with
// --fmad=false reproduces the reference's last bits.
#pragma once

#include "physics.cuh"

namespace ath {

constexpr int kJac = 25;

// fluxJacobian::InvFluxJacobian (include/fluxJacobian.hpp:432): convective
// flux Jacobian along the unit normal n times 0.5 |A|
template <typename T>
__device__ __forceinline__ void InvFluxJac(const Prim<T> &s, const Gas<T> &g, T nx, T ny,
                                           T nz, T mag, T J[kJac]) {
  const T velNorm = Dot(s.u, s.v, s.w, nx, ny, nz);
  const T mf = s.rho / s.rho;  // mass fraction of the single species
  const T gamma = g.Gamma();
  const T gm1 = gamma - T(1);
  const T phi = T(0.5) * gm1 * Dot(s.u, s.v, s.w, s.u, s.v, s.w);
  const T a1 = gamma * Energy(s, g) - phi;
  const T a3 = gamma - T(2);
  J[0] = velNorm * (T(1) - mf);
  J[1] = mf * nx;
  J[2] = mf * ny;
  J[3] = mf * nz;
  J[4] = T(0);
  J[5] = phi * nx - s.u * velNorm;
  J[6] = velNorm - a3 * nx * s.u;
  J[7] = s.u * ny - gm1 * s.v * nx;
  J[8] = s.u * nz - gm1 * s.w * nx;
  J[9] = gm1 * nx;
  J[10] = phi * ny - s.v * velNorm;
  J[11] = s.v * nx - gm1 * s.u * ny;
  J[12] = velNorm - a3 * ny * s.v;
  J[13] = s.v * nz - gm1 * s.w * ny;
  J[14] = gm1 * ny;
  J[15] = phi * nz - s.w * velNorm;
  J[16] = s.w * nx - gm1 * s.u * nz;
  J[17] = s.w * ny - gm1 * s.v * nz;
  J[18] = velNorm - a3 * nz * s.w;
  J[19] = gm1 * nz;
  J[20] = velNorm * (phi - a1);
  J[21] = a1 * nx - gm1 * s.u * velNorm;
  J[22] = a1 * ny - gm1 * s.v * velNorm;
  J[23] = a1 * nz - gm1 * s.w * velNorm;
  J[24] = gamma * velNorm;
  const T f = T(0.5) * mag;
#pragma unroll
  for (int e = 0; e < kJac; ++e) J[e] *= f;
}

// fluxJacobian::RusanovFluxJacobian (include/fluxJacobian.hpp:405):
// J = A(W) 0.5|A| +/- lambda_face I, the dissipation added element by element
template <typename T>
__device__ __forceinline__ void RusanovJac(const Prim<T> &s, const Gas<T> &g, T nx, T ny,
                                           T nz, T mag, bool positive, T J[kJac]) {
  const T specRad = InvFaceSpecRad(s, g, nx, ny, nz, mag);
  InvFluxJac(s, g, nx, ny, nz, mag, J);
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      const T dis = (r == c) ? T(1) * specRad : T(0);
      J[r * 5 + c] = positive ? J[r * 5 + c] + dis : J[r * 5 + c] - dis;
    }
}

// TauNormal (src/utility.cpp:426) with the velocity-gradient tensor g[r][c]
// (row r: derivative along axis r)
template <typename T>
__device__ __forceinline__ void TauNormal(const T vg[9], T nx, T ny, T nz, T mu, T mut,
                                          T tau[3]) {
  const T nrm[3] = {nx, ny, nz};
  const T lambda = T(0) - (T(2) / T(3)) * (mu + mut);
  const T trace = vg[0] + vg[4] + vg[8];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const T sn = (vg[r * 3 + 0] + vg[0 * 3 + r]) * nrm[0] +
                 (vg[r * 3 + 1] + vg[1 * 3 + r]) * nrm[1] +
                 (vg[r * 3 + 2] + vg[2 * 3 + r]) * nrm[2];
    tau[r] = lambda * trace * nrm[r] + (mu + mut) * sn;
  }
}

// Laminar transport of the thin-shear-layer Jacobian: nondimensional
// scaling and Sutherland conductivity coefficients.
template <typename T>
struct TslCoeffs {
  T scale, t_ref, k_c1, k_s, k_ref;
  T prt;  // turbulent Prandtl number of the solve's model
};

// J <- J - T(W) (subtract) or J + T(W) with T the approximate thin-shear-
// layer Jacobian (fluxJacobian::ApproxTSLJacobian, include/fluxJacobian.hpp:
// 667) multiplied by dW/dU (DelprimitiveDelConservative :626) through
// MatrixMultiply (src/matrix.cpp:197); laminar, one species, no diffusion
// model.  `left` is the reference's flag (sign of the tau term).
template <typename T>
__device__ __forceinline__ void TslJacAccum(const Prim<T> &s, T mu_lam, T mut_lam,
                                            const Gas<T> &g, const TslCoeffs<T> &k_, T nx,
                                            T ny, T nz, T mag, T dist, bool left,
                                            const T vg[9], bool subtract, T J[kJac]) {
  const T t = Temperature(s, g);
  const T mu = k_.scale * mu_lam;
  const T mut = k_.scale * mut_lam;
  const T velNorm = Dot(s.u, s.v, s.w, nx, ny, nz);
  const T rho = s.rho;
  const T k = SutherlandRatio(t, k_.t_ref, k_.k_c1, k_.k_s, k_.k_ref) * k_.scale;
  const T kt = mut * g.Cp() / k_.prt;
  T tau[3];
  TauNormal(vg, nx, ny, nz, mu, mut, tau);
  const T fac = left ? T(-1) : T(1);
  const T third = T(1) / T(3);
  const T f = mag * (mu + mut) / dist;
  T M[kJac];
#pragma unroll
  for (int e = 0; e < kJac; ++e) M[e] = T(0);
  M[20] = -(k + kt) * t / ((mu + mut) * rho) + T(0);
  M[6] = third * nx * nx + T(1);
  M[11] = third * nx * ny;
  M[16] = third * nx * nz;
  M[21] = fac * T(0.5) * dist / (mu + mut) * tau[0] + third * nx * velNorm + s.u;
  M[7] = third * ny * nx;
  M[12] = third * ny * ny + T(1);
  M[17] = third * ny * nz;
  M[22] = fac * T(0.5) * dist / (mu + mut) * tau[1] + third * ny * velNorm + s.v;
  M[8] = third * nz * nx;
  M[13] = third * nz * ny;
  M[18] = third * nz * nz + T(1);
  M[23] = fac * T(0.5) * dist / (mu + mut) * tau[2] + third * nz * velNorm + s.w;
  M[24] = (k + kt) / ((mu + mut) * rho);
#pragma unroll
  for (int e = 0; e < kJac; ++e) M[e] *= f;
  const T gm1 = g.Gamma() - T(1);
  const T invRho = T(1) / rho;
  T Pm[kJac];
#pragma unroll
  for (int e = 0; e < kJac; ++e) Pm[e] = T(0);
  Pm[0] = T(1);
  Pm[5] = -invRho * s.u;
  Pm[10] = -invRho * s.v;
  Pm[15] = -invRho * s.w;
  Pm[20] = T(0.5) * gm1 * Dot(s.u, s.v, s.w, s.u, s.v, s.w);
  Pm[6] = invRho;
  Pm[21] = -gm1 * s.u;
  Pm[12] = invRho;
  Pm[22] = -gm1 * s.v;
  Pm[18] = invRho;
  Pm[23] = -gm1 * s.w;
  Pm[24] = gm1;
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      T acc = T(0);
#pragma unroll
      for (int c = 0; c < 5; ++c) acc = acc + M[r * 5 + c] * Pm[c * 5 + i];
      J[r * 5 + i] = subtract ? J[r * 5 + i] - acc : J[r * 5 + i] + acc;
    }
}

// ArrayMultiplication (include/fluxJacobian.hpp:46): out = M x, each row
// accumulated from zero
template <typename T>
__device__ __forceinline__ void MatVec5(const T M[kJac], const T x[5], T out[5]) {
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    T s = T(0);
#pragma unroll
    for (int c = 0; c < 5; ++c) s = s + M[r * 5 + c] * x[c];
    out[r] = s;
  }
}

// 2x2 turbulence parts of the block operator: Rusanov Jacobian 0.5 conv
// +/- 0.5 diss (turbModel::InviscidConvectiveJacobian /
// InviscidDissipationJacobian, src/turbulence.cpp:73-92) and the SST
// viscous Jacobian times fac (turbKWSst::ViscJac, :764).
template <typename T>
__device__ __forceinline__ void TurbRusanovJac(const Prim<T> &s, T nx, T ny, T nz, T mag,
                                               bool positive, T J[4]) {
  const T vn = Dot(s.u, s.v, s.w, nx, ny, nz);
  const T conv = vn * mag, diss = fabs(vn) * mag;
  const T cj[4] = {T(0.5) * conv, T(0.5) * T(0), T(0.5) * T(0), T(0.5) * conv};
  const T dj[4] = {T(0.5) * diss, T(0.5) * T(0), T(0.5) * T(0), T(0.5) * diss};
#pragma unroll
  for (int e = 0; e < 4; ++e) J[e] = positive ? cj[e] + dj[e] : cj[e] - dj[e];
}
// The k and omega equations' diffusivities mu + sigma mu_t of the
// turbulence radii and Jacobians: SST-2003 blends sigma with F1 and takes
// the limited eddy viscosity mut, Wilcox k-omega 2006 takes sigma* = 0.6,
// sigma = 0.5 and the unlimited rho k / omega (nut) of the state
// (turbKWSst / turbKWWilcox ::ViscJac, ViscousCell/FaceSpectralRadius,
// src/turbulence.cpp:485-547,764-797)
template <typename T>
struct TurbDiff {
  T k, w;
};
template <typename T>
__device__ __forceinline__ TurbDiff<T> TurbDiffOf(bool wilcox, T mu, T mut, T f1, T nut) {
  if (wilcox) return TurbDiff<T>{mu + T(0.6) * nut, mu + T(0.5) * nut};
  const T sk = f1 * T(0.85) + (T(1) - f1) * T(1.0);
  const T sw = f1 * T(0.5) + (T(1) - f1) * T(0.856);
  return TurbDiff<T>{mu + sk * mut, mu + sw * mut};
}
template <typename T>
__device__ __forceinline__ void TurbViscJac(T rho, T mag, const TurbDiff<T> &df, T dist,
                                            T scale, T fac, T J[4]) {
  const T length = mag / dist;
  const T j00 = scale * length / rho * df.k;
  const T j11 = scale * length / rho * df.w;
  J[0] = fac * j00;
  J[1] = fac * T(0);
  J[2] = fac * T(0);
  J[3] = fac * j11;
}
// MatrixInverse of the 2x2 turbulence block (src/matrix.cpp:57)
template <typename T>
__device__ __forceinline__ void Inverse2(T a[4]) {
  T I[4] = {T(1), T(0), T(0), T(1)};
  // column 0: pivot among rows 0, 1 (row 0 when both are zero)
  const int rp = (fabs(a[2]) > fabs(a[0])) ? 1 : 0;
  if (rp == 1) {
    T t = a[0]; a[0] = a[2]; a[2] = t;
    t = a[1]; a[1] = a[3]; a[3] = t;
    t = I[0]; I[0] = I[2]; I[2] = t;
    t = I[1]; I[1] = I[3]; I[3] = t;
  }
  T nf = T(1) / a[0];
  a[0] *= nf;
  a[1] *= nf;
  I[0] *= nf;
  I[1] *= nf;
  // column 1: only row 1 remains
  const T factor = a[2] / a[0];
  a[2] = a[2] - factor * a[0];
  a[3] = a[3] - factor * a[1];
  I[2] = I[2] - factor * I[0];
  I[3] = I[3] - factor * I[1];
  nf = T(1) / a[3];
  a[3] *= nf;
  I[2] *= nf;
  I[3] *= nf;
  // back substitution
  const T f2 = a[1];
  a[0] = a[0] - f2 * a[2];
  a[1] = a[1] - f2 * a[3];
  I[0] = I[0] - f2 * I[2];
  I[1] = I[1] - f2 * I[3];
#pragma unroll
  for (int e = 0; e < 4; ++e) a[e] = I[e];
}
template <typename T>
__device__ __forceinline__ void MatVec2(const T M[4], const T x[2], T out[2]) {
  T s0 = T(0), s1 = T(0);
  s0 = s0 + M[0] * x[0];
  s0 = s0 + M[1] * x[1];
  s1 = s1 + M[2] * x[0];
  s1 = s1 + M[3] * x[1];
  out[0] = s0;
  out[1] = s1;
}

// MatrixInverse (src/matrix.cpp:57): Gauss-Jordan with the reference's pivot
// rule (largest magnitude in the column among the rows not yet reduced,
// searched before the row is reduced; row 0 when the column is all zero).
// Row swaps are predicated register moves.
template <typename T>
__device__ __forceinline__ void Inverse5(T a[kJac]) {
  T I[kJac];
#pragma unroll
  for (int e = 0; e < kJac; ++e) I[e] = (e % 6 == 0) ? T(1) : T(0);
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    T maxv = T(0);
    int rp = 0;
#pragma unroll
    for (int ii = r; ii < 5; ++ii) {
      const T m = fabs(a[ii * 5 + r]);
      if (m > maxv) {
        maxv = m;
        rp = ii;
      }
    }
#pragma unroll
    for (int ii = 0; ii < 5; ++ii) {
      if (ii == r) continue;
      const bool sw = rp == ii;
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        const T ta = a[r * 5 + c], tb = a[ii * 5 + c];
        a[r * 5 + c] = sw ? tb : ta;
        a[ii * 5 + c] = sw ? ta : tb;
        const T ia = I[r * 5 + c], ib = I[ii * 5 + c];
        I[r * 5 + c] = sw ? ib : ia;
        I[ii * 5 + c] = sw ? ia : ib;
      }
    }
#pragma unroll
    for (int ii = 0; ii < r; ++ii) {
      const T factor = a[r * 5 + ii] / a[ii * 5 + ii];
#pragma unroll
      for (int c = 0; c < 5; ++c) a[r * 5 + c] = a[r * 5 + c] - factor * a[ii * 5 + c];
#pragma unroll
      for (int c = 0; c < 5; ++c) I[r * 5 + c] = I[r * 5 + c] - factor * I[ii * 5 + c];
    }
    const T normFactor = T(1) / a[r * 5 + r];
#pragma unroll
    for (int c = r; c < 5; ++c) a[r * 5 + c] *= normFactor;
#pragma unroll
    for (int c = 0; c < 5; ++c) I[r * 5 + c] *= normFactor;
  }
#pragma unroll
  for (int r = 3; r >= 0; --r)
#pragma unroll
    for (int ii = 4; ii > r; --ii) {
      const T factor = a[r * 5 + ii];
#pragma unroll
      for (int c = 0; c < 5; ++c) a[r * 5 + c] = a[r * 5 + c] - factor * a[ii * 5 + c];
#pragma unroll
      for (int c = 0; c < 5; ++c) I[r * 5 + c] = I[r * 5 + c] - factor * I[ii * 5 + c];
    }
#pragma unroll
  for (int e = 0; e < kJac; ++e) a[e] = I[e];
}

}  // namespace ath
