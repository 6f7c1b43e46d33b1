/* CPU oracle of the per-iteration solver step -- TEST INFRASTRUCTURE ONLY.
 * See aither_oracle.h.  Every function names the reference function it
 * restates (paths inside the reference project).  Arithmetic is written in
 * the reference's evaluation order; build with -ffp-contract=off. */
#include <float.h>
#include "aither_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NV 5

typedef struct {
  double r, n, hf;
} gas_t;

typedef struct {
  int ni, nj, nk, ng, NI, NJ, NK, solve;
  int64_t nc, nf[3];
  double *vol, *width; /* width: [3][nc] */
  double *fa[3];       /* [4][nf] */
  double *W;           /* [nc][5] primitive, AoS as in the reference */
  double *R;           /* [nc][5] */
  double *dU;          /* [nc][5] */
  double *Un, *Unm1;   /* [nc][7] conserved state of time levels n, n-1 */
  double *lam, *dt, *A, *Ainv; /* [nc] */
  double *Ab, *Ainvb;  /* [nc][25] block diagonal and its inverse (blusgs) */
  double *vg;          /* [nc][9] cell-averaged velocity gradient (blusgs) */
  uint8_t *wallf[3];   /* [nf] face is a viscous wall */
  /* RANS (SST-2003): turbulence variables beside the five flow variables */
  double *Wt, *Rt, *dUt;        /* [nc][2] k, omega; residual; update */
  double *lamt, *At, *Ainvt;    /* [nc] turbulence radius, scalar diagonal */
  double *Abt, *Ainvbt;         /* [nc][4] 2x2 block diagonal */
  double *mutc, *f1c, *f2c;     /* [nc] cell eddy viscosity, blending */
  double *kgc, *wgc;            /* [nc][3] cell k, omega gradients */
  double *wd;                   /* [nc] wall distance */
  double force[6];     /* wall forces of the last residual: p A, tau |A| */
  uint8_t *mask;
  double *center;      /* [3][nc] */
  double *T, *mu;      /* [nc] temperature, laminar viscosity (aux) */
  uint8_t *corner;     /* [nc] ghost in all three directions */
  int nops;
  ath_ghost_op *ops;
  int nedge, nvops, nvedge;
  ath_ghost_op *edge, *vops, *vedge;
  int nplanes;
  int32_t *plane_off, *plane_cells;
  int n_nr, n_nr_surf;     /* nonreflecting surfaces: cells, surfaces */
  ath_nr_cell *nr;
  double *nr_mach;         /* [n_nr_surf][2] average, largest Mach */
  double *nrg;  /* [nc][12] velocity (9) and pressure (3) gradients of the
                   previous residual at the cells nonreflecting pressure
                   outlets read (NULL without such outlets) */
  /* multigrid: forcing of a coarse level's linear system (gridLevel
   * mgForcing_), the matrix residual of this level's last relaxation, and
   * the transfer to the next coarser level (its block, and per physical
   * cell the coarse cell, restriction weight, 7 prolongation coefficients) */
  double *F, *mr;      /* [nc][5], NULL without multigrid */
  double *og;          /* [nc][24] output gradients of the last residual
                          (orc_set_output_grads; NULL otherwise) */
  int mg_coarse;
  int32_t *mg_cell;
  double *mg_volfac, *mg_coef;
} oblock;

typedef struct {
  ath_solve_view v;
  ath_bc_state *states;
  gas_t gas;
  double cfl;
  int viscous;
  int block;   /* blusgs: 5x5 Jacobian diagonal and off-diagonals */
  int rans;    /* k-omega turbulence equations (SST-2003 or Wilcox 2006) */
  int wilcox;  /* Wilcox k-omega 2006 instead of SST-2003 */
  int sweeps;  /* matrixSweeps */
  int jacobi;  /* dplur / bdplur: Jacobi sweeps instead of LU-SGS */
  int nm1_given; /* time n-1 set from a restart: kept at the first step */
} osolve;

struct orc_case {
  int nb, ns;
  oblock *b;
  osolve *s;
  int64_t iter;
  int nthreads;
  int matrix_resid;     /* compute the logged matrix residual */
  double *mres;         /* [ns] last matrix residual */
  double *forces;       /* [ns][6] wall forces of the last residual */
  struct orc_case *coarse;  /* next coarser multigrid level (NULL: none) */
  int mg_cycle;             /* 1 V, 2 W */
  /* visits of this (coarse) level in the current iteration: its implicit
   * diagonal is zeroed only after each update (gridLevel::ResetDiagonal,
   * src/mgSolution.cpp:225-228), so a level a W cycle visits again adds its
   * new spectral radii to the diagonal of the previous visit */
  int mg_visits;
};

/* ---------------------------------------------------------------- thermo */
/* caloricallyPerfect (include/thermodynamic.hpp:102-115) and idealGas
 * (src/eos.cpp), one species, mass fraction 1. */
static double cv_of(const gas_t *g) { return g->r * g->n; }
static double cp_of(const gas_t *g) { return g->r * (g->n + 1.0); }
static double gamma_of(const gas_t *g) { return cp_of(g) / cv_of(g); }
static double temp_of(const double *w, const gas_t *g) { return w[4] / (w[0] * g->r); }
static double velmag(const double *w) {
  return sqrt(w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
}
/* SpeedOfSound (include/arrayView.hpp:384) */
static double sos_of(const double *w, const gas_t *g) {
  return sqrt(gamma_of(g) * w[4] / w[0]);
}
/* EnthalpyFunc (include/arrayView.hpp:401) */
static double enthalpy_of(const double *w, const gas_t *g) {
  const double t = temp_of(w, g);
  const double vm = velmag(w);
  return (g->hf + cp_of(g) * t) + 0.5 * vm * vm;
}
/* InternalEnergy (include/arrayView.hpp:436) */
static double energy_of(const double *w, const gas_t *g) {
  const double t = temp_of(w, g);
  const double vm = velmag(w);
  return (g->hf + cv_of(g) * t) + 0.5 * vm * vm;
}
/* PrimToCons (include/primitive.hpp:183) */
static void prim_to_cons(const double *w, const gas_t *g, double *c) {
  c[0] = w[0];
  c[1] = w[0] * w[1];
  c[2] = w[0] * w[2];
  c[3] = w[0] * w[3];
  c[4] = w[0] * energy_of(w, g);
}
/* primitive(conserved) (include/primitive.hpp:137), PressFromEnergy
 * (src/eos.cpp:40), TemperatureFromSpecEnergy (src/thermodynamic.cpp:107) */
static void cons_to_prim(const double *c, const gas_t *g, double *w) {
  const double rho = c[0];
  w[0] = rho;
  w[1] = c[1] / rho;
  w[2] = c[2] / rho;
  w[3] = c[3] / rho;
  const double energy = c[4] / rho;
  const double vel = velmag(w);
  const double spec = energy - 0.5 * vel * vel;
  const double t = (spec - g->hf) / cv_of(g);
  w[4] = rho * g->r * t;
}
/* UpdatePrimWithCons (include/primitive.hpp:206) */
static void update_with_cons(const double *w, const gas_t *g, const double *du,
                             double *out) {
  double c[NV];
  prim_to_cons(w, g, c);
  for (int v = 0; v < NV; ++v) c[v] = c[v] + du[v];
  cons_to_prim(c, g, out);
}
/* inviscidFlux::ConstructFromPrim (include/inviscidFlux.hpp:129) */
static void inv_flux(const double *w, const gas_t *g, const double *n, double *f) {
  const double vn = w[1] * n[0] + w[2] * n[1] + w[3] * n[2];
  f[0] = w[0] * vn;
  f[1] = w[0] * vn * w[1] + w[4] * n[0];
  f[2] = w[0] * vn * w[2] + w[4] * n[1];
  f[3] = w[0] * vn * w[3] + w[4] * n[2];
  f[4] = w[0] * vn * enthalpy_of(w, g);
}

/* ------------------------------------------------------- reconstruction */
static double lim_minmod(double r) {
  const double m = (r < 1.0) ? r : 1.0; /* std::min(1.0, r) */
  return (0.0 < m) ? m : 0.0;           /* std::max(0.0, m) */
}
static double lim_vanalbada(double r) {
  const double r2 = r * r;
  const double l = (r + r2) / (1.0 + r2);
  return (0.0 < l) ? l : 0.0;
}
/* FaceReconMUSCL (include/reconstruction.hpp:110), limiters
 * src/limiter.cpp:24,36 */
static void muscl_n(const double *up2, const double *up1, const double *dw1,
                    double kappa, int limiter, double uw2, double uw, double dw,
                    double *out, int n) {
  const double dPlus = (uw + uw) / (uw + dw);
  const double dMinus = (uw + uw) / (uw + uw2);
  for (int v = 0; v < n; ++v) {
    const double r = (1.0e-30 + (dw1[v] - up1[v]) * dPlus) /
                     (1.0e-30 + (up1[v] - up2[v]) * dMinus);
    double l, il;
    if (limiter == ATH_LIMITER_MINMOD) {
      l = lim_minmod(r);
      il = lim_minmod(1.0 / r);
    } else if (limiter == ATH_LIMITER_VANALBADA) {
      l = lim_vanalbada(r);
      il = lim_vanalbada(1.0 / r);
    } else {
      l = 1.0;
      il = 1.0;
    }
    out[v] = up1[v] + 0.25 * ((up1[v] - up2[v]) * dMinus) *
                          ((1.0 - kappa) * l + (1.0 + kappa) * r * il);
  }
}

/* ------------------------------------------------------------- Roe flux */
/* RoeFlux (include/inviscidFlux.hpp:260), RoeAveragedState
 * (include/primitive.hpp:245), inviscidFlux::RoeFlux (src/inviscidFlux.cpp:27) */
static void roe_flux(const double *L, const double *R, const double *Lt, const double *Rt,
                     const gas_t *g, const double *n, double *f, double *ft) {
  const double denRatio = sqrt(R[0] / L[0]);
  double roe[NV];
  roe[0] = L[0] * denRatio;
  roe[1] = (L[1] + denRatio * R[1]) / (1.0 + denRatio);
  roe[2] = (L[2] + denRatio * R[2]) / (1.0 + denRatio);
  roe[3] = (L[3] + denRatio * R[3]) / (1.0 + denRatio);
  roe[4] = (L[4] + denRatio * R[4]) / (1.0 + denRatio);
  const double hR = enthalpy_of(roe, g);
  const double aR = sos_of(roe, g);
  const double rhoR = roe[0];
  const double velNormR = roe[1] * n[0] + roe[2] * n[1] + roe[3] * n[2];
  const double mfR = roe[0] / rhoR;
  double delta[NV];
  for (int v = 0; v < NV; ++v) delta[v] = R[v] - L[v];
  const double nvd = delta[1] * n[0] + delta[2] * n[1] + delta[3] * n[2];
  double d[NV] = {0, 0, 0, 0, 0};
  const double fix = 0.1;

  double ws = fabs(velNormR - aR);
  if (ws < fix) ws = 0.5 * (ws * ws / fix + fix);
  double st = (delta[4] - rhoR * aR * nvd) / (2.0 * aR * aR);
  double wss = ws * st;
  const double wssL = wss;
  d[0] += wss * mfR;
  d[1] += wss * (roe[1] - aR * n[0]);
  d[2] += wss * (roe[2] - aR * n[1]);
  d[3] += wss * (roe[3] - aR * n[2]);
  d[4] += wss * (hR - aR * velNormR);

  ws = fabs(velNormR);
  st = -delta[4] / (aR * aR);
  wss = ws * st;
  d[0] += wss * mfR + ws * delta[0];
  st = delta[0] - delta[4] / (aR * aR);
  wss = ws * st;
  d[1] += wss * roe[1];
  d[2] += wss * roe[2];
  d[3] += wss * roe[3];
  d[4] += wss * 0.5 * (roe[1] * roe[1] + roe[2] * roe[2] + roe[3] * roe[3]);

  st = rhoR;
  wss = ws * st;
  d[1] += wss * (delta[1] - nvd * n[0]);
  d[2] += wss * (delta[2] - nvd * n[1]);
  d[3] += wss * (delta[3] - nvd * n[2]);
  d[4] += wss * ((roe[1] * delta[1] + roe[2] * delta[2] + roe[3] * delta[3]) -
                 velNormR * nvd);

  ws = fabs(velNormR + aR);
  if (ws < fix) ws = 0.5 * (ws * ws / fix + fix);
  st = (delta[4] + rhoR * aR * nvd) / (2.0 * aR * aR);
  wss = ws * st;
  d[0] += wss * mfR;
  d[1] += wss * (roe[1] + aR * n[0]);
  d[2] += wss * (roe[2] + aR * n[1]);
  d[3] += wss * (roe[3] + aR * n[2]);
  d[4] += wss * (hR + aR * velNormR);

  double fl[NV], fr[NV];
  inv_flux(L, g, n, fl);
  inv_flux(R, g, n, fr);
  for (int v = 0; v < NV; ++v) {
    f[v] = fl[v] + (fr[v] - d[v]);
    f[v] *= 0.5;
  }
  if (ft) {
    /* turbulence: both acoustic waves carry the Roe-averaged k, omega, plus
     * the turbulence waves (include/inviscidFlux.hpp:311-368) */
    const double vnL = L[1] * n[0] + L[2] * n[1] + L[3] * n[2];
    const double vnR = R[1] * n[0] + R[2] * n[1] + R[3] * n[2];
    for (int q = 0; q < 2; ++q) {
      const double rt = (Lt[q] + denRatio * Rt[q]) / (1.0 + denRatio);
      double dq = 0.0;
      dq += wssL * rt;
      dq += wss * rt;
      const double wsT = fabs(velNormR);
      const double stT = rhoR * (Rt[q] - Lt[q]) + rt * delta[0] - delta[4] * rt / (aR * aR);
      dq += wsT * stT * 1.0;
      const double flt = L[0] * vnL * Lt[q], frt = R[0] * vnR * Rt[q];
      ft[q] = flt + (frt - dq);
      ft[q] *= 0.5;
    }
  }
}

/* ------------------------------------------------------------ WENO5 */
/* StencilWidth (include/utility.hpp:104) */
static double stencil_width(const double *w, int start, int end) {
  double width = 0.0;
  if (end > start) {
    for (int q = start; q < end; ++q) width += w[q];
  } else if (start > end) {
    double a = 0.0;
    for (int q = end; q < start; ++q) a += w[q];
    width = -1.0 * a;
  }
  return width;
}
/* LagrangeCoeff (src/utility.cpp:449): weights of the cell averages that
 * reconstruct the value at the upper face of cell ii on a non-uniform
 * stencil starting rr cells left of ii */
static void lagrange_coeff(const double *w, int degree, int rr, int ii, double *coeffs) {
  for (int jj = 0; jj <= degree; ++jj) {
    coeffs[jj] = 0.0;
    for (int mm = jj + 1; mm <= degree + 1; ++mm) {
      double numer = 0.0, denom = 1.0;
      for (int ll = 0; ll <= degree + 1; ++ll) {
        if (ll != mm) {
          double numProd = 1.0;
          for (int qq = 0; qq <= degree + 1; ++qq)
            if (qq != mm && qq != ll) numProd *= stencil_width(w, ii - rr + qq, ii + 1);
          numer += numProd;
          denom *= stencil_width(w, ii - rr + ll, ii - rr + mm);
        }
      }
      coeffs[jj] += numer / denom;
    }
    coeffs[jj] *= w[ii - rr + jj];
  }
}
/* Derivative2nd (include/utility.hpp:117) */
static double deriv2nd(double x0, double x1, double x2, double y0, double y1, double y2) {
  const double fwd = (y2 - y1) / (0.5 * (x2 + x1));
  const double bck = (y1 - y0) / (0.5 * (x1 + x0));
  return (fwd - bck) / (0.25 * (x2 + x0) + 0.5 * x1);
}
/* BetaIntegral (include/reconstruction.hpp:157,171) */
static double beta_int(double d1, double d2, double dx, double x) {
  return (d1 * d1 * x + d1 * d2 * x * x + d2 * d2 * pow(x, 3.0) / 3.0) * dx +
         d2 * d2 * x * pow(dx, 3.0);
}
static double beta_int2(double d1, double d2, double dx, double xl, double xh) {
  return beta_int(d1, d2, dx, xh) - beta_int(d1, d2, dx, xl);
}
/* FaceReconWENO (include/reconstruction.hpp:244) with Beta0/1/2 (:186-240);
 * c[5] = (upwind3, upwind2, upwind1, downwind1, downwind2), w[5] widths */
static void weno_n(const double *const c[5], const double w[5], int wenoz, double *out, int n) {
  double c0[3], c1[3], c2[3], full[5];
  lagrange_coeff(w, 2, 2, 2, c0);
  lagrange_coeff(w, 2, 1, 2, c1);
  lagrange_coeff(w, 2, 0, 2, c2);
  lagrange_coeff(w, 4, 2, 2, full);
  const double lw0 = full[0] / c0[0];
  const double lw1 = full[4] / c2[2];
  const double lw2 = 1.0 - lw0 - lw1;
  for (int v = 0; v < n; ++v) {
    const double y3 = c[0][v], y2 = c[1][v], y1 = c[2][v], d1 = c[3][v], d2 = c[4][v];
    const double st0 = c0[0] * y3 + c0[1] * y2 + c0[2] * y1;
    const double st1 = c1[0] * y2 + c1[1] * y1 + c1[2] * d1;
    const double st2 = c2[0] * y1 + c2[1] * d1 + c2[2] * d2;
    double b0, b1, b2;
    {
      const double dd = deriv2nd(w[0], w[1], w[2], y3, y2, y1);
      const double d = (y1 - y2) / (0.5 * (w[2] + w[1])) + 0.5 * w[2] * dd;
      b0 = beta_int2(d, dd, w[2], -0.5 * w[2], 0.5 * w[2]);
    }
    {
      const double dd = deriv2nd(w[1], w[2], w[3], y2, y1, d1);
      const double d = (d1 - y1) / (0.5 * (w[3] + w[2])) - 0.5 * w[2] * dd;
      b1 = beta_int2(d, dd, w[2], -0.5 * w[2], 0.5 * w[2]);
    }
    {
      const double dd = deriv2nd(w[2], w[3], w[4], y1, d1, d2);
      const double d = (d1 - y1) / (0.5 * (w[3] + w[2])) - 0.5 * w[2] * dd;
      b2 = beta_int2(d, dd, w[2], -0.5 * w[2], 0.5 * w[2]);
    }
    double n0, n1, n2;
    if (wenoz) {
      const double tau5 = fabs(b0 - b2);
      const double t0 = tau5 / (1.0e-40 + b0), t1 = tau5 / (1.0e-40 + b1),
                   t2 = tau5 / (1.0e-40 + b2);
      n0 = lw0 * (1.0 + t0 * t0);
      n1 = lw1 * (1.0 + t1 * t1);
      n2 = lw2 * (1.0 + t2 * t2);
    } else {
      n0 = lw0 / ((1.0e-6 + b0) * (1.0e-6 + b0));
      n1 = lw1 / ((1.0e-6 + b1) * (1.0e-6 + b1));
      n2 = lw2 / ((1.0e-6 + b2) * (1.0e-6 + b2));
    }
    const double sum = n0 + n1 + n2;
    n0 /= sum;
    n1 /= sum;
    n2 /= sum;
    out[v] = n0 * st0 + n1 * st1 + n2 * st2;
  }
}

/* ---------------------------------------------------------- AUSMPW+ flux */
/* AUSMFlux (include/inviscidFlux.hpp:396) and inviscidFlux::AUSMFlux
 * (:162), Sign (include/utility.hpp:126) */
static double sign_of(double x) { return (double)((0.0 < x) - (x < 0.0)); }
static void ausm_flux(const double *L, const double *R, const double *Lt, const double *Rt,
                      const gas_t *g, const double *n, double *f, double *ft) {
  const double vnL = L[1] * n[0] + L[2] * n[1] + L[3] * n[2];
  const double vnR = R[1] * n[0] + R[2] * n[1] + R[3] * n[2];
  const double sosL = sos_of(L, g), sosR = sos_of(R, g);
  const double sosStar = sqrt(sosL * sosR);
  const double vel = 0.5 * (vnL + vnR);
  double sos = sosStar;
  if (vel < 0.0) {
    sos = sosStar * sosStar / ((vnR < sosStar) ? sosStar : vnR);
  } else if (vel > 0.0) {
    sos = sosStar * sosStar / ((vnL < sosStar) ? sosStar : vnL);
  }
  const double ml = vnL / sos, mr = vnR / sos;
  const double mPlusL = fabs(ml) <= 1.0 ? 0.25 * pow(ml + 1.0, 2.0) : 0.5 * (ml + fabs(ml));
  const double mMinusR = fabs(mr) <= 1.0 ? -0.25 * pow(mr - 1.0, 2.0) : 0.5 * (mr - fabs(mr));
  const double pPlus = fabs(ml) <= 1.0 ? 0.25 * pow(ml + 1.0, 2.0) * (2.0 - ml)
                                       : 0.5 * (1.0 + sign_of(ml));
  const double pMinus = fabs(mr) <= 1.0 ? 0.25 * pow(mr - 1.0, 2.0) * (2.0 + mr)
                                        : 0.5 * (1.0 - sign_of(mr));
  const double ps = pPlus * L[4] + pMinus * R[4];
  const double ra = L[4] / R[4], rb = R[4] / L[4];
  const double w = 1.0 - pow((rb < ra) ? rb : ra, 3.0);
  const double fl = fabs(ml) < 1.0 ? L[4] / ps - 1.0 : 0.0;
  const double fr = fabs(mr) < 1.0 ? R[4] / ps - 1.0 : 0.0;
  const double mavg = mPlusL + mMinusR;
  const double mPlusLBar = mavg >= 0.0 ? mPlusL + mMinusR * ((1.0 - w) * (1.0 + fr) - fl)
                                       : mPlusL * w * (1.0 + fl);
  const double mMinusRBar = mavg >= 0.0 ? mMinusR * w * (1.0 + fr)
                                        : mMinusR + mPlusL * ((1.0 - w) * (1.0 + fl) - fr);
  const double vl = mPlusLBar * sos;
  f[0] = L[0] * vl;
  f[1] = L[0] * vl * L[1] + pPlus * L[4] * n[0];
  f[2] = L[0] * vl * L[2] + pPlus * L[4] * n[1];
  f[3] = L[0] * vl * L[3] + pPlus * L[4] * n[2];
  f[4] = L[0] * vl * enthalpy_of(L, g);
  const double vr = mMinusRBar * sos;
  f[0] += R[0] * vr;
  f[1] += R[0] * vr * R[1] + pMinus * R[4] * n[0];
  f[2] += R[0] * vr * R[2] + pMinus * R[4] * n[1];
  f[3] += R[0] * vr * R[3] + pMinus * R[4] * n[2];
  f[4] += R[0] * vr * enthalpy_of(R, g);
  if (ft)
    for (int q = 0; q < 2; ++q) {
      ft[q] = L[0] * vl * Lt[q];
      ft[q] += R[0] * vr * Rt[q];
    }
}

/* ------------------------------------------------------ spectral radius */
/* InvCellSpectralRadius (include/spectralRadius.hpp:44) */
static double inv_cell_specrad(const double *w, const gas_t *g, const double *lo,
                               double lom, const double *hi, double him) {
  double a[3];
  for (int q = 0; q < 3; ++q) a[q] = 0.5 * (lo[q] + hi[q]);
  const double m = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  for (int q = 0; q < 3; ++q) a[q] = a[q] / m;
  const double fMag = 0.5 * (lom + him);
  return (fabs(w[1] * a[0] + w[2] * a[1] + w[3] * a[2]) + sos_of(w, g)) * fMag;
}

/* RusanovScalarOffDiagonal (src/fluxJacobian.cpp:122) with
 * ConvectiveFluxUpdate (include/inviscidFlux.hpp:544) and
 * InvFaceSpectralRadius (include/spectralRadius.hpp:67); inviscid */
static void scalar_offdiag(const double *w, const double *du, const gas_t *g,
                           const double *n, double mag, int positive, double visc_sr,
                           double *out) {
  double wu[NV], fo[NV], fn[NV];
  update_with_cons(w, g, du, wu);
  inv_flux(w, g, n, fo);
  inv_flux(wu, g, n, fn);
  double lam =
      0.5 * mag * (fabs(w[1] * n[0] + w[2] * n[1] + w[3] * n[2]) + sos_of(w, g));
  lam += visc_sr; /* FaceSpectralRadius (include/spectralRadius.hpp:182) */
  for (int v = 0; v < NV; ++v) {
    const double fc = 0.5 * mag * (fn[v] - fo[v]);
    out[v] = positive ? fc + lam * du[v] : fc - lam * du[v];
  }
}

/* ------------------------------------------------------------- helpers */
static inline int64_t cell_idx(const oblock *b, int i, int j, int k) {
  return (int64_t)(i + b->ng) + (int64_t)b->NI * ((j + b->ng) + (int64_t)b->NJ * (k + b->ng));
}
static inline int64_t face_idx(const oblock *b, int d, int i, int j, int k) {
  const int fi = b->NI + (d == 0), fj = b->NJ + (d == 1);
  return (int64_t)(i + b->ng) + (int64_t)fi * ((j + b->ng) + (int64_t)fj * (k + b->ng));
}
static inline void face_normal(const oblock *b, int d, int64_t f, double *n, double *mag) {
  const int64_t nf = b->nf[d];
  n[0] = b->fa[d][f];
  n[1] = b->fa[d][nf + f];
  n[2] = b->fa[d][2 * nf + f];
  *mag = b->fa[d][3 * nf + f];
}

static void *dup_arr(const void *src, size_t bytes) {
  void *p = malloc(bytes ? bytes : 1);
  if (src && bytes) memcpy(p, src, bytes);
  else memset(p, 0, bytes ? bytes : 1);
  return p;
}

/* --------------------------------------------------------- viscous terms */
/* sutherland (src/transport.cpp:100-195) */
static double visc_of(double t, const ath_solve_view *v) {
  const double temp = t * v->t_ref;
  const double mu = (v->mu_c1 * pow(temp, 1.5)) / (temp + v->mu_s);
  return mu / v->mu_ref;
}
static double cond_eff(double t, const ath_solve_view *v) {
  const double temp = t * v->t_ref;
  const double k = (v->k_c1 * pow(temp, 1.5)) / (temp + v->k_s);
  return (k / v->k_ref) * v->visc_scale;
}
/* thermodynamic::Prandtl (include/thermodynamic.hpp:61) */
static double prandtl_of(const gas_t *g) {
  const double gamma = gamma_of(g);
  return (4.0 * gamma) / (9.0 * gamma - 5.0);
}
/* ViscCellSpectralRadius / ViscFaceSpectralRadius
 * (include/spectralRadius.hpp:94,126), laminar (mut = 0, Prt 0.9) */
static double visc_max_term(const double *w, const gas_t *g) {
  const double a = 4.0 / (3.0 * w[0]), b = gamma_of(g) / w[0];
  return (a < b) ? b : a;
}
/* turbModel::TurbPrandtlNumber: 0.9, Wilcox 2006 8/9 (include/turbulence.hpp:70,462) */
static double prt_of(const ath_solve_view *v) {
  return v->turb == ATH_TURB_KW2006 ? 8.0 / 9.0 : 0.9;
}
static double visc_term(double mu, double mut, const ath_solve_view *v, const gas_t *g) {
  return v->visc_scale * (mu / prandtl_of(g) + mut / prt_of(v));
}
/* FaceReconCentral (include/reconstruction.hpp:315): coefficients of the
 * lower (upwind) and upper (downwind) cell */
static void central_coeffs(double wl, double wu, double *cd, double *cu) {
  const double w[2] = {wl, wu};
  double c[2];
  lagrange_coeff(w, 1, 0, 0, c);
  *cd = c[0];
  *cu = c[1];
}
static inline void area_vec(const oblock *b, int d, int64_t f, double *a) {
  double n[3], m;
  face_normal(b, d, f, n, &m);
  a[0] = n[0] * m;
  a[1] = n[1] * m;
  a[2] = n[2] * m;
}

/* GetGhostState for viscousWall, low-Re treatment
 * (src/ghostStates.cpp:130-200, 230-241, 243-266); wd is the wall distance
 * of the wall-adjacent cell */
static double cond_eff(double t, const ath_solve_view *v);
static void viscous_wall_ghost(const double *in, const ath_bc_state *bs, const gas_t *g,
                               const ath_solve_view *v, double wd, double *out) {
  memcpy(out, in, 8 * NV);
  out[1] = 2.0 * bs->wall_u - in[1];
  out[2] = 2.0 * bs->wall_v - in[2];
  out[3] = 2.0 * bs->wall_w - in[3];
  if (bs->isothermal) {
    const double tGhost = 2.0 * bs->wall_t - temp_of(in, g);
    const double rho = out[4] / ((0.0 + 1.0 * g->r) * tGhost);
    out[0] = rho * (in[0] / in[0]);
  } else if (bs->heat_flux) {
    const double t = temp_of(in, g);
    const double kappa = cond_eff(t, v);
    const double tGhost = temp_of(in, g) - bs->wall_q / kappa * 2.0 * wd;
    const double rho = out[4] / ((0.0 + 1.0 * g->r) * tGhost);
    out[0] = rho * (in[0] / in[0]);
  }
}

/* edge ghost cells (procBlock::AssignInviscidGhostCellsEdge /
 * AssignViscousGhostCellsEdge) */
static void apply_edge_ops(oblock *b, int n, const ath_ghost_op *ops) {
  for (int o = 0; o < n; ++o) {
    const ath_ghost_op *op = &ops[o];
    double g[NV];
    const double *a = &b->W[op->src * NV];
    if (b->Wt) {
      /* turbulence: copied, or averaged for the averaged edges */
      double *gt = &b->Wt[op->dst * 2];
      const double *at = &b->Wt[op->src * 2];
      if (op->type == ATH_EDGE_AVG) {
        const double *ct = &b->Wt[op->src2 * 2];
        gt[0] = 0.5 * (at[0] + ct[0]);
        gt[1] = 0.5 * (at[1] + ct[1]);
      } else {
        gt[0] = at[0];
        gt[1] = at[1];
      }
    }
    if (op->type == ATH_EDGE_COPY) {
      memcpy(g, a, sizeof(g));
    } else if (op->type == ATH_EDGE_AVG) {
      const double *c2 = &b->W[op->src2 * NV];
      for (int v = 0; v < NV; ++v) g[v] = 0.5 * (a[v] + c2[v]);
    } else {
      double nrm[3], mag;
      face_normal(b, op->dir, op->face, nrm, &mag);
      if (op->lower) {
        nrm[0] = -1.0 * nrm[0];
        nrm[1] = -1.0 * nrm[1];
        nrm[2] = -1.0 * nrm[2];
      }
      memcpy(g, a, sizeof(g));
      const double vn = a[1] * nrm[0] + a[2] * nrm[1] + a[3] * nrm[2];
      g[1] = a[1] - 2.0 * nrm[0] * vn;
      g[2] = a[2] - 2.0 * nrm[1] * vn;
      g[3] = a[3] - 2.0 * nrm[2] * vn;
    }
    memcpy(&b->W[op->dst * NV], g, sizeof(g));
  }
}

/* procBlock::CalcViscFluxI/J/K (src/procBlock.cpp:1233,1556,1879) with
 * CalcGradsI/J/K (:5173,5378,5584), VectorGradGG/ScalarGradGG
 * (src/utility.cpp:59,138), viscousFlux::CalcFlux (src/viscousFlux.cpp:58),
 * TauNormal (src/utility.cpp:426); laminar */
/* ------------------------------------------------ block implicit operator */
/* 5x5 matrices are row-major, m[r * 5 + c] (fluxJacobian flow part with
 * one species and no turbulence equations, include/fluxJacobian.hpp:92). */
#define NJAC (NV * NV)

/* fluxJacobian::InvFluxJacobian (include/fluxJacobian.hpp:432): convective
 * flux Jacobian along the unit normal n, times 0.5|A| */
static void inv_flux_jac(const double *w, const gas_t *g, const double *n, double mag,
                         double *J) {
  const double velNorm = w[1] * n[0] + w[2] * n[1] + w[3] * n[2];
  const double mf = w[0] / w[0];
  const double gamma = gamma_of(g);
  const double gm1 = gamma - 1.0;
  const double phi = 0.5 * gm1 * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
  const double a1 = gamma * energy_of(w, g) - phi;
  const double a3 = gamma - 2.0;
  for (int e = 0; e < NJAC; ++e) J[e] = 0.0;
  J[0 * 5 + 0] = velNorm * (1.0 - mf);
  J[0 * 5 + 1] = mf * n[0];
  J[0 * 5 + 2] = mf * n[1];
  J[0 * 5 + 3] = mf * n[2];
  J[1 * 5 + 0] = phi * n[0] - w[1] * velNorm;
  J[2 * 5 + 0] = phi * n[1] - w[2] * velNorm;
  J[3 * 5 + 0] = phi * n[2] - w[3] * velNorm;
  J[4 * 5 + 0] = velNorm * (phi - a1);
  J[1 * 5 + 1] = velNorm - a3 * n[0] * w[1];
  J[2 * 5 + 1] = w[2] * n[0] - gm1 * w[1] * n[1];
  J[3 * 5 + 1] = w[3] * n[0] - gm1 * w[1] * n[2];
  J[4 * 5 + 1] = a1 * n[0] - gm1 * w[1] * velNorm;
  J[1 * 5 + 2] = w[1] * n[1] - gm1 * w[2] * n[0];
  J[2 * 5 + 2] = velNorm - a3 * n[1] * w[2];
  J[3 * 5 + 2] = w[3] * n[1] - gm1 * w[2] * n[2];
  J[4 * 5 + 2] = a1 * n[1] - gm1 * w[2] * velNorm;
  J[1 * 5 + 3] = w[1] * n[2] - gm1 * w[3] * n[0];
  J[2 * 5 + 3] = w[2] * n[2] - gm1 * w[3] * n[1];
  J[3 * 5 + 3] = velNorm - a3 * n[2] * w[3];
  J[4 * 5 + 3] = a1 * n[2] - gm1 * w[3] * velNorm;
  J[1 * 5 + 4] = gm1 * n[0];
  J[2 * 5 + 4] = gm1 * n[1];
  J[3 * 5 + 4] = gm1 * n[2];
  J[4 * 5 + 4] = gamma * velNorm;
  const double f = 0.5 * mag;
  for (int e = 0; e < NJAC; ++e) J[e] *= f;
}

/* fluxJacobian::RusanovFluxJacobian (include/fluxJacobian.hpp:405):
 * J = A(W) 0.5|A| +/- lambda_face I */
static void rusanov_jac(const double *w, const gas_t *g, const double *n, double mag,
                        int positive, double *J) {
  const double specRad =
      0.5 * mag * (fabs(w[1] * n[0] + w[2] * n[1] + w[3] * n[2]) + sos_of(w, g));
  inv_flux_jac(w, g, n, mag, J);
  for (int r = 0; r < NV; ++r)
    for (int cc = 0; cc < NV; ++cc) {
      const double dis = (r == cc) ? 1.0 * specRad : 0.0;
      J[r * 5 + cc] = positive ? J[r * 5 + cc] + dis : J[r * 5 + cc] - dis;
    }
}

/* fluxJacobian::ApproxTSLJacobian (include/fluxJacobian.hpp:667), laminar,
 * one species, no diffusion model; vg[r][c] is the velocity gradient
 * tensor (row = derivative direction, as TauNormal reads it) */
static void tsl_jac(const double *w, double mu_lam, double mut_lam, const gas_t *g,
                    const ath_solve_view *v, const double *n, double mag, double dist,
                    int left, const double *vg, double *J) {
  const double t = temp_of(w, g);
  const double mu = v->visc_scale * mu_lam;
  const double mut = v->visc_scale * mut_lam;
  const double velNorm = w[1] * n[0] + w[2] * n[1] + w[3] * n[2];
  const double rho = w[0];
  const double k = cond_eff(t, v);
  const double kt = mut * cp_of(g) / prt_of(v);  /* turbulent Prandtl number */
  /* TauNormal (src/utility.cpp:426) */
  const double lambda = 0.0 - (2.0 / 3.0) * (mu + mut);
  const double trace = vg[0] + vg[4] + vg[8];
  double tau[3];
  for (int r = 0; r < 3; ++r) {
    const double sn = (vg[r * 3 + 0] + vg[0 * 3 + r]) * n[0] +
                      (vg[r * 3 + 1] + vg[1 * 3 + r]) * n[1] +
                      (vg[r * 3 + 2] + vg[2 * 3 + r]) * n[2];
    tau[r] = lambda * trace * n[r] + (mu + mut) * sn;
  }
  const double fac = left ? -1.0 : 1.0;
  const double third = 1.0 / 3.0;
  double T[NJAC];
  for (int e = 0; e < NJAC; ++e) T[e] = 0.0;
  /* species row and column: DiffCoeff = 0 (no diffusion model) */
  const double speciesEnthalpy = 0.0;
  T[4 * 5 + 0] = -(k + kt) * t / ((mu + mut) * rho) + speciesEnthalpy;
  T[1 * 5 + 1] = third * n[0] * n[0] + 1.0;
  T[2 * 5 + 1] = third * n[0] * n[1];
  T[3 * 5 + 1] = third * n[0] * n[2];
  T[4 * 5 + 1] = fac * 0.5 * dist / (mu + mut) * tau[0] + third * n[0] * velNorm + w[1];
  T[1 * 5 + 2] = third * n[1] * n[0];
  T[2 * 5 + 2] = third * n[1] * n[1] + 1.0;
  T[3 * 5 + 2] = third * n[1] * n[2];
  T[4 * 5 + 2] = fac * 0.5 * dist / (mu + mut) * tau[1] + third * n[1] * velNorm + w[2];
  T[1 * 5 + 3] = third * n[2] * n[0];
  T[2 * 5 + 3] = third * n[2] * n[1];
  T[3 * 5 + 3] = third * n[2] * n[2] + 1.0;
  T[4 * 5 + 3] = fac * 0.5 * dist / (mu + mut) * tau[2] + third * n[2] * velNorm + w[3];
  T[4 * 5 + 4] = (k + kt) / ((mu + mut) * rho);
  const double f = mag * (mu + mut) / dist;
  for (int e = 0; e < NJAC; ++e) T[e] *= f;
  /* DelprimitiveDelConservative (include/fluxJacobian.hpp:626) */
  const double gm1 = gamma_of(g) - 1.0;
  const double invRho = 1.0 / rho;
  double P[NJAC];
  for (int e = 0; e < NJAC; ++e) P[e] = 0.0;
  P[0 * 5 + 0] = 1.0;
  P[1 * 5 + 0] = -invRho * w[1];
  P[2 * 5 + 0] = -invRho * w[2];
  P[3 * 5 + 0] = -invRho * w[3];
  P[4 * 5 + 0] = 0.5 * gm1 * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
  P[1 * 5 + 1] = invRho;
  P[4 * 5 + 1] = -gm1 * w[1];
  P[2 * 5 + 2] = invRho;
  P[4 * 5 + 2] = -gm1 * w[2];
  P[3 * 5 + 3] = invRho;
  P[4 * 5 + 3] = -gm1 * w[3];
  P[4 * 5 + 4] = gm1;
  /* MatrixMultiply (src/matrix.cpp:197): column of the left operand
   * outermost, accumulated from zero */
  for (int e = 0; e < NJAC; ++e) J[e] = 0.0;
  for (int cc = 0; cc < NV; ++cc)
    for (int r = 0; r < NV; ++r)
      for (int i = 0; i < NV; ++i) J[r * 5 + i] += T[r * 5 + cc] * P[cc * 5 + i];
}

/* ArrayMultiplication (include/fluxJacobian.hpp:46): out = M x, each row
 * accumulated from zero */
static void mat_vec(const double *M, const double *x, double *out) {
  for (int r = 0; r < NV; ++r) {
    double s = 0.0;
    for (int cc = 0; cc < NV; ++cc) s += M[r * 5 + cc] * x[cc];
    out[r] = s;
  }
}

/* MatrixInverse (src/matrix.cpp:57): Gauss-Jordan with the reference's
 * pivot search (FindMaxInColumn before the row is reduced) */
static void mat_inverse(double *a) {
  double I[NJAC];
  for (int r = 0; r < NV; ++r)
    for (int cc = 0; cc < NV; ++cc) I[r * 5 + cc] = (r == cc) ? 1.0 : 0.0;
  for (int r = 0; r < NV; ++r) {
    const int cp = r;
    double maxVal = 0.0;
    int rp = 0;
    for (int ii = cp; ii <= NV - 1; ++ii)
      if (fabs(a[ii * 5 + r]) > maxVal) {
        maxVal = fabs(a[ii * 5 + r]);
        rp = ii;
      }
    if (rp != r)
      for (int cc = 0; cc < NV; ++cc) {
        double t = a[r * 5 + cc]; a[r * 5 + cc] = a[rp * 5 + cc]; a[rp * 5 + cc] = t;
        t = I[r * 5 + cc]; I[r * 5 + cc] = I[rp * 5 + cc]; I[rp * 5 + cc] = t;
      }
    if (r != 0)
      for (int ii = 0; ii < cp; ++ii) {
        const double factor = a[r * 5 + ii] / a[ii * 5 + ii];
        for (int cc = 0; cc < NV; ++cc) a[r * 5 + cc] = a[r * 5 + cc] - factor * a[ii * 5 + cc];
        for (int cc = 0; cc < NV; ++cc) I[r * 5 + cc] = I[r * 5 + cc] - factor * I[ii * 5 + cc];
      }
    const double normFactor = 1.0 / a[r * 5 + cp];
    for (int cc = cp; cc < NV; ++cc) a[r * 5 + cc] *= normFactor;
    for (int cc = 0; cc < NV; ++cc) I[r * 5 + cc] *= normFactor;
  }
  for (int cp = NV - 2, r = NV - 2; r >= 0; --r, --cp)
    for (int ii = NV - 1; ii > cp; --ii) {
      const double factor = a[r * 5 + ii];
      for (int cc = 0; cc < NV; ++cc) a[r * 5 + cc] = a[r * 5 + cc] - factor * a[ii * 5 + cc];
      for (int cc = 0; cc < NV; ++cc) I[r * 5 + cc] = I[r * 5 + cc] - factor * I[ii * 5 + cc];
    }
  memcpy(a, I, sizeof(I));
}

/* ------------------------------------------------------- SST-2003 model */
/* turbKWSst constants (include/turbulence.hpp:489-501) and the turbulence
 * floors of turbModel (include/turbulence.hpp:63-64) */
#define SST_BETASTAR 0.09
#define SST_SIGMAK1 0.85
#define SST_SIGMAK2 1.0
#define SST_SIGMAW1 0.5
#define SST_SIGMAW2 0.856
#define SST_BETA1 0.075
#define SST_BETA2 0.0828
#define SST_GAMMA1 (5.0 / 9.0)
#define SST_GAMMA2 0.44
#define SST_A1 0.31
#define SST_PRT 0.9
#define SST_PROD2DEST 10.0
#define TURB_MIN 1.0e-20

/* std::max / std::min */
static double cmax(double a, double b) { return (a < b) ? b : a; }
static double cmin(double a, double b) { return (b < a) ? b : a; }
/* turbKWSst::BlendedCoeff (src/turbulence.cpp:598) */
static double blended(double c1, double c2, double f1) { return f1 * c1 + (1.0 - f1) * c2; }

/* primitive::ApplyFarfieldTurbBC (src/primitive.cpp:83) + LimitTurb (:100):
 * k, omega of state w from the velocity vel, intensity and viscosity ratio */
static void farfield_turb(const double *w, const double *vel, double tint, double ratio,
                          const gas_t *g, const ath_solve_view *v, double *kw) {
  const double vmag = sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
  kw[0] = 1.5 * pow(tint * vmag, 2.0);
  kw[1] = w[0] * kw[0] / (ratio * visc_of(temp_of(w, g), v));
  kw[0] = cmax(kw[0], TURB_MIN);
  kw[1] = cmax(kw[1], TURB_MIN);
}

/* ExtrapolateHoldMixture (src/ghostStates.cpp:693) over the flow and the
 * turbulence variables */
static void extrap_hold7(double *g, double *gt, double factor, const double *in,
                         const double *int_) {
  const double ghostRho = factor * g[0] - in[0];
  if (ghostRho <= 0.0) return;
  const double mf = g[0] / g[0];
  for (int v = 0; v < NV; ++v) g[v] = factor * g[v] - in[v];
  for (int v = 0; v < 2; ++v) gt[v] = factor * gt[v] - int_[v];
  const double r = ghostRho * mf;
  g[0] = (r > 0.0) ? r : 0.0;
}

/* tensor DoubleDotTrans of two tensors (include/tensor.hpp:353): sum of the
 * element-by-element products, accumulated from zero in storage order */
static double ddot(const double *a, const double *b) {
  double s = 0.0;
  for (int e = 0; e < 9; ++e) s += a[e] * b[e];
  return s;
}

/* turbKWSst::EddyViscAndBlending (src/turbulence.cpp:668) with Alpha1-3,
 * CDkw, F1, F2 and EddyVisc (:573-634, include/turbulence.hpp:529); mu is
 * the (unscaled) laminar viscosity, wd the wall distance, vg the velocity
 * gradient tensor (row = derivative axis) */
static void sst_eddy_visc(const double *w, const double *kw, const double *vg,
                          const double *kg, const double *wg, double mu, double wd,
                          double scale, double *mut, double *f1, double *f2) {
  const double k = kw[0], om = kw[1], rho = w[0];
  const double a1 = scale * sqrt(k) / (SST_BETASTAR * om * (wd + 1.0e-30));
  const double a2 = scale * scale * 500.0 * mu / ((wd + 1.0e-30) * (wd + 1.0e-30) * rho * om);
  const double cd = cmax(2.0 * rho * SST_SIGMAW2 / om * (kg[0] * wg[0] + kg[1] * wg[1] +
                                                          kg[2] * wg[2]),
                         1.0e-10);
  const double a3 = 4.0 * rho * SST_SIGMAW2 * k / (cd * (wd + 1.0e-30) * (wd + 1.0e-30));
  *f1 = tanh(pow(cmin(cmax(a1, a2), a3), 4.0));
  const double arg2 = cmax(2.0 * a1, a2);
  *f2 = tanh(arg2 * arg2);
  double S[9];
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) S[r * 3 + q] = 0.5 * (vg[r * 3 + q] + vg[q * 3 + r]);
  const double msr = sqrt(2.0 * ddot(S, S));
  *mut = rho * SST_A1 * k / cmax(SST_A1 * om, scale * msr * *f2);
}

/* turbKWSst::CalcTurbSrc (src/turbulence.cpp:637) with the Boussinesq
 * Reynolds stress (turbModel::ReynoldsStressDDotVelGrad, :53); returns the
 * blended beta for the source Jacobian */
static double sst_source(const double *w, const double *kw, const double *vg,
                         const double *kg, const double *wg, double mut, double f1,
                         double scale, double *src) {
  const double k = kw[0], om = kw[1], rho = w[0];
  const double inv = 1.0 / scale;
  const double cd = cmax(2.0 * rho * SST_SIGMAW2 / om * (kg[0] * wg[0] + kg[1] * wg[1] +
                                                          kg[2] * wg[2]),
                         1.0e-10);
  const double gamma = blended(SST_GAMMA1, SST_GAMMA2, f1);
  const double beta = blended(SST_BETA1, SST_BETA2, f1);
  const double tkeDest = inv * SST_BETASTAR * (rho * k * om * 1.0);
  const double omgDest = inv * beta * (rho * om * om);
  const double lambda = 0.0 - (2.0 / 3.0) * mut;
  const double tr = vg[0] + vg[4] + vg[8];
  const double c23 = 2.0 / 3.0 * rho * k;
  double tau[9];
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) {
      const double I = (r == q) ? 1.0 : 0.0;
      tau[r * 3 + q] = (I * (lambda * tr) + (vg[r * 3 + q] + vg[q * 3 + r]) * mut) - I * c23;
    }
  double tkeProd = cmin(scale * ddot(tau, vg), SST_PROD2DEST * tkeDest);
  tkeProd = cmax(tkeProd, 0.0);
  double omgProd = gamma * rho / mut * tkeProd;
  omgProd = cmax(omgProd, 0.0);
  const double omgCd = scale * (1.0 - f1) * cd;
  src[0] = tkeProd - tkeDest;
  src[1] = omgProd - omgDest + omgCd;
  return beta;
}

/* ---------------------------------------------- Wilcox k-omega 2006 */
/* turbKWWilcox (include/turbulence.hpp:390-398) */
#define WK_GAMMA 0.52
#define WK_BETASTAR 0.09
#define WK_SIGMA 0.5
#define WK_SIGMASTAR 0.6
#define WK_SIGMAD0 0.125
#define WK_BETA0 0.0708
#define WK_CLIM 0.875

/* turbKWWilcox::EddyVisc / OmegaTilda (src/turbulence.cpp:270,339): rho k
 * over omega limited below by clim sqrt(2 S^:S^ / beta*), S^ the traceless
 * strain rate */
static double wk_eddy_visc(const double *w, const double *kw, const double *vg, double scale) {
  const double tr = (vg[0] + vg[4]) + vg[8];
  const double c = 1.0 / 3.0 * tr;
  double sh[9];
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q)
      sh[r * 3 + q] = 0.5 * (vg[r * 3 + q] + vg[q * 3 + r]) - c * (r == q ? 1.0 : 0.0);
  const double omt = cmax(kw[1], scale * WK_CLIM * sqrt(2.0 * ddot(sh, sh) / WK_BETASTAR));
  return w[0] * kw[0] / omt;
}

/* turbModel::EddyViscosityNoLim (src/turbulence.cpp:38): rho k / omega */
static double eddy_visc_nolim(const double *w, const double *kw) { return w[0] * kw[0] / kw[1]; }

/* turbKWWilcox::CalcTurbSrc (src/turbulence.cpp:359) with Beta / FBeta /
 * Xw / StrainKI / SigmaD (:283-337); returns beta for the source Jacobian */
static double wk_source(const double *w, const double *kw, const double *vg, const double *kg,
                        const double *wg, double mut, double scale, double *src) {
  const double k = kw[0], om = kw[1], rho = w[0];
  const double inv = 1.0 / scale;
  const double tkeDest = inv * WK_BETASTAR * (rho * k * om * 1.0);
  /* vortex stretching: vorticity squared double-dotted with the strain */
  double vo[9], skI[9], vv[9];
  const double tr = (vg[0] + vg[4]) + vg[8];
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) {
      vo[r * 3 + q] = 0.5 * (vg[r * 3 + q] - vg[q * 3 + r]);
      skI[r * 3 + q] = 0.5 * ((vg[r * 3 + q] + vg[q * 3 + r]) - tr * (r == q ? 1.0 : 0.0));
    }
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) {
      double t = 0.0;
      for (int m = 0; m < 3; ++m) t += vo[r * 3 + m] * vo[m * 3 + q];
      vv[r * 3 + q] = t;
    }
  const double xw = fabs(ddot(vv, skI) / pow(WK_BETASTAR * om, 3.0)) * pow(scale, 3.0);
  const double fbeta = (1.0 + 85.0 * xw) / (1.0 + 100.0 * xw);
  const double beta = WK_BETA0 * fbeta;
  const double omgDest = inv * beta * (rho * om * om);
  const double lambda = 0.0 - (2.0 / 3.0) * mut;
  const double c23 = 2.0 / 3.0 * rho * k;
  double tau[9];
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) {
      const double I = (r == q) ? 1.0 : 0.0;
      tau[r * 3 + q] = (I * (lambda * tr) + (vg[r * 3 + q] + vg[q * 3 + r]) * mut) - I * c23;
    }
  double tkeProd = scale * ddot(tau, vg);
  tkeProd = cmax(tkeProd, 0.0);
  double omgProd = WK_GAMMA * om / k * tkeProd;
  omgProd = cmax(omgProd, 0.0);
  const double kdw = ((0.0 + kg[0] * wg[0]) + kg[1] * wg[1]) + kg[2] * wg[2];
  const double sigd = kdw <= 0.0 ? 0.0 : WK_SIGMAD0;
  const double omgCd = scale * sigd * (rho / om * kdw);
  src[0] = tkeProd - tkeDest;
  src[1] = omgProd - omgDest + omgCd;
  return beta;
}

/* turbulence spectral radii and Jacobians (src/turbulence.cpp:105-160,
 * 749-797): inviscid cell radius |v.n_avg| |A|; viscous cell radius
 * scale |A|^2/(V rho) (mu + sigma_k mut); face radii; viscous Jacobian */
static double turb_inv_cell_sr(const double *w, const double *lo, double lom,
                               const double *hi, double him) {
  double a[3];
  for (int q = 0; q < 3; ++q) a[q] = 0.5 * (lo[q] + hi[q]);
  const double m = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  for (int q = 0; q < 3; ++q) a[q] = a[q] / m;
  const double fMag = 0.5 * (lom + him);
  return fabs(w[1] * a[0] + w[2] * a[1] + w[3] * a[2]) * fMag;
}
/* the k equation's diffusivity mu + sigma_k mu_t of the radii and
 * Jacobians: SST blends sigma_k with F1 and takes the limited mu_t, Wilcox
 * 2006 takes sigma* and the unlimited rho k / omega of the state (kw) */
static double turb_diff_k(int wilcox, const double *w, const double *kw, double mu, double mut,
                          double f1) {
  return wilcox ? mu + WK_SIGMASTAR * eddy_visc_nolim(w, kw)
                : mu + blended(SST_SIGMAK1, SST_SIGMAK2, f1) * mut;
}
static double turb_visc_cell_sr(int wilcox, const double *w, const double *kw, double lom,
                                double him, double vol, double mu, double mut, double f1,
                                double scale) {
  const double fMag = 0.5 * (lom + him);
  const double length = fMag * fMag / vol;
  return scale * length / w[0] * turb_diff_k(wilcox, w, kw, mu, mut, f1);
}
static double turb_face_sr(int wilcox, const double *w, const double *kw, const double *n,
                           double mag, double mu, double mut, double f1, double dist,
                           double scale, int positive, int viscous) {
  const double vn = w[1] * n[0] + w[2] * n[1] + w[3] * n[2];
  double sr = positive ? 0.5 * mag * fabs(vn + fabs(vn)) : 0.5 * mag * fabs(vn - fabs(vn));
  if (viscous) {
    const double length = mag / dist;
    sr += scale * length / w[0] * turb_diff_k(wilcox, w, kw, mu, mut, f1);
  }
  return sr;
}
/* 2x2 turbulence part of RusanovFluxJacobian: 0.5 conv +/- 0.5 diss */
static void turb_rusanov_jac(const double *w, const double *n, double mag, int positive,
                             double *J) {
  const double vn = w[1] * n[0] + w[2] * n[1] + w[3] * n[2];
  const double conv = vn * mag, diss = fabs(vn) * mag;
  const double cj[4] = {0.5 * conv, 0.5 * 0.0, 0.5 * 0.0, 0.5 * conv};
  const double dj[4] = {0.5 * diss, 0.5 * 0.0, 0.5 * 0.0, 0.5 * diss};
  for (int e = 0; e < 4; ++e) J[e] = positive ? cj[e] + dj[e] : cj[e] - dj[e];
}
/* turbKWSst::ViscJac (src/turbulence.cpp:764), turbKWWilcox::ViscJac
 * (:485) times the sign factor */
static void turb_visc_jac(int wilcox, const double *w, const double *kw, double mag, double mu,
                          double mut, double f1, double dist, double scale, double fac,
                          double *J) {
  const double length = mag / dist;
  const double j00 = scale * length / w[0] * turb_diff_k(wilcox, w, kw, mu, mut, f1);
  const double j11 = scale * length / w[0] *
                     (wilcox ? mu + WK_SIGMA * eddy_visc_nolim(w, kw)
                             : mu + blended(SST_SIGMAW1, SST_SIGMAW2, f1) * mut);
  J[0] = fac * j00;
  J[1] = fac * 0.0;
  J[2] = fac * 0.0;
  J[3] = fac * j11;
}
/* MatrixInverse of a 2x2 (src/matrix.cpp:57) */
static void mat_inverse2(double *a) {
  double I[4] = {1.0, 0.0, 0.0, 1.0};
  for (int r = 0; r < 2; ++r) {
    double maxVal = 0.0;
    int rp = 0;
    for (int ii = r; ii <= 1; ++ii)
      if (fabs(a[ii * 2 + r]) > maxVal) {
        maxVal = fabs(a[ii * 2 + r]);
        rp = ii;
      }
    if (rp != r)
      for (int cc = 0; cc < 2; ++cc) {
        double t = a[r * 2 + cc]; a[r * 2 + cc] = a[rp * 2 + cc]; a[rp * 2 + cc] = t;
        t = I[r * 2 + cc]; I[r * 2 + cc] = I[rp * 2 + cc]; I[rp * 2 + cc] = t;
      }
    if (r != 0)
      for (int ii = 0; ii < r; ++ii) {
        const double factor = a[r * 2 + ii] / a[ii * 2 + ii];
        for (int cc = 0; cc < 2; ++cc) a[r * 2 + cc] = a[r * 2 + cc] - factor * a[ii * 2 + cc];
        for (int cc = 0; cc < 2; ++cc) I[r * 2 + cc] = I[r * 2 + cc] - factor * I[ii * 2 + cc];
      }
    const double normFactor = 1.0 / a[r * 2 + r];
    for (int cc = r; cc < 2; ++cc) a[r * 2 + cc] *= normFactor;
    for (int cc = 0; cc < 2; ++cc) I[r * 2 + cc] *= normFactor;
  }
  {
    const double factor = a[0 * 2 + 1];
    for (int cc = 0; cc < 2; ++cc) a[0 * 2 + cc] = a[0 * 2 + cc] - factor * a[1 * 2 + cc];
    for (int cc = 0; cc < 2; ++cc) I[0 * 2 + cc] = I[0 * 2 + cc] - factor * I[1 * 2 + cc];
  }
  memcpy(a, I, sizeof(I));
}
static void mat_vec2(const double *M, const double *x, double *out) {
  for (int r = 0; r < 2; ++r) {
    double s = 0.0;
    for (int cc = 0; cc < 2; ++cc) s += M[r * 2 + cc] * x[cc];
    out[r] = s;
  }
}

/* Dual-cell Green-Gauss gradients of velocity and pressure at the face of
 * direction d below cell cu (procBlock::CalcGradsI/J/K, src/procBlock.cpp:
 * 5173; VectorGradGG / ScalarGradGG, src/utility.cpp:59,138). */
static void face_grad_vp(const oblock *b, int d, int64_t cu, double grad[3][3], double pg[3]) {
  const int64_t st[3] = {1, b->NI, (int64_t)b->NI * b->NJ};
  const int64_t cl = cu - st[d];
  const double *Wl = &b->W[cl * NV], *Wu = &b->W[cu * NV];
  double vlo[3][3], vhi[3][3], plo[3], phi[3], alo[3][3], ahi[3][3];
  const int uI = (int)(cu % b->NI) - b->ng, uJ = (int)((cu / b->NI) % b->NJ) - b->ng,
            uK = (int)(cu / ((int64_t)b->NI * b->NJ)) - b->ng;
  const int lI = (int)(cl % b->NI) - b->ng, lJ = (int)((cl / b->NI) % b->NJ) - b->ng,
            lK = (int)(cl / ((int64_t)b->NI * b->NJ)) - b->ng;
  for (int e = 0; e < 3; ++e) {
    if (e == d) {
      for (int q = 0; q < 3; ++q) {
        vlo[e][q] = Wl[1 + q];
        vhi[e][q] = Wu[1 + q];
      }
      plo[e] = Wl[4];
      phi[e] = Wu[4];
      double A0[3], A1[3], A2[3];
      area_vec(b, d, face_idx(b, d, uI, uJ, uK), A0);
      area_vec(b, d, face_idx(b, d, uI + (d == 0), uJ + (d == 1), uK + (d == 2)), A1);
      area_vec(b, d, face_idx(b, d, uI - (d == 0), uJ - (d == 1), uK - (d == 2)), A2);
      for (int q = 0; q < 3; ++q) {
        ahi[e][q] = 0.5 * (A0[q] + A1[q]);
        alo[e][q] = 0.5 * (A0[q] + A2[q]);
      }
    } else {
      const int64_t cup = cu + st[e], clp = cl + st[e], cum = cu - st[e], clm = cl - st[e];
      const double *Wup = &b->W[cup * NV], *Wlp = &b->W[clp * NV], *Wum = &b->W[cum * NV],
                   *Wlm = &b->W[clm * NV];
      for (int q = 0; q < 3; ++q) {
        vhi[e][q] = 0.25 * (((Wl[1 + q] + Wu[1 + q]) + Wup[1 + q]) + Wlp[1 + q]);
        vlo[e][q] = 0.25 * (((Wl[1 + q] + Wu[1 + q]) + Wum[1 + q]) + Wlm[1 + q]);
      }
      phi[e] = 0.25 * (((Wl[4] + Wu[4]) + Wup[4]) + Wlp[4]);
      plo[e] = 0.25 * (((Wl[4] + Wu[4]) + Wum[4]) + Wlm[4]);
      double Au[3], Al[3], Aup[3], Alp[3];
      area_vec(b, e, face_idx(b, e, uI, uJ, uK), Au);
      area_vec(b, e, face_idx(b, e, lI, lJ, lK), Al);
      area_vec(b, e, face_idx(b, e, uI + (e == 0), uJ + (e == 1), uK + (e == 2)), Aup);
      area_vec(b, e, face_idx(b, e, lI + (e == 0), lJ + (e == 1), lK + (e == 2)), Alp);
      for (int q = 0; q < 3; ++q) {
        ahi[e][q] = 0.5 * (Aup[q] + Alp[q]);
        alo[e][q] = 0.5 * (Au[q] + Al[q]);
      }
    }
  }
  const double vol = 0.5 * (b->vol[cl] + b->vol[cu]);
  const double invVol = 1.0 / vol;
  for (int r = 0; r < 3; ++r) {
    for (int q = 0; q < 3; ++q) {
      grad[r][q] = vhi[0][q] * ahi[0][r] - vlo[0][q] * alo[0][r] + vhi[1][q] * ahi[1][r] -
                   vlo[1][q] * alo[1][r] + vhi[2][q] * ahi[2][r] - vlo[2][q] * alo[2][r];
      grad[r][q] *= invVol;
    }
    pg[r] = phi[0] * ahi[0][r] - plo[0] * alo[0][r] + phi[1] * ahi[1][r] -
            plo[1] * alo[1][r] + phi[2] * ahi[2][r] - plo[2] * alo[2][r];
    pg[r] *= invVol;
  }
}

/* Cell-averaged velocity and pressure gradients (one sixth per face, i low,
 * i high, j low, ... as the reference accumulates them, src/procBlock.cpp:
 * 5790) of the cells nonreflecting pressure outlets read; used at the next
 * ghost fill. */
static void nr_grads(const orc_case *c, oblock *b) {
  const osolve *sv = &c->s[b->solve];
  const int64_t st[3] = {1, b->NI, (int64_t)b->NI * b->NJ};
  for (int o = 0; o < b->nops; ++o) {
    const ath_ghost_op *op = &b->ops[o];
    if (op->type != ATH_BC_PRESSURE_OUTLET || !sv->states[op->state].nonreflecting) continue;
    const int64_t x = op->src;
    double vg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, pg[3] = {0, 0, 0};
    const double sixth = 1.0 / 6.0;
    for (int d = 0; d < 3; ++d)
      for (int side = 0; side < 2; ++side) {
        double grad[3][3], p[3];
        face_grad_vp(b, d, side ? x + st[d] : x, grad, p);
        for (int r = 0; r < 3; ++r) {
          for (int q = 0; q < 3; ++q) vg[r * 3 + q] += sixth * grad[r][q];
          pg[r] += sixth * p[r];
        }
      }
    memcpy(&b->nrg[x * 12], vg, sizeof(vg));
    memcpy(&b->nrg[x * 12 + 9], pg, sizeof(pg));
  }
}

/* Green-Gauss gradients at the face of direction d below cell cu of the
 * cell scalars u, v, w, T, rho, p and, with RANS, k, omega
 * (procBlock::CalcGradsI/J/K, src/procBlock.cpp:5173-5790): face_grad_vp's
 * dual cell with every scalar; temperature p / (rho R) of the state. */
static double cell_scalar(const oblock *b, const gas_t *g, int64_t x, int k) {
  const double *w = &b->W[x * NV];
  switch (k) {
    case 0: return w[1];
    case 1: return w[2];
    case 2: return w[3];
    case 3: return w[4] / (0.0 + w[0] * g->r);
    case 4: return w[0];
    case 5: return w[4];
    default: return b->Wt[x * 2 + (k - 6)];
  }
}
static void face_grads_all(const oblock *b, const gas_t *g, int d, int64_t cu, int ns,
                           double grad[8][3]) {
  const int64_t st[3] = {1, b->NI, (int64_t)b->NI * b->NJ};
  const int64_t cl = cu - st[d];
  double lo[3][8], hi[3][8], alo[3][3], ahi[3][3];
  const int uI = (int)(cu % b->NI) - b->ng, uJ = (int)((cu / b->NI) % b->NJ) - b->ng,
            uK = (int)(cu / ((int64_t)b->NI * b->NJ)) - b->ng;
  const int lI = (int)(cl % b->NI) - b->ng, lJ = (int)((cl / b->NI) % b->NJ) - b->ng,
            lK = (int)(cl / ((int64_t)b->NI * b->NJ)) - b->ng;
  for (int e = 0; e < 3; ++e) {
    if (e == d) {
      for (int k = 0; k < ns; ++k) {
        lo[e][k] = cell_scalar(b, g, cl, k);
        hi[e][k] = cell_scalar(b, g, cu, k);
      }
      double A0[3], A1[3], A2[3];
      area_vec(b, d, face_idx(b, d, uI, uJ, uK), A0);
      area_vec(b, d, face_idx(b, d, uI + (d == 0), uJ + (d == 1), uK + (d == 2)), A1);
      area_vec(b, d, face_idx(b, d, uI - (d == 0), uJ - (d == 1), uK - (d == 2)), A2);
      for (int q = 0; q < 3; ++q) {
        ahi[e][q] = 0.5 * (A0[q] + A1[q]);
        alo[e][q] = 0.5 * (A0[q] + A2[q]);
      }
    } else {
      const int64_t cup = cu + st[e], clp = cl + st[e], cum = cu - st[e], clm = cl - st[e];
      for (int k = 0; k < ns; ++k) {
        const double sl = cell_scalar(b, g, cl, k), su = cell_scalar(b, g, cu, k);
        hi[e][k] = 0.25 * (((sl + su) + cell_scalar(b, g, cup, k)) + cell_scalar(b, g, clp, k));
        lo[e][k] = 0.25 * (((sl + su) + cell_scalar(b, g, cum, k)) + cell_scalar(b, g, clm, k));
      }
      double Au[3], Al[3], Aup[3], Alp[3];
      area_vec(b, e, face_idx(b, e, uI, uJ, uK), Au);
      area_vec(b, e, face_idx(b, e, lI, lJ, lK), Al);
      area_vec(b, e, face_idx(b, e, uI + (e == 0), uJ + (e == 1), uK + (e == 2)), Aup);
      area_vec(b, e, face_idx(b, e, lI + (e == 0), lJ + (e == 1), lK + (e == 2)), Alp);
      for (int q = 0; q < 3; ++q) {
        ahi[e][q] = 0.5 * (Aup[q] + Alp[q]);
        alo[e][q] = 0.5 * (Au[q] + Al[q]);
      }
    }
  }
  const double vol = 0.5 * (b->vol[cl] + b->vol[cu]);
  const double invVol = 1.0 / vol;
  for (int k = 0; k < ns; ++k)
    for (int r = 0; r < 3; ++r) {
      const double v = hi[0][k] * ahi[0][r] - lo[0][k] * alo[0][r] + hi[1][k] * ahi[1][r] -
                       lo[1][k] * alo[1][r] + hi[2][k] * ahi[2][r] - lo[2][k] * alo[2][r];
      grad[k][r] = v * invVol;
    }
}

/* The cell-averaged gradients the reference keeps from every residual
 * (velocityGrad_ ... omegaGrad_; one sixth of each face's, faces i low,
 * i high, j low, ...) for its output files: [24] per cell = velocity
 * gradient (9, row = derivative axis), T, rho, p, k, omega gradients. */
static void out_grads(const orc_case *c, oblock *b) {
  const gas_t *g = &c->s[b->solve].gas;
  const int ns = b->Wt ? 8 : 6;
  const int64_t st[3] = {1, b->NI, (int64_t)b->NI * b->NJ};
  const double sixth = 1.0 / 6.0;
  for (int k = 0; k < b->nk; ++k)
    for (int j = 0; j < b->nj; ++j)
      for (int i = 0; i < b->ni; ++i) {
        const int64_t x = cell_idx(b, i, j, k);
        double acc[8][3];
        memset(acc, 0, sizeof(acc));
        for (int d = 0; d < 3; ++d)
          for (int side = 0; side < 2; ++side) {
            double gr[8][3];
            face_grads_all(b, g, d, side ? x + st[d] : x, ns, gr);
            for (int q = 0; q < ns; ++q)
              for (int r = 0; r < 3; ++r) acc[q][r] += sixth * gr[q][r];
          }
        double *o = &b->og[x * 24];
        for (int r = 0; r < 3; ++r)
          for (int q = 0; q < 3; ++q) o[r * 3 + q] = acc[q][r];
        for (int q = 3; q < 8; ++q)
          for (int r = 0; r < 3; ++r) o[9 + (q - 3) * 3 + r] = acc[q][r];
      }
}

void orc_set_output_grads(orc_case *c, int on) {
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    if (on && !b->og) b->og = (double *)calloc((size_t)b->nc * 24, sizeof(double));
    if (!on) {
      free(b->og);
      b->og = NULL;
    }
  }
}

static void viscous_fluxes(orc_case *c, oblock *b) {
  const osolve *sv = &c->s[b->solve];
  const ath_solve_view *v = &sv->v;
  const gas_t *g = &sv->gas;
  const int64_t st[3] = {1, b->NI, (int64_t)b->NI * b->NJ};
  const double coeff = v->visc_cfl_coeff;
  for (int d = 0; d < 3; ++d) {
    const int ei = b->ni + (d == 0), ej = b->nj + (d == 1), ek = b->nk + (d == 2);
    const int nd = d == 0 ? b->ni : (d == 1 ? b->nj : b->nk);
    const double *wd = &b->width[d * b->nc];
    for (int k = 0; k < ek; ++k)
      for (int j = 0; j < ej; ++j)
        for (int i = 0; i < ei; ++i) {
          const int fpos = d == 0 ? i : (d == 1 ? j : k);
          const int64_t cu = cell_idx(b, i, j, k), cl = cu - st[d];
          /* dual-cell face values and area vectors, axes i, j, k */
          double vlo[3][3], vhi[3][3], tlo[3], thi[3], alo[3][3], ahi[3][3];
          double klo[3] = {0, 0, 0}, khi[3] = {0, 0, 0}, olo[3] = {0, 0, 0}, ohi[3] = {0, 0, 0};
          const int rans = sv->rans;
          const double *Tt = b->Wt;
          for (int e = 0; e < 3; ++e) {
            const double *Wl = &b->W[cl * NV], *Wu = &b->W[cu * NV];
            if (rans) {
              if (e == d) {
                klo[e] = Tt[cl * 2];
                khi[e] = Tt[cu * 2];
                olo[e] = Tt[cl * 2 + 1];
                ohi[e] = Tt[cu * 2 + 1];
              } else {
                const int64_t up = cu + st[e], lp = cl + st[e], um = cu - st[e], lm = cl - st[e];
                khi[e] = 0.25 * (((Tt[cl * 2] + Tt[cu * 2]) + Tt[up * 2]) + Tt[lp * 2]);
                klo[e] = 0.25 * (((Tt[cl * 2] + Tt[cu * 2]) + Tt[um * 2]) + Tt[lm * 2]);
                ohi[e] = 0.25 * (((Tt[cl * 2 + 1] + Tt[cu * 2 + 1]) + Tt[up * 2 + 1]) +
                                 Tt[lp * 2 + 1]);
                olo[e] = 0.25 * (((Tt[cl * 2 + 1] + Tt[cu * 2 + 1]) + Tt[um * 2 + 1]) +
                                 Tt[lm * 2 + 1]);
              }
            }
            if (e == d) {
              for (int q = 0; q < 3; ++q) {
                vlo[e][q] = Wl[1 + q];
                vhi[e][q] = Wu[1 + q];
              }
              tlo[e] = b->T[cl];
              thi[e] = b->T[cu];
              double A0[3], A1[3], A2[3];
              area_vec(b, d, face_idx(b, d, i, j, k), A0);
              area_vec(b, d, face_idx(b, d, i + (d == 0), j + (d == 1), k + (d == 2)), A1);
              area_vec(b, d, face_idx(b, d, i - (d == 0), j - (d == 1), k - (d == 2)), A2);
              for (int q = 0; q < 3; ++q) {
                ahi[e][q] = 0.5 * (A0[q] + A1[q]);
                alo[e][q] = 0.5 * (A0[q] + A2[q]);
              }
            } else {
              const int64_t cup = cu + st[e], clp = cl + st[e], cum = cu - st[e], clm = cl - st[e];
              const double *Wup = &b->W[cup * NV], *Wlp = &b->W[clp * NV],
                           *Wum = &b->W[cum * NV], *Wlm = &b->W[clm * NV];
              for (int q = 0; q < 3; ++q) {
                vhi[e][q] = 0.25 * (((Wl[1 + q] + Wu[1 + q]) + Wup[1 + q]) + Wlp[1 + q]);
                vlo[e][q] = 0.25 * (((Wl[1 + q] + Wu[1 + q]) + Wum[1 + q]) + Wlm[1 + q]);
              }
              thi[e] = 0.25 * (((b->T[cl] + b->T[cu]) + b->T[cup]) + b->T[clp]);
              tlo[e] = 0.25 * (((b->T[cl] + b->T[cu]) + b->T[cum]) + b->T[clm]);
              /* faces of direction e: cell index (i,j,k) of cu/cl shifted */
              const int64_t xu = cu, xl = cl;
              const int uI = (int)(xu % b->NI) - b->ng, uJ = (int)((xu / b->NI) % b->NJ) - b->ng,
                        uK = (int)(xu / ((int64_t)b->NI * b->NJ)) - b->ng;
              const int lI = (int)(xl % b->NI) - b->ng, lJ = (int)((xl / b->NI) % b->NJ) - b->ng,
                        lK = (int)(xl / ((int64_t)b->NI * b->NJ)) - b->ng;
              double Au[3], Al[3], Aup[3], Alp[3];
              area_vec(b, e, face_idx(b, e, uI, uJ, uK), Au);
              area_vec(b, e, face_idx(b, e, lI, lJ, lK), Al);
              area_vec(b, e, face_idx(b, e, uI + (e == 0), uJ + (e == 1), uK + (e == 2)), Aup);
              area_vec(b, e, face_idx(b, e, lI + (e == 0), lJ + (e == 1), lK + (e == 2)), Alp);
              for (int q = 0; q < 3; ++q) {
                ahi[e][q] = 0.5 * (Aup[q] + Alp[q]);
                alo[e][q] = 0.5 * (Au[q] + Al[q]);
              }
            }
          }
          const double vol = 0.5 * (b->vol[cl] + b->vol[cu]);
          const double invVol = 1.0 / vol;
          double grad[3][3], tg[3];
          for (int r = 0; r < 3; ++r) {     /* area component */
            for (int q = 0; q < 3; ++q) {   /* velocity component */
              grad[r][q] = vhi[0][q] * ahi[0][r] - vlo[0][q] * alo[0][r] +
                           vhi[1][q] * ahi[1][r] - vlo[1][q] * alo[1][r] +
                           vhi[2][q] * ahi[2][r] - vlo[2][q] * alo[2][r];
              grad[r][q] *= invVol;
            }
            tg[r] = thi[0] * ahi[0][r] - tlo[0] * alo[0][r] + thi[1] * ahi[1][r] -
                    tlo[1] * alo[1][r] + thi[2] * ahi[2][r] - tlo[2] * alo[2][r];
            tg[r] *= invVol;
          }
          double kg[3] = {0, 0, 0}, wg[3] = {0, 0, 0};
          if (rans)
            for (int r = 0; r < 3; ++r) {
              kg[r] = khi[0] * ahi[0][r] - klo[0] * alo[0][r] + khi[1] * ahi[1][r] -
                      klo[1] * alo[1][r] + khi[2] * ahi[2][r] - klo[2] * alo[2][r];
              kg[r] *= invVol;
              wg[r] = ohi[0] * ahi[0][r] - olo[0] * alo[0][r] + ohi[1] * ahi[1][r] -
                      olo[1] * alo[1][r] + ohi[2] * ahi[2][r] - olo[2] * alo[2][r];
              wg[r] *= invVol;
            }
          /* face state and viscosity by central reconstruction */
          double cd, cuw;
          central_coeffs(wd[cl], wd[cu], &cd, &cuw);
          double fs[NV];
          for (int q = 0; q < NV; ++q) fs[q] = cd * b->W[cu * NV + q] + cuw * b->W[cl * NV + q];
          const double muf = cd * b->mu[cu] + cuw * b->mu[cl];
          /* SST at the face: k, omega by central reconstruction with the
           * turbulence floors, wall distance likewise (clipped to 0 within
           * WALL_DIST_NEG_TOL), eddy viscosity and blending */
          double fst[2] = {0, 0}, mutf = 0.0, f1f = 0.0, f2f = 0.0;
          if (rans) {
            for (int q = 0; q < 2; ++q)
              fst[q] = cmax(cd * Tt[cu * 2 + q] + cuw * Tt[cl * 2 + q], TURB_MIN);
            double wdf = cd * b->wd[cu] + cuw * b->wd[cl];
            if (wdf < 0.0 && wdf > -1.0e-10) wdf = 0.0;
            if (sv->wilcox) {
              /* turbKWWilcox::EddyViscAndBlending (src/turbulence.cpp:412) */
              f1f = 1.0;
              f2f = 0.0;
              mutf = wk_eddy_visc(fs, fst, &grad[0][0], v->visc_scale);
            } else {
              sst_eddy_visc(fs, fst, &grad[0][0], kg, wg, muf, wdf, v->visc_scale, &mutf, &f1f,
                            &f2f);
            }
          }
          /* viscous flux */
          double n[3], mag;
          face_normal(b, d, face_idx(b, d, i, j, k), n, &mag);
          const double mus = v->visc_scale * muf, muts = v->visc_scale * mutf;
          double Ft[2] = {0, 0};
          if (rans && sv->wilcox) {
            /* the unlimited eddy viscosity in the turbulence diffusion
             * (viscousFlux::CalcFlux src/viscousFlux.cpp:126) */
            const double mutt = v->visc_scale * eddy_visc_nolim(fs, fst);
            Ft[0] = (mus + WK_SIGMASTAR * mutt) * (kg[0] * n[0] + kg[1] * n[1] + kg[2] * n[2]);
            Ft[1] = (mus + WK_SIGMA * mutt) * (wg[0] * n[0] + wg[1] * n[1] + wg[2] * n[2]);
          } else if (rans) {
            Ft[0] = (mus + blended(SST_SIGMAK1, SST_SIGMAK2, f1f) * muts) *
                    (kg[0] * n[0] + kg[1] * n[1] + kg[2] * n[2]);
            Ft[1] = (mus + blended(SST_SIGMAW1, SST_SIGMAW2, f1f) * muts) *
                    (wg[0] * n[0] + wg[1] * n[1] + wg[2] * n[2]);
          }
          const double lambda = 0.0 - (2.0 / 3.0) * (mus + muts);
          const double trace = grad[0][0] + grad[1][1] + grad[2][2];
          double tau[3];
          for (int r = 0; r < 3; ++r) {
            const double sn = (grad[r][0] + grad[0][r]) * n[0] + (grad[r][1] + grad[1][r]) * n[1] +
                              (grad[r][2] + grad[2][r]) * n[2];
            tau[r] = lambda * trace * n[r] + (mus + muts) * sn;
          }
          const double tf = temp_of(fs, g);
          const double kk_ = cond_eff(tf, v);
          const double kt = muts * cp_of(g) / prt_of(v);
          double F[NV];
          F[0] = 0.0;
          F[1] = tau[0];
          F[2] = tau[1];
          F[3] = tau[2];
          F[4] = (tau[0] * fs[1] + tau[1] * fs[2] + tau[2] * fs[3]) +
                 (kk_ + kt) * (tg[0] * n[0] + tg[1] * n[1] + tg[2] * n[2]) + 0.0;
          if (b->wallf[d][face_idx(b, d, i, j, k)]) {
            /* wall data (viscousFlux::CalcWallFlux, src/viscousFlux.cpp:137)
             * and wallData::WallPressure (src/wallData.cpp:140) */
            const double pw = fs[0] * g->r * tf;
            for (int q = 0; q < 3; ++q) b->force[q] += pw * n[q] * mag;
            for (int q = 0; q < 3; ++q) b->force[3 + q] += tau[q] * mag;
          }
          /* block diagonal: ApproxTSLJacobian at the face with the face
           * state, viscosity and gradient, ProjC2CDist as the length; cell
           * gradients: one sixth of each face gradient */
          double c2c = 0.0, Jt[NJAC], Jtt[4];
          const double sixth = 1.0 / 6.0;
          if (sv->block) {
            const double dc[3] = {b->center[cu] - b->center[cl],
                                  b->center[b->nc + cu] - b->center[b->nc + cl],
                                  b->center[2 * b->nc + cu] - b->center[2 * b->nc + cl]};
            c2c = dc[0] * n[0] + dc[1] * n[1] + dc[2] * n[2];
          }
          if (fpos > 0) {
            for (int q = 0; q < NV; ++q) b->R[cl * NV + q] -= F[q] * mag;
            if (rans) {
              for (int q = 0; q < 2; ++q) b->Rt[cl * 2 + q] -= Ft[q] * mag;
              b->mutc[cl] += sixth * mutf;
              for (int q = 0; q < 3; ++q) b->kgc[cl * 3 + q] += sixth * kg[q];
              for (int q = 0; q < 3; ++q) b->wgc[cl * 3 + q] += sixth * wg[q];
              b->f1c[cl] += sixth * f1f;
              b->f2c[cl] += sixth * f2f;
            }
            if (b->vg)
              for (int e = 0; e < 9; ++e) b->vg[cl * 9 + e] += sixth * grad[e / 3][e % 3];
            if (sv->block) {
              tsl_jac(fs, muf, mutf, g, v, n, mag, c2c, 1, &grad[0][0], Jt);
              for (int e = 0; e < NJAC; ++e) b->Ab[cl * NJAC + e] -= Jt[e];
              if (rans) {
                turb_visc_jac(sv->wilcox, fs, fst, mag, muf, mutf, f1f, c2c, v->visc_scale, -1.0,
                              Jtt);
                for (int e = 0; e < 4; ++e) b->Abt[cl * 4 + e] -= Jtt[e];
              }
            }
          }
          if (fpos < nd) {
            for (int q = 0; q < NV; ++q) b->R[cu * NV + q] += F[q] * mag;
            if (rans) {
              for (int q = 0; q < 2; ++q) b->Rt[cu * 2 + q] += Ft[q] * mag;
              b->mutc[cu] += sixth * mutf;
              for (int q = 0; q < 3; ++q) b->kgc[cu * 3 + q] += sixth * kg[q];
              for (int q = 0; q < 3; ++q) b->wgc[cu * 3 + q] += sixth * wg[q];
              b->f1c[cu] += sixth * f1f;
              b->f2c[cu] += sixth * f2f;
            }
            if (b->vg)
              for (int e = 0; e < 9; ++e) b->vg[cu * 9 + e] += sixth * grad[e / 3][e % 3];
            double nl[3], ml, nh[3], mh;
            face_normal(b, d, face_idx(b, d, i, j, k), nl, &ml);
            face_normal(b, d, face_idx(b, d, i + (d == 0), j + (d == 1), k + (d == 2)), nh, &mh);
            const double *Wc = &b->W[cu * NV];
            const double fMag = 0.5 * (ml + mh);
            const double lv = visc_max_term(Wc, g) * visc_term(b->mu[cu], mutf, v, g) * fMag *
                              fMag / b->vol[cu];
            b->lam[cu] += lv * coeff;
            const double lvt = rans ? turb_visc_cell_sr(sv->wilcox, Wc, &Tt[cu * 2], ml, mh,
                                                        b->vol[cu], b->mu[cu], mutf, f1f,
                                                        v->visc_scale)
                                    : 0.0;
            if (rans) b->lamt[cu] += lvt * coeff;
            if (sv->block) {
              tsl_jac(fs, muf, mutf, g, v, n, mag, c2c, 0, &grad[0][0], Jt);
              for (int e = 0; e < NJAC; ++e) b->Ab[cu * NJAC + e] += Jt[e];
              if (rans) {
                turb_visc_jac(sv->wilcox, fs, fst, mag, muf, mutf, f1f, c2c, v->visc_scale, 1.0,
                              Jtt);
                for (int e = 0; e < 4; ++e) b->Abt[cu * 4 + e] += Jtt[e];
              }
            } else {
              b->A[cu] += 2.0 * lv;
              if (rans) b->At[cu] += 2.0 * lvt;
            }
          }
        }
  }
}

/* ---------------------------------------------------------------- API */
orc_case *orc_create(int nblocks, const ath_block_view *bv, int nsolves,
                     const ath_solve_view *sv) {
  orc_case *c = (orc_case *)calloc(1, sizeof(orc_case));
  c->nb = nblocks;
  c->ns = nsolves;
  c->b = (oblock *)calloc(nblocks, sizeof(oblock));
  c->s = (osolve *)calloc(nsolves, sizeof(osolve));
  c->mres = (double *)calloc(nsolves, sizeof(double));
  c->forces = (double *)calloc((size_t)nsolves * 6, sizeof(double));
  for (int s = 0; s < nsolves; ++s) {
    c->s[s].v = sv[s];
    c->s[s].states = (ath_bc_state *)dup_arr(sv[s].states, sizeof(ath_bc_state) * sv[s].nstates);
    c->s[s].v.states = c->s[s].states;
    c->s[s].gas.r = sv[s].gas_r;
    c->s[s].gas.n = sv[s].gas_n;
    c->s[s].gas.hf = sv[s].gas_hf;
    c->s[s].viscous = sv[s].eqn != ATH_EQN_EULER;
    c->s[s].block = sv[s].solver == ATH_SOLVER_BLUSGS || sv[s].solver == ATH_SOLVER_BDPLUR;
    c->s[s].jacobi = sv[s].solver == ATH_SOLVER_DPLUR || sv[s].solver == ATH_SOLVER_BDPLUR;
    c->s[s].rans = sv[s].eqn == ATH_EQN_RANS;
    c->s[s].wilcox = sv[s].turb == ATH_TURB_KW2006;
    c->s[s].sweeps = sv[s].sweeps > 0 ? sv[s].sweeps : 1;
  }
  for (int bi = 0; bi < nblocks; ++bi) {
    const ath_block_view *v = &bv[bi];
    oblock *b = &c->b[bi];
    b->ni = v->ni; b->nj = v->nj; b->nk = v->nk; b->ng = v->ng;
    b->NI = v->ni + 2 * v->ng; b->NJ = v->nj + 2 * v->ng; b->NK = v->nk + 2 * v->ng;
    b->solve = v->solve;
    b->nc = v->ncell_padded;
    b->vol = (double *)dup_arr(v->vol, 8 * b->nc);
    b->width = (double *)dup_arr(v->width, 8 * 3 * b->nc);
    for (int d = 0; d < 3; ++d) {
      b->nf[d] = v->nface_padded[d];
      b->fa[d] = (double *)dup_arr(v->farea[d], 8 * 4 * b->nf[d]);
    }
    const int rans = c->s[b->solve].rans;
    b->W = (double *)dup_arr(NULL, 8 * NV * b->nc);
    for (int64_t x = 0; x < b->nc; ++x)
      for (int q = 0; q < NV; ++q) b->W[x * NV + q] = v->state0[x * v->nv + q];
    if (rans) {
      b->Wt = (double *)dup_arr(NULL, 8 * 2 * b->nc);
      for (int64_t x = 0; x < b->nc; ++x)
        for (int q = 0; q < 2; ++q) b->Wt[x * 2 + q] = v->state0[x * v->nv + 5 + q];
      b->Rt = (double *)dup_arr(NULL, 8 * 2 * b->nc);
      b->dUt = (double *)dup_arr(NULL, 8 * 2 * b->nc);
      b->lamt = (double *)dup_arr(NULL, 8 * b->nc);
      b->At = (double *)dup_arr(NULL, 8 * b->nc);
      b->Ainvt = (double *)dup_arr(NULL, 8 * b->nc);
      b->Abt = (double *)dup_arr(NULL, 8 * 4 * b->nc);
      b->Ainvbt = (double *)dup_arr(NULL, 8 * 4 * b->nc);
      b->mutc = (double *)dup_arr(NULL, 8 * b->nc);
      b->f1c = (double *)dup_arr(NULL, 8 * b->nc);
      b->f2c = (double *)dup_arr(NULL, 8 * b->nc);
      b->kgc = (double *)dup_arr(NULL, 8 * 3 * b->nc);
      b->wgc = (double *)dup_arr(NULL, 8 * 3 * b->nc);
    }
    b->wd = v->wall_dist ? (double *)dup_arr(v->wall_dist, 8 * b->nc) : NULL;
    b->R = (double *)dup_arr(NULL, 8 * NV * b->nc);
    b->dU = (double *)dup_arr(NULL, 8 * NV * b->nc);
    b->lam = (double *)dup_arr(NULL, 8 * b->nc);
    b->dt = (double *)dup_arr(NULL, 8 * b->nc);
    b->Un = (double *)dup_arr(NULL, 8 * 7 * b->nc);
    b->Unm1 = (double *)dup_arr(NULL, 8 * 7 * b->nc);
    b->A = (double *)dup_arr(NULL, 8 * b->nc);
    b->Ainv = (double *)dup_arr(NULL, 8 * b->nc);
    if (c->s[b->solve].viscous) {
      /* cell-averaged velocity gradients (block diagonal, SST sources, output) */
      b->vg = (double *)dup_arr(NULL, 8 * 9 * b->nc);
    }
    if (c->s[b->solve].block) {
      b->Ab = (double *)dup_arr(NULL, 8 * NJAC * b->nc);
      b->Ainvb = (double *)dup_arr(NULL, 8 * NJAC * b->nc);
    }
    b->mask = (uint8_t *)dup_arr(v->nbr_mask, b->nc);
    b->center = (double *)dup_arr(v->center, 8 * 3 * b->nc);
    b->T = (double *)dup_arr(NULL, 8 * b->nc);
    b->mu = (double *)dup_arr(NULL, 8 * b->nc);
    b->corner = (uint8_t *)dup_arr(NULL, b->nc);
    for (int64_t x = 0; x < b->nc; ++x) {
      const int64_t ii = x % b->NI, jj = (x / b->NI) % b->NJ, kk = x / ((int64_t)b->NI * b->NJ);
      const int gi = ii < b->ng || ii >= b->NI - b->ng, gj = jj < b->ng || jj >= b->NJ - b->ng,
                gk = kk < b->ng || kk >= b->NK - b->ng;
      b->corner[x] = (uint8_t)(gi && gj && gk);
    }
    /* gridLevel::AuxillaryAndWidths (src/gridLevel.cpp:433): temperature
     * and viscosity of the physical cells of the initial state */
    if (c->s[b->solve].viscous)
      for (int k = 0; k < b->nk; ++k)
        for (int j = 0; j < b->nj; ++j)
          for (int i = 0; i < b->ni; ++i) {
            const int64_t x = cell_idx(b, i, j, k);
            b->T[x] = temp_of(&b->W[x * NV], &c->s[b->solve].gas);
            b->mu[x] = visc_of(b->T[x], &c->s[b->solve].v);
          }
    b->nops = v->nops;
    b->ops = (ath_ghost_op *)dup_arr(v->ops, sizeof(ath_ghost_op) * v->nops);
    b->nedge = v->nedge_ops;
    b->edge = (ath_ghost_op *)dup_arr(v->edge_ops, sizeof(ath_ghost_op) * v->nedge_ops);
    b->nvops = v->nvops;
    b->vops = (ath_ghost_op *)dup_arr(v->vops, sizeof(ath_ghost_op) * v->nvops);
    b->nvedge = v->nvedge_ops;
    b->vedge = (ath_ghost_op *)dup_arr(v->vedge_ops, sizeof(ath_ghost_op) * v->nvedge_ops);
    b->n_nr = v->n_nr;
    b->nr = (ath_nr_cell *)dup_arr(v->nr, sizeof(ath_nr_cell) * v->n_nr);
    b->n_nr_surf = 0;
    for (int i = 0; i < b->n_nr; ++i)
      if (b->nr[i].surf + 1 > b->n_nr_surf) b->n_nr_surf = b->nr[i].surf + 1;
    b->nr_mach = (double *)dup_arr(NULL, 16 * (size_t)b->n_nr_surf);
    b->nrg = NULL;
    for (int o = 0; o < v->nops; ++o)
      if (v->ops[o].type == ATH_BC_PRESSURE_OUTLET && v->ops[o].state >= 0 &&
          c->s[v->solve].states[v->ops[o].state].nonreflecting) {
        b->nrg = (double *)dup_arr(NULL, sizeof(double) * 12 * (size_t)b->nc);
        break;
      }
    b->nplanes = v->nplanes;
    b->plane_off = (int32_t *)dup_arr(v->plane_offsets, 4 * (v->nplanes + 1));
    b->plane_cells = (int32_t *)dup_arr(v->plane_cells, 4 * (size_t)v->ni * v->nj * v->nk);
    for (int d = 0; d < 3; ++d) b->wallf[d] = (uint8_t *)dup_arr(NULL, b->nf[d]);
    for (int o = 0; o < b->nvops; ++o)
      if (b->vops[o].layer == 1) b->wallf[b->vops[o].dir][b->vops[o].face] = 1;
  }
  return c;
}

void orc_destroy(orc_case *c) {
  if (!c) return;
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    free(b->vol); free(b->width);
    for (int d = 0; d < 3; ++d) free(b->fa[d]);
    free(b->W); free(b->R); free(b->dU); free(b->lam); free(b->dt); free(b->A);
    free(b->Un); free(b->Unm1);
    free(b->nr); free(b->nr_mach); free(b->nrg);
    free(b->Ainv); free(b->mask); free(b->ops); free(b->plane_off); free(b->plane_cells);
    free(b->center); free(b->T); free(b->mu); free(b->corner);
    free(b->edge); free(b->vops); free(b->vedge);
    free(b->Ab); free(b->Ainvb); free(b->vg);
    free(b->Wt); free(b->Rt); free(b->dUt); free(b->lamt); free(b->At); free(b->Ainvt);
    free(b->Abt); free(b->Ainvbt); free(b->mutc); free(b->f1c); free(b->f2c);
    free(b->kgc); free(b->wgc); free(b->wd);
    for (int d = 0; d < 3; ++d) free(b->wallf[d]);
    free(b->F); free(b->mr); free(b->mg_cell); free(b->mg_volfac); free(b->mg_coef);
    free(b->og);
  }
  for (int s = 0; s < c->ns; ++s) free(c->s[s].states);
  free(c->b);
  free(c->s);
  free(c->mres);
  free(c->forces);
  free(c);
}

void orc_set_threads(orc_case *c, int n) { c->nthreads = n; }
void orc_set_matrix_resid(orc_case *c, int on) { c->matrix_resid = on; }
void orc_forces(const orc_case *c, int solve, double *out) {
  for (int q = 0; q < 6; ++q) out[q] = (solve >= 0 && solve < c->ns) ? c->forces[solve * 6 + q] : 0.0;
}
double orc_matrix_resid(const orc_case *c, int solve) {
  return (solve >= 0 && solve < c->ns) ? c->mres[solve] : 0.0;
}

#ifdef _OPENMP
#define PAR_BLOCKS _Pragma("omp parallel for schedule(dynamic, 1) num_threads(nth)")
#define NTH int nth = c->nthreads > 0 ? c->nthreads : omp_get_max_threads();
#else
#define PAR_BLOCKS
#define NTH
#endif

/* ExtrapolateHoldMixture (src/ghostStates.cpp:693), one species */
static void extrap_hold(double *g, double factor, const double *in) {
  const double ghostRho = factor * g[0] - in[0];
  if (ghostRho <= 0.0) return;
  const double mf = g[0] / g[0];
  for (int v = 0; v < NV; ++v) g[v] = factor * g[v] - in[v];
  const double r = ghostRho * mf;
  g[0] = (r > 0.0) ? r : 0.0;
}

/* GetGhostState (src/ghostStates.cpp:62) for the supported types;
 * interblock/periodic: copy of the partner cell (SwapStateSlice). */
void orc_fill_ghosts(orc_case *c) {
  /* CalcCFL of the time step (src/input.cpp:647); at a time step's first
   * nonlinear iteration StoreOldSolution (src/mgSolution.cpp:103): the
   * conserved state of time n, and of time n-1 too at the first step of a
   * multilevel (bdf2) solve */
  for (int s = 0; s < c->ns; ++s) {
    const ath_solve_view *v = &c->s[s].v;
    const int nl = v->nl_iters > 0 ? v->nl_iters : 1;
    const double cfl = v->cfl_start + (double)(c->iter / nl) * v->cfl_step;
    c->s[s].cfl = cfl < v->cfl_max ? cfl : v->cfl_max;
  }
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const ath_solve_view *v = &c->s[b->solve].v;
    const int nl = v->nl_iters > 0 ? v->nl_iters : 1;
    if (c->iter % nl != 0) continue;
    for (int k = 0; k < b->nk; ++k)
      for (int j = 0; j < b->nj; ++j)
        for (int i = 0; i < b->ni; ++i) {
          const int64_t x = cell_idx(b, i, j, k);
          double *un = &b->Un[x * 7];
          prim_to_cons(&b->W[x * NV], &c->s[b->solve].gas, un);
          un[5] = b->Wt ? b->W[x * NV] * b->Wt[x * 2] : 0.0;
          un[6] = b->Wt ? b->W[x * NV] * b->Wt[x * 2 + 1] : 0.0;
          /* a restarted run keeps the file's time n-1 (!IsRestart()) */
          if (v->multilevel && c->iter == 0 && !c->s[b->solve].nm1_given)
            memcpy(&b->Unm1[x * 7], un, 8 * 7);
        }
  }
  NTH
  PAR_BLOCKS
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const osolve *sv = &c->s[b->solve];
    /* average and largest outward normal Mach number of each nonreflecting
     * surface over its boundary-adjacent cells, summed in the surface's
     * k, j, i order (procBlock::GetGhostStates src/procBlock.cpp:6235-6260) */
    for (int sf = 0; sf < b->n_nr_surf; ++sf) {
      double avg = 0.0, mx = -1.0 * DBL_MAX;
      int cnt = 0;
      for (int i = 0; i < b->n_nr; ++i) {
        const ath_nr_cell *x = &b->nr[i];
        if (x->surf != sf) continue;
        double nn[3], mg;
        face_normal(b, x->dir, x->face, nn, &mg);
        if (x->lower)
          for (int e = 0; e < 3; ++e) nn[e] = -1.0 * nn[e];
        const double *w = &b->W[x->cell * NV];
        const double mach = (w[1] * nn[0] + w[2] * nn[1] + w[3] * nn[2]) / sos_of(w, &sv->gas);
        mx = mx < mach ? mach : mx;
        avg += mach;
        ++cnt;
      }
      avg /= (double)cnt;
      b->nr_mach[2 * sf] = avg;
      b->nr_mach[2 * sf + 1] = mx;
    }
    for (int o = 0; o < b->nops; ++o) {
      const ath_ghost_op *op = &b->ops[o];
      const oblock *src = &c->b[op->src_block];
      const double *in = &src->W[op->src * NV];
      double g[NV];
      memcpy(g, in, sizeof(g));
      const int rans = sv->rans;
      const double *int_ = rans ? &src->Wt[op->src * 2] : NULL;
      double gt[2] = {0.0, 0.0};
      if (rans) {
        gt[0] = int_[0];
        gt[1] = int_[1];
      }
      if (op->type != ATH_BC_PERIODIC && op->type != ATH_BC_INTERBLOCK) {
        double n[3], mag;
        face_normal(b, op->dir, op->face, n, &mag);
        if (op->lower) {
          n[0] = -1.0 * n[0];
          n[1] = -1.0 * n[1];
          n[2] = -1.0 * n[2];
        }
        if (op->type == ATH_BC_SLIP_WALL) {
          const double vn = in[1] * n[0] + in[2] * n[1] + in[3] * n[2];
          g[1] = in[1] - 2.0 * n[0] * vn;
          g[2] = in[2] - 2.0 * n[1] * vn;
          g[3] = in[3] - 2.0 * n[2] * vn;
        } else if (op->type == ATH_BC_CHARACTERISTIC) {
          const ath_bc_state *bs = &sv->states[op->state];
          const double fr[NV] = {bs->rho, bs->u, bs->v, bs->w, bs->p};
          const double freeVel[3] = {bs->u, bs->v, bs->w};
          const double vin = in[1] * n[0] + in[2] * n[1] + in[3] * n[2];
          const double sosInt = sos_of(in, &sv->gas);
          const double machInt = fabs(vin) / sosInt;
          if (machInt >= 1.0 && vin < 0.0) {
            memcpy(g, fr, sizeof(g));
            if (rans)
              farfield_turb(g, freeVel, bs->turb_intensity, bs->eddy_visc_ratio, &sv->gas,
                            &sv->v, gt);
          } else if (machInt >= 1.0 && vin >= 0.0) {
          } else if (machInt < 1.0 && vin < 0.0) {
            const double rhoSoSInt = in[0] * sosInt;
            const double dv[3] = {fr[1] - in[1], fr[2] - in[2], fr[3] - in[3]};
            g[4] = 0.5 * (fr[4] + in[4] -
                          rhoSoSInt * (n[0] * dv[0] + n[1] * dv[1] + n[2] * dv[2]));
            const double dp = fr[4] - g[4];
            const double rho = fr[0] - dp / (sosInt * sosInt);
            g[0] = rho * (fr[0] / fr[0]);
            g[1] = fr[1] - n[0] * dp / rhoSoSInt;
            g[2] = fr[2] - n[1] * dp / rhoSoSInt;
            g[3] = fr[3] - n[2] * dp / rhoSoSInt;
            if (rans)
              farfield_turb(g, freeVel, bs->turb_intensity, bs->eddy_visc_ratio, &sv->gas,
                            &sv->v, gt);
          } else {
            const double rhoSoSInt = in[0] * sosInt;
            const double dp = in[4] - fr[4];
            const double rho = in[0] - dp / (sosInt * sosInt);
            g[0] = rho * (in[0] / in[0]);
            g[1] = in[1] + n[0] * dp / rhoSoSInt;
            g[2] = in[2] + n[1] * dp / rhoSoSInt;
            g[3] = in[3] + n[2] * dp / rhoSoSInt;
            g[4] = fr[4];
          }
          if (rans) {
            extrap_hold7(g, gt, 2.0, in, int_);
            if (op->layer > 1) {
              extrap_hold7(g, gt, (double)op->layer, in, int_);
              farfield_turb(g, freeVel, bs->turb_intensity, bs->eddy_visc_ratio, &sv->gas,
                            &sv->v, gt);
            }
          } else {
            extrap_hold(g, 2.0, in);
            if (op->layer > 1) extrap_hold(g, (double)op->layer, in);
          }
        } else if (op->type == ATH_BC_PRESSURE_OUTLET) {
          /* src/ghostStates.cpp:605-672, reflecting form */
          const ath_bc_state *bs = &sv->states[op->state];
          const double sosInt = sos_of(in, &sv->gas);
          const double rhoSoSInt = in[0] * sosInt;
          g[4] = bs->p_out;
          if (bs->nonreflecting) {
            /* LODI relaxation with transverse terms (src/ghostStates.cpp:
             * 612-638): time-n state, previous dt and gradients of the
             * cell, average and largest normal Mach number of the surface */
            double sN[NV];
            cons_to_prim(&b->Un[op->src * 7], &sv->gas, sN);
            const double dt = b->dt[op->src];
            const double avgMach = b->nr_mach[2 * op->src2];
            const double maxMach = b->nr_mach[2 * op->src2 + 1];
            const double *vg = &b->nrg[op->src * 12], *pgr = &b->nrg[op->src * 12 + 9];
            const double deltaVel =
                (in[1] - sN[1]) * n[0] + (in[2] - sN[2]) * n[1] + (in[3] - sN[3]) * n[2];
            const double sigma = 0.25;
            const double sosN = sos_of(sN, &sv->gas);
            const double rhoSoSN = sN[0] * sosN;
            const double k = sigma * sosN * (1.0 - maxMach * maxMach) / bs->length_scale;
            const double beta = avgMach;
            const double pgn = pgr[0] * n[0] + pgr[1] * n[1] + pgr[2] * n[2];
            double pgT[3], velT[3], gT[9], dVn[3];
            const double vnN = sN[1] * n[0] + sN[2] * n[1] + sN[3] * n[2];
            for (int e = 0; e < 3; ++e) {
              pgT[e] = pgr[e] - pgn * n[e];
              velT[e] = sN[1 + e] - vnN * n[e];
            }
            /* tensor::RemoveComponent, LinearCombination, Sum
             * (include/tensor.hpp:371-389) */
            for (int r = 0; r < 3; ++r) {
              const double rn = vg[r * 3] * n[0] + vg[r * 3 + 1] * n[1] + vg[r * 3 + 2] * n[2];
              for (int q = 0; q < 3; ++q) gT[r * 3 + q] = vg[r * 3 + q] - rn * n[q];
            }
            for (int q = 0; q < 3; ++q) {
              dVn[q] = gT[q] * n[0];
              dVn[q] += gT[3 + q] * n[1];
              dVn[q] += gT[6 + q] * n[2];
            }
            double gsum = 0.0;
            for (int e = 0; e < 9; ++e) gsum += gT[e];
            const double dVelT = gsum - (((0.0 + dVn[0]) + dVn[1]) + dVn[2]);
            const double gam = gamma_of(&sv->gas);
            const double w0 = pgT[0] - rhoSoSN * dVn[0], w1 = pgT[1] - rhoSoSN * dVn[1],
                         w2 = pgT[2] - rhoSoSN * dVn[2];
            const double tr = -0.5 * ((velT[0] * w0 + velT[1] * w1 + velT[2] * w2) +
                                      gam * sN[4] * dVelT);
            g[4] = (sN[4] + rhoSoSN * deltaVel + dt * k * bs->p_out - dt * beta * tr) /
                   (1.0 + dt * k);
          }
          const double dp = in[4] - g[4];
          const double rho = in[0] - dp / (sosInt * sosInt);
          g[0] = rho * (in[0] / in[0]);
          g[1] = in[1] + n[0] * dp / rhoSoSInt;
          g[2] = in[2] + n[1] * dp / rhoSoSInt;
          g[3] = in[3] + n[2] * dp / rhoSoSInt;
          if ((g[1] * n[0] + g[2] * n[1] + g[3] * n[2]) / sos_of(g, &sv->gas) >= 1.0) {
            memcpy(g, in, sizeof(g));
            if (rans) {
              gt[0] = int_[0];
              gt[1] = int_[1];
            }
          }
          for (int v = 0; v < NV; ++v) g[v] = 2.0 * g[v] - in[v];
          if (rans)
            for (int v = 0; v < 2; ++v) gt[v] = 2.0 * gt[v] - int_[v];
          if (op->layer > 1) {
            for (int v = 0; v < NV; ++v) g[v] = (double)op->layer * g[v] - in[v];
            if (rans)
              for (int v = 0; v < 2; ++v) gt[v] = (double)op->layer * gt[v] - int_[v];
          }
        } else if (op->type == ATH_BC_STAGNATION_INLET) {
          /* src/ghostStates.cpp:535-604 */
          const ath_bc_state *bs = &sv->states[op->state];
          const double gm1 = gamma_of(&sv->gas) - 1.0;
          const double vn = in[1] * n[0] + in[2] * n[1] + in[3] * n[2];
          const double sosInt = sos_of(in, &sv->gas);
          const double rNeg = vn - 2.0 * sosInt / gm1;
          const double cosTheta = -1.0 * vn / velmag(in);
          /* pow(sos, 2.0) is the correctly rounded square */
          const double stagSoSsq =
              sosInt * sosInt + 0.5 * gm1 * (in[1] * in[1] + in[2] * in[2] + in[3] * in[3]);
          const double sosB = -1.0 * rNeg * gm1 / (gm1 * cosTheta * cosTheta + 2.0) *
                              (1.0 + cosTheta * sqrt((gm1 * cosTheta * cosTheta + 2.0) *
                                                         stagSoSsq / (gm1 * rNeg * rNeg) -
                                                     0.5 * gm1));
          const double tb = bs->t0 * (sosB * sosB / stagSoSsq);
          const double pb = bs->p0 * pow(sosB * sosB / stagSoSsq, gamma_of(&sv->gas) / gm1);
          const double vbMag = sqrt(2.0 / gm1 * (bs->t0 - tb));
          const double rhoGhost = pb / ((0.0 + 1.0 * sv->gas.r) * tb);
          g[0] = rhoGhost * 1.0;
          g[1] = vbMag * bs->dir[0];
          g[2] = vbMag * bs->dir[1];
          g[3] = vbMag * bs->dir[2];
          g[4] = pb;
          if (rans) {
            const double vel[3] = {g[1], g[2], g[3]};
            farfield_turb(g, vel, bs->turb_intensity, bs->eddy_visc_ratio, &sv->gas, &sv->v,
                          gt);
            extrap_hold7(g, gt, 2.0, in, int_);
            if (op->layer > 1) {
              extrap_hold7(g, gt, (double)op->layer, in, int_);
              const double vel2[3] = {g[1], g[2], g[3]};
              farfield_turb(g, vel2, bs->turb_intensity, bs->eddy_visc_ratio, &sv->gas,
                            &sv->v, gt);
            }
          } else {
            extrap_hold(g, 2.0, in);
            if (op->layer > 1) extrap_hold(g, (double)op->layer, in);
          }
        } else if (op->type == ATH_BC_INLET) {
          /* src/ghostStates.cpp:392-493, reflecting form */
          const ath_bc_state *bs = &sv->states[op->state];
          const double fr[NV] = {bs->rho, bs->u, bs->v, bs->w, bs->p};
          const double freeVel[3] = {bs->u, bs->v, bs->w};
          const double vin = in[1] * n[0] + in[2] * n[1] + in[3] * n[2];
          const double sosInt = sos_of(in, &sv->gas);
          const double machInt = fabs(vin) / sosInt;
          if (machInt >= 1.0) {
            memcpy(g, fr, sizeof(g));
            if (rans)
              farfield_turb(g, freeVel, bs->turb_intensity, bs->eddy_visc_ratio, &sv->gas,
                            &sv->v, gt);
          } else {
            const double rhoSoSInt = in[0] * sosInt;
            const double dv[3] = {fr[1] - in[1], fr[2] - in[2], fr[3] - in[3]};
            g[4] = 0.5 * (fr[4] + in[4] -
                          rhoSoSInt * (n[0] * dv[0] + n[1] * dv[1] + n[2] * dv[2]));
            if (bs->nonreflecting) {
              /* LODI relaxation of the incoming characteristic
               * (src/ghostStates.cpp:433-461) */
              double sN[NV];
              cons_to_prim(&b->Un[op->src * 7], &sv->gas, sN);
              const double dt = b->dt[op->src];
              const double maxMach = b->nr_mach[2 * op->src2 + 1];
              const double sigma = 0.25;
              const double rhoN = sN[0];
              const double sosN = sos_of(sN, &sv->gas);
              const double rhoSoSN = rhoN * sosN;
              const double dp = g[4] - sN[4];
              const double alpha = sigma * sosN / bs->length_scale;
              const double rhoNp1 =
                  (rhoN + dt * alpha * fr[0] + dp / (sosN * sosN)) / (1.0 + dt * alpha);
              g[0] = rhoNp1 * (fr[0] / fr[0]);
              const double k = alpha * (1.0 - maxMach * maxMach);
              for (int e = 0; e < 3; ++e)
                g[1 + e] = (sN[1 + e] + dt * k * fr[1 + e] - n[e] * dp / rhoSoSN) / (1.0 + dt * k);
            } else {
              const double dp = fr[4] - g[4];
              const double rho = fr[0] - dp / (sosInt * sosInt);
              g[0] = rho * (fr[0] / fr[0]);
              g[1] = fr[1] - n[0] * dp / rhoSoSInt;
              g[2] = fr[2] - n[1] * dp / rhoSoSInt;
              g[3] = fr[3] - n[2] * dp / rhoSoSInt;
            }
            if (rans) {
              farfield_turb(g, freeVel, bs->turb_intensity, bs->eddy_visc_ratio, &sv->gas,
                            &sv->v, gt);
              extrap_hold7(g, gt, 2.0, in, int_);
              if (op->layer > 1) extrap_hold7(g, gt, (double)op->layer, in, int_);
            } else {
              extrap_hold(g, 2.0, in);
              if (op->layer > 1) extrap_hold(g, (double)op->layer, in);
            }
          }
        } else if (op->type == ATH_BC_SUPERSONIC_INFLOW) {
          const ath_bc_state *bs = &sv->states[op->state];
          g[0] = bs->rho; g[1] = bs->u; g[2] = bs->v; g[3] = bs->w; g[4] = bs->p;
          if (rans) {
            const double vel[3] = {bs->u, bs->v, bs->w};
            farfield_turb(g, vel, bs->turb_intensity, bs->eddy_visc_ratio, &sv->gas, &sv->v,
                          gt);
          }
        } else if (op->type == ATH_BC_SUPERSONIC_OUTFLOW) {
          if (op->layer > 1) {
            for (int v = 0; v < NV; ++v) g[v] = (double)op->layer * in[v] - in[v];
            if (rans)
              for (int v = 0; v < 2; ++v) gt[v] = (double)op->layer * int_[v] - int_[v];
          }
        }
      }
      memcpy(&b->W[op->dst * NV], g, sizeof(g));
      if (rans) memcpy(&b->Wt[op->dst * 2], gt, sizeof(gt));
    }
  }
  PAR_BLOCKS
  for (int bi = 0; bi < c->nb; ++bi) apply_edge_ops(&c->b[bi], c->b[bi].nedge, c->b[bi].edge);
}

/* procBlock::CalcResidualNoSource (src/procBlock.cpp:6111) for inviscid
 * flow: ResetResidWS, then CalcInvFluxI/J/K (src/procBlock.cpp:384,522,660):
 * per face, MUSCL states, Roe flux, scatter +F|A| to the lower cell and
 * -F|A| to the upper cell, cell spectral radius and scalar diagonal for the
 * upper cell. */
void orc_residual(orc_case *c) {
  NTH
  PAR_BLOCKS
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const osolve *sv = &c->s[b->solve];
    const gas_t *g = &sv->gas;
    memset(b->R, 0, 8 * NV * b->nc);
    memset(b->lam, 0, 8 * b->nc);
    if (c->mg_visits <= 1) memset(b->A, 0, 8 * b->nc);
    memset(b->force, 0, sizeof(b->force));
    if (sv->rans) {
      memset(b->Rt, 0, 8 * 2 * b->nc);
      memset(b->lamt, 0, 8 * b->nc);
      memset(b->At, 0, 8 * b->nc);
      memset(b->Abt, 0, 8 * 4 * b->nc);
      memset(b->mutc, 0, 8 * b->nc);
      memset(b->f1c, 0, 8 * b->nc);
      memset(b->f2c, 0, 8 * b->nc);
      memset(b->kgc, 0, 8 * 3 * b->nc);
      memset(b->wgc, 0, 8 * 3 * b->nc);
    }
    if (sv->block && c->mg_visits <= 1) memset(b->Ab, 0, 8 * NJAC * b->nc);
    if (b->vg) memset(b->vg, 0, 8 * 9 * b->nc);
    for (int d = 0; d < 3; ++d) {
      const int ei = b->ni + (d == 0), ej = b->nj + (d == 1), ek = b->nk + (d == 2);
      const int nd = d == 0 ? b->ni : (d == 1 ? b->nj : b->nk);
      const int64_t st = d == 0 ? 1 : (d == 1 ? b->NI : (int64_t)b->NI * b->NJ);
      const double *wd = &b->width[d * b->nc];
      for (int k = 0; k < ek; ++k)
        for (int j = 0; j < ej; ++j)
          for (int i = 0; i < ei; ++i) {
            const int fpos = d == 0 ? i : (d == 1 ? j : k);
            const int64_t cu = cell_idx(b, i, j, k); /* upper cell of the face */
            const int64_t cl = cu - st;
            const double *wm1 = &b->W[cl * NV], *w0 = &b->W[cu * NV];
            double fL[NV], fR[NV], f[NV], n[3], mag;
            double fLt[2] = {0, 0}, fRt[2] = {0, 0}, ft[2] = {0, 0};
            const int recon = sv->v.recon;
            const int rans = sv->rans;
            if (rans) {
              /* k, omega reconstructed like the flow variables */
              const double *T_ = b->Wt;
              if (recon == ATH_RECON_CONSTANT) {
                memcpy(fLt, &T_[cl * 2], sizeof(fLt));
                memcpy(fRt, &T_[cu * 2], sizeof(fRt));
              } else if (recon == ATH_RECON_MUSCL) {
                muscl_n(&T_[(cl - st) * 2], &T_[cl * 2], &T_[cu * 2], sv->v.kappa,
                        sv->v.limiter, wd[cl - st], wd[cl], wd[cu], fLt, 2);
                muscl_n(&T_[(cu + st) * 2], &T_[cu * 2], &T_[cl * 2], sv->v.kappa,
                        sv->v.limiter, wd[cu + st], wd[cu], wd[cl], fRt, 2);
              } else {
                const double *cl5[5] = {&T_[(cl - 2 * st) * 2], &T_[(cl - st) * 2],
                                        &T_[cl * 2], &T_[cu * 2], &T_[(cu + st) * 2]};
                const double wl5[5] = {wd[cl - 2 * st], wd[cl - st], wd[cl], wd[cu],
                                       wd[cu + st]};
                const double *cu5[5] = {&T_[(cu + 2 * st) * 2], &T_[(cu + st) * 2],
                                        &T_[cu * 2], &T_[cl * 2], &T_[(cl - st) * 2]};
                const double wu5[5] = {wd[cu + 2 * st], wd[cu + st], wd[cu], wd[cl],
                                       wd[cl - st]};
                weno_n(cl5, wl5, recon == ATH_RECON_WENOZ, fLt, 2);
                weno_n(cu5, wu5, recon == ATH_RECON_WENOZ, fRt, 2);
              }
            }
            if (recon == ATH_RECON_CONSTANT) {
              memcpy(fL, wm1, sizeof(fL));
              memcpy(fR, w0, sizeof(fR));
            } else if (recon == ATH_RECON_MUSCL) {
              const double *wm2 = &b->W[(cl - st) * NV], *wp1 = &b->W[(cu + st) * NV];
              muscl_n(wm2, wm1, w0, sv->v.kappa, sv->v.limiter, wd[cl - st], wd[cl],
                      wd[cu], fL, NV);
              muscl_n(wp1, w0, wm1, sv->v.kappa, sv->v.limiter, wd[cu + st], wd[cu],
                      wd[cl], fR, NV);
            } else {
              const double *wm3 = &b->W[(cl - 2 * st) * NV], *wm2 = &b->W[(cl - st) * NV],
                           *wp1 = &b->W[(cu + st) * NV], *wp2 = &b->W[(cu + 2 * st) * NV];
              const double *cl5[5] = {wm3, wm2, wm1, w0, wp1};
              const double wl5[5] = {wd[cl - 2 * st], wd[cl - st], wd[cl], wd[cu], wd[cu + st]};
              const double *cu5[5] = {wp2, wp1, w0, wm1, wm2};
              const double wu5[5] = {wd[cu + 2 * st], wd[cu + st], wd[cu], wd[cl], wd[cl - st]};
              weno_n(cl5, wl5, recon == ATH_RECON_WENOZ, fL, NV);
              weno_n(cu5, wu5, recon == ATH_RECON_WENOZ, fR, NV);
            }
            face_normal(b, d, face_idx(b, d, i, j, k), n, &mag);
            if (sv->v.flux == ATH_FLUX_AUSM)
              ausm_flux(fL, fR, fLt, fRt, g, n, f, rans ? ft : NULL);
            else
              roe_flux(fL, fR, fLt, fRt, g, n, f, rans ? ft : NULL);
            double J[NJAC], Jt[4];
            if (fpos > 0) {
              for (int v = 0; v < NV; ++v) b->R[cl * NV + v] += f[v] * mag;
              if (rans)
                for (int v = 0; v < 2; ++v) b->Rt[cl * 2 + v] += ft[v] * mag;
              if (sv->block) {
                rusanov_jac(fL, g, n, mag, 1, J);
                for (int e = 0; e < NJAC; ++e) b->Ab[cl * NJAC + e] += J[e];
                if (rans) {
                  turb_rusanov_jac(fL, n, mag, 1, Jt);
                  for (int e = 0; e < 4; ++e) b->Abt[cl * 4 + e] += Jt[e];
                }
              }
            }
            if (fpos < nd) {
              for (int v = 0; v < NV; ++v) b->R[cu * NV + v] -= f[v] * mag;
              if (rans)
                for (int v = 0; v < 2; ++v) b->Rt[cu * 2 + v] -= ft[v] * mag;
              double nl[3], ml, nh[3], mh;
              face_normal(b, d, face_idx(b, d, i, j, k), nl, &ml);
              face_normal(b, d,
                          face_idx(b, d, i + (d == 0), j + (d == 1), k + (d == 2)), nh, &mh);
              const double lam = inv_cell_specrad(w0, g, nl, ml, nh, mh);
              b->lam[cu] += lam;
              const double lamt = rans ? turb_inv_cell_sr(w0, nl, ml, nh, mh) : 0.0;
              if (rans) b->lamt[cu] += lamt;
              if (sv->block) {
                rusanov_jac(fR, g, n, mag, 0, J);
                for (int e = 0; e < NJAC; ++e) b->Ab[cu * NJAC + e] -= J[e];
                if (rans) {
                  turb_rusanov_jac(fR, n, mag, 0, Jt);
                  for (int e = 0; e < 4; ++e) b->Abt[cu * 4 + e] -= Jt[e];
                }
              } else {
                b->A[cu] += lam;
                if (rans) b->At[cu] += lamt;
              }
            }
          }
    }
    if (sv->viscous) {
      /* AssignViscousGhostCells (src/procBlock.cpp:2760) + edges */
      for (int o = 0; o < b->nvops; ++o) {
        const ath_ghost_op *op = &b->vops[o];
        double gw[NV];
        viscous_wall_ghost(&b->W[op->src * NV], &sv->states[op->state], g, &sv->v,
                           b->wd ? b->wd[op->src2] : 0.0, gw);
        memcpy(&b->W[op->dst * NV], gw, sizeof(gw));
        if (sv->rans) {
          /* low-Re wall: k = 0 and omega = 60 nu / (beta1 d^2) at the face
           * (src/ghostStates.cpp:262-275); nu and d of the wall-adjacent
           * cell, nu from the previous auxiliary update */
          const double *it = &b->Wt[op->src * 2];
          const int64_t a = op->src2;
          const double nuW = b->mu[a] / b->W[a * NV];
          const double s_ = sv->v.visc_scale;
          /* turbModel::WallBeta: SST beta1, Wilcox 2006 beta0 */
          const double wallBeta = c->s[b->solve].wilcox ? WK_BETA0 : SST_BETA1;
          const double wWall = s_ * s_ * 60.0 * nuW / (b->wd[a] * b->wd[a] * wallBeta);
          double *gt = &b->Wt[op->dst * 2];
          gt[0] = -1.0 * it[0];
          gt[1] = 2.0 * wWall - it[1];
          if (op->layer > 1) gt[1] = (double)op->layer * gt[1] - wWall;
        }
      }
      apply_edge_ops(b, b->nvedge, b->vedge);
      /* UpdateAuxillaryVariables (src/procBlock.cpp:6171): all but corners */
      for (int64_t x = 0; x < b->nc; ++x) {
        if (b->corner[x]) continue;
        b->T[x] = temp_of(&b->W[x * NV], g);
        b->mu[x] = visc_of(b->T[x], &sv->v);
      }
      viscous_fluxes(c, b);
    }
    if (b->nrg) nr_grads(c, b);
    if (b->og) out_grads(c, b);
  }
  memset(c->forces, 0, sizeof(double) * 6 * c->ns);
  for (int bi = 0; bi < c->nb; ++bi)
    for (int q = 0; q < 6; ++q) c->forces[c->b[bi].solve * 6 + q] += c->b[bi].force[q];
  /* SwapEddyViscAndGradients (src/gridLevel.cpp:343): cell gradients of
   * the connection ghosts from the partner block */
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const int rans = c->s[b->solve].rans;
    if (!c->s[b->solve].block && !rans) continue;
    for (int o = 0; o < b->nops; ++o) {
      const ath_ghost_op *op = &b->ops[o];
      if (op->type != ATH_BC_PERIODIC && op->type != ATH_BC_INTERBLOCK) continue;
      const oblock *sb = &c->b[op->src_block];
      memcpy(&b->vg[op->dst * 9], &sb->vg[op->src * 9], 8 * 9);
      if (rans) {
        /* and SwapTurbVars (src/gridLevel.cpp:321): eddy viscosity,
         * blending functions, k and omega gradients */
        b->mutc[op->dst] = sb->mutc[op->src];
        b->f1c[op->dst] = sb->f1c[op->src];
        b->f2c[op->dst] = sb->f2c[op->src];
        memcpy(&b->kgc[op->dst * 3], &sb->kgc[op->src * 3], 8 * 3);
        memcpy(&b->wgc[op->dst * 3], &sb->wgc[op->src * 3], 8 * 3);
      }
    }
  }
  /* procBlock::CalcSrcTerms (src/procBlock.cpp:5956): SST sources of the
   * physical cells from the cell-averaged gradients, eddy viscosity and
   * blending; the source Jacobian's radius (negative) is subtracted from
   * the turbulence radius and diagonal */
  PAR_BLOCKS
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const osolve *sv = &c->s[b->solve];
    if (!sv->rans) continue;
    const double scale = sv->v.visc_scale;
    const double inv = 1.0 / scale;
    for (int k = 0; k < b->nk; ++k)
      for (int j = 0; j < b->nj; ++j)
        for (int i = 0; i < b->ni; ++i) {
          const int64_t x = cell_idx(b, i, j, k);
          const double *w = &b->W[x * NV], *kw = &b->Wt[x * 2];
          double src[2];
          const double beta =
              c->s[b->solve].wilcox
                  ? wk_source(w, kw, &b->vg[x * 9], &b->kgc[x * 3], &b->wgc[x * 3], b->mutc[x],
                              scale, src)
                  : sst_source(w, kw, &b->vg[x * 9], &b->kgc[x * 3], &b->wgc[x * 3], b->mutc[x],
                               b->f1c[x], scale, src);
          const double vol = b->vol[x];
          const double srcSR = -2.0 * SST_BETASTAR * kw[1] * vol * inv;
          b->lamt[x] -= srcSR;
          if (sv->block) {
            const double j00 = -2.0 * SST_BETASTAR * kw[1] * 1.0 * vol * inv;
            const double j11 = -2.0 * beta * kw[1] * vol * inv;
            b->Abt[x * 4 + 0] -= j00;
            b->Abt[x * 4 + 1] -= 0.0;
            b->Abt[x * 4 + 2] -= 0.0;
            b->Abt[x * 4 + 3] -= j11;
          } else {
            b->A[x] -= 0.0;
            b->At[x] -= srcSR;
          }
          for (int q = 0; q < 2; ++q) b->Rt[x * 2 + q] -= src[q] * vol;
        }
  }
}

/* procBlock::CalcBlockTimeStep / CalcCellDt (src/procBlock.cpp:782,798) */
void orc_timestep(orc_case *c) {
  NTH
  PAR_BLOCKS
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const double cfl = c->s[b->solve].cfl;
    for (int k = 0; k < b->nk; ++k)
      for (int j = 0; j < b->nj; ++j)
        for (int i = 0; i < b->ni; ++i) {
          const int64_t x = cell_idx(b, i, j, k);
          /* global time step when given, else local from the CFL with
           * uncoupledScalar::Max of the flow and turbulence radii */
          const double dtg = c->s[b->solve].v.dt_global;
          const double lm = b->Wt ? cmax(b->lam[x], b->lamt[x]) : b->lam[x];
          b->dt[x] = dtg > 0.0 ? dtg : cfl * (b->vol[x] / lm);
        }
  }
}

/* linearSolver::AddDiagonalTerms / Invert (src/linearSolver.cpp:146,177),
 * scalar diagonal or 5x5 block (MatrixInverse, src/matrix.cpp:57) */
void orc_diag_invert(orc_case *c) {
  NTH
  PAR_BLOCKS
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const ath_solve_view *v = &c->s[b->solve].v;
    for (int k = 0; k < b->nk; ++k)
      for (int j = 0; j < b->nj; ++j)
        for (int i = 0; i < b->ni; ++i) {
          const int64_t x = cell_idx(b, i, j, k);
          double diagVolTime = (b->vol[x] * (1.0 + v->zeta)) / (b->dt[x] * v->theta);
          if (v->dual_cfl > 0.0) {
            /* dual time stepping: volume / tau */
            const double lm = b->Wt ? cmax(b->lam[x], b->lamt[x]) : cmax(b->lam[x], 0.0);
            diagVolTime += lm / v->dual_cfl;
          }
          if (c->s[b->solve].block) {
            double *a = &b->Ab[x * NJAC];
            for (int r = 0; r < NV; ++r) a[r * 5 + r] *= v->relax;
            for (int r = 0; r < NV; ++r) a[r * 5 + r] += diagVolTime;
            memcpy(&b->Ainvb[x * NJAC], a, 8 * NJAC);
            mat_inverse(&b->Ainvb[x * NJAC]);
            if (b->Wt) {
              double *at = &b->Abt[x * 4];
              at[0] *= v->relax;
              at[3] *= v->relax;
              at[0] += diagVolTime;
              at[3] += diagVolTime;
              memcpy(&b->Ainvbt[x * 4], at, 8 * 4);
              mat_inverse2(&b->Ainvbt[x * 4]);
            }
            continue;
          }
          b->A[x] *= v->relax;
          b->A[x] += diagVolTime;
          b->Ainv[x] = 1.0 / b->A[x];
          if (b->Wt) {
            b->At[x] *= v->relax;
            b->At[x] += diagVolTime;
            b->Ainvt[x] = 1.0 / b->At[x];
          }
        }
  }
}

/* off-diagonal sum of one cell: procBlock::ImplicitLower (forward) or
 * ImplicitUpper (backward), src/procBlock.cpp:1056,1106 */
static void offdiag_sum(const orc_case *c, const oblock *b, int64_t x, int lower,
                        double *acc) {
  const gas_t *g = &c->s[b->solve].gas;
  const int64_t st[3] = {1, b->NI, (int64_t)b->NI * b->NJ};
  for (int v = 0; v < NV + 2; ++v) acc[v] = 0.0;
  /* padded (i,j,k) of x */
  const int64_t ii = x % b->NI, jj = (x / b->NI) % b->NJ, kk = x / ((int64_t)b->NI * b->NJ);
  for (int d = 0; d < 3; ++d) {
    if (!(b->mask[x] & (1u << (2 * d + (lower ? 0 : 1))))) continue;
    const int64_t nb = lower ? x - st[d] : x + st[d];
    const int fi = (int)ii - b->ng + (!lower && d == 0);
    const int fj = (int)jj - b->ng + (!lower && d == 1);
    const int fk = (int)kk - b->ng + (!lower && d == 2);
    double n[3], mag, o[NV];
    face_normal(b, d, face_idx(b, d, fi, fj, fk), n, &mag);
    double vsr = 0.0, dist = 0.0;
    const osolve *sv = &c->s[b->solve];
    const double *wn = &b->W[nb * NV];
    if (sv->viscous) {
      /* ProjC2CDist (src/procBlock.cpp:6316): centre of the cell above the
       * face minus the one below, along the face normal */
      const int64_t up = lower ? x : nb, lo = lower ? nb : x;
      const double dc[3] = {b->center[up] - b->center[lo],
                            b->center[b->nc + up] - b->center[b->nc + lo],
                            b->center[2 * b->nc + up] - b->center[2 * b->nc + lo]};
      dist = dc[0] * n[0] + dc[1] * n[1] + dc[2] * n[2];
      vsr = mag / dist * visc_max_term(wn, g) *
            visc_term(b->mu[nb], sv->rans ? b->mutc[nb] : 0.0, &sv->v, g);
    }
    if (sv->block) {
      /* RusanovBlockOffDiagonal (src/fluxJacobian.cpp:164) */
      double J[NJAC];
      rusanov_jac(wn, g, n, mag, lower, J);
      if (sv->viscous) {
        double Tj[NJAC];
        tsl_jac(wn, b->mu[nb], sv->rans ? b->mutc[nb] : 0.0, g, &sv->v, n, mag, dist, lower,
                &b->vg[nb * 9], Tj);
        for (int e = 0; e < NJAC; ++e) J[e] = lower ? J[e] - Tj[e] : J[e] + Tj[e];
      }
      mat_vec(J, &b->dU[nb * NV], o);
    } else {
      scalar_offdiag(wn, &b->dU[nb * NV], g, n, mag, lower, vsr, o);
    }
    for (int v = 0; v < NV; ++v) acc[v] += o[v];
    if (sv->rans) {
      /* turbulence rows: the turbulence face radius (scalar) or the 2x2
       * Rusanov and viscous Jacobians (block) times the update */
      const double *dut = &b->dUt[nb * 2];
      const double scale = sv->v.visc_scale;
      double ot[2];
      if (sv->block) {
        double Jt[4];
        turb_rusanov_jac(wn, n, mag, lower, Jt);
        if (sv->viscous) {
          double Tv[4];
          turb_visc_jac(sv->wilcox, wn, &b->Wt[nb * 2], mag, b->mu[nb], b->mutc[nb], b->f1c[nb],
                        dist, scale, lower ? -1.0 : 1.0, Tv);
          for (int e = 0; e < 4; ++e) Jt[e] = lower ? Jt[e] - Tv[e] : Jt[e] + Tv[e];
        }
        mat_vec2(Jt, dut, ot);
      } else {
        const double srt = turb_face_sr(sv->wilcox, wn, &b->Wt[nb * 2], n, mag, b->mu[nb],
                                        b->mutc[nb], b->f1c[nb], dist, scale, lower,
                                        sv->viscous);
        for (int q = 0; q < 2; ++q) ot[q] = lower ? 0.0 + dut[q] * srt : 0.0 - dut[q] * srt;
      }
      for (int q = 0; q < 2; ++q) acc[NV + q] += ot[q];
    }
  }
}

/* SwapImplicitUpdate (src/utility.cpp:400) */
static void swap_du(orc_case *c) {
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    for (int o = 0; o < b->nops; ++o) {
      const ath_ghost_op *op = &b->ops[o];
      if (op->type != ATH_BC_PERIODIC && op->type != ATH_BC_INTERBLOCK) continue;
      memcpy(&b->dU[op->dst * NV], &c->b[op->src_block].dU[op->src * NV], 8 * NV);
      if (b->dUt)
        memcpy(&b->dUt[op->dst * 2], &c->b[op->src_block].dUt[op->src * 2], 8 * 2);
    }
  }
}

/* update of cell x as 7 values (flow, then k and omega when present) */
static void get_du(const oblock *b, int64_t x, double *u) {
  memcpy(u, &b->dU[x * NV], 8 * NV);
  u[NV] = b->dUt ? b->dUt[x * 2] : 0.0;
  u[NV + 1] = b->dUt ? b->dUt[x * 2 + 1] : 0.0;
}
static void set_du(oblock *b, int64_t x, const double *u) {
  memcpy(&b->dU[x * NV], u, 8 * NV);
  if (b->dUt) memcpy(&b->dUt[x * 2], u + NV, 8 * 2);
}
static void get_rhs(const orc_case *c, const oblock *b, int64_t x, double *r) {
  (void)c;
  memcpy(r, &b->R[x * NV], 8 * NV);
  r[NV] = b->Rt ? b->Rt[x * 2] : 0.0;
  r[NV + 1] = b->Rt ? b->Rt[x * 2 + 1] : 0.0;
}

/* right-hand side b of the linear system per equation: -R/theta +
 * SolDeltaNm1 - SolDeltaMmN (src/linearSolver.cpp:350-352, procBlock::
 * SolDeltaNm1 / SolDeltaMmN src/procBlock.cpp:1015-1034): the change since
 * time n times V(1+zeta)/(dt theta), and for bdf2 the change from n-1 to n
 * times V zeta/(dt theta); without time levels (one nonlinear iteration of
 * a one-level scheme) both are zero */
static void rhs_b(const orc_case *c, const oblock *b, int64_t x, double *bb) {
  const ath_solve_view *v = &c->s[b->solve].v;
  const double thetaInv = 1.0 / v->theta;
  double r[NV + 2];
  get_rhs(c, b, x, r);
  const int unsteady = v->multilevel || v->nl_iters > 1;
  if (!unsteady) {
    for (int q = 0; q < NV + 2; ++q) bb[q] = -thetaInv * r[q] + 0.0 + 0.0 - 0.0;
    return;
  }
  double cn[7];
  prim_to_cons(&b->W[x * NV], &c->s[b->solve].gas, cn);
  cn[5] = b->Wt ? b->W[x * NV] * b->Wt[x * 2] : 0.0;
  cn[6] = b->Wt ? b->W[x * NV] * b->Wt[x * 2 + 1] : 0.0;
  const double coeffN = (b->vol[x] * (1.0 + v->zeta)) / (b->dt[x] * v->theta);
  const double coeffNm1 = (b->vol[x] * v->zeta) / (b->dt[x] * v->theta);
  for (int q = 0; q < NV + 2; ++q) {
    const double dMmN = coeffN * (cn[q] - b->Un[x * 7 + q]);
    const double dNm1 = v->multilevel ? coeffNm1 * (b->Un[x * 7 + q] - b->Unm1[x * 7 + q]) : 0.0;
    bb[q] = -thetaInv * r[q] + dNm1 - dMmN;
  }
}

/* b with the multigrid forcing f as the LU-SGS sweeps form it (src/
 * linearSolver.cpp:350-352, 407-409): -R/theta + f + SolDeltaNm1 -
 * SolDeltaMmN */
static void rhs_bf(const orc_case *c, const oblock *b, int64_t x, double *bb) {
  const ath_solve_view *v = &c->s[b->solve].v;
  const int unsteady = v->multilevel || v->nl_iters > 1;
  if (!b->F || unsteady) {
    rhs_b(c, b, x, bb);
    return;
  }
  const double thetaInv = 1.0 / v->theta;
  double r[NV + 2];
  get_rhs(c, b, x, r);
  for (int q = 0; q < NV + 2; ++q) {
    const double f = q < NV ? b->F[x * NV + q] : 0.0;
    bb[q] = -thetaInv * r[q] + f + 0.0 - 0.0;
  }
}
static double forcing_of(const oblock *b, int64_t x, int v) {
  return (b->F && v < NV) ? b->F[x * NV + v] : 0.0;
}

/* linearSolver::Residual / AXmB (src/linearSolver.cpp:58,92) and the L2 of
 * mgSolution::CycleAtLevel (src/mgSolution.cpp:196-206) with the second
 * normalisation of src/main.cpp:271: sqrt(sum(r^2)/padded_size/(cells*nv)),
 * r = f - (A x - (L x - U x) - b), f = 0 on the finest level; with
 * multigrid the per-cell r is kept for the restriction. */
static void matrix_residual(orc_case *c) {
  for (int s = 0; s < c->ns; ++s) {
    double sum = 0.0, padded = 0.0, cells = 0.0;
    const int nv = c->s[s].rans ? NV + 2 : NV;
    for (int bi = 0; bi < c->nb; ++bi) {
      oblock *b = &c->b[bi];
      if (b->solve != s) continue;
      const double thetaInv = 1.0 / c->s[s].v.theta;
      double bsum = 0.0; /* std::accumulate per block (src/mgSolution.cpp:199-203) */
      for (int k = 0; k < b->nk; ++k)
        for (int j = 0; j < b->nj; ++j)
          for (int i = 0; i < b->ni; ++i) {
            const int64_t x = cell_idx(b, i, j, k);
            double L[NV + 2], U[NV + 2], u[NV + 2], r[NV + 2], Ax[NV + 2];
            offdiag_sum(c, b, x, 1, L);
            offdiag_sum(c, b, x, 0, U);
            get_du(b, x, u);
            rhs_b(c, b, x, r);
            if (c->s[s].block) {
              mat_vec(&b->Ab[x * NJAC], u, Ax);
              if (b->Wt) mat_vec2(&b->Abt[x * 4], u + NV, Ax + NV);
            } else {
              for (int v = 0; v < NV; ++v) Ax[v] = u[v] * b->A[x];
              if (b->Wt)
                for (int v = 0; v < 2; ++v) Ax[NV + v] = u[NV + v] * b->At[x];
            }
            for (int v = 0; v < nv; ++v) {
              const double off = L[v] - U[v];
              const double bb = r[v];
              const double axmb = Ax[v] - off - bb;
              const double rr = forcing_of(b, x, v) - axmb;
              if (b->mr && v < NV) b->mr[x * NV + v] = rr;
              bsum += rr * rr;
            }
          }
      sum += bsum;
      padded += (double)b->nc * nv;
      cells += (double)b->ni * b->nj * b->nk;
    }
    c->mres[s] = sqrt((sum / padded) / (cells * nv));
  }
}

/* x = A^-1 v: scalar (orig * A^-1) or 5x5 block (ArrayMultiplication) */
static void apply_ainv(const orc_case *c, const oblock *b, int64_t x, const double *in,
                       double *out) {
  if (c->s[b->solve].block) {
    mat_vec(&b->Ainvb[x * NJAC], in, out);
    if (b->Wt) mat_vec2(&b->Ainvbt[x * 4], in + NV, out + NV);
  } else {
    for (int v = 0; v < NV; ++v) out[v] = in[v] * b->Ainv[x];
    if (b->Wt)
      for (int v = 0; v < 2; ++v) out[NV + v] = in[NV + v] * b->Ainvt[x];
  }
}

/* lusgs::Relax (src/linearSolver.cpp:430) with LUSGS_Forward :341 and
 * LUSGS_Backward :385: matrixSweeps sweeps; with more than one sweep the
 * update starts from A^-1 b (InitializeMatrixUpdate :111) and every sweep
 * uses both triangles, otherwise from zero with one triangle per pass.
 * dplur::Relax (:501) with DPLUR (:473): from A^-1 b (MatrixRequires-
 * Initialization, src/input.cpp:1120), matrixSweeps Jacobi sweeps, each
 * after a ghost swap: x = A^-1 (b + L(x_old) - U(x_old)) */
/* the sweeps of one relaxation: matrixSweeps of each solve, or (half = 1)
 * the multigrid pre- and post-relaxation count max(matrixSweeps/2, 1)
 * (mgSolution::CycleAtLevel src/mgSolution.cpp:175) */
static int sweeps_of(const osolve *sv, int half) {
  if (!half) return sv->sweeps;
  return sv->sweeps / 2 > 1 ? sv->sweeps / 2 : 1;
}

/* linearSolver::InitializeMatrixUpdate (src/linearSolver.cpp:111) */
static void relax_init(orc_case *c) {
  NTH
  PAR_BLOCKS
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const osolve *sv = &c->s[b->solve];
    const int nv = sv->rans ? NV + 2 : NV;
    if (sv->sweeps <= 1 && !sv->jacobi) {
      memset(b->dU, 0, 8 * NV * b->nc);
      if (b->dUt) memset(b->dUt, 0, 8 * 2 * b->nc);
      continue;
    }
    const double thetaInv = 1.0 / sv->v.theta;
    for (int k = 0; k < b->nk; ++k)
      for (int j = 0; j < b->nj; ++j)
        for (int i = 0; i < b->ni; ++i) {
          const int64_t x = cell_idx(b, i, j, k);
          double in[NV + 2], r[NV + 2], out[NV + 2];
          rhs_b(c, b, x, r);
          for (int v = 0; v < nv; ++v) in[v] = r[v];
          apply_ainv(c, b, x, in, out);
          set_du(b, x, out);
        }
  }
}

static void relax_sweeps(orc_case *c, int half) {
  NTH
  int maxsw = 0, maxj = 0;
  for (int s = 0; s < c->ns; ++s) {
    const int n = sweeps_of(&c->s[s], half);
    if (c->s[s].jacobi) maxj = n > maxj ? n : maxj;
    else maxsw = n > maxsw ? n : maxsw;
  }
  for (int sw = 0; sw < maxj; ++sw) {
    swap_du(c);
    PAR_BLOCKS
    for (int bi = 0; bi < c->nb; ++bi) {
      oblock *b = &c->b[bi];
      const osolve *sv = &c->s[b->solve];
      if (!sv->jacobi || sw >= sweeps_of(sv, half)) continue;
      const int nv = sv->rans ? NV + 2 : NV;
      const double thetaInv = 1.0 / sv->v.theta;
      /* new iterate beside the old one (ghosts keep the swapped values) */
      double *nu = (double *)dup_arr(b->dU, 8 * NV * b->nc);
      double *nut = b->dUt ? (double *)dup_arr(b->dUt, 8 * 2 * b->nc) : NULL;
      for (int k = 0; k < b->nk; ++k)
        for (int j = 0; j < b->nj; ++j)
          for (int i = 0; i < b->ni; ++i) {
            const int64_t x = cell_idx(b, i, j, k);
            double L[NV + 2], U[NV + 2], in[NV + 2], r[NV + 2], out[NV + 2];
            offdiag_sum(c, b, x, 1, L);
            offdiag_sum(c, b, x, 0, U);
            rhs_b(c, b, x, r);
            for (int v = 0; v < nv; ++v) {
              const double bb = r[v];
              in[v] = bb + forcing_of(b, x, v) + (L[v] - U[v]);
            }
            apply_ainv(c, b, x, in, out);
            memcpy(&nu[x * NV], out, 8 * NV);
            if (nut) memcpy(&nut[x * 2], out + NV, 8 * 2);
          }
      memcpy(b->dU, nu, 8 * NV * b->nc);
      if (nut) memcpy(b->dUt, nut, 8 * 2 * b->nc);
      free(nu);
      free(nut);
    }
  }
  for (int sw = 0; sw < maxsw; ++sw) {
    swap_du(c);
    PAR_BLOCKS
    for (int bi = 0; bi < c->nb; ++bi) {
      oblock *b = &c->b[bi];
      const osolve *sv = &c->s[b->solve];
      if (sv->jacobi || sw >= sweeps_of(sv, half)) continue;
      const int nv = sv->rans ? NV + 2 : NV;
      const int full = sw > 0 || sv->sweeps > 1;
      const double thetaInv = 1.0 / sv->v.theta;
      const int ncell = b->ni * b->nj * b->nk;
      for (int q = 0; q < ncell; ++q) {
        const int64_t x = b->plane_cells[q];
        double L[NV + 2], U[NV + 2], in[NV + 2], r[NV + 2], out[NV + 2];
        offdiag_sum(c, b, x, 1, L);
        if (full) {
          offdiag_sum(c, b, x, 0, U);
          for (int v = 0; v < nv; ++v) L[v] -= U[v];
        }
        rhs_bf(c, b, x, r);
        for (int v = 0; v < nv; ++v) {
          const double bb = r[v];
          in[v] = bb + L[v];
        }
        apply_ainv(c, b, x, in, out);
        set_du(b, x, out);
      }
    }
    swap_du(c);
    PAR_BLOCKS
    for (int bi = 0; bi < c->nb; ++bi) {
      oblock *b = &c->b[bi];
      const osolve *sv = &c->s[b->solve];
      if (sv->jacobi || sw >= sweeps_of(sv, half)) continue;
      const int nv = sv->rans ? NV + 2 : NV;
      const int full = sw > 0 || sv->sweeps > 1;
      const double thetaInv = 1.0 / sv->v.theta;
      const int ncell = b->ni * b->nj * b->nk;
      for (int q = ncell - 1; q >= 0; --q) {
        const int64_t x = b->plane_cells[q];
        double U[NV + 2], L[NV + 2], in[NV + 2], t[NV + 2], r[NV + 2], out[NV + 2];
        offdiag_sum(c, b, x, 0, U);
        if (full) {
          offdiag_sum(c, b, x, 1, L);
          rhs_bf(c, b, x, r);
          for (int v = 0; v < nv; ++v) {
            const double bb = r[v];
            in[v] = bb + L[v] - U[v];
          }
          apply_ainv(c, b, x, in, out);
          set_du(b, x, out);
        } else {
          double cur[NV + 2];
          apply_ainv(c, b, x, U, t);
          get_du(b, x, cur);
          for (int v = 0; v < nv; ++v) out[v] = cur[v] - t[v];
          set_du(b, x, out);
        }
      }
    }
  }
}

/* ---------------------------------------------------------- multigrid */
/* coarse cell (padded index) of fine physical cell number x of block b */
static int64_t mg_coarse_cell(const oblock *b, const oblock *cb, int64_t x) {
  const int cc = b->mg_cell[x];
  const int ci = cc % cb->ni, cj = (cc / cb->ni) % cb->nj, ck = cc / (cb->ni * cb->nj);
  return cell_idx(cb, ci, cj, ck);
}

/* BlockRestriction (include/procBlock.hpp:637,656): the coarse array is
 * zeroed (ghosts included), then every fine physical cell, in k, j, i
 * order, adds its value times its volume weight (weighted) or its value
 * (sum) to its coarse cell */
static void mg_restrict(orc_case *c, int what) {
  orc_case *cc = c->coarse;
  for (int bi = 0; bi < cc->nb; ++bi) {
    oblock *cb = &cc->b[bi];
    double *dst = what == 0 ? cb->W : what == 1 ? cb->dU : cb->F;
    memset(dst, 0, 8 * NV * cb->nc);
  }
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    oblock *cb = &cc->b[b->mg_coarse];
    const double *src = what == 0 ? b->W : what == 1 ? b->dU : b->mr;
    double *dst = what == 0 ? cb->W : what == 1 ? cb->dU : cb->F;
    int64_t x = 0;
    for (int k = 0; k < b->nk; ++k)
      for (int j = 0; j < b->nj; ++j)
        for (int i = 0; i < b->ni; ++i, ++x) {
          const int64_t f = cell_idx(b, i, j, k), q = mg_coarse_cell(b, cb, x);
          for (int v = 0; v < NV; ++v) {
            const double t = what == 2 ? src[f * NV + v] : b->mg_volfac[x] * src[f * NV + v];
            dst[q * NV + v] = dst[q * NV + v] + t;
          }
        }
  }
}

/* BlockProlongation (include/gridLevel.hpp:160): the coarse correction at
 * the coarse nodes (ConvertCellToNode without ghosts, include/utility.hpp:
 * 187: each cell, in k, j, i order, adds to its 8 nodes; corner nodes of
 * the block keep the sum, nodes on a block edge take half of it, all others
 * an eighth), interpolated trilinearly to every fine cell centre
 * (TrilinearInterp include/utility.hpp:357) and added to the fine update */
static double lin(double d0, double d1, double c) { return (1.0 - c) * d0 + c * d1; }
static void mg_prolong(orc_case *c) {
  orc_case *cc = c->coarse;
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const oblock *cb = &cc->b[b->mg_coarse];
    const int ni = cb->ni + 1, nj = cb->nj + 1, nk = cb->nk + 1;
    double *nd = (double *)calloc((size_t)ni * nj * nk * NV, sizeof(double));
#define NODE(i, j, k) (nd + (((size_t)(k) * nj + (j)) * ni + (i)) * NV)
    for (int k = 0; k < cb->nk; ++k)
      for (int j = 0; j < cb->nj; ++j)
        for (int i = 0; i < cb->ni; ++i) {
          const double *u = &cb->dU[cell_idx(cb, i, j, k) * NV];
          double *t[8] = {NODE(i, j, k),         NODE(i, j + 1, k),
                          NODE(i, j + 1, k + 1), NODE(i, j, k + 1),
                          NODE(i + 1, j, k),     NODE(i + 1, j + 1, k),
                          NODE(i + 1, j + 1, k + 1), NODE(i + 1, j, k + 1)};
          for (int n = 0; n < 8; ++n)
            for (int v = 0; v < NV; ++v) t[n][v] += u[v];
        }
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j < nj; ++j)
        for (int i = 0; i < ni; ++i) {
          const int ei = i == 0 || i == ni - 1, ej = j == 0 || j == nj - 1,
                    ek = k == 0 || k == nk - 1;
          const double f = (ei && ej && ek) ? 1.0 : (ei + ej + ek == 2) ? 1.0 / 2.0 : 1.0 / 8.0;
          for (int v = 0; v < NV; ++v) NODE(i, j, k)[v] *= f;
        }
    int64_t x = 0;
    for (int k = 0; k < b->nk; ++k)
      for (int j = 0; j < b->nj; ++j)
        for (int i = 0; i < b->ni; ++i, ++x) {
          const int cc = b->mg_cell[x];
          const int ci = cc % cb->ni, cj = (cc / cb->ni) % cb->nj, ck = cc / (cb->ni * cb->nj);
          const double *co = &b->mg_coef[7 * x];
          const double *d[8] = {NODE(ci, cj, ck),         NODE(ci + 1, cj, ck),
                                NODE(ci, cj + 1, ck),     NODE(ci + 1, cj + 1, ck),
                                NODE(ci, cj, ck + 1),     NODE(ci + 1, cj, ck + 1),
                                NODE(ci, cj + 1, ck + 1), NODE(ci + 1, cj + 1, ck + 1)};
          const int64_t f = cell_idx(b, i, j, k);
          for (int v = 0; v < NV; ++v) {
            const double d04 = lin(d[0][v], d[4][v], co[0]);
            const double d15 = lin(d[1][v], d[5][v], co[1]);
            const double d26 = lin(d[2][v], d[6][v], co[2]);
            const double d37 = lin(d[3][v], d[7][v], co[3]);
            const double d0415 = lin(d04, d15, co[4]);
            const double d2637 = lin(d26, d37, co[5]);
            b->dU[f * NV + v] = b->dU[f * NV + v] + lin(d0415, d2637, co[6]);
          }
        }
#undef NODE
    free(nd);
  }
}

/* A x - (L x - U x) - b per physical cell of every block of level c
 * (linearSolver::AXmB src/linearSolver.cpp:58), added to the restricted
 * matrix residual already in F: the coarse level's forcing (gridLevel::
 * Restriction src/gridLevel.cpp:571-589) */
static void mg_forcing(orc_case *c) {
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const int s = b->solve;
    for (int k = 0; k < b->nk; ++k)
      for (int j = 0; j < b->nj; ++j)
        for (int i = 0; i < b->ni; ++i) {
          const int64_t x = cell_idx(b, i, j, k);
          double L[NV + 2], U[NV + 2], u[NV + 2], r[NV + 2], Ax[NV + 2];
          offdiag_sum(c, b, x, 1, L);
          offdiag_sum(c, b, x, 0, U);
          get_du(b, x, u);
          rhs_b(c, b, x, r);
          if (c->s[s].block) {
            mat_vec(&b->Ab[x * NJAC], u, Ax);
          } else {
            for (int v = 0; v < NV; ++v) Ax[v] = u[v] * b->A[x];
          }
          for (int v = 0; v < NV; ++v) {
            const double off = L[v] - U[v];
            const double axmb = Ax[v] - off - r[v];
            b->F[x * NV + v] = axmb + b->F[x * NV + v];
          }
        }
  }
}

/* mgSolution::CycleAtLevel (src/mgSolution.cpp:160-207) from level c:
 * relaxation (the coarsest level: matrixSweeps; the others max(matrixSweeps
 * / 2, 1) before and after the coarse-grid correction), each ending with a
 * ghost swap and the matrix residual f - (A x - b) */
static void mg_cycle(orc_case *c) {
  orc_case *cc = c->coarse;
  if (!cc) {
    relax_sweeps(c, 0);
    swap_du(c);
    matrix_residual(c);
    return;
  }
  relax_sweeps(c, 1);
  swap_du(c);
  matrix_residual(c);
  /* gridLevel::Restriction (src/gridLevel.cpp:538): the state, then the
   * coarse residual, time step and diagonal from it, the update, and the
   * forcing */
  mg_restrict(c, 0);
  cc->iter = c->iter;
  cc->mg_visits += 1;
  orc_fill_ghosts(cc);
  orc_residual(cc);
  orc_timestep(cc);
  orc_diag_invert(cc);
  mg_restrict(c, 1);
  swap_du(cc);
  mg_restrict(c, 2);
  mg_forcing(cc);
  size_t tot = 0;
  for (int bi = 0; bi < cc->nb; ++bi) tot += (size_t)cc->b[bi].nc * NV;
  double *du0 = (double *)malloc(8 * (tot ? tot : 1));
  size_t o = 0;
  for (int bi = 0; bi < cc->nb; ++bi) {
    memcpy(du0 + o, cc->b[bi].dU, 8 * NV * cc->b[bi].nc);
    o += (size_t)cc->b[bi].nc * NV;
  }
  for (int n = 0; n < c->mg_cycle; ++n) mg_cycle(cc);
  o = 0;
  for (int bi = 0; bi < cc->nb; ++bi) {
    oblock *cb = &cc->b[bi];
    for (int64_t q = 0; q < cb->nc * NV; ++q) cb->dU[q] -= du0[o + q];
    o += (size_t)cb->nc * NV;
  }
  free(du0);
  mg_prolong(c);
  relax_sweeps(c, 1);
  swap_du(c);
  matrix_residual(c);
}

/* Links level c to its next coarser level: maps[b] is the transfer of
 * block b of c (ath_setup_mg_map) */
void orc_set_coarse(orc_case *c, orc_case *coarse, int cycle, const ath_mg_map *maps) {
  c->coarse = coarse;
  c->mg_cycle = cycle;
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const int64_t n = maps[bi].ncells;
    b->mg_coarse = maps[bi].coarse_block;
    b->mg_cell = (int32_t *)dup_arr(maps[bi].coarse_cell, 4 * n);
    b->mg_volfac = (double *)dup_arr(maps[bi].volfac, 8 * n);
    b->mg_coef = (double *)dup_arr(maps[bi].coef, 8 * 7 * n);
    if (!b->mr) b->mr = (double *)calloc((size_t)b->nc * NV, sizeof(double));
  }
  for (int bi = 0; bi < coarse->nb; ++bi) {
    oblock *cb = &coarse->b[bi];
    if (!cb->F) cb->F = (double *)calloc((size_t)cb->nc * NV, sizeof(double));
    if (!cb->mr) cb->mr = (double *)calloc((size_t)cb->nc * NV, sizeof(double));
  }
}

void orc_relax(orc_case *c) {
  relax_init(c);
  if (c->coarse) {
    for (orc_case *l = c->coarse; l; l = l->coarse) l->mg_visits = 0;
    mg_cycle(c);
    return;
  }
  relax_sweeps(c, 0);
  swap_du(c);
  if (c->matrix_resid) matrix_residual(c);
}

/* procBlock::UpdateBlock / ImplicitTimeAdvance (src/procBlock.cpp:826,902)
 * and the L2 sums of src/main.cpp:254-268 */
int orc_update(orc_case *c, double *l2_out, double *linf_out) {
  int bad = 0;
  double *l2 = (double *)calloc((size_t)c->ns * (NV + 2), sizeof(double));
  double *linf = (double *)calloc((size_t)c->ns, sizeof(double));
  NTH
  PAR_BLOCKS
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const gas_t *g = &c->s[b->solve].gas;
    for (int k = 0; k < b->nk; ++k)
      for (int j = 0; j < b->nj; ++j)
        for (int i = 0; i < b->ni; ++i) {
          const int64_t x = cell_idx(b, i, j, k);
          double w[NV];
          const double rho0 = b->W[x * NV];
          update_with_cons(&b->W[x * NV], g, &b->dU[x * NV], w);
          if (!(w[0] > 0.0) || !(w[4] > 0.0) || !isfinite(w[1]) || !isfinite(w[2]) ||
              !isfinite(w[3]))
            bad = 1;
          memcpy(&b->W[x * NV], w, sizeof(w));
          if (b->Wt) {
            /* conserved rho k, rho omega updated, divided by the new density
             * and held above the floors (primitive(conserved), LimitTurb) */
            const double rho1 = rho0 + b->dU[x * NV];
            for (int q = 0; q < 2; ++q) {
              const double cq = rho0 * b->Wt[x * 2 + q] + b->dUt[x * 2 + q];
              b->Wt[x * 2 + q] = cmax(cq / rho1, TURB_MIN);
            }
          }
        }
  }
  /* sequential norm sums in the reference's block, k, j, i order */
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    for (int k = 0; k < b->nk; ++k)
      for (int j = 0; j < b->nj; ++j)
        for (int i = 0; i < b->ni; ++i) {
          const int64_t x = cell_idx(b, i, j, k);
          double rr[NV + 2];
          get_rhs(c, b, x, rr);
          const int nv = b->Wt ? NV + 2 : NV;
          for (int v = 0; v < nv; ++v) {
            const double r = rr[v];
            l2[b->solve * (NV + 2) + v] += r * r;
            if (r > linf[b->solve]) linf[b->solve] = r;
          }
        }
  }
  for (int q = 0; q < c->ns * (NV + 2); ++q)
    if (l2_out) l2_out[q] = sqrt(l2[q]);
  for (int s = 0; s < c->ns; ++s)
    if (linf_out) linf_out[s] = linf[s];
  free(l2);
  free(linf);
  /* gridLevel::UpdateBlocks (src/gridLevel.cpp:418): time n becomes n-1
   * after the last nonlinear iteration of a multilevel step */
  for (int bi = 0; bi < c->nb; ++bi) {
    oblock *b = &c->b[bi];
    const ath_solve_view *v = &c->s[b->solve].v;
    const int nl = v->nl_iters > 0 ? v->nl_iters : 1;
    if (v->multilevel && c->iter % nl == nl - 1) memcpy(b->Unm1, b->Un, 8 * 7 * b->nc);
  }
  c->iter += 1;
  return bad ? ATH_ERR_NONPHYSICAL : 0;
}

int orc_iterate(orc_case *c, int n, double *l2_out) {
  int rc = 0;
  for (int it = 0; it < n; ++it) {
    orc_fill_ghosts(c);
    orc_residual(c);
    orc_timestep(c);
    orc_diag_invert(c);
    orc_relax(c);
    const int r = orc_update(c, l2_out ? l2_out + (size_t)it * c->ns * (NV + 2) : NULL, NULL);
    if (r) rc = r;
  }
  return rc;
}

int orc_get_field(orc_case *c, int block, int field, double *out) {
  if (block < 0 || block >= c->nb) return ATH_ERR_ARG;
  oblock *b = &c->b[block];
  const int nv = b->Wt ? NV + 2 : NV;
  size_t q = 0;
  if (field == ATH_FIELD_STATE_GHOSTS) {
    for (int64_t x = 0; x < b->nc; ++x) {
      memcpy(out + nv * x, &b->W[x * NV], 8 * NV);
      if (b->Wt) memcpy(out + nv * x + NV, &b->Wt[x * 2], 8 * 2);
    }
    return 0;
  }
  for (int k = 0; k < b->nk; ++k)
    for (int j = 0; j < b->nj; ++j)
      for (int i = 0; i < b->ni; ++i) {
        const int64_t x = cell_idx(b, i, j, k);
        double u[NV + 2];
        switch (field) {
          case ATH_FIELD_STATE:
            memcpy(out + nv * q, &b->W[x * NV], 8 * NV);
            if (b->Wt) memcpy(out + nv * q + NV, &b->Wt[x * 2], 8 * 2);
            break;
          case ATH_FIELD_RESID:
            get_rhs(c, b, x, u);
            memcpy(out + nv * q, u, 8 * nv);
            break;
          case ATH_FIELD_DU:
            get_du(b, x, u);
            memcpy(out + nv * q, u, 8 * nv);
            break;
          case ATH_FIELD_DT: out[q] = b->dt[x]; break;
          case ATH_FIELD_SPECRAD:
            out[2 * q] = b->lam[x];
            out[2 * q + 1] = b->lamt ? b->lamt[x] : 0.0;
            break;
          case ATH_FIELD_AINV: out[q] = b->Ainv[x]; break;
          case ATH_FIELD_AUX: {
            /* temperature and viscosity of the last auxiliary update (Euler:
             * temperature of the current state), eddy viscosity, F1, F2 */
            const osolve *sv = &c->s[b->solve];
            out[5 * q] = sv->viscous ? b->T[x] : temp_of(&b->W[x * NV], &sv->gas);
            out[5 * q + 1] = sv->viscous ? b->mu[x] : 0.0;
            out[5 * q + 2] = b->mutc ? b->mutc[x] : 0.0;
            out[5 * q + 3] = b->f1c ? b->f1c[x] : 0.0;
            out[5 * q + 4] = b->f2c ? b->f2c[x] : 0.0;
            break;
          }
          case ATH_FIELD_VELGRAD:
            if (!b->vg) return ATH_ERR_UNSUPPORTED;
            memcpy(out + 9 * q, &b->vg[x * 9], 8 * 9);
            break;
          case ATH_FIELD_WALLDIST: out[q] = b->wd ? b->wd[x] : 1.0e10; break;
          case ATH_FIELD_GRADS:
            if (!b->og) return ATH_ERR_UNSUPPORTED;
            memcpy(out + 24 * q, &b->og[x * 24], 8 * 24);
            break;
          case ATH_FIELD_CONS_N:
          case ATH_FIELD_CONS_NM1: {
            const ath_solve_view *v = &c->s[b->solve].v;
            const int nm1 = field == ATH_FIELD_CONS_NM1;
            if (nm1 ? !v->multilevel : !(v->multilevel || v->nl_iters > 1))
              return ATH_ERR_UNSUPPORTED;
            memcpy(out + nv * q, nm1 ? &b->Unm1[x * 7] : &b->Un[x * 7], 8 * nv);
            break;
          }
          default: return ATH_ERR_ARG;
        }
        ++q;
      }
  return 0;
}

/* Time n-1 of a bdf2 solve's block from a restart (GetSolNm1FromRestart,
 * src/procBlock.cpp:6418; nv conserved values per cell), or, with cons
 * NULL, the current state into both levels (AssignSolToTimeN and
 * AssignSolToTimeNm1 of a one-level restart, src/output.cpp:892).  The
 * solve then keeps time n-1 through its first time step. */
int orc_set_state_nm1(orc_case *c, int block, const double *cons) {
  if (block < 0 || block >= c->nb) return ATH_ERR_ARG;
  oblock *b = &c->b[block];
  osolve *sv = &c->s[b->solve];
  if (!sv->v.multilevel) return ATH_ERR_UNSUPPORTED;
  const int nv = b->Wt ? NV + 2 : NV;
  size_t q = 0;
  for (int k = 0; k < b->nk; ++k)
    for (int j = 0; j < b->nj; ++j)
      for (int i = 0; i < b->ni; ++i) {
        const int64_t x = cell_idx(b, i, j, k);
        double *um = &b->Unm1[x * 7];
        if (cons) {
          for (int v = 0; v < 7; ++v) um[v] = v < nv ? cons[nv * q + v] : 0.0;
        } else {
          double *un = &b->Un[x * 7];
          prim_to_cons(&b->W[x * NV], &sv->gas, un);
          un[5] = b->Wt ? b->W[x * NV] * b->Wt[x * 2] : 0.0;
          un[6] = b->Wt ? b->W[x * NV] * b->Wt[x * 2 + 1] : 0.0;
          memcpy(um, un, 8 * 7);
        }
        ++q;
      }
  sv->nm1_given = 1;
  return 0;
}

int orc_set_state(orc_case *c, int block, const double *prim) {
  if (block < 0 || block >= c->nb) return ATH_ERR_ARG;
  oblock *b = &c->b[block];
  const int nv = b->Wt ? NV + 2 : NV;
  size_t q = 0;
  for (int k = 0; k < b->nk; ++k)
    for (int j = 0; j < b->nj; ++j)
      for (int i = 0; i < b->ni; ++i) {
        const int64_t x = cell_idx(b, i, j, k);
        memcpy(&b->W[x * NV], prim + nv * q, 8 * NV);
        if (b->Wt) memcpy(&b->Wt[x * 2], prim + nv * q + NV, 8 * 2);
        /* temperature and viscosity of the loaded state, as after
         * ReadRestart (gridLevel::AuxillaryAndWidths src/gridLevel.cpp:433);
         * the lagged eddy viscosity stays that of the initial condition */
        if (c->s[b->solve].viscous) {
          b->T[x] = temp_of(&b->W[x * NV], &c->s[b->solve].gas);
          b->mu[x] = visc_of(b->T[x], &c->s[b->solve].v);
        }
        ++q;
      }
  return 0;
}
