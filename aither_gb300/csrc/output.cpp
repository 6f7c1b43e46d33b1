// Output files of resident solutions in the reference's formats (C ABI,
// include/aither_gb300.h):
//   * restart files, WriteRestart / ReadRestart / ReadSolFromRestart
//     (src/output.cpp:591,756,1177): dimensional primitives per physical
//     cell, one time level;
//   * Plot3D cell-centre function files, WriteFunFile (src/output.cpp:209),
//     the cell-centre grid, WriteCellCenter (:57), and the Paraview meta file,
//     WriteMeta (:903), with WriteBlockDims (include/output.hpp:109);
//   * the residual history, PrintHeaders / PrintResiduals (:1007,1028).
// Derived output variables follow the reference's evaluation order so the
// files match its own byte for byte on the same state.  Host code only: the
// batch-level entry points gather fields through ath_batch_get_field.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "aither_gb300.h"
#include "errors.hpp"
#include "setup.hpp"

namespace ath {
namespace {

const Solve &SolveOf(const ath_setup *st, int solve) {
  if (!st) throw Error(ATH_ERR_ARG, "null setup");
  if (solve < 0 || solve >= (int)st->s.solves.size()) throw Error(ATH_ERR_ARG, "solve index");
  return st->s.solves[solve];
}

size_t Cells(const Block &b) { return (size_t)b.ni * b.nj * b.nk; }

std::ofstream OpenOut(const char *path, bool binary) {
  if (!path) throw Error(ATH_ERR_ARG, "null path");
  std::ofstream f(path, binary ? std::ios::out | std::ios::binary : std::ios::out);
  if (!f) throw Error(ATH_ERR_IO, std::string("cannot open ") + path);
  return f;
}

template <typename V>
void Put(std::ofstream &f, const V &v) {
  f.write(reinterpret_cast<const char *>(&v), sizeof(v));
}
template <typename V>
void Get(std::ifstream &f, V &v) {
  f.read(reinterpret_cast<char *>(&v), sizeof(v));
  if (!f) throw Error(ATH_ERR_IO, "restart file ends early");
}

// WriteBlockDims (include/output.hpp:109): block count, then per block the
// physical cell counts and, when numVars > 0, the variable count
void BlockDims(std::ofstream &f, const Setup &s, const Solve &sv, int nvars) {
  Put(f, (int)sv.blocks.size());
  for (int bi : sv.blocks) {
    const Block &b = s.blocks[bi];
    Put(f, b.ni);
    Put(f, b.nj);
    Put(f, b.nk);
    if (nvars > 0) Put(f, nvars);
  }
}

std::vector<std::string> SplitVars(const char *vars, const Solve &sv) {
  if (!vars || !*vars) return sv.output_vars;
  std::set<std::string> out;  // the reference keeps a sorted set
  std::stringstream ss(vars);
  std::string tok;
  while (std::getline(ss, tok, ',')) {
    size_t a = tok.find_first_not_of(" \t"), z = tok.find_last_not_of(" \t");
    if (a != std::string::npos) out.insert(tok.substr(a, z - a + 1));
  }
  return std::vector<std::string>(out.begin(), out.end());
}

// Dimensional scales of one solve (input::RRef/ARef/LRef/TRef,
// transport::MuRef)
struct Scales {
  double r, a, l, t, mu;
};
Scales ScalesOf(const Solve &sv) {
  return {sv.phys.r_ref, sv.phys.a_ref, sv.phys.l_ref, sv.phys.t_ref, sv.phys.mu_ref};
}

// One output variable of one physical cell (WriteFunFile,
// src/output.cpp:232-425).  Thermodynamics of one calorically perfect
// species: mass and mole fraction rho/rho, Cp = R(n+1), Cv = R n
// (include/thermodynamic.hpp:102-115), temperature p / (rho R)
// (src/eos.cpp:100).
double FunValue(const std::string &var, const Solve &sv, int pos, const ath_block_fields &fl,
                size_t q, int nv) {
  const Scales sc = ScalesOf(sv);
  const ath_solve_view &ph = sv.phys;
  auto need = [&](const double *p, const char *what) {
    if (!p) throw Error(ATH_ERR_ARG, std::string("output variable ") + var + " needs " + what);
    return p;
  };
  const double *w = need(fl.prim, "the state") + q * nv;
  const double rho = w[0], u = w[1], v = w[2], wz = w[3], p = w[4];
  const double R = ph.gas_r, n = ph.gas_n, hf = ph.gas_hf;
  const double mf = rho / rho;
  auto cp_of = [&](double) { return 0.0 + mf * (R * (n + 1.0)); };
  auto cv_of = [&](double) { return 0.0 + mf * (R * n); };
  auto temp_state = [&]() { return p / (0.0 + rho * R); };
  auto velmag = [&]() { return std::sqrt(u * u + v * v + wz * wz); };
  auto sos = [&]() {
    const double t = temp_state();
    return std::sqrt(cp_of(t) / cv_of(t) * p / rho);
  };
  auto aux = [&](int k) { return need(fl.aux, "auxiliary fields")[q * 5 + k]; };
  auto vgrad = [&](int k) {
    if (fl.grads) return fl.grads[q * 24 + k];
    return need(fl.velgrad, "velocity gradients")[q * 9 + k];
  };
  auto grad = [&](int k) { return need(fl.grads, "the cell gradients")[q * 24 + k]; };
  auto res = [&](int k) {
    if (k >= nv) throw Error(ATH_ERR_ARG, "output variable " + var + " needs SST");
    return need(fl.resid, "the residual")[q * nv + k];
  };
  auto turb = [&](int k) {
    if (nv < 7) throw Error(ATH_ERR_ARG, "output variable " + var + " needs SST");
    return w[5 + k];
  };
  if (var == "density") return rho * sc.r;
  if (var == "vel_x") return u * sc.a;
  if (var == "vel_y") return v * sc.a;
  if (var == "vel_z") return wz * sc.a;
  if (var == "pressure") return p * (sc.r * sc.a * sc.a);
  if (var == "mach") return velmag() / sos();
  if (var == "sos") return sos() * sc.a;
  if (var == "dt") return need(fl.dt, "the time step")[q] / (sc.a * sc.l);
  if (var == "temperature") return aux(0) * sc.t;
  // SpecEnergy / SpecEnthalpy (src/thermodynamic.cpp): mass-fraction sums
  // of the species hf + Cv t and hf + Cp t; plus 0.5 |v|^2 (src/eos.cpp:70,80)
  if (var == "energy") {
    const double t = temp_state(), vm = velmag();
    const double e = 0.0 + mf * (hf + (R * n) * t);
    return (e + 0.5 * vm * vm) * (sc.a * sc.a);
  }
  if (var == "enthalpy") {
    const double t = temp_state(), vm = velmag();
    const double h = 0.0 + mf * (hf + (R * (n + 1.0)) * t);
    return (h + 0.5 * vm * vm) * (sc.a * sc.a);
  }
  if (var == "cp") return cp_of(aux(0)) * (sc.a * sc.a / sc.t);
  if (var == "cv") return cv_of(aux(0)) * (sc.a * sc.a / sc.t);
  if (var == "rank") return 0.0;
  if (var == "globalPosition") return (double)pos;
  if (var == "viscosityRatio") return nv == 7 ? aux(2) / aux(1) : 0.0;
  if (var == "turbulentViscosity") return aux(2) * sc.mu;
  if (var == "viscosity") return aux(1) * sc.mu;
  if (var == "tke") return turb(0) * (sc.a * sc.a);
  if (var == "sdr") return turb(1) * (sc.a * sc.a * sc.r / sc.mu);
  if (var == "f1") return aux(3);
  if (var == "f2") return aux(4);
  if (var == "wallDistance") return need(fl.wall_dist, "the wall distance")[q] * sc.l;
  static const char *vg_names[9] = {"velGrad_ux", "velGrad_vx", "velGrad_wx",
                                    "velGrad_uy", "velGrad_vy", "velGrad_wy",
                                    "velGrad_uz", "velGrad_vz", "velGrad_wz"};
  for (int k = 0; k < 9; ++k)
    if (var == vg_names[k]) return vgrad(k) * (sc.a / sc.l);
  // scalar gradients and their dimensional scales (src/output.cpp:336-395)
  static const char *axes = "xyz";
  for (int r = 0; r < 3; ++r) {
    const std::string ax(1, axes[r]);
    if (var == "tempGrad_" + ax) return grad(9 + r) * (sc.t / sc.l);
    if (var == "densityGrad_" + ax) return grad(12 + r) * (sc.r / sc.l);
    if (var == "pressGrad_" + ax) return grad(15 + r) * (sc.r * sc.a * sc.a / sc.l);
    if (var == "tkeGrad_" + ax) {
      if (nv < 7) throw Error(ATH_ERR_ARG, "output variable " + var + " needs SST");
      return grad(18 + r) * (sc.a * sc.a / sc.l);
    }
    if (var == "omegaGrad_" + ax) {
      if (nv < 7) throw Error(ATH_ERR_ARG, "output variable " + var + " needs SST");
      return grad(21 + r) * (sc.a * sc.a * sc.r / (sc.mu * sc.l));
    }
  }
  if (var == "resid_mass") return res(0) * (sc.r * sc.a * sc.l * sc.l);
  if (var == "resid_mom_x") return res(1) * (sc.r * sc.a * sc.a * sc.l * sc.l);
  if (var == "resid_mom_y") return res(2) * (sc.r * sc.a * sc.a * sc.l * sc.l);
  if (var == "resid_mom_z") return res(3) * (sc.r * sc.a * sc.a * sc.l * sc.l);
  if (var == "resid_energy") return res(4) * (sc.r * std::pow(sc.a, 3.0) * sc.l * sc.l);
  if (var == "resid_tke") return res(5) * (sc.r * std::pow(sc.a, 3.0) * sc.l * sc.l);
  if (var == "resid_sdr")
    return res(6) * (sc.r * sc.r * std::pow(sc.a, 4.0) * sc.l * sc.l / sc.mu);
  if (var == "mf_" + sv.species) return mf;
  if (var == "vf_" + sv.species) {
    const double x = mf;  // one species: mole fraction x / (0 + x)
    return x / (0.0 + x);
  }
  throw Error(ATH_ERR_UNSUPPORTED, "output variable " + var + " is not supported");
}

void CheckFields(const Solve &sv, const ath_block_fields *fields) {
  if (!fields) throw Error(ATH_ERR_ARG, "null fields");
  for (size_t k = 0; k < sv.blocks.size(); ++k)
    if (!fields[k].prim) throw Error(ATH_ERR_ARG, "every block needs its state");
}

void WriteFunction(const Setup &s, const Solve &sv, const std::vector<std::string> &vars,
                   const ath_block_fields *fields, const char *path) {
  CheckFields(sv, fields);
  // evaluate everything before opening the file, so an unsupported
  // variable leaves no partial file
  std::vector<std::vector<double>> vals(sv.blocks.size());
  for (size_t k = 0; k < sv.blocks.size(); ++k) {
    const Block &b = s.blocks[sv.blocks[k]];
    const size_t m = Cells(b);
    vals[k].resize(vars.size() * m);
    for (size_t vi = 0; vi < vars.size(); ++vi)
      for (size_t q = 0; q < m; ++q)
        vals[k][vi * m + q] = FunValue(vars[vi], sv, (int)k, fields[k], q, b.nv);
  }
  auto f = OpenOut(path, true);
  BlockDims(f, s, sv, (int)vars.size());
  for (auto &blk : vals) f.write(reinterpret_cast<const char *>(blk.data()), blk.size() * 8);
  if (!f) throw Error(ATH_ERR_IO, std::string("write failed: ") + path);
}

// WriteRestart (src/output.cpp:591): the state, and for a bdf2 solve the
// conserved state of time n-1 as a second time level
void WriteRestart(const Setup &s, const Solve &sv, int iteration, const double *resid_first,
                  const ath_block_fields *fields, const char *path) {
  CheckFields(sv, fields);
  if (!resid_first) throw Error(ATH_ERR_ARG, "null residual normalisation");
  const int nv = sv.phys.nv;
  const int levels = sv.phys.multilevel ? 2 : 1;
  if (levels == 2)
    for (size_t k = 0; k < sv.blocks.size(); ++k)
      if (!fields[k].cons_nm1) throw Error(ATH_ERR_ARG, "bdf2 restart needs time n-1");
  auto f = OpenOut(path, true);
  Put(f, levels);          // time levels
  Put(f, iteration);       // solution iteration
  Put(f, nv);              // equations
  Put(f, (int)1);          // species
  const size_t len = sv.species.size();
  Put(f, len);
  f.write(sv.species.data(), (std::streamsize)len);
  f.write(reinterpret_cast<const char *>(resid_first), nv * sizeof(double));
  BlockDims(f, s, sv, nv + 1);
  const Scales sc = ScalesOf(sv);
  for (size_t k = 0; k < sv.blocks.size(); ++k) {
    const Block &b = s.blocks[sv.blocks[k]];
    const size_t m = Cells(b);
    std::vector<double> out;
    out.reserve(m * (nv + 1));
    for (size_t q = 0; q < m; ++q) {
      const double *w = fields[k].prim + q * nv;
      out.push_back(w[0] * sc.r);
      out.push_back(w[1] * sc.a);
      out.push_back(w[2] * sc.a);
      out.push_back(w[3] * sc.a);
      out.push_back(w[4] * (sc.r * sc.a * sc.a));
      if (nv == 7) {
        out.push_back(w[5] * (sc.a * sc.a));
        out.push_back(w[6] * (sc.a * sc.a * sc.r / sc.mu));
      }
      out.push_back(w[0] / w[0]);  // mass fraction of the one species
    }
    f.write(reinterpret_cast<const char *>(out.data()), out.size() * 8);
  }
  // time n-1: rho, rho u, rho v, rho w, rho E [, rho k, rho omega] times
  // their reference scales, then the species' share of the density
  for (size_t k = 0; levels == 2 && k < sv.blocks.size(); ++k) {
    const Block &b = s.blocks[sv.blocks[k]];
    const size_t m = Cells(b);
    std::vector<double> out;
    out.reserve(m * (nv + 1));
    for (size_t q = 0; q < m; ++q) {
      const double *u = fields[k].cons_nm1 + q * nv;
      out.push_back(u[0] * sc.r);
      out.push_back(u[1] * (sc.a * sc.r));
      out.push_back(u[2] * (sc.a * sc.r));
      out.push_back(u[3] * (sc.a * sc.r));
      out.push_back(u[4] * (sc.a * sc.a * sc.r));
      if (nv == 7) {
        out.push_back(u[5] * (sc.a * sc.a * sc.r));
        out.push_back(u[6] * (sc.a * sc.a * sc.r * sc.r / sc.mu));
      }
      out.push_back(u[0] / u[0]);
    }
    f.write(reinterpret_cast<const char *>(out.data()), out.size() * 8);
  }
  if (!f) throw Error(ATH_ERR_IO, std::string("write failed: ") + path);
}

// ReadRestart / ReadSolFromRestart (src/output.cpp:756,1177): the header is
// checked against the solve (equations, species, blocks and their sizes);
// values are made nondimensional and the species density is rho * mf
void ReadRestart(const Setup &s, const Solve &sv, const char *path, int *iteration,
                 double *resid_first, double *const *prim_out, int *levels,
                 double *const *cons_nm1_out) {
  if (!path) throw Error(ATH_ERR_ARG, "null path");
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) throw Error(ATH_ERR_IO, std::string("cannot open ") + path);
  int nsol = 0, iter = 0, neq = 0, nspec = 0;
  Get(f, nsol);
  Get(f, iter);
  Get(f, neq);
  Get(f, nspec);
  const int nv = sv.phys.nv;
  if (nsol < 1) throw Error(ATH_ERR_IO, "restart file holds no time level");
  if (nspec != 1) throw Error(ATH_ERR_UNSUPPORTED, "restart file has more than one species");
  if (neq != nv) throw Error(ATH_ERR_ARG, "restart file equations do not match the solve");
  size_t len = 0;
  Get(f, len);
  if (len > 4096) throw Error(ATH_ERR_IO, "bad species name length");
  std::string name(len, '\0');
  f.read(&name[0], (std::streamsize)len);
  if (name != sv.species) throw Error(ATH_ERR_ARG, "restart species " + name + " not in case");
  std::vector<double> rf(neq);
  f.read(reinterpret_cast<char *>(rf.data()), neq * sizeof(double));
  int nb = 0;
  Get(f, nb);
  if (nb != (int)sv.blocks.size())
    throw Error(ATH_ERR_ARG, "restart file block count does not match the grid");
  for (int k = 0; k < nb; ++k) {
    int ni = 0, nj = 0, nk = 0, nvars = 0;
    Get(f, ni);
    Get(f, nj);
    Get(f, nk);
    Get(f, nvars);
    const Block &b = s.blocks[sv.blocks[k]];
    if (ni != b.ni || nj != b.nj || nk != b.nk || nvars - 1 != neq)
      throw Error(ATH_ERR_ARG, "restart block size or variable count does not match");
  }
  const Scales sc = ScalesOf(sv);
  for (int k = 0; k < nb; ++k) {
    const Block &b = s.blocks[sv.blocks[k]];
    const size_t m = Cells(b);
    std::vector<double> in(m * (nv + 1));
    f.read(reinterpret_cast<char *>(in.data()), in.size() * 8);
    if (!f) throw Error(ATH_ERR_IO, "restart file ends early");
    if (!prim_out || !prim_out[k]) continue;
    for (size_t q = 0; q < m; ++q) {
      const double *x = &in[q * (nv + 1)];
      double *w = prim_out[k] + q * nv;
      const double rho = x[0] / sc.r;
      w[1] = x[1] / sc.a;
      w[2] = x[2] / sc.a;
      w[3] = x[3] / sc.a;
      w[4] = x[4] / (sc.r * sc.a * sc.a);
      if (nv == 7) {
        w[5] = x[5] / (sc.a * sc.a);
        w[6] = x[6] / (sc.a * sc.a * sc.r / sc.mu);
      }
      w[0] = 0.0 + rho * x[nv];  // species density, then their sum
    }
  }
  // ReadSolNm1FromRestart (src/output.cpp:1242): conserved values over
  // their scales, the species density rho * mf
  for (int k = 0; nsol >= 2 && cons_nm1_out && k < nb; ++k) {
    const Block &b = s.blocks[sv.blocks[k]];
    const size_t m = Cells(b);
    std::vector<double> in(m * (nv + 1));
    f.read(reinterpret_cast<char *>(in.data()), in.size() * 8);
    if (!f) throw Error(ATH_ERR_IO, "restart file ends early");
    if (!cons_nm1_out[k]) continue;
    for (size_t q = 0; q < m; ++q) {
      const double *x = &in[q * (nv + 1)];
      double *u = cons_nm1_out[k] + q * nv;
      const double rho = x[0] / sc.r;
      u[1] = x[1] / (sc.a * sc.r);
      u[2] = x[2] / (sc.a * sc.r);
      u[3] = x[3] / (sc.a * sc.r);
      u[4] = x[4] / (sc.r * sc.a * sc.a);
      if (nv == 7) {
        u[5] = x[5] / (sc.a * sc.a * sc.r);
        u[6] = x[6] / (sc.a * sc.a * sc.r * sc.r / sc.mu);
      }
      u[0] = rho * x[nv];
    }
  }
  if (levels) *levels = nsol;
  if (iteration) *iteration = iter;
  if (resid_first) std::memcpy(resid_first, rf.data(), neq * sizeof(double));
}

// WriteCellCenter (src/output.cpp:57): per block x of every physical cell,
// then y, then z, times the reference length
void WriteCenters(const Setup &s, const Solve &sv, const char *path) {
  auto f = OpenOut(path, true);
  BlockDims(f, s, sv, 0);
  for (int bi : sv.blocks) {
    const Block &b = s.blocks[bi];
    const int64_t nc = b.NCell();
    std::vector<double> out;
    out.reserve(3 * Cells(b));
    for (int c = 0; c < 3; ++c)
      for (int k = 0; k < b.nk; ++k)
        for (int j = 0; j < b.nj; ++j)
          for (int i = 0; i < b.ni; ++i)
            out.push_back(b.center[c * nc + b.Cell(i, j, k)] * sv.phys.l_ref);
    f.write(reinterpret_cast<const char *>(out.data()), out.size() * 8);
  }
  if (!f) throw Error(ATH_ERR_IO, std::string("write failed: ") + path);
}

// WriteMeta (src/output.cpp:903), steady form
void WriteMeta(const Solve &sv, const std::vector<std::string> &vars, int iteration,
               const char *path) {
  auto f = OpenOut(path, false);
  f << "{\n";
  f << "\"auto-detect-format\" : true,\n";
  f << "\"format\" : \"binary\",\n";
  f << "\"language\" : \"C\",\n";
  f << "\"filenames\" : [{ \"time\" : " << iteration << ", \"xyz\" : \"" << sv.grid_name
    << "_center.xyz\", \"function\" : \"" << sv.sim_root << "_" << iteration
    << "_center.fun\" }],\n";
  f << "\"function-names\" : [ ";
  for (size_t k = 0; k < vars.size(); ++k) {
    f << "\"" << vars[k] << "\"";
    if (k + 1 < vars.size()) f << ", ";
  }
  f << " ]\n";
  f << "}\n";
  if (!f) throw Error(ATH_ERR_IO, std::string("write failed: ") + path);
}

// std::left << setw(w) << value, scientific with 4 digits for doubles
void Cell(std::string &out, const std::string &txt, int w) {
  out += txt;
  if ((int)txt.size() < w) out.append(w - txt.size(), ' ');
}
std::string Sci(double x) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.4e", x);
  return buf;
}

// PrintHeaders (src/output.cpp:1007) as the residual file gets it: the
// file's header is written when the log opens, before the first CFL is set,
// so it has no CFL column although every row carries one
std::string ResidHeader(bool rans, bool time_step) {
  std::string h;
  Cell(h, "Step", 7);
  Cell(h, "NL-Iter", 8);
  // the CFL column has no header: the reference prints the header while
  // its CFL is still 0
  if (time_step) Cell(h, "Time-Step", 12);
  for (const char *t : {"Res-Mass", "Res-Mom-X", "Res-Mom-Y", "Res-Mom-Z", "Res-Energy"})
    Cell(h, t, 12);
  if (rans) {
    Cell(h, "Res-Tke", 12);
    Cell(h, "Res-Omega", 12);
  }
  for (const char *t : {"Max-Eqn", "Max-Blk", "Max-I", "Max-J", "Max-K"}) Cell(h, t, 8);
  Cell(h, "Max-Res", 12);
  Cell(h, "Res-Matrix", 12);
  return h + "\n";
}

// PrintResiduals (src/output.cpp:1028): time step nn, nonlinear iteration
// mm; the normalisation is the L2 of the first time step's first nonlinear
// iteration, raised to the largest of each equation over the first
// nonlinear iterations of time steps 1-4 (never changed in a restarted
// run); every L2 is shown as (L2 + EPS) / (L2_first + EPS), EPS = 1e-30;
// the third column is the input's timeStep, or else the CFL
std::string ResidLine(bool rans, int nn, int mm, double time_step, bool restarted,
                      const ath_norms &nm, double *first) {
  const int nv = rans ? 7 : 5;
  if (!restarted && mm == 0) {
    if (nn == 0) {
      for (int v = 0; v < nv; ++v) first[v] = nm.l2[v];
    } else if (nn < 5) {
      if (nm.l2[0] > first[0]) first[0] = nm.l2[0];
      for (int v = 1; v < nv; ++v) first[v] = first[v] < nm.l2[v] ? nm.l2[v] : first[v];
    }
  }
  const double eps = 1.0e-30;
  std::string r;
  Cell(r, std::to_string(nn), 7);
  Cell(r, std::to_string(mm), 8);
  Cell(r, Sci(time_step > 0.0 ? time_step : nm.cfl), 12);
  for (int v = 0; v < nv; ++v) Cell(r, Sci((nm.l2[v] + eps) / (first[v] + eps)), 12);
  Cell(r, std::to_string(nm.linf_eqn), 8);
  Cell(r, std::to_string(nm.linf_block), 8);
  Cell(r, std::to_string(nm.linf_i), 8);
  Cell(r, std::to_string(nm.linf_j), 8);
  Cell(r, std::to_string(nm.linf_k), 8);
  Cell(r, Sci(nm.linf), 12);
  Cell(r, Sci(nm.matrix_resid), 12);
  return r + "\n";
}

// per-block fields of one solve gathered from a batch
struct Gathered {
  std::vector<std::vector<double>> prim, dt, resid, aux, velgrad, wd, nm1, grads;
  std::vector<ath_block_fields> f;
};

void GatherFields(ath_batch *batch, const Setup &s, const Solve &sv, bool want_dt,
                  bool want_resid, bool want_aux, bool want_velgrad, bool want_wd, Gathered &g,
                  bool want_nm1 = false, bool want_grads = false) {
  const size_t nb = sv.blocks.size();
  g.prim.resize(nb);
  g.nm1.resize(nb);
  g.dt.resize(nb);
  g.resid.resize(nb);
  g.aux.resize(nb);
  g.velgrad.resize(nb);
  g.wd.resize(nb);
  g.grads.resize(nb);
  g.f.assign(nb, ath_block_fields{});
  auto get = [&](int bi, int field, std::vector<double> &out, size_t w) {
    out.resize(Cells(s.blocks[bi]) * w);
    const int rc = ath_batch_get_field(batch, bi, field, out.data());
    if (rc != ATH_OK) throw Error(rc, ath_last_error());
    return out.data();
  };
  for (size_t k = 0; k < nb; ++k) {
    const int bi = sv.blocks[k];
    const int nv = s.blocks[bi].nv;
    g.f[k].prim = get(bi, ATH_FIELD_STATE, g.prim[k], nv);
    if (want_dt) g.f[k].dt = get(bi, ATH_FIELD_DT, g.dt[k], 1);
    if (want_resid) g.f[k].resid = get(bi, ATH_FIELD_RESID, g.resid[k], nv);
    if (want_aux) g.f[k].aux = get(bi, ATH_FIELD_AUX, g.aux[k], 5);
    if (want_grads) g.f[k].grads = get(bi, ATH_FIELD_GRADS, g.grads[k], 24);
    if (want_velgrad && !want_grads) g.f[k].velgrad = get(bi, ATH_FIELD_VELGRAD, g.velgrad[k], 9);
    if (want_wd) g.f[k].wall_dist = get(bi, ATH_FIELD_WALLDIST, g.wd[k], 1);
    if (want_nm1) g.f[k].cons_nm1 = get(bi, ATH_FIELD_CONS_NM1, g.nm1[k], nv);
  }
}

bool Wants(const std::vector<std::string> &vars, std::initializer_list<const char *> names,
           const char *prefix = nullptr) {
  for (const auto &v : vars) {
    for (const char *n : names)
      if (v == n) return true;
    if (prefix && v.compare(0, std::strlen(prefix), prefix) == 0) return true;
  }
  return false;
}

}  // namespace
}  // namespace ath

using namespace ath;

extern "C" {

int ath_output_function(const ath_setup *setup, int solve, const char *variables,
                        const ath_block_fields *fields, const char *path) {
  return Guard([&] {
    const Solve &sv = SolveOf(setup, solve);
    WriteFunction(setup->s, sv, SplitVars(variables, sv), fields, path);
  });
}

int ath_output_restart(const ath_setup *setup, int solve, int iteration,
                       const double *resid_first, const ath_block_fields *fields,
                       const char *path) {
  return Guard([&] {
    WriteRestart(setup->s, SolveOf(setup, solve), iteration, resid_first, fields, path);
  });
}

int ath_input_restart(const ath_setup *setup, int solve, const char *path, int *iteration,
                      double *resid_first, double *const *prim_out, int *levels,
                      double *const *cons_nm1_out) {
  return Guard([&] {
    ReadRestart(setup->s, SolveOf(setup, solve), path, iteration, resid_first, prim_out,
                levels, cons_nm1_out);
  });
}

int ath_output_center_grid(const ath_setup *setup, int solve, const char *path) {
  return Guard([&] { WriteCenters(setup->s, SolveOf(setup, solve), path); });
}

int ath_output_meta(const ath_setup *setup, int solve, const char *variables, int iteration,
                    const char *path) {
  return Guard([&] {
    const Solve &sv = SolveOf(setup, solve);
    WriteMeta(sv, SplitVars(variables, sv), iteration, path);
  });
}

int ath_output_resid(const ath_setup *setup, int solve, const char *path, int flags,
                     int first_step, int n, const ath_norms *norms, double *resid_first) {
  return Guard([&] {
    const Solve &sv = SolveOf(setup, solve);
    if (n < 0 || (n > 0 && !norms) || !resid_first || first_step < 0)
      throw Error(ATH_ERR_ARG, "bad argument");
    if (!path) throw Error(ATH_ERR_ARG, "null path");
    const bool rans = sv.phys.nv == 7;
    const bool append = (flags & ATH_RESID_APPEND) != 0;
    const bool restarted = (flags & ATH_RESID_RESTARTED) != 0;
    const int nl = std::max(1, (int)sv.phys.nl_iters);
    std::ofstream f(path, append ? std::ios::app : std::ios::out);
    if (!f) throw Error(ATH_ERR_IO, std::string("cannot open ") + path);
    if (!append) f << ResidHeader(rans, sv.time_step > 0.0);
    for (int k = 0; k < n; ++k) {
      const int it = first_step + k;
      f << ResidLine(rans, it / nl, it % nl, sv.time_step, restarted, norms[k], resid_first);
    }
    if (!f) throw Error(ATH_ERR_IO, std::string("write failed: ") + path);
  });
}

int ath_batch_write_function(ath_batch *batch, const ath_setup *setup, int solve,
                             const char *variables, const char *path) {
  return Guard([&] {
    const Solve &sv = SolveOf(setup, solve);
    const auto vars = SplitVars(variables, sv);
    Gathered g;
    // the scalar gradients come from the batch's kept gradients, and the
    // velocity gradient too where the batch keeps them
    const bool scalar_grads = Wants(vars, {}, "tempGrad_") || Wants(vars, {}, "densityGrad_") ||
                              Wants(vars, {}, "pressGrad_") || Wants(vars, {}, "tkeGrad_") ||
                              Wants(vars, {}, "omegaGrad_");
    int flags = 0;
    const int rc = ath_batch_flags(batch, &flags);
    if (rc != ATH_OK) throw Error(rc, ath_last_error());
    const bool kept = (flags & ATH_BATCH_OUTPUT_GRADS) != 0;
    GatherFields(batch, setup->s, sv, Wants(vars, {"dt"}), Wants(vars, {}, "resid_"),
                 Wants(vars, {"temperature", "cp", "cv", "viscosity", "viscosityRatio",
                              "turbulentViscosity", "f1", "f2"}),
                 Wants(vars, {}, "velGrad_"), Wants(vars, {"wallDistance"}), g, false,
                 scalar_grads || (kept && Wants(vars, {}, "velGrad_")));
    WriteFunction(setup->s, sv, vars, g.f.data(), path);
  });
}

int ath_batch_write_restart(ath_batch *batch, const ath_setup *setup, int solve,
                            int iteration, const double *resid_first, const char *path) {
  return Guard([&] {
    const Solve &sv = SolveOf(setup, solve);
    Gathered g;
    GatherFields(batch, setup->s, sv, false, false, false, false, false, g,
                 sv.phys.multilevel != 0);
    WriteRestart(setup->s, sv, iteration, resid_first, g.f.data(), path);
  });
}

int ath_batch_read_restart(ath_batch *batch, const ath_setup *setup, int solve,
                           const char *path, int *iteration, double *resid_first) {
  return Guard([&] {
    const Solve &sv = SolveOf(setup, solve);
    const size_t nb = sv.blocks.size();
    std::vector<std::vector<double>> prim(nb), nm1(nb);
    std::vector<double *> ptr(nb), ptr1(nb);
    for (size_t k = 0; k < nb; ++k) {
      const Block &b = setup->s.blocks[sv.blocks[k]];
      prim[k].resize(Cells(b) * b.nv);
      ptr[k] = prim[k].data();
      if (sv.phys.multilevel) {
        nm1[k].resize(Cells(b) * b.nv);
        ptr1[k] = nm1[k].data();
      }
    }
    int levels = 0;
    ReadRestart(setup->s, sv, path, iteration, resid_first, ptr.data(), &levels,
                sv.phys.multilevel ? ptr1.data() : nullptr);
    for (size_t k = 0; k < nb; ++k) {
      const int rc = ath_batch_set_state(batch, sv.blocks[k], prim[k].data());
      if (rc != ATH_OK) throw Error(rc, ath_last_error());
    }
    // bdf2: time n-1 from the file, or the state itself (ReadRestart
    // src/output.cpp:869-895)
    for (size_t k = 0; sv.phys.multilevel && k < nb; ++k) {
      const int rc =
          ath_batch_set_state_nm1(batch, sv.blocks[k], levels >= 2 ? nm1[k].data() : nullptr);
      if (rc != ATH_OK) throw Error(rc, ath_last_error());
    }
  });
}

}  // extern "C"
