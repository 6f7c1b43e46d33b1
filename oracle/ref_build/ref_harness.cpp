// Driver for the unmodified reference solver built as a CPU oracle.
//
// It follows the reference's own program setup (src/main.cpp:55-230: input
// parse, nondimensionalisation, Plot3D read, decomposition on one rank,
// finest grid level, auxiliary variables, wall distance) and its nonlinear
// iteration loop (src/main.cpp:231-277), then writes the per-cell fields the
// parity tests compare against.  Optionally the initial primitive state of
// every block is replaced by nondimensional values read from a file, so that
// analytic initial conditions reach the reference bit for bit.
//
// usage: ref_harness case.inp iterations out.bin [state_override.bin]
//
// out.bin is a sequence of records:
//   char name[32]; int64 ndim; int64 dims[ndim]; double data[prod(dims)]
// Test infrastructure only.
#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "boundaryConditions.hpp"
#include "fluxJacobian.hpp"
#include "gridLevel.hpp"
#include "input.hpp"
#include "kdtree.hpp"
#include "matMultiArray3d.hpp"
#include "mgSolution.hpp"
#include "multiArray3d.hpp"
#include "output.hpp"
#include "parallel.hpp"
#include "physicsModels.hpp"
#include "plot3d.hpp"
#include "primitive.hpp"
#include "procBlock.hpp"
#include "resid.hpp"
#include "utility.hpp"
#include "varArray.hpp"
#include "vector3d.hpp"

namespace {

class Writer {
 public:
  explicit Writer(const std::string &path) : f_(path, std::ios::binary) {
    if (!f_) {
      std::cerr << "cannot open " << path << std::endl;
      std::exit(2);
    }
  }
  void Put(const std::string &name, const std::vector<int64_t> &dims,
           const std::vector<double> &data) {
    char buf[32] = {0};
    std::strncpy(buf, name.c_str(), 31);
    f_.write(buf, 32);
    const int64_t nd = dims.size();
    f_.write(reinterpret_cast<const char *>(&nd), sizeof(nd));
    f_.write(reinterpret_cast<const char *>(dims.data()), nd * sizeof(int64_t));
    f_.write(reinterpret_cast<const char *>(data.data()),
             data.size() * sizeof(double));
  }

 private:
  std::ofstream f_;
};

void DumpBlock(Writer &w, const procBlock &blk, const linearSolver *,
               const blkMultiArray3d<varArray> &du, const physics &phys,
               int bb) {
  const auto pre = "b" + std::to_string(bb) + "_";
  const int ng = blk.NumGhosts();
  const int ni = blk.NumI(), nj = blk.NumJ(), nk = blk.NumK();
  const int nv = blk.NumEquations();
  const int NI = ni + 2 * ng, NJ = nj + 2 * ng, NK = nk + 2 * ng;

  // primitive state including ghost cells, [k][j][i][v]
  {
    std::vector<double> d;
    d.reserve(static_cast<size_t>(NI) * NJ * NK * nv);
    const auto &st = blk.States();
    for (int k = -ng; k < nk + ng; ++k)
      for (int j = -ng; j < nj + ng; ++j)
        for (int i = -ng; i < ni + ng; ++i)
          for (int v = 0; v < nv; ++v) d.push_back(st(i, j, k, v));
    w.Put(pre + "state", {NK, NJ, NI, nv}, d);
  }
  // residual, dt, spectral radius over physical cells
  {
    std::vector<double> r, dt, sr, up;
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j < nj; ++j)
        for (int i = 0; i < ni; ++i) {
          for (int v = 0; v < nv; ++v) r.push_back(blk.Residual(i, j, k, v));
          dt.push_back(blk.Dt(i, j, k));
          sr.push_back(blk.SpectralRadius(i, j, k).FlowVariable());
          sr.push_back(blk.SpectralRadius(i, j, k).TurbVariable());
          for (int v = 0; v < nv; ++v) up.push_back(du(i, j, k, v));
        }
    w.Put(pre + "resid", {nk, nj, ni, nv}, r);
    w.Put(pre + "dt", {nk, nj, ni}, dt);
    w.Put(pre + "specrad", {nk, nj, ni, 2}, sr);
    w.Put(pre + "du", {nk, nj, ni, nv}, up);
  }
  // geometry: volume, centre, cell widths (with ghosts)
  {
    std::vector<double> vol, cen, wid;
    for (int k = -ng; k < nk + ng; ++k)
      for (int j = -ng; j < nj + ng; ++j)
        for (int i = -ng; i < ni + ng; ++i) {
          vol.push_back(blk.Vol(i, j, k));
          const auto c = blk.Center(i, j, k);
          cen.push_back(c.X());
          cen.push_back(c.Y());
          cen.push_back(c.Z());
          wid.push_back(blk.CellWidthI(i, j, k));
          wid.push_back(blk.CellWidthJ(i, j, k));
          wid.push_back(blk.CellWidthK(i, j, k));
        }
    w.Put(pre + "vol", {NK, NJ, NI}, vol);
    w.Put(pre + "center", {NK, NJ, NI, 3}, cen);
    w.Put(pre + "width", {NK, NJ, NI, 3}, wid);
  }
  // face areas with ghosts: unit vector (3) + magnitude
  {
    std::vector<double> fa;
    for (int k = -ng; k < nk + ng; ++k)
      for (int j = -ng; j < nj + ng; ++j)
        for (int i = -ng; i < ni + ng + 1; ++i) {
          const auto &a = blk.FAreaI(i, j, k);
          fa.push_back(a.UnitVector().X());
          fa.push_back(a.UnitVector().Y());
          fa.push_back(a.UnitVector().Z());
          fa.push_back(a.Mag());
        }
    w.Put(pre + "fareai", {NK, NJ, NI + 1, 4}, fa);
    fa.clear();
    for (int k = -ng; k < nk + ng; ++k)
      for (int j = -ng; j < nj + ng + 1; ++j)
        for (int i = -ng; i < ni + ng; ++i) {
          const auto &a = blk.FAreaJ(i, j, k);
          fa.push_back(a.UnitVector().X());
          fa.push_back(a.UnitVector().Y());
          fa.push_back(a.UnitVector().Z());
          fa.push_back(a.Mag());
        }
    w.Put(pre + "fareaj", {NK, NJ + 1, NI, 4}, fa);
    fa.clear();
    for (int k = -ng; k < nk + ng + 1; ++k)
      for (int j = -ng; j < nj + ng; ++j)
        for (int i = -ng; i < ni + ng; ++i) {
          const auto &a = blk.FAreaK(i, j, k);
          fa.push_back(a.UnitVector().X());
          fa.push_back(a.UnitVector().Y());
          fa.push_back(a.UnitVector().Z());
          fa.push_back(a.Mag());
        }
    w.Put(pre + "fareak", {NK + 1, NJ, NI, 4}, fa);
  }
  // auxiliary fields used by viscous paths
  {
    std::vector<double> t, mu, wd, mut, f1, f2;
    for (int k = -ng; k < nk + ng; ++k)
      for (int j = -ng; j < nj + ng; ++j)
        for (int i = -ng; i < ni + ng; ++i) {
          t.push_back(blk.Temperature(i, j, k));
          mu.push_back(blk.Viscosity(i, j, k));
          wd.push_back(blk.WallDist(i, j, k));
          mut.push_back(blk.EddyViscosity(i, j, k));
          f1.push_back(blk.F1(i, j, k));
          f2.push_back(blk.F2(i, j, k));
        }
    w.Put(pre + "temperature", {NK, NJ, NI}, t);
    w.Put(pre + "viscosity", {NK, NJ, NI}, mu);
    w.Put(pre + "walldist", {NK, NJ, NI}, wd);
    w.Put(pre + "eddyvisc", {NK, NJ, NI}, mut);
    w.Put(pre + "f1", {NK, NJ, NI}, f1);
    w.Put(pre + "f2", {NK, NJ, NI}, f2);
  }
  (void)phys;
}

}  // namespace

int main(int argc, char *argv[]) {
  if (argc < 4) {
    std::cerr << "usage: ref_harness case.inp iterations out.bin "
                 "[state_override.bin]"
              << std::endl;
    return 2;
  }
  MPI_Init(&argc, &argv);
  const int rank = 0;
  std::string inputFile = argv[1];
  const int niter = std::stoi(argv[2]);
  const std::string outFile = argv[3];
  const std::string overrideFile = argc > 4 ? argv[4] : "";

  auto totalCells = 0.0;
  input inp(inputFile, "none");
  decomposition decomp;
  auto numProcBlock = 0;
  inp.ReadInput(rank);
  inp.NondimensionalizeFluid();
  const auto phys = inp.AssignPhysicsModels();
  inp.NondimensionalizeStateData(phys.EoS());

  mgSolution solution;
  std::vector<vector3d<double>> viscFaces;
  std::vector<double> l2First;
  {
    auto mesh = ReadP3dGrid(inp.GridName(), inp.LRef(), totalCells);
    auto bcs = inp.AllBC();
    decomp = CubicDecomposition(mesh, bcs, 1);
    residual dummy(inp.NumEquations(), inp.NumSpecies());
    solution.ConstructFinestLevel(mesh, bcs, decomp, phys, "none", inp, dummy);
    viscFaces = GetViscousFaceCenters(solution.Finest().Blocks());
  }
  MPI_Datatype MPI_vec3d, MPI_procBlockInts, MPI_connection, MPI_DOUBLE_5INT,
      MPI_vec3dMag, MPI_uncoupledScalar, MPI_tensorDouble;
  SetDataTypesMPI(MPI_vec3d, MPI_procBlockInts, MPI_connection, MPI_DOUBLE_5INT,
                  MPI_vec3dMag, MPI_uncoupledScalar, MPI_tensorDouble);
  decomp.Broadcast();
  SendNumProcBlocks(decomp.NumBlocksOnAllProc(), numProcBlock);
  auto local = solution.SendFinestGridLevel(rank, numProcBlock, MPI_vec3d,
                                            MPI_vec3dMag, MPI_connection, inp);
  local.ConstructMultigrids(decomp, inp, phys, rank, MPI_connection, MPI_vec3d,
                            MPI_vec3dMag);

  // optional analytic initial state, nondimensional, [block][k][j][i][v]
  if (!overrideFile.empty()) {
    std::ifstream f(overrideFile, std::ios::binary);
    if (!f) {
      std::cerr << "cannot open " << overrideFile << std::endl;
      return 2;
    }
    auto &lvl = const_cast<gridLevel &>(local.Finest());
    for (int bb = 0; bb < lvl.NumBlocks(); ++bb) {
      auto &blk = lvl.Block(bb);
      blkMultiArray3d<primitive> st(blk.NumI(), blk.NumJ(), blk.NumK(), 0,
                                    blk.NumEquations(), blk.NumSpecies());
      for (int k = 0; k < blk.NumK(); ++k)
        for (int j = 0; j < blk.NumJ(); ++j)
          for (int i = 0; i < blk.NumI(); ++i)
            for (int v = 0; v < blk.NumEquations(); ++v) {
              double val;
              f.read(reinterpret_cast<char *>(&val), sizeof(val));
              st(i, j, k, v) = val;
            }
      if (!f) {
        std::cerr << "override file too short" << std::endl;
        return 2;
      }
      blk.GetStatesFromRestart(st);
    }
  }
  local.AuxillaryAndWidths(phys);

  {
    kdtree tree(viscFaces);
    if (tree.Size() > 0) {
      local.CalcWallDistance(tree);
      local.SwapWallDist(rank, inp.NumberGhostLayers());
    }
  }

  Writer w(outFile);
  // initial state (before any iteration) for every block
  for (int bb = 0; bb < local.Finest().NumBlocks(); ++bb) {
    const auto &blk = local.Finest().Block(bb);
    const int ni = blk.NumI(), nj = blk.NumJ(), nk = blk.NumK();
    const int nv = blk.NumEquations();
    std::vector<double> d;
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j < nj; ++j)
        for (int i = 0; i < ni; ++i)
          for (int v = 0; v < nv; ++v) d.push_back(blk.States()(i, j, k, v));
    w.Put("b" + std::to_string(bb) + "_state0", {nk, nj, ni, nv}, d);
  }

  std::vector<double> l2hist, mresHist;
  for (int nn = 0; nn < niter; ++nn) {
    inp.CalcCFL(nn);
    local.StoreOldSolution(inp, phys, nn);
    for (int mm = 0; mm < inp.NonlinearIterations(); ++mm) {
      residual residL2(inp.NumEquations(), inp.NumSpecies());
      resid residLinf;
      auto matrixResid = local.Iterate(inp, phys, MPI_tensorDouble, MPI_vec3d,
                                       mm, rank, residL2, residLinf);
      residL2.GlobalReduceMPI(rank);
      residL2.SquareRoot();
      matrixResid = std::sqrt(matrixResid / (totalCells * inp.NumEquations()));
      for (int v = 0; v < inp.NumEquations(); ++v)
        l2hist.push_back(residL2[v]);
      mresHist.push_back(matrixResid);
    }
  }
  const int nv = inp.NumEquations();
  w.Put("l2", {static_cast<int64_t>(l2hist.size() / nv), nv}, l2hist);
  w.Put("matrix_resid", {static_cast<int64_t>(mresHist.size())}, mresHist);
  {
    const auto du = local.Finest().Update();
    for (int bb = 0; bb < local.Finest().NumBlocks(); ++bb) {
      DumpBlock(w, local.Finest().Block(bb), nullptr, du[bb], phys, bb);
    }
  }
  {
    // integrated wall forces from the wall data of the last residual:
    // sum over viscous-wall faces of p_w A (area vector) and tau_w |A|,
    // blocks in order, wall surfaces in wall-data order, faces k, j, i
    std::vector<double> forces(6, 0.0);
    for (int bb = 0; bb < local.Finest().NumBlocks(); ++bb) {
      const auto &blk = local.Finest().Block(bb);
      for (int ss = 0; ss < blk.WallDataSize(); ++ss) {
        const auto surf = blk.WallSurface(ss);
        const int dir = (surf.SurfaceType() - 1) / 2;
        const int i1 = dir == 0 ? surf.IMin() + 1 : surf.IMax();
        const int j1 = dir == 1 ? surf.JMin() + 1 : surf.JMax();
        const int k1 = dir == 2 ? surf.KMin() + 1 : surf.KMax();
        for (int kk = surf.KMin(); kk < k1; ++kk)
          for (int jj = surf.JMin(); jj < j1; ++jj)
            for (int ii = surf.IMin(); ii < i1; ++ii) {
              const double p = blk.WallPressure(ss, ii, jj, kk, phys.EoS());
              const auto tau = blk.WallShearStress(ss, ii, jj, kk);
              const auto n = dir == 0 ? blk.FAreaUnitI(ii, jj, kk)
                             : dir == 1 ? blk.FAreaUnitJ(ii, jj, kk)
                                        : blk.FAreaUnitK(ii, jj, kk);
              const double mag = dir == 0 ? blk.FAreaMagI(ii, jj, kk)
                                 : dir == 1 ? blk.FAreaMagJ(ii, jj, kk)
                                            : blk.FAreaMagK(ii, jj, kk);
              forces[0] += p * n.X() * mag;
              forces[1] += p * n.Y() * mag;
              forces[2] += p * n.Z() * mag;
              forces[3] += tau.X() * mag;
              forces[4] += tau.Y() * mag;
              forces[5] += tau.Z() * mag;
            }
      }
    }
    w.Put("forces", {6}, forces);
  }
  std::vector<double> consts = {inp.ARef(), inp.RRef(), inp.TRef(), inp.LRef(),
                                inp.CFL()};
  w.Put("refs", {static_cast<int64_t>(consts.size())}, consts);
  MPI_Finalize();
  return 0;
}
