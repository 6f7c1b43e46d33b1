// Host-side case setup: the reference's input/Plot3D formats, its
// nondimensionalisation, block geometry and boundary bookkeeping, turned
// into flat arrays that the device batch and the CPU oracle consume.
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "aither_gb300.h"

namespace ath {

// One boundary surface of a block as written in the reference input file:
// "type imin imax jmin jmax kmin kmax tag" (node indices).
struct Surface {
  std::string name;
  int type = 0;  // ATH_BC_*
  int i1 = 0, i2 = 0, j1 = 0, j2 = 0, k1 = 0, k2 = 0;
  int tag = 0;
  // surface id as in the reference: 1 i-lower, 2 i-upper, 3 j-lower,
  // 4 j-upper, 5 k-lower, 6 k-upper
  int SurfaceId() const;
  int Dir() const { return (SurfaceId() - 1) / 2; }
  bool Lower() const { return SurfaceId() % 2 == 1; }
};

struct BCStateIn {
  ath_bc_state s{};
  // periodic pairing
  int start_tag = -1, end_tag = -1;
  double translation[3] = {0, 0, 0};
};

struct Block {
  int ni = 0, nj = 0, nk = 0, ng = 0, nv = 0, solve = 0;
  int NI = 0, NJ = 0, NK = 0;
  std::vector<double> nodes;  // [3][(ni+1)(nj+1)(nk+1)], nondimensional
  std::vector<Surface> surfs;
  // padded geometry
  std::vector<double> vol, center, width, fcenter[3], farea[3], wall_dist;
  std::vector<double> state0;  // padded AoS primitive
  std::vector<ath_ghost_op> ops, edge_ops, vops, vedge_ops;
  std::vector<ath_nr_cell> nr_cells;  // cells of nonreflecting surfaces
  std::vector<int32_t> plane_offsets, plane_cells;
  std::vector<uint8_t> nbr_mask;
  // multigrid: this block's block on the next coarser level (its index in
  // that level's setup) and, per physical cell in k, j, i order, the coarse
  // physical cell it lies in (i + ni*(j + nj*k) of the coarse block), its
  // volume weight in the restriction and its 7 trilinear prolongation
  // coefficients (gridLevel::Coarsen, src/gridLevel.cpp:440-535)
  int mg_coarse = -1;
  std::vector<int32_t> mg_cell;
  std::vector<double> mg_volfac, mg_coef;  // [cells], [cells][7]

  int64_t Cell(int i, int j, int k) const {
    return (int64_t)(i + ng) + (int64_t)NI * ((j + ng) + (int64_t)NJ * (k + ng));
  }
  int64_t NCell() const { return (int64_t)NI * NJ * NK; }
  // face of direction d at (i,j,k): arrays are one longer along d
  int64_t Face(int d, int i, int j, int k) const {
    const int fi = NI + (d == 0), fj = NJ + (d == 1);
    return (int64_t)(i + ng) + (int64_t)fi * ((j + ng) + (int64_t)fj * (k + ng));
  }
  int64_t NFace(int d) const {
    return (int64_t)(NI + (d == 0)) * (NJ + (d == 1)) * (NK + (d == 2));
  }
  double Node(int c, int i, int j, int k) const {
    return nodes[(size_t)c * (ni + 1) * (nj + 1) * (nk + 1) +
                 (size_t)i + (size_t)(ni + 1) * (j + (size_t)(nj + 1) * k)];
  }
};

struct Solve {
  std::string name;
  // output controls of the input file: outputVariables (a sorted set, as
  // the reference keeps it), outputFrequency, restartFrequency, iterations;
  // the simulation name root (input file name up to its first '.') and the
  // grid name
  std::vector<std::string> output_vars;
  int output_freq = 1, restart_freq = 0, iterations = 1;
  std::string sim_root, grid_name;
  std::string species = "air";  // the one fluid of the case (fluids key)
  double time_step = -1.0;      // timeStep as written (dimensional; <= 0: none)
  ath_solve_view phys{};  // states pointer refreshed on access
  std::vector<ath_bc_state> states;
  std::vector<BCStateIn> states_in;
  std::vector<int> blocks;  // global block indices
};

struct Setup {
  std::vector<Block> blocks;
  std::vector<Solve> solves;
  // CUDA device that computes the physical cells' geometry and wall
  // distance (-1: the host does)
  int geom_device = -1;
  // coarser multigrid levels: levels[l-1] holds level l of every solve with
  // more than l levels, in the order of the solves (mgSolution::
  // ConstructMultigrids, src/mgSolution.cpp:86)
  std::vector<std::unique_ptr<Setup>> levels;
};

// Parse an input file and append its blocks as a new solve.
void AppendInput(Setup &setup, const std::string &path);

// Geometry and boundary bookkeeping for the blocks of one solve.
void BuildGeometry(Block &b, int device = -1);
// The physical cells' and faces' geometry (DeviceGeometry) and the physical
// cells' wall distance to the centres wf (DeviceWallDistance) computed on a
// CUDA device, bit for bit the host's (geometry.cu).
void DeviceGeometry(Block &b, int device);
void DeviceWallDistance(const std::vector<double> &wf, Block &b, int device);
void BuildGhostGeometry(Block &b);
void BuildCellWidths(Block &b);
void BuildGhostOps(Setup &setup, int solve);
void BuildHyperplanes(Block &b);
void BuildEdgeOps(Setup &setup, int solve);
// Coarser multigrid levels of a solve with more than one level.
void BuildCoarseLevels(Setup &setup, int solve);

// Reads the binary multi-block Plot3D grid format.
std::vector<Block> ReadPlot3d(const std::string &path, double lref);

}  // namespace ath

// Block (5x5) solvers and Jacobi (DP-LUR) solvers among ATH_SOLVER_*
inline bool IsBlockSolver(int s) { return s == ATH_SOLVER_BLUSGS || s == ATH_SOLVER_BDPLUR; }
inline bool IsJacobiSolver(int s) { return s == ATH_SOLVER_DPLUR || s == ATH_SOLVER_BDPLUR; }

// The C handle of a host setup.
struct ath_setup {
  ath::Setup s;
};
