// C ABI for the host-side setup (see include/aither_gb300.h).
#include <cstring>
#include <exception>
#include <string>

#include "aither_gb300.h"
#include "errors.hpp"
#include "setup.hpp"


namespace ath {
namespace {
thread_local std::string g_last_error;
}
void SetError(const std::string &msg) { g_last_error = msg; }
const char *LastError() { return g_last_error.c_str(); }
}  // namespace ath

using ath::Guard;

namespace {
// level 0 is the setup itself, level l > 0 its l-th coarser multigrid level
const ath::Setup &LevelOf(const ath_setup *setup, int level) {
  if (!setup) throw ath::Error(ATH_ERR_ARG, "null setup");
  if (level < 0 || level > (int)setup->s.levels.size())
    throw ath::Error(ATH_ERR_ARG, "multigrid level out of range");
  return level == 0 ? setup->s : *setup->s.levels[level - 1];
}
}  // namespace

extern "C" {

const char *ath_last_error(void) { return ath::LastError(); }

int ath_setup_from_input(const char *inp_path, ath_setup **out) {
  return Guard([&] {
    if (!inp_path || !out) throw ath::Error(ATH_ERR_ARG, "null argument");
    auto *s = new ath_setup();
    try {
      ath::AppendInput(s->s, inp_path);
    } catch (...) {
      delete s;
      throw;
    }
    *out = s;
  });
}

int ath_setup_from_input_dev(const char *inp_path, int device, ath_setup **out) {
  return Guard([&] {
    if (!inp_path || !out || device < 0) throw ath::Error(ATH_ERR_ARG, "bad argument");
    auto *s = new ath_setup();
    s->s.geom_device = device;
    try {
      ath::AppendInput(s->s, inp_path);
    } catch (...) {
      delete s;
      throw;
    }
    *out = s;
  });
}

int ath_setup_append(ath_setup *setup, const char *inp_path) {
  return Guard([&] {
    if (!setup || !inp_path) throw ath::Error(ATH_ERR_ARG, "null argument");
    ath::AppendInput(setup->s, inp_path);
  });
}

int ath_setup_destroy(ath_setup *setup) {
  delete setup;
  return ATH_OK;
}

int ath_setup_level_counts(const ath_setup *setup, int level, int *nsolves, int *nblocks,
                           int64_t *ncells) {
  return Guard([&] {
    const ath::Setup &st = LevelOf(setup, level);
    if (nsolves) *nsolves = (int)st.solves.size();
    if (nblocks) *nblocks = (int)st.blocks.size();
    if (ncells) {
      int64_t n = 0;
      for (auto &b : st.blocks) n += (int64_t)b.ni * b.nj * b.nk;
      *ncells = n;
    }
  });
}

int ath_setup_level_block(const ath_setup *setup, int level, int block, ath_block_view *out) {
  return Guard([&] {
    const ath::Setup &st = LevelOf(setup, level);
    if (!out) throw ath::Error(ATH_ERR_ARG, "null argument");
    if (block < 0 || block >= (int)st.blocks.size())
      throw ath::Error(ATH_ERR_ARG, "block index out of range");
    const auto &b = st.blocks[block];
    std::memset(out, 0, sizeof(*out));
    out->ni = b.ni;
    out->nj = b.nj;
    out->nk = b.nk;
    out->ng = b.ng;
    out->nv = b.nv;
    out->solve = b.solve;
    out->ncell_padded = b.NCell();
    for (int d = 0; d < 3; ++d) {
      out->nface_padded[d] = b.NFace(d);
      out->farea[d] = b.farea[d].data();
    }
    out->vol = b.vol.data();
    out->center = b.center.data();
    out->width = b.width.data();
    out->wall_dist = b.wall_dist.data();
    out->state0 = b.state0.data();
    out->nops = (int32_t)b.ops.size();
    out->ops = b.ops.data();
    out->nedge_ops = (int32_t)b.edge_ops.size();
    out->edge_ops = b.edge_ops.data();
    out->nvops = (int32_t)b.vops.size();
    out->vops = b.vops.data();
    out->nvedge_ops = (int32_t)b.vedge_ops.size();
    out->vedge_ops = b.vedge_ops.data();
    out->nplanes = (int32_t)b.plane_offsets.size() - 1;
    out->plane_offsets = b.plane_offsets.data();
    out->plane_cells = b.plane_cells.data();
    out->nbr_mask = b.nbr_mask.data();
    out->n_nr = (int32_t)b.nr_cells.size();
    out->nr = b.nr_cells.data();
  });
}

int ath_setup_level_solve(const ath_setup *setup, int level, int solve, ath_solve_view *out) {
  return Guard([&] {
    const ath::Setup &st = LevelOf(setup, level);
    if (!out) throw ath::Error(ATH_ERR_ARG, "null argument");
    if (solve < 0 || solve >= (int)st.solves.size())
      throw ath::Error(ATH_ERR_ARG, "solve index out of range");
    const auto &sv = st.solves[solve];
    *out = sv.phys;
    out->nstates = (int32_t)sv.states.size();
    out->states = sv.states.data();
  });
}

int ath_setup_counts(const ath_setup *setup, int *nsolves, int *nblocks, int64_t *ncells) {
  return ath_setup_level_counts(setup, 0, nsolves, nblocks, ncells);
}

int ath_setup_block(const ath_setup *setup, int block, ath_block_view *out) {
  return ath_setup_level_block(setup, 0, block, out);
}

int ath_setup_solve(const ath_setup *setup, int solve, ath_solve_view *out) {
  return ath_setup_level_solve(setup, 0, solve, out);
}

int ath_setup_levels(const ath_setup *setup, int *nlevels) {
  return Guard([&] {
    if (!setup || !nlevels) throw ath::Error(ATH_ERR_ARG, "null argument");
    *nlevels = 1 + (int)setup->s.levels.size();
  });
}

int ath_setup_mg_map(const ath_setup *setup, int level, int block, ath_mg_map *out) {
  return Guard([&] {
    const ath::Setup &st = LevelOf(setup, level);
    if (!out) throw ath::Error(ATH_ERR_ARG, "null argument");
    if (block < 0 || block >= (int)st.blocks.size())
      throw ath::Error(ATH_ERR_ARG, "block index out of range");
    const auto &b = st.blocks[block];
    if (b.mg_coarse < 0) throw ath::Error(ATH_ERR_ARG, "block has no coarser level");
    out->coarse_block = b.mg_coarse;
    out->ncells = (int64_t)b.ni * b.nj * b.nk;
    out->coarse_cell = b.mg_cell.data();
    out->volfac = b.mg_volfac.data();
    out->coef = b.mg_coef.data();
  });
}

int ath_setup_set_state(ath_setup *setup, int block, const double *prim) {
  return Guard([&] {
    if (!setup || !prim) throw ath::Error(ATH_ERR_ARG, "null argument");
    if (block < 0 || block >= (int)setup->s.blocks.size())
      throw ath::Error(ATH_ERR_ARG, "block index out of range");
    auto &b = setup->s.blocks[block];
    size_t n = 0;
    for (int k = 0; k < b.nk; ++k)
      for (int j = 0; j < b.nj; ++j)
        for (int i = 0; i < b.ni; ++i)
          for (int v = 0; v < b.nv; ++v)
            b.state0[(size_t)b.Cell(i, j, k) * b.nv + v] = prim[n++];
  });
}

}  // extern "C"
