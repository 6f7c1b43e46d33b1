// Host-side case setup.  Restates, in this project's own code, the parts of
// the reference that run once before the iteration loop:
//   input file format           src/input.cpp:167-643
//   fluid data and reference    src/fluid.cpp:89-101, src/input.cpp:604-621
//     speed of sound, BC-state  src/inputStates.cpp:464,590,674,775
//     nondimensionalisation
//   Plot3D grid                 src/plot3d.cpp:363-445
//   cell geometry               src/plot3d.cpp:36-360 (centroid, six-pyramid
//                               volume, diagonal cross-product face areas)
//   ghost-cell geometry         src/procBlock.cpp:2160-2294
//   cell widths                 src/procBlock.cpp:6397
//   connections (periodic,      src/boundaryConditions.cpp:293-1150
//     interblock) by patch-corner matching
//   hyperplane visit order      src/utility.cpp:377
// The arithmetic of the geometry follows the reference operation by
// operation so the device path sees the same metric terms.
#include "setup.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <memory>
#include <set>
#include <sstream>
#include <stdexcept>

namespace ath {

namespace {

std::string Trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) ++a;
  while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) --b;
  return s.substr(a, b - a);
}

std::vector<std::string> Split(const std::string &s, char sep) {
  std::vector<std::string> out;
  std::string cur;
  for (char c : s) {
    if (c == sep) {
      out.push_back(Trim(cur));
      cur.clear();
    } else {
      cur += c;
    }
  }
  out.push_back(Trim(cur));
  return out;
}

[[noreturn]] void Fail(const std::string &msg) { throw std::runtime_error(msg); }

int BCType(const std::string &name) {
  if (name == "slipWall") return ATH_BC_SLIP_WALL;
  if (name == "viscousWall") return ATH_BC_VISCOUS_WALL;
  if (name == "characteristic") return ATH_BC_CHARACTERISTIC;
  if (name == "stagnationInlet") return ATH_BC_STAGNATION_INLET;
  if (name == "pressureOutlet") return ATH_BC_PRESSURE_OUTLET;
  if (name == "supersonicInflow") return ATH_BC_SUPERSONIC_INFLOW;
  if (name == "supersonicOutflow") return ATH_BC_SUPERSONIC_OUTFLOW;
  if (name == "periodic") return ATH_BC_PERIODIC;
  if (name == "interblock") return ATH_BC_INTERBLOCK;
  if (name == "inlet") return ATH_BC_INLET;
  Fail("unsupported boundary condition type '" + name + "'");
}

bool IsConnection(int type) {
  return type == ATH_BC_PERIODIC || type == ATH_BC_INTERBLOCK;
}

// "[a, b, c]" -> 3 doubles
void ParseVec3(const std::string &s, double out[3]) {
  std::string t = s;
  for (auto &c : t)
    if (c == '[' || c == ']' || c == ',') c = ' ';
  std::istringstream is(t);
  for (int i = 0; i < 3; ++i) {
    if (!(is >> out[i])) Fail("bad vector '" + s + "'");
  }
}

// name(k1=v1; k2=v2; ...) -> name, map
std::pair<std::string, std::map<std::string, std::string>> ParseCall(
    const std::string &s) {
  const auto open = s.find('(');
  const auto close = s.rfind(')');
  if (open == std::string::npos || close == std::string::npos || close < open)
    Fail("bad state definition '" + s + "'");
  std::map<std::string, std::string> kv;
  for (auto &tok : Split(s.substr(open + 1, close - open - 1), ';')) {
    if (tok.empty()) continue;
    const auto eq = tok.find('=');
    if (eq == std::string::npos) Fail("bad parameter '" + tok + "'");
    kv[Trim(tok.substr(0, eq))] = Trim(tok.substr(eq + 1));
  }
  return {Trim(s.substr(0, open)), kv};
}

// split "<a(...), b(...)>" into the individual calls
std::vector<std::string> SplitList(const std::string &s) {
  std::vector<std::string> out;
  std::string body = Trim(s);
  if (!body.empty() && body.front() == '<') body = body.substr(1);
  if (!body.empty() && body.back() == '>') body.pop_back();
  int depth = 0;
  std::string cur;
  for (char c : body) {
    if (c == '(') ++depth;
    if (c == ')') --depth;
    if (c == ',' && depth == 0) {
      if (!Trim(cur).empty()) out.push_back(Trim(cur));
      cur.clear();
    } else {
      cur += c;
    }
  }
  if (!Trim(cur).empty()) out.push_back(Trim(cur));
  return out;
}

struct Fluid {
  double n = 2.5;
  double molar_mass = 28.97 / 1000.;  // kg/mol
  double hf = 0.0;
  double mu_c1 = 1.458e-6, mu_s = 110.4;
  double k_c1 = 2.495e-3, k_s = 194.0;
};

// Reads "key: value" lines of a fluid database file (air.dat format).
bool ReadFluidFile(const std::string &path, Fluid &f) {
  std::ifstream in(path);
  if (!in) return false;
  std::string line;
  while (std::getline(in, line)) {
    line = Trim(line);
    if (line.empty() || line[0] == '#') continue;
    const auto c = line.find(':');
    if (c == std::string::npos) continue;
    const auto key = Trim(line.substr(0, c));
    const auto val = Trim(line.substr(c + 1));
    if (key == "n") f.n = std::stod(val);
    else if (key == "molarMass") f.molar_mass = std::stod(val) / 1000.;
    else if (key == "heatOfFormation") f.hf = std::stod(val);
    else if (key == "sutherlandViscosityC1") f.mu_c1 = std::stod(val);
    else if (key == "sutherlandViscosityS") f.mu_s = std::stod(val);
    else if (key == "sutherlandConductivityC1") f.k_c1 = std::stod(val);
    else if (key == "sutherlandConductivityS") f.k_s = std::stod(val);
  }
  return true;
}

std::string DirName(const std::string &p) {
  const auto s = p.find_last_of('/');
  return s == std::string::npos ? std::string(".") : p.substr(0, s);
}

}  // namespace

int Surface::SurfaceId() const {
  if (i1 == i2) return i1 == 0 ? 1 : 2;
  if (j1 == j2) return j1 == 0 ? 3 : 4;
  if (k1 == k2) return k1 == 0 ? 5 : 6;
  Fail("boundary surface is not a constant-index plane");
}

std::vector<Block> ReadPlot3d(const std::string &path, double lref) {
  std::ifstream in(path, std::ios::binary);
  if (!in) Fail("cannot open grid file " + path);
  int32_t nb = 0;
  in.read(reinterpret_cast<char *>(&nb), 4);
  if (!in || nb <= 0 || nb > 1000000) Fail("bad Plot3D header in " + path);
  std::vector<std::array<int32_t, 3>> dims(nb);
  for (auto &d : dims) {
    in.read(reinterpret_cast<char *>(d.data()), 12);
    if (!in || d[0] < 2 || d[1] < 2 || d[2] < 2) Fail("bad block size in " + path);
  }
  std::vector<Block> blocks(nb);
  for (int b = 0; b < nb; ++b) {
    auto &blk = blocks[b];
    blk.ni = dims[b][0] - 1;
    blk.nj = dims[b][1] - 1;
    blk.nk = dims[b][2] - 1;
    const size_t nn = (size_t)dims[b][0] * dims[b][1] * dims[b][2];
    blk.nodes.resize(3 * nn);
    in.read(reinterpret_cast<char *>(blk.nodes.data()), 3 * nn * sizeof(double));
    if (!in) Fail("truncated Plot3D file " + path);
    for (auto &x : blk.nodes) x = x / lref;
  }
  return blocks;
}

// ---------------------------------------------------------------------------
// geometry
namespace {
struct V3 {
  double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double Dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 Cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, -1.0 * (a.x * b.z - a.z * b.x),
          a.x * b.y - a.y * b.x};
}
inline double Mag(V3 a) { return std::sqrt(Dot(a, a)); }

V3 NodeV(const Block &b, int i, int j, int k) {
  return {b.Node(0, i, j, k), b.Node(1, i, j, k), b.Node(2, i, j, k)};
}

double Pyramid(V3 p, V3 a, V3 bb, V3 c, V3 d) {
  const V3 xp = 0.25 * ((((a - p) + (bb - p)) + (c - p)) + (d - p));
  const V3 xac = c - a;
  const V3 xbd = d - bb;
  return 1.0 / 6.0 * Dot(xp, Cross(xac, xbd));
}

void StoreArea(std::vector<double> &fa, int64_t nf, int64_t idx, V3 a) {
  const double m = Mag(a);
  fa[idx] = a.x / m;
  fa[nf + idx] = a.y / m;
  fa[2 * nf + idx] = a.z / m;
  fa[3 * nf + idx] = m;
}

V3 GetV(const std::vector<double> &v, int64_t n, int64_t idx) {
  return {v[idx], v[n + idx], v[2 * n + idx]};
}
void SetV(std::vector<double> &v, int64_t n, int64_t idx, V3 a) {
  v[idx] = a.x;
  v[n + idx] = a.y;
  v[2 * n + idx] = a.z;
}
}  // namespace

void BuildGeometry(Block &b, int device) {
  b.NI = b.ni + 2 * b.ng;
  b.NJ = b.nj + 2 * b.ng;
  b.NK = b.nk + 2 * b.ng;
  const int64_t nc = b.NCell();
  b.vol.assign(nc, 0.0);
  b.center.assign(3 * nc, 0.0);
  b.width.assign(3 * nc, 0.0);
  b.wall_dist.assign(nc, 1.0e10);
  for (int d = 0; d < 3; ++d) {
    b.farea[d].assign(4 * b.NFace(d), 0.0);
    b.fcenter[d].assign(3 * b.NFace(d), 0.0);
  }
  if (device >= 0) {
    DeviceGeometry(b, device);
    return;
  }
  for (int k = 0; k < b.nk; ++k)
    for (int j = 0; j < b.nj; ++j)
      for (int i = 0; i < b.ni; ++i) {
        const V3 c0 = NodeV(b, i, j, k), c1 = NodeV(b, i + 1, j, k),
                 c2 = NodeV(b, i, j + 1, k), c3 = NodeV(b, i + 1, j + 1, k),
                 c4 = NodeV(b, i, j, k + 1), c5 = NodeV(b, i + 1, j, k + 1),
                 c6 = NodeV(b, i, j + 1, k + 1),
                 c7 = NodeV(b, i + 1, j + 1, k + 1);
        const V3 cen =
            0.125 * (((((((c0 + c1) + c2) + c3) + c4) + c5) + c6) + c7);
        double v = 0.0;
        v += Pyramid(cen, c0, c4, c6, c2);
        v += Pyramid(cen, c1, c3, c7, c5);
        v += Pyramid(cen, c0, c1, c5, c4);
        v += Pyramid(cen, c2, c6, c7, c3);
        v += Pyramid(cen, c0, c2, c3, c1);
        v += Pyramid(cen, c4, c5, c7, c6);
        if (!(v > 0)) Fail("non-positive cell volume in grid");
        const auto id = b.Cell(i, j, k);
        b.vol[id] = v;
        SetV(b.center, nc, id, cen);
      }
  // i-faces
  {
    const int64_t nf = b.NFace(0);
    for (int k = 0; k < b.nk; ++k)
      for (int j = 0; j < b.nj; ++j)
        for (int i = 0; i <= b.ni; ++i) {
          const V3 xac = NodeV(b, i, j + 1, k + 1) - NodeV(b, i, j, k);
          const V3 xbd = NodeV(b, i, j + 1, k) - NodeV(b, i, j, k + 1);
          const auto id = b.Face(0, i, j, k);
          StoreArea(b.farea[0], nf, id, 0.5 * Cross(xbd, xac));
          SetV(b.fcenter[0], nf, id,
               0.25 * (((NodeV(b, i, j, k) + NodeV(b, i, j + 1, k)) +
                        NodeV(b, i, j, k + 1)) +
                       NodeV(b, i, j + 1, k + 1)));
        }
  }
  // j-faces
  {
    const int64_t nf = b.NFace(1);
    for (int k = 0; k < b.nk; ++k)
      for (int j = 0; j <= b.nj; ++j)
        for (int i = 0; i < b.ni; ++i) {
          const V3 xac = NodeV(b, i, j, k + 1) - NodeV(b, i + 1, j, k);
          const V3 xbd = NodeV(b, i, j, k) - NodeV(b, i + 1, j, k + 1);
          const auto id = b.Face(1, i, j, k);
          StoreArea(b.farea[1], nf, id, 0.5 * Cross(xbd, xac));
          SetV(b.fcenter[1], nf, id,
               0.25 * (((NodeV(b, i, j, k) + NodeV(b, i + 1, j, k)) +
                        NodeV(b, i, j, k + 1)) +
                       NodeV(b, i + 1, j, k + 1)));
        }
  }
  // k-faces
  {
    const int64_t nf = b.NFace(2);
    for (int k = 0; k <= b.nk; ++k)
      for (int j = 0; j < b.nj; ++j)
        for (int i = 0; i < b.ni; ++i) {
          const V3 xac = NodeV(b, i, j + 1, k) - NodeV(b, i + 1, j, k);
          const V3 xbd = NodeV(b, i + 1, j + 1, k) - NodeV(b, i, j, k);
          const auto id = b.Face(2, i, j, k);
          StoreArea(b.farea[2], nf, id, 0.5 * Cross(xbd, xac));
          SetV(b.fcenter[2], nf, id,
               0.25 * (((NodeV(b, i, j, k) + NodeV(b, i + 1, j, k)) +
                        NodeV(b, i, j + 1, k)) +
                       NodeV(b, i + 1, j + 1, k)));
        }
  }
}

namespace {
// Index helpers for a surface-normal direction d and in-plane directions
// (d1, d2) following the reference's convention: i-surface (j, k),
// j-surface (k, i), k-surface (i, j).
inline void InPlane(int d, int &d1, int &d2) {
  d1 = (d + 1) % 3;
  d2 = (d + 2) % 3;
}
inline std::array<int, 3> Ijk(int d, int a, int d1, int b1, int d2, int b2) {
  std::array<int, 3> r{};
  r[d] = a;
  r[d1] = b1;
  r[d2] = b2;
  return r;
}
inline int Ncell(const Block &b, int d) {
  return d == 0 ? b.ni : (d == 1 ? b.nj : b.nk);
}
inline void SurfRange(const Surface &s, int d, int &lo, int &hi) {
  if (d == 0) { lo = s.i1; hi = s.i2; }
  else if (d == 1) { lo = s.j1; hi = s.j2; }
  else { lo = s.k1; hi = s.k2; }
}
}  // namespace

void BuildGhostGeometry(Block &b) {
  const int64_t nc = b.NCell();
  for (int layer = 1; layer <= b.ng; ++layer) {
    for (const auto &s : b.surfs) {
      if (s.type == ATH_BC_INTERBLOCK) continue;
      const int d = s.Dir();
      int d1, d2;
      InPlane(d, d1, d2);
      const int n = Ncell(b, d);
      const bool lower = s.Lower();
      int g, ic, pc, pic, ifc, pifc;
      if (!lower) {
        g = n + layer - 1;
        ic = n - layer;
        pc = g - 1;
        if (ic < 0) ic = 0;
        pic = ic + 1;
        ifc = n - layer;
        if (ifc < 0) ifc = 0;
        pifc = ifc + 1;
      } else {
        g = -layer;
        ic = layer - 1;
        pc = g + 1;
        if (ic >= n) ic = n - 1;
        pic = ic - 1;
        ifc = layer;
        if (ifc > n) ifc = n;
        pifc = ifc - 1;
      }
      int lo1, hi1, lo2, hi2;
      SurfRange(s, d1, lo1, hi1);
      SurfRange(s, d2, lo2, hi2);
      for (int b2 = lo2; b2 < hi2; ++b2)
        for (int b1 = lo1; b1 < hi1; ++b1) {
          const auto G = Ijk(d, g, d1, b1, d2, b2);
          const auto I = Ijk(d, ic, d1, b1, d2, b2);
          const auto P = Ijk(d, pc, d1, b1, d2, b2);
          const auto PI = Ijk(d, pic, d1, b1, d2, b2);
          const auto gid = b.Cell(G[0], G[1], G[2]);
          const auto iid = b.Cell(I[0], I[1], I[2]);
          b.vol[gid] = b.vol[iid];
          // face areas: the ghost's outward face takes the interior cell's
          // face on the same side (lower: face g <- face ic; upper: face
          // g+1 <- face ic+1); the other faces copy straight over
          for (int fd = 0; fd < 3; ++fd) {
            const int64_t nf = b.NFace(fd);
            auto copy_face = [&](std::array<int, 3> to, std::array<int, 3> from) {
              const auto t = b.Face(fd, to[0], to[1], to[2]);
              const auto f = b.Face(fd, from[0], from[1], from[2]);
              for (int c = 0; c < 4; ++c) b.farea[fd][c * nf + t] = b.farea[fd][c * nf + f];
            };
            if (fd == d) {
              auto to = G, from = I;
              if (!lower) {
                to[d] = g + 1;
                from[d] = ic + 1;
              }
              copy_face(to, from);
            } else {
              copy_face(G, I);
              auto G2 = G, I2 = I;
              G2[fd] += 1;
              I2[fd] += 1;
              copy_face(G2, I2);
            }
          }
          // centres
          auto FcAt = [&](int fd, std::array<int, 3> c) {
            return GetV(b.fcenter[fd], b.NFace(fd), b.Face(fd, c[0], c[1], c[2]));
          };
          auto IF = Ijk(d, ifc, d1, b1, d2, b2);
          auto PIF = Ijk(d, pifc, d1, b1, d2, b2);
          const V3 distF2F = FcAt(d, PIF) - FcAt(d, IF);
          const V3 distC2C =
              layer > 1 ? GetV(b.center, nc, b.Cell(PI[0], PI[1], PI[2])) -
                              GetV(b.center, nc, iid)
                        : distF2F;
          for (int fd = 0; fd < 3; ++fd) {
            const int64_t nf = b.NFace(fd);
            if (fd == d) {
              auto to = G, from = P;
              if (!lower) { to[d] = g + 1; from[d] = pc + 1; }
              SetV(b.fcenter[fd], nf, b.Face(fd, to[0], to[1], to[2]),
                   distF2F + FcAt(fd, from));
            } else {
              SetV(b.fcenter[fd], nf, b.Face(fd, G[0], G[1], G[2]),
                   distC2C + FcAt(fd, P));
              auto G2 = G, P2 = P;
              G2[fd] += 1;
              P2[fd] += 1;
              SetV(b.fcenter[fd], nf, b.Face(fd, G2[0], G2[1], G2[2]),
                   distC2C + FcAt(fd, P2));
            }
          }
          SetV(b.center, nc, gid,
               GetV(b.center, nc, b.Cell(P[0], P[1], P[2])) + distC2C);
        }
    }
  }
}

void BuildCellWidths(Block &b) {
  const int64_t nc = b.NCell();
  for (int k = -b.ng; k < b.nk + b.ng; ++k)
    for (int j = -b.ng; j < b.nj + b.ng; ++j)
      for (int i = -b.ng; i < b.ni + b.ng; ++i) {
        const auto id = b.Cell(i, j, k);
        for (int d = 0; d < 3; ++d) {
          const int64_t nf = b.NFace(d);
          const V3 a = GetV(b.fcenter[d], nf, b.Face(d, i, j, k));
          const V3 c = GetV(b.fcenter[d], nf,
                            b.Face(d, i + (d == 0), j + (d == 1), k + (d == 2)));
          b.width[d * nc + id] = Mag(a - c);
        }
      }
}

void BuildHyperplanes(Block &b) {
  const int np = b.ni + b.nj + b.nk - 2;
  b.plane_offsets.assign(np + 1, 0);
  b.plane_cells.clear();
  b.plane_cells.reserve((size_t)b.ni * b.nj * b.nk);
  // planes p = i+j+k; inside a plane k, then j, then i ascending (the
  // reference's visit order; cells of one plane are independent)
  std::vector<int32_t> count(np, 0);
  for (int k = 0; k < b.nk; ++k)
    for (int j = 0; j < b.nj; ++j)
      for (int i = 0; i < b.ni; ++i) count[i + j + k]++;
  for (int p = 0; p < np; ++p) b.plane_offsets[p + 1] = b.plane_offsets[p] + count[p];
  b.plane_cells.resize(b.plane_offsets[np]);
  std::vector<int32_t> fill(b.plane_offsets.begin(), b.plane_offsets.end() - 1);
  for (int k = 0; k < b.nk; ++k)
    for (int j = 0; j < b.nj; ++j)
      for (int i = 0; i < b.ni; ++i)
        b.plane_cells[fill[i + j + k]++] = (int32_t)b.Cell(i, j, k);
}

// ---------------------------------------------------------------------------
// ghost-cell operations and connections
namespace {

struct Patch {
  int block, surf;
  int d, d1, d2;
  bool lower;
  int lo1, hi1, lo2, hi2;  // node ranges in d1, d2
  int plane;               // node index of the plane along d
  V3 Corner(const Block &b, int a1, int a2) const {
    const auto c = Ijk(d, plane, d1, a1, d2, a2);
    return NodeV(b, c[0], c[1], c[2]);
  }
};

bool Close(V3 a, V3 b, double tol) {
  return std::fabs(a.x - b.x) < tol && std::fabs(a.y - b.y) < tol &&
         std::fabs(a.z - b.z) < tol;
}

// Maps each node (a1, a2) of patch A to a node of patch B.  Returns false
// when the four corners of the patches do not coincide (after shifting A by
// `shift`) in any of the 8 orientations.
bool MatchPatches(const Setup &st, const Patch &A, const Patch &B, V3 shift,
                  int m[2][3]) {
  const Block &ba = st.blocks[A.block], &bb = st.blocks[B.block];
  const int na1 = A.hi1 - A.lo1, na2 = A.hi2 - A.lo2;
  const int nb1 = B.hi1 - B.lo1, nb2 = B.hi2 - B.lo2;
  if (!((na1 == nb1 && na2 == nb2) || (na1 == nb2 && na2 == nb1))) return false;
  double scale = 0.0;
  for (int a2 : {A.lo2, A.hi2})
    for (int a1 : {A.lo1, A.hi1}) scale = std::max(scale, Mag(A.Corner(ba, a1, a2)));
  const double tol = 1e-10 * std::max(1.0, scale);
  const V3 oA = A.Corner(ba, A.lo1, A.lo2) + shift;
  const V3 cA1 = A.Corner(ba, A.hi1, A.lo2) + shift;
  const V3 cA2 = A.Corner(ba, A.lo1, A.hi2) + shift;
  // candidate B node for a corner of A: try all four B corners
  const int cb1[2] = {B.lo1, B.hi1}, cb2[2] = {B.lo2, B.hi2};
  for (int o = 0; o < 4; ++o) {
    const int ob1 = cb1[o & 1], ob2 = cb2[o >> 1];
    if (!Close(oA, B.Corner(bb, ob1, ob2), tol)) continue;
    for (int c = 0; c < 4; ++c) {
      const int x1 = cb1[c & 1], x2 = cb2[c >> 1];
      if (!Close(cA1, B.Corner(bb, x1, x2), tol)) continue;
      for (int e = 0; e < 4; ++e) {
        const int y1 = cb1[e & 1], y2 = cb2[e >> 1];
        if (!Close(cA2, B.Corner(bb, y1, y2), tol)) continue;
        // b = o + a1*(c-o)/na1 + a2*(e-o)/na2 in node space
        const int s11 = (x1 - ob1) / std::max(na1, 1), s12 = (x2 - ob2) / std::max(na1, 1);
        const int s21 = (y1 - ob1) / std::max(na2, 1), s22 = (y2 - ob2) / std::max(na2, 1);
        if (std::abs(s11) + std::abs(s12) != 1 || std::abs(s21) + std::abs(s22) != 1)
          continue;
        m[0][0] = ob1 - (A.lo1 * s11 + A.lo2 * s21);
        m[0][1] = s11;
        m[0][2] = s21;
        m[1][0] = ob2 - (A.lo1 * s12 + A.lo2 * s22);
        m[1][1] = s12;
        m[1][2] = s22;
        return true;
      }
    }
  }
  return false;
}

// Sides of patch A's surface that touch another surface of the same block
// face: [direction 1 start, direction 1 end, direction 2 start, direction 2
// end] (boundaryConditions::BordersSurface, src/boundaryConditions.cpp:193:
// any surface of the same face, whatever its type, whose range ends where
// A's begins or begins where A's ends).
std::array<bool, 4> PatchBorders(const Block &b, const Patch &A) {
  std::array<bool, 4> r{false, false, false, false};
  const int id = b.surfs[A.surf].SurfaceId();
  for (const auto &o : b.surfs) {
    if (o.SurfaceId() != id) continue;
    int lo1, hi1, lo2, hi2;
    SurfRange(o, A.d1, lo1, hi1);
    SurfRange(o, A.d2, lo2, hi2);
    if (A.lo1 == hi1) r[0] = true;
    if (A.hi1 == lo1) r[1] = true;
    if (A.lo2 == hi2) r[2] = true;
    if (A.hi2 == lo2) r[3] = true;
  }
  return r;
}

// Adds the ghost ops that copy B's interior into A's ghost layers and, for
// interblock connections, the ghost geometry of those cells.
//
// Geometry follows the reference's order of construction: every ghost layer
// of a non-interblock surface, periodic ones included, is a mirror of the
// block's own boundary cells (procBlock::AssignGhostCellsGeom,
// src/procBlock.cpp:2201, built before this); interblock ghosts then take
// the partner's volume, centroid and faces (SwapGeomSlice,
// src/utility.cpp:213 -> procBlock::PutGeomSlice src/procBlock.cpp:3167):
// the faces normal to the patch from the boundary face outwards, and of
// each in-plane direction the ghost's lower face; the upper face of the
// patch's last cell along an in-plane direction only when that end of the
// patch does not border another surface of the block face (there the
// reference's insertion stops short of the patch end and the face keeps its
// mirror value).  Cell widths are formed afterwards from the face centres of
// the assembled geometry (procBlock::CalcCellWidths src/procBlock.cpp:6397).
// Geometry of a block as it was before a connection's swap: both sides of a
// swap read the partner's values from before either side was written, as
// the reference extracts both slices first (src/utility.cpp:213-232).
struct GeomSnap {
  std::vector<double> vol, center, farea[3], fcenter[3];
  explicit GeomSnap(const Block &b) : vol(b.vol), center(b.center) {
    for (int d = 0; d < 3; ++d) {
      farea[d] = b.farea[d];
      fcenter[d] = b.fcenter[d];
    }
  }
};

void ConnectOneWay(Setup &st, const Patch &A, const Patch &B, const GeomSnap *snap,
                   const int m[2][3], int type) {
  Block &ba = st.blocks[A.block];
  const Block &bb = st.blocks[B.block];
  const int nA = Ncell(ba, A.d), nB = Ncell(bb, B.d);
  const int64_t ncA = ba.NCell(), ncB = bb.NCell();
  const bool geom = snap != nullptr;  // interblock connections only
  const auto bord = PatchBorders(ba, A);
  for (int layer = 1; layer <= ba.ng; ++layer) {
    const int g = A.lower ? -layer : nA + layer - 1;
    int s = B.lower ? layer - 1 : nB - layer;
    if (s < 0) s = 0;
    if (s >= nB) s = nB - 1;
    for (int a2 = A.lo2; a2 < A.hi2; ++a2)
      for (int a1 = A.lo1; a1 < A.hi1; ++a1) {
        // the cell spans nodes a1..a1+1, a2..a2+1 of A; map both ends
        int bn1[2], bn2[2];
        for (int t = 0; t < 2; ++t) {
          const int n1 = a1 + t, n2 = a2 + t;
          bn1[t] = m[0][0] + n1 * m[0][1] + n2 * m[0][2];
          bn2[t] = m[1][0] + n1 * m[1][1] + n2 * m[1][2];
        }
        const int c1 = std::min(bn1[0], bn1[1]), c2 = std::min(bn2[0], bn2[1]);
        const auto G = Ijk(A.d, g, A.d1, a1, A.d2, a2);
        const auto S = Ijk(B.d, s, B.d1, c1, B.d2, c2);
        ath_ghost_op op{};
        op.dst = ba.Cell(G[0], G[1], G[2]);
        op.src = bb.Cell(S[0], S[1], S[2]);
        op.src_block = B.block;
        op.type = type;
        op.layer = layer;
        op.dir = A.d;
        op.lower = A.lower ? 1 : 0;
        op.state = -1;
        {
          auto F = Ijk(A.d, A.lower ? 0 : nA, A.d1, a1, A.d2, a2);
          op.face = ba.Face(A.d, F[0], F[1], F[2]);
        }
        op.src2 = -1;
        ba.ops.push_back(op);
        if (!geom) continue;
        const GeomSnap &bg = *snap;
        ba.vol[op.dst] = bg.vol[op.src];
        for (int c = 0; c < 3; ++c) ba.center[c * ncA + op.dst] = bg.center[c * ncB + op.src];
        // per A direction, the matching B direction and whether increasing
        // index runs the same way; a reversed axis swaps the ghost's low and
        // high faces and flips the unit normal
        const int dir_of_a1 = (m[0][1] != 0) ? B.d1 : B.d2;
        const int dir_of_a2 = (m[0][2] != 0) ? B.d1 : B.d2;
        const int bdir[3] = {B.d, dir_of_a1, dir_of_a2};
        const int sgn_d = (A.lower ? -1 : 1) * (B.lower ? 1 : -1);
        const int sgn1 = m[0][1] != 0 ? m[0][1] : m[1][1];
        const int sgn2 = m[0][2] != 0 ? m[0][2] : m[1][2];
        const int sgn[3] = {sgn_d, sgn1, sgn2};
        const int adir[3] = {A.d, A.d1, A.d2};
        const bool upper_face[3] = {true, a1 == A.hi1 - 1 && !bord[1],
                                    a2 == A.hi2 - 1 && !bord[3]};
        for (int q = 0; q < 3; ++q) {
          const int ea = adir[q], eb = bdir[q];
          const int64_t nfa = ba.NFace(ea), nfb = bb.NFace(eb);
          for (int side = 0; side < 2; ++side) {
            if (side == 1 && !upper_face[q]) continue;
            auto gf = G;
            gf[ea] += side;
            auto sf = S;
            sf[eb] += (sgn[q] > 0) ? side : 1 - side;
            const int64_t ta = ba.Face(ea, gf[0], gf[1], gf[2]);
            const int64_t fb = bb.Face(eb, sf[0], sf[1], sf[2]);
            const double flip = sgn[q] > 0 ? 1.0 : -1.0;
            for (int comp = 0; comp < 3; ++comp) {
              ba.farea[ea][comp * nfa + ta] = flip * bg.farea[eb][comp * nfb + fb];
              ba.fcenter[ea][comp * nfa + ta] = bg.fcenter[eb][comp * nfb + fb];
            }
            ba.farea[ea][3 * nfa + ta] = bg.farea[eb][3 * nfb + fb];
          }
        }
      }
  }
}

}  // namespace

void BuildGhostOps(Setup &st, int solve) {
  auto &sv = st.solves[solve];
  // boundary-state lookup by tag
  auto state_of_tag = [&](int tag) {
    for (size_t i = 0; i < sv.states.size(); ++i)
      if (sv.states[i].tag == tag) return (int)i;
    return -1;
  };
  std::vector<Patch> conns;
  for (int bi : sv.blocks) {
    Block &b = st.blocks[bi];
    b.ops.clear();
    b.vops.clear();
    b.nr_cells.clear();
    int nr_surfs = 0;
    for (size_t si = 0; si < b.surfs.size(); ++si) {
      const auto &s = b.surfs[si];
      const int d = s.Dir();
      int d1, d2;
      InPlane(d, d1, d2);
      Patch p{bi, (int)si, d, d1, d2, s.Lower(), 0, 0, 0, 0, 0};
      SurfRange(s, d1, p.lo1, p.hi1);
      SurfRange(s, d2, p.lo2, p.hi2);
      int lo, hi;
      SurfRange(s, d, lo, hi);
      p.plane = lo;
      if (IsConnection(s.type)) {
        conns.push_back(p);
        continue;
      }
      int st_idx = -1;
      if (s.type != ATH_BC_SLIP_WALL && s.type != ATH_BC_SUPERSONIC_OUTFLOW) {
        st_idx = state_of_tag(s.tag);
        if (st_idx < 0)
          Fail("no boundary state for tag " + std::to_string(s.tag));
      }
      const int n = Ncell(b, d);
      // nonreflecting inlet / pressureOutlet: the surface's boundary-
      // adjacent cells in the slice's k, j, i order for its Mach numbers
      int nr_surf = -1;
      if ((s.type == ATH_BC_INLET || s.type == ATH_BC_PRESSURE_OUTLET) &&
          sv.states[st_idx].nonreflecting) {
        nr_surf = nr_surfs++;
        int lo3[3], hi3[3];
        lo3[d] = s.Lower() ? 0 : n - 1;
        hi3[d] = lo3[d] + 1;
        lo3[d1] = p.lo1;
        hi3[d1] = p.hi1;
        lo3[d2] = p.lo2;
        hi3[d2] = p.hi2;
        for (int k = lo3[2]; k < hi3[2]; ++k)
          for (int j = lo3[1]; j < hi3[1]; ++j)
            for (int i = lo3[0]; i < hi3[0]; ++i) {
              int f3[3] = {i, j, k};
              f3[d] = s.Lower() ? 0 : n;
              ath_nr_cell x{};
              x.cell = b.Cell(i, j, k);
              x.face = b.Face(d, f3[0], f3[1], f3[2]);
              x.surf = nr_surf;
              x.dir = d;
              x.lower = s.Lower() ? 1 : 0;
              b.nr_cells.push_back(x);
            }
      }
      for (int layer = 1; layer <= b.ng; ++layer) {
        int g, ic, ac;
        if (s.Lower()) {
          g = -layer;
          ic = std::min(layer - 1, n - 1);
          ac = 0;
        } else {
          g = n + layer - 1;
          ic = std::max(n - layer, 0);
          ac = n - 1;
        }
        const bool reflect =
            s.type == ATH_BC_SLIP_WALL || s.type == ATH_BC_VISCOUS_WALL;
        // inviscid ghosts treat a viscous wall as a slip wall
        // (AssignInviscidGhostCells); the viscous-wall state is applied
        // before the viscous fluxes (AssignViscousGhostCells)
        const int inv_type = s.type == ATH_BC_VISCOUS_WALL ? ATH_BC_SLIP_WALL : s.type;
        for (int b2 = p.lo2; b2 < p.hi2; ++b2)
          for (int b1 = p.lo1; b1 < p.hi1; ++b1) {
            const auto G = Ijk(d, g, d1, b1, d2, b2);
            const auto I = Ijk(d, reflect ? ic : ac, d1, b1, d2, b2);
            const auto F = Ijk(d, s.Lower() ? 0 : n, d1, b1, d2, b2);
            ath_ghost_op op{};
            op.dst = b.Cell(G[0], G[1], G[2]);
            op.src = b.Cell(I[0], I[1], I[2]);
            op.src_block = bi;
            op.type = inv_type;
            op.layer = layer;
            op.dir = d;
            op.lower = s.Lower() ? 1 : 0;
            op.state = st_idx;
            op.face = b.Face(d, F[0], F[1], F[2]);
            op.src2 = nr_surf;  // -1 unless a nonreflecting surface
            b.ops.push_back(op);
            if (s.type == ATH_BC_VISCOUS_WALL) {
              // the wall-adjacent cell supplies the wall distance and the
              // kinematic viscosity of the omega wall value at every layer
              const auto A = Ijk(d, ac, d1, b1, d2, b2);
              op.type = ATH_BC_VISCOUS_WALL;
              op.src2 = b.Cell(A[0], A[1], A[2]);
              b.vops.push_back(op);
            }
          }
      }
    }
  }
  // pair up connection patches: periodic by tag pairs, interblock by
  // coincident corners
  std::vector<bool> used(conns.size(), false);
  for (size_t a = 0; a < conns.size(); ++a) {
    if (used[a]) continue;
    const Patch &A = conns[a];
    const Surface &sa = st.blocks[A.block].surfs[A.surf];
    bool found = false;
    for (size_t c = a + 1; c < conns.size() && !found; ++c) {
      if (used[c]) continue;
      const Patch &B = conns[c];
      const Surface &sb = st.blocks[B.block].surfs[B.surf];
      if (sa.type != sb.type) continue;
      if (sa.type == ATH_BC_INTERBLOCK) {
        // interblock tag = partner surface * 1000 + partner block
        // (boundarySurface::PartnerBlock/PartnerSurface)
        const auto &blks = sv.blocks;
        const int pb = sa.tag % 1000, ps = sa.tag / 1000;
        if (pb < 0 || pb >= (int)blks.size() || blks[pb] != B.block || ps != sb.SurfaceId())
          continue;
      }
      V3 shift{0, 0, 0};
      if (sa.type == ATH_BC_PERIODIC) {
        const BCStateIn *ps = nullptr;
        for (auto &si : sv.states_in)
          if ((si.start_tag == sa.tag && si.end_tag == sb.tag) ||
              (si.start_tag == sb.tag && si.end_tag == sa.tag))
            ps = &si;
        if (!ps) continue;
        shift = {ps->translation[0], ps->translation[1], ps->translation[2]};
        if (ps->start_tag == sb.tag) shift = -1.0 * shift;
      }
      int mab[2][3], mba[2][3];
      if (!MatchPatches(st, A, B, shift, mab)) continue;
      if (!MatchPatches(st, B, A, -1.0 * shift, mba))
        Fail("connection patches match one way only");
      if (sa.type == ATH_BC_INTERBLOCK) {
        const GeomSnap ga(st.blocks[A.block]), gb(st.blocks[B.block]);
        ConnectOneWay(st, A, B, &gb, mab, sa.type);
        ConnectOneWay(st, B, A, &ga, mba, sa.type);
      } else {
        ConnectOneWay(st, A, B, nullptr, mab, sa.type);
        ConnectOneWay(st, B, A, nullptr, mba, sa.type);
      }
      used[a] = used[c] = true;
      found = true;
    }
    if (!found)
      Fail("no partner found for connection surface with tag " +
           std::to_string(sa.tag));
  }
  // neighbour masks for the implicit off-diagonal sums
  for (int bi : sv.blocks) {
    Block &b = st.blocks[bi];
    b.nbr_mask.assign(b.NCell(), 0);
    std::vector<uint8_t> conn_face[3];
    for (int d = 0; d < 3; ++d) conn_face[d].assign(b.NFace(d), 0);
    for (const auto &s : b.surfs) {
      if (!IsConnection(s.type)) continue;
      const int d = s.Dir();
      int d1, d2;
      InPlane(d, d1, d2);
      int lo1, hi1, lo2, hi2, lo, hi;
      SurfRange(s, d1, lo1, hi1);
      SurfRange(s, d2, lo2, hi2);
      SurfRange(s, d, lo, hi);
      for (int b2 = lo2; b2 < hi2; ++b2)
        for (int b1 = lo1; b1 < hi1; ++b1) {
          const auto F = Ijk(d, lo, d1, b1, d2, b2);
          conn_face[d][b.Face(d, F[0], F[1], F[2])] = 1;
        }
    }
    const int n[3] = {b.ni, b.nj, b.nk};
    for (int k = 0; k < b.nk; ++k)
      for (int j = 0; j < b.nj; ++j)
        for (int i = 0; i < b.ni; ++i) {
          const int c[3] = {i, j, k};
          uint8_t m = 0;
          for (int d = 0; d < 3; ++d) {
            int lc[3] = {i, j, k}, uc[3] = {i, j, k};
            uc[d] += 1;
            if (c[d] > 0 || conn_face[d][b.Face(d, lc[0], lc[1], lc[2])])
              m |= (uint8_t)(1u << (2 * d));
            if (c[d] < n[d] - 1 || conn_face[d][b.Face(d, uc[0], uc[1], uc[2])])
              m |= (uint8_t)(1u << (2 * d + 1));
          }
          b.nbr_mask[b.Cell(i, j, k)] = m;
        }
  }
}

// ---------------------------------------------------------------------------
// block-edge ghost cells
namespace {

// boundary surface of id surf (1..6) holding the face at cell indices
// (i, j, k), the index along the surface normal being the face index
// (boundaryConditions::GetBCSurface)
const Surface &SurfaceAt(const Block &b, int i, int j, int k, int surf) {
  for (const auto &s : b.surfs) {
    if (s.SurfaceId() != surf) continue;
    const int d = s.Dir();
    const int c[3] = {i, j, k};
    int lo, hi;
    SurfRange(s, d, lo, hi);
    if (c[d] != lo) continue;
    bool inside = true;
    for (int e = 0; e < 3 && inside; ++e) {
      if (e == d) continue;
      SurfRange(s, e, lo, hi);
      if (c[e] < lo || c[e] >= hi) inside = false;
    }
    if (inside) return s;
  }
  Fail("no boundary surface covers a block edge");
}

}  // namespace

// procBlock::AssignInviscidGhostCellsEdge (src/procBlock.cpp:2565) and
// AssignViscousGhostCellsEdge (:2840): for each of the 12 block edges, each
// pair of ghost layers and each cell along the edge, one op; phases
// (layer3-1)*ng + layer2-1 run in order, cells inside a phase are
// independent.
void BuildEdgeOps(Setup &st, int solve) {
  const bool viscous = st.solves[solve].phys.eqn != ATH_EQN_EULER;
  for (int bi : st.solves[solve].blocks) {
    Block &b = st.blocks[bi];
    b.edge_ops.clear();
    b.vedge_ops.clear();
    const int n[3] = {b.ni, b.nj, b.nk};
    for (int dd = 0; dd < 3; ++dd) {
      const int a2 = (dd + 1) % 3, a3 = (dd + 2) % 3;  // j,k for i; k,i for j; i,j for k
      const int max1 = n[dd], max2 = n[a2], max3 = n[a3];
      const int surfStart2 = 2 * a2 + 1, surfStart3 = 2 * a3 + 1;
      auto ijk = [&](int d1, int x2, int x3) {
        std::array<int, 3> c{};
        c[dd] = d1;
        c[a2] = x2;
        c[a3] = x3;
        return c;
      };
      for (int layer3 = 1; layer3 <= b.ng; ++layer3)
        for (int layer2 = 1; layer2 <= b.ng; ++layer2)
          for (int cc = 0; cc < 4; ++cc) {
            const bool upper2 = cc > 1, upper3 = cc % 2 == 1;
            const int pCellD2 = upper2 ? max2 + layer2 - 2 : 1 - layer2;
            const int gCellD2 = upper2 ? pCellD2 + 1 : pCellD2 - 1;
            const int pCellD3 = upper3 ? max3 + layer3 - 2 : 1 - layer3;
            const int gCellD3 = upper3 ? pCellD3 + 1 : pCellD3 - 1;
            const int surf2 = upper2 ? surfStart2 + 1 : surfStart2;
            const int surf3 = upper3 ? surfStart3 + 1 : surfStart3;
            const int cFaceD2_2 = upper2 ? max2 : 0;
            const int cFaceD2_3 = upper3 ? max3 - 1 : 0;
            const int cFaceD3_2 = upper2 ? max2 - 1 : 0;
            const int cFaceD3_3 = upper3 ? max3 : 0;
            const int phase = (layer3 - 1) * b.ng + (layer2 - 1);
            for (int d1 = 0; d1 < max1; ++d1) {
              const auto s2c = ijk(d1, cFaceD2_2, cFaceD2_3);
              const auto s3c = ijk(d1, cFaceD3_2, cFaceD3_3);
              const Surface &bs2 = SurfaceAt(b, s2c[0], s2c[1], s2c[2], surf2);
              const Surface &bs3 = SurfaceAt(b, s3c[0], s3c[1], s3c[2], surf3);
              const auto dst = ijk(d1, gCellD2, gCellD3);
              const auto from2 = ijk(d1, pCellD2, gCellD3);
              const auto from3 = ijk(d1, gCellD2, pCellD3);
              const auto f2 = ijk(d1, cFaceD2_2, gCellD3);  // face along a2
              const auto f3 = ijk(d1, gCellD2, cFaceD3_3);  // face along a3
              ath_ghost_op op{};
              op.dst = b.Cell(dst[0], dst[1], dst[2]);
              op.src_block = bi;
              op.layer = phase;
              op.state = -1;
              op.src2 = -1;
              auto slip2 = [&]() {
                op.type = ATH_EDGE_SLIP;
                op.src = b.Cell(from2[0], from2[1], from2[2]);
                op.dir = a2;
                op.face = b.Face(a2, f2[0], f2[1], f2[2]);
                op.lower = surf2 % 2 == 1;
              };
              auto slip3 = [&]() {
                op.type = ATH_EDGE_SLIP;
                op.src = b.Cell(from3[0], from3[1], from3[2]);
                op.dir = a3;
                op.face = b.Face(a3, f3[0], f3[1], f3[2]);
                op.lower = surf3 % 2 == 1;
              };
              auto average = [&]() {
                if (layer2 == layer3) {
                  op.type = ATH_EDGE_AVG;
                  op.src = b.Cell(from2[0], from2[1], from2[2]);
                  op.src2 = b.Cell(from3[0], from3[1], from3[2]);
                } else if (layer2 > layer3) {
                  op.type = ATH_EDGE_COPY;
                  op.src = b.Cell(from3[0], from3[1], from3[2]);
                } else {
                  op.type = ATH_EDGE_COPY;
                  op.src = b.Cell(from2[0], from2[1], from2[2]);
                }
              };
              // inviscid: viscous walls count as slip walls
              {
                const bool w2 = bs2.type == ATH_BC_SLIP_WALL || bs2.type == ATH_BC_VISCOUS_WALL;
                const bool w3 = bs3.type == ATH_BC_SLIP_WALL || bs3.type == ATH_BC_VISCOUS_WALL;
                if (w2 && !w3) slip2();
                else if (!w2 && w3) slip3();
                else average();
                b.edge_ops.push_back(op);
              }
              if (viscous) {
                op.src2 = -1;
                const bool s2 = bs2.type == ATH_BC_SLIP_WALL, s3 = bs3.type == ATH_BC_SLIP_WALL;
                const bool v2 = bs2.type == ATH_BC_VISCOUS_WALL, v3 = bs3.type == ATH_BC_VISCOUS_WALL;
                bool add = true;
                if (s2 && !s3) slip2();
                else if (!s2 && s3) slip3();
                else if (v2 && v3) average();
                else add = false;
                if (add) b.vedge_ops.push_back(op);
              }
            }
          }
    }
    auto by_phase = [](const ath_ghost_op &x, const ath_ghost_op &y) { return x.layer < y.layer; };
    std::stable_sort(b.edge_ops.begin(), b.edge_ops.end(), by_phase);
    std::stable_sort(b.vedge_ops.begin(), b.vedge_ops.end(), by_phase);
  }
}

// ---------------------------------------------------------------------------
// input file
// primitive::ApplyFarfieldTurbBC (src/primitive.cpp:83) with
// primitive::LimitTurb (:100): k = 1.5 (I |v|)^2, omega = rho k / (ratio mu(T)),
// floors 1e-20 (turbModel::TkeMin / OmegaMin, include/turbulence.hpp:63)
void FarfieldTurbulence(double *w, double tint, double ratio, const ath_solve_view &ph) {
  const double vmag = std::sqrt(w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
  w[5] = 1.5 * std::pow(tint * vmag, 2.0);
  const double t = w[4] / (w[0] * ph.gas_r);
  const double temp = t * ph.t_ref;
  const double mu = (ph.mu_c1 * std::pow(temp, 1.5)) / (temp + ph.mu_s) / ph.mu_ref;
  w[6] = w[0] * w[5] / (ratio * mu);
  w[5] = std::max(w[5], 1.0e-20);
  w[6] = std::max(w[6], 1.0e-20);
}

// procBlock::CalcWallDistance (src/procBlock.cpp:6030): distance of every
// physical cell centre to the nearest viscous-wall face centre of the solve
// (the reference's k-d tree returns the exact nearest neighbour: the
// minimum of |c - f|^2, then its square root); non-edge ghost cells take
// minus the mirrored interior value across a viscous wall, the value of the
// boundary cell elsewhere; edge ghosts keep the default 1e10.
// Nearest wall-face centre: a k-d tree over the centres (split on the axis
// of largest extent at the median), searched with the same squared distance
// dx*dx + dy*dy + dz*dz as an exhaustive scan, so the minimum is the same
// value (kdtree::NearestNeighbor, src/kdtree.cpp, is also an exact search).
class WallTree {
 public:
  explicit WallTree(std::vector<double> pts) : p_(std::move(pts)) {
    const size_t n = p_.size() / 3;
    idx_.resize(n);
    for (size_t q = 0; q < n; ++q) idx_[q] = (int32_t)q;
    axis_.assign(n, 0);
    Build(0, n);
  }
  double MinDist2(double x, double y, double z) const {
    double best = std::numeric_limits<double>::max();
    Search(0, idx_.size(), x, y, z, best);
    return best;
  }

 private:
  void Build(size_t lo, size_t hi) {
    if (hi - lo <= 1) return;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (size_t q = lo; q < hi; ++q)
      for (int e = 0; e < 3; ++e) {
        mn[e] = std::min(mn[e], p_[3 * idx_[q] + e]);
        mx[e] = std::max(mx[e], p_[3 * idx_[q] + e]);
      }
    int ax = 0;
    for (int e = 1; e < 3; ++e)
      if (mx[e] - mn[e] > mx[ax] - mn[ax]) ax = e;
    const size_t mid = (lo + hi) / 2;
    std::nth_element(idx_.begin() + lo, idx_.begin() + mid, idx_.begin() + hi,
                     [&](int32_t a, int32_t b) { return p_[3 * a + ax] < p_[3 * b + ax]; });
    axis_[mid] = (int8_t)ax;
    Build(lo, mid);
    Build(mid + 1, hi);
  }
  void Search(size_t lo, size_t hi, double x, double y, double z, double &best) const {
    if (lo >= hi) return;
    const size_t mid = (lo + hi) / 2;
    const double *c = &p_[3 * idx_[mid]];
    const double dx = x - c[0], dy = y - c[1], dz = z - c[2];
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < best) best = d2;
    if (hi - lo == 1) return;
    const int ax = axis_[mid];
    const double diff = (ax == 0 ? x : ax == 1 ? y : z) - c[ax];
    const bool left_first = diff < 0.0;
    Search(left_first ? lo : mid + 1, left_first ? mid : hi, x, y, z, best);
    // the other side can only hold a closer centre within |diff| of the plane
    if (diff * diff <= best) Search(left_first ? mid + 1 : lo, left_first ? hi : mid, x, y, z, best);
  }
  std::vector<double> p_;
  std::vector<int32_t> idx_;
  std::vector<int8_t> axis_;
};

// x, y, z of the centre of every viscous-wall face of a solve's blocks
std::vector<double> WallFaceCentres(const Setup &setup, int solve) {
  std::vector<double> wf;
  for (int bi : setup.solves[solve].blocks) {
    const Block &b = setup.blocks[bi];
    for (const auto &sf : b.surfs) {
      if (sf.type != ATH_BC_VISCOUS_WALL) continue;
      const int d = sf.Dir();
      const int64_t nf = b.NFace(d);
      const int ib = d == 0 ? sf.i1 + 1 : sf.i2;
      const int jb = d == 1 ? sf.j1 + 1 : sf.j2;
      const int kb = d == 2 ? sf.k1 + 1 : sf.k2;
      for (int k = sf.k1; k < kb; ++k)
        for (int j = sf.j1; j < jb; ++j)
          for (int i = sf.i1; i < ib; ++i) {
            const int64_t f = b.Face(d, i, j, k);
            wf.push_back(b.fcenter[d][f]);
            wf.push_back(b.fcenter[d][nf + f]);
            wf.push_back(b.fcenter[d][2 * nf + f]);
          }
    }
  }
  return wf;
}

// Wall distance of a solve's cells to the wall-face centres wf (by default
// its own walls; the coarse multigrid levels use the finest level's, as
// the reference's k-d tree of the finest faces serves every level,
// src/main.cpp:186-201)
void BuildWallDistance(Setup &setup, int solve, const std::vector<double> *faces = nullptr) {
  const std::vector<double> wf = faces ? *faces : WallFaceCentres(setup, solve);
  if (wf.empty()) return;
  std::unique_ptr<WallTree> tree;
  if (setup.geom_device < 0) tree.reset(new WallTree(wf));
  for (int bi : setup.solves[solve].blocks) {
    Block &b = setup.blocks[bi];
    const int64_t nc = b.NCell();
    if (tree) {
      for (int k = 0; k < b.nk; ++k)
        for (int j = 0; j < b.nj; ++j)
          for (int i = 0; i < b.ni; ++i) {
            const int64_t c = b.Cell(i, j, k);
            const double cx = b.center[c], cy = b.center[nc + c], cz = b.center[2 * nc + c];
            b.wall_dist[c] = std::sqrt(tree->MinDist2(cx, cy, cz));
          }
    } else {
      DeviceWallDistance(wf, b, setup.geom_device);
    }
    // boundary condition of the block face crossed by a non-edge ghost
    auto bc_at = [&](int d, bool lower, const int p[3]) {
      for (const auto &sf : b.surfs) {
        if (sf.Dir() != d || sf.Lower() != lower) continue;
        const int lo[3] = {sf.i1, sf.j1, sf.k1}, hi[3] = {sf.i2, sf.j2, sf.k2};
        bool in = true;
        for (int e = 0; e < 3; ++e)
          if (e != d && (p[e] < lo[e] || p[e] >= hi[e])) in = false;
        if (in) return sf.type;
      }
      return -1;
    };
    const int n3[3] = {b.ni, b.nj, b.nk};
    for (int k = -b.ng; k < b.nk + b.ng; ++k)
      for (int j = -b.ng; j < b.nj + b.ng; ++j)
        for (int i = -b.ng; i < b.ni + b.ng; ++i) {
          const int p[3] = {i, j, k};
          int d = -1, nout = 0;
          for (int e = 0; e < 3; ++e)
            if (p[e] < 0 || p[e] >= n3[e]) {
              d = e;
              ++nout;
            }
          if (nout != 1) continue;
          const bool lower = p[d] < 0;
          int q[3] = {i, j, k};
          if (bc_at(d, lower, p) == ATH_BC_VISCOUS_WALL) {
            q[d] = lower ? -p[d] - 1 : n3[d] - (p[d] - n3[d] + 1);
            b.wall_dist[b.Cell(i, j, k)] = -1.0 * b.wall_dist[b.Cell(q[0], q[1], q[2])];
          } else {
            q[d] = lower ? 0 : n3[d] - 1;
            b.wall_dist[b.Cell(i, j, k)] = b.wall_dist[b.Cell(q[0], q[1], q[2])];
          }
        }
  }
  // connection ghosts take the partner's value (SwapWallDistSlice,
  // src/procBlock.cpp:3105); block-edge ghosts are left as they are
  for (int bi : setup.solves[solve].blocks) {
    Block &b = setup.blocks[bi];
    for (const auto &op : b.ops)
      if (op.type == ATH_BC_PERIODIC || op.type == ATH_BC_INTERBLOCK)
        b.wall_dist[op.dst] = setup.blocks[op.src_block].wall_dist[op.src];
  }
}

// ---------------------------------------------------------------------------
// Multigrid levels (gridLevel::Coarsen, src/gridLevel.cpp:440-535;
// procBlock::GetCoarseMeshAndBCs, src/procBlock.cpp:6471-6590).

// std::inner_product's order: the sum starts from zero
inline double DotIP(V3 a, V3 b) { return ((0.0 + a.x * b.x) + a.y * b.y) + a.z * b.z; }
inline double MagIP(V3 a) { return std::sqrt(DotIP(a, a)); }

// LinearInterpCoeff (src/utility.cpp:625): the position of x along x0 -> x1
double LinearCoeff(V3 x0, V3 x1, V3 x) {
  const V3 d = x1 - x0;
  const double m = MagIP(d);
  const V3 dir{d.x / m, d.y / m, d.z / m};
  const double dist = MagIP(x0 - x1);
  return DotIP(x - x0, dir) / dist;
}
V3 LinearAt(V3 x0, V3 x1, double c) { return (1.0 - c) * x0 + c * x1; }

// The node indices of one direction a coarse level keeps: every node a
// boundary surface starts or ends on, and otherwise every other node; with
// the surfaces' indices along that direction renumbered on the copy
std::vector<int> KeptNodes(const Block &fb, int dir, std::vector<Surface> &coarse_surfs) {
  const int nn = (dir == 0 ? fb.ni : dir == 1 ? fb.nj : fb.nk) + 1;
  std::vector<int> keep;
  int since = 0;
  for (int n = 0; n < nn; ++n) {
    bool boundary = false;
    for (const auto &sf : fb.surfs) {
      const int lo = dir == 0 ? sf.i1 : dir == 1 ? sf.j1 : sf.k1;
      const int hi = dir == 0 ? sf.i2 : dir == 1 ? sf.j2 : sf.k2;
      if (lo == n || hi == n) boundary = true;
    }
    if (boundary) {
      keep.push_back(n);
      const int m = (int)keep.size() - 1;
      for (auto &sf : coarse_surfs) {
        int &lo = dir == 0 ? sf.i1 : dir == 1 ? sf.j1 : sf.k1;
        int &hi = dir == 0 ? sf.i2 : dir == 1 ? sf.j2 : sf.k2;
        if (lo == n) lo = m;
        if (hi == n) hi = m;
      }
      since = 0;
    } else if (since > 0) {
      keep.push_back(n);
      since = 0;
    } else {
      ++since;
    }
  }
  return keep;
}

// The coarse block of fine block fb (nodes and renumbered surfaces) and
// fb's fine-to-coarse cell map and volume weights; the prolongation
// coefficients need the coarse nodes and are formed by MgCoefficients
Block CoarsenBlock(Block &fb) {
  Block cb;
  cb.surfs = fb.surfs;
  std::vector<int> keep[3];
  for (int d = 0; d < 3; ++d) keep[d] = KeptNodes(fb, d, cb.surfs);
  cb.ni = (int)keep[0].size() - 1;
  cb.nj = (int)keep[1].size() - 1;
  cb.nk = (int)keep[2].size() - 1;
  const size_t cnn = (size_t)(cb.ni + 1) * (cb.nj + 1) * (cb.nk + 1);
  cb.nodes.assign(3 * cnn, 0.0);
  for (int k = 0; k <= cb.nk; ++k)
    for (int j = 0; j <= cb.nj; ++j)
      for (int i = 0; i <= cb.ni; ++i) {
        const size_t o = (size_t)i + (size_t)(cb.ni + 1) * (j + (size_t)(cb.nj + 1) * k);
        for (int c = 0; c < 3; ++c) cb.nodes[c * cnn + o] = fb.Node(c, keep[0][i], keep[1][j], keep[2][k]);
      }
  // coarse cell of each fine cell: the last kept node at or below it
  auto coarse_of = [](const std::vector<int> &kp, int f) {
    int pos = 0;
    while (pos < (int)kp.size() && !(kp[pos] > f)) ++pos;
    return pos != 0 ? pos - 1 : pos;
  };
  const int64_t nfc = (int64_t)fb.ni * fb.nj * fb.nk;
  fb.mg_cell.assign(nfc, 0);
  fb.mg_volfac.assign(nfc, 0.0);
  const int64_t ncc = (int64_t)cb.ni * cb.nj * cb.nk;
  std::vector<double> vsum(ncc, 0.0);
  int64_t x = 0;
  for (int k = 0; k < fb.nk; ++k)
    for (int j = 0; j < fb.nj; ++j)
      for (int i = 0; i < fb.ni; ++i, ++x) {
        const int ci = coarse_of(keep[0], i), cj = coarse_of(keep[1], j),
                  ck = coarse_of(keep[2], k);
        fb.mg_cell[x] = ci + cb.ni * (cj + cb.nj * ck);
      }
  // fine volumes summed per coarse cell in the fine cells' k, j, i order
  x = 0;
  for (int k = 0; k < fb.nk; ++k)
    for (int j = 0; j < fb.nj; ++j)
      for (int i = 0; i < fb.ni; ++i, ++x) vsum[fb.mg_cell[x]] += fb.vol[fb.Cell(i, j, k)];
  x = 0;
  for (int k = 0; k < fb.nk; ++k)
    for (int j = 0; j < fb.nj; ++j)
      for (int i = 0; i < fb.ni; ++i, ++x)
        fb.mg_volfac[x] = fb.vol[fb.Cell(i, j, k)] / vsum[fb.mg_cell[x]];
  return cb;
}

// TrilinearInterpCoeff (src/utility.cpp:633) of every fine cell centre in
// the hexahedron of its coarse cell's nodes
void MgCoefficients(Block &fb, const Block &cb) {
  const int64_t nfc = (int64_t)fb.ni * fb.nj * fb.nk;
  const int64_t nc = fb.NCell();
  fb.mg_coef.assign(7 * nfc, 0.0);
  int64_t x = 0;
  for (int k = 0; k < fb.nk; ++k)
    for (int j = 0; j < fb.nj; ++j)
      for (int i = 0; i < fb.ni; ++i, ++x) {
        const int cc = fb.mg_cell[x];
        const int ci = cc % cb.ni, cj = (cc / cb.ni) % cb.nj, ck = cc / (cb.ni * cb.nj);
        const V3 c0 = NodeV(cb, ci, cj, ck), c1 = NodeV(cb, ci + 1, cj, ck),
                 c2 = NodeV(cb, ci, cj + 1, ck), c3 = NodeV(cb, ci + 1, cj + 1, ck),
                 c4 = NodeV(cb, ci, cj, ck + 1), c5 = NodeV(cb, ci + 1, cj, ck + 1),
                 c6 = NodeV(cb, ci, cj + 1, ck + 1), c7 = NodeV(cb, ci + 1, cj + 1, ck + 1);
        const int64_t c = fb.Cell(i, j, k);
        const V3 p{fb.center[c], fb.center[nc + c], fb.center[2 * nc + c]};
        double *co = &fb.mg_coef[7 * x];
        co[0] = LinearCoeff(c0, c4, p);
        const V3 x04 = LinearAt(c0, c4, co[0]);
        co[1] = LinearCoeff(c1, c5, p);
        const V3 x15 = LinearAt(c1, c5, co[1]);
        co[2] = LinearCoeff(c2, c6, p);
        const V3 x26 = LinearAt(c2, c6, co[2]);
        co[3] = LinearCoeff(c3, c7, p);
        const V3 x37 = LinearAt(c3, c7, co[3]);
        co[4] = LinearCoeff(x04, x15, p);
        const V3 x0415 = LinearAt(x04, x15, co[4]);
        co[5] = LinearCoeff(x26, x37, p);
        const V3 x2637 = LinearAt(x26, x37, co[5]);
        co[6] = LinearCoeff(x0415, x2637, p);
      }
}

// Levels 1 .. L-1 of a solve: each level's blocks from the finer level's
// (CoarsenBlock), then the same geometry, boundary and connection
// bookkeeping as the finest level (the coarse procBlocks are built from
// their plot3dBlock and boundary conditions like the fine ones,
// src/gridLevel.cpp:455-500), with the wall distance to the finest level's
// wall faces
void BuildCoarseLevels(Setup &st, int solve) {
  const int nl = st.solves[solve].phys.mg_levels;
  std::vector<double> wf;
  if (st.solves[solve].phys.eqn != ATH_EQN_EULER) wf = WallFaceCentres(st, solve);
  Setup *fine = &st;
  int fsolve = solve;
  for (int l = 1; l < nl; ++l) {
    while ((int)st.levels.size() < l) {
      st.levels.emplace_back(new Setup());
      st.levels.back()->geom_device = st.geom_device;
    }
    Setup &cs = *st.levels[l - 1];
    const int csolve = (int)cs.solves.size();
    Solve csv = fine->solves[fsolve];
    csv.blocks.clear();
    for (int fbi : fine->solves[fsolve].blocks) {
      Block &fb = fine->blocks[fbi];
      Block cb = CoarsenBlock(fb);
      cb.ng = fb.ng;
      cb.nv = fb.nv;
      cb.solve = csolve;
      BuildGeometry(cb, st.geom_device);
      BuildGhostGeometry(cb);
      BuildHyperplanes(cb);
      MgCoefficients(fb, cb);
      // initial state: the volume-weighted restriction of the fine one
      // (the coarse level's state is replaced by a restriction before each
      // use)
      cb.state0.assign((size_t)cb.NCell() * cb.nv, 0.0);
      int64_t x = 0;
      for (int k = 0; k < fb.nk; ++k)
        for (int j = 0; j < fb.nj; ++j)
          for (int i = 0; i < fb.ni; ++i, ++x) {
            const int cc = fb.mg_cell[x];
            const int ci = cc % cb.ni, cj = (cc / cb.ni) % cb.nj, ck = cc / (cb.ni * cb.nj);
            const int64_t o = cb.Cell(ci, cj, ck) * cb.nv, f = fb.Cell(i, j, k) * fb.nv;
            for (int v = 0; v < cb.nv; ++v) cb.state0[o + v] += fb.mg_volfac[x] * fb.state0[f + v];
          }
      fb.mg_coarse = (int)cs.blocks.size();
      csv.blocks.push_back((int)cs.blocks.size());
      cs.blocks.push_back(std::move(cb));
    }
    cs.solves.push_back(std::move(csv));
    BuildGhostOps(cs, csolve);
    BuildEdgeOps(cs, csolve);
    for (int bi : cs.solves[csolve].blocks) BuildCellWidths(cs.blocks[bi]);
    if (!wf.empty()) BuildWallDistance(cs, csolve, &wf);
    fine = &cs;
    fsolve = csolve;
  }
}

void AppendInput(Setup &st, const std::string &path) {
  std::ifstream in(path);
  if (!in) Fail("cannot open input file " + path);
  std::map<std::string, std::string> kv;
  std::vector<std::string> bc_lines;
  std::string line;
  std::string pending_key, pending_val;
  bool reading_bcs = false;
  while (std::getline(in, line)) {
    const auto hash = line.find('#');
    if (hash != std::string::npos) line = line.substr(0, hash);
    line = Trim(line);
    if (line.empty()) continue;
    if (!pending_key.empty()) {
      pending_val += " " + line;
      if (line.find('>') != std::string::npos) {
        kv[pending_key] = pending_val;
        pending_key.clear();
      }
      continue;
    }
    if (reading_bcs) {
      bc_lines.push_back(line);
      continue;
    }
    const auto colon = line.find(':');
    if (colon == std::string::npos) Fail("cannot parse input line '" + line + "'");
    const auto key = Trim(line.substr(0, colon));
    const auto val = Trim(line.substr(colon + 1));
    if (key == "boundaryConditions") {
      kv[key] = val;
      reading_bcs = true;
      continue;
    }
    if (val.find('<') != std::string::npos && val.find('>') == std::string::npos) {
      pending_key = key;
      pending_val = val;
      continue;
    }
    kv[key] = val;
  }
  auto get = [&](const std::string &k, const std::string &def) {
    auto it = kv.find(k);
    return it == kv.end() ? def : it->second;
  };
  auto getd = [&](const std::string &k, double def) {
    auto it = kv.find(k);
    return it == kv.end() ? def : std::stod(it->second);
  };

  Solve sv;
  sv.name = path;
  {
    // input::SimNameRoot (src/input.cpp:872) and the output keys
    // (src/input.cpp:321-327,463-467); the default output set is the
    // reference's
    const auto slash = path.find_last_of('/');
    const auto file = slash == std::string::npos ? path : path.substr(slash + 1);
    sv.sim_root = file.substr(0, file.find('.'));
    sv.grid_name = get("gridName", "");
    sv.output_freq = (int)getd("outputFrequency", 1);
    sv.restart_freq = (int)getd("restartFrequency", 0);
    sv.iterations = (int)getd("iterations", 1);
    std::set<std::string> vars = {"density", "vel_x", "vel_y", "vel_z", "pressure"};
    const auto ov = get("outputVariables", "");
    if (!ov.empty()) {
      vars.clear();
      std::string body = ov;
      const auto a = body.find('<'), z = body.rfind('>');
      if (a != std::string::npos && z != std::string::npos && z > a)
        body = body.substr(a + 1, z - a - 1);
      std::stringstream ss(body);
      std::string tok;
      while (std::getline(ss, tok, ',')) {
        tok = Trim(tok);
        if (!tok.empty()) vars.insert(tok);
      }
    }
    sv.output_vars.assign(vars.begin(), vars.end());
    // fluids: <fluid(name=air; ...)> -- one species, whose properties are
    // read from <name>.dat
    const auto fl = get("fluids", "");
    const auto np = fl.find("name=");
    if (np != std::string::npos) {
      auto e = fl.find_first_of(";) ", np + 5);
      sv.species = Trim(fl.substr(np + 5, e == std::string::npos ? std::string::npos : e - np - 5));
      if (fl.find("fluid(", fl.find("fluid(") + 1) != std::string::npos)
        Fail("only one fluid species is supported");
    }
  }
  auto &ph = sv.phys;
  // scheme
  const auto eqn = get("equationSet", "euler");
  ph.eqn = eqn == "euler" ? ATH_EQN_EULER
           : eqn == "navierStokes" ? ATH_EQN_NAVIER_STOKES
           : eqn == "rans" ? ATH_EQN_RANS
           : (Fail("unsupported equationSet " + eqn), 0);
  // input::ReadInput (src/input.cpp:255-267): theta and zeta of the
  // implicit schemes; nonlinear iterations per time step (:353)
  const auto ti = get("timeIntegration", "explicitEuler");
  ph.multilevel = 0;
  if (ti == "implicitEuler") {
    ph.theta = 1.0;
    ph.zeta = 0.0;
  } else if (ti == "crankNicholson") {
    ph.theta = 0.5;
    ph.zeta = 0.0;
  } else if (ti == "bdf2") {
    ph.theta = 1.0;
    ph.zeta = 0.5;
    ph.multilevel = 1;
  } else {
    Fail("only the implicit time integrations (implicitEuler, crankNicholson, bdf2) are "
         "supported");
  }
  ph.nl_iters = (int)getd("nonlinearIterations", 1);
  if (ph.nl_iters < 1) Fail("nonlinearIterations must be at least 1");
  ph.dual_cfl = getd("dualTimeCFL", -1.0) > 0.0 ? getd("dualTimeCFL", -1.0) : 0.0;
  const auto fr = get("faceReconstruction", "constant");
  ph.kappa = -2.0;
  if (fr == "upwind") { ph.recon = ATH_RECON_MUSCL; ph.kappa = -1.0; }
  else if (fr == "fromm") { ph.recon = ATH_RECON_MUSCL; ph.kappa = 0.0; }
  else if (fr == "quick") { ph.recon = ATH_RECON_MUSCL; ph.kappa = 0.5; }
  else if (fr == "central") { ph.recon = ATH_RECON_MUSCL; ph.kappa = 1.0; }
  else if (fr == "thirdOrder") { ph.recon = ATH_RECON_MUSCL; ph.kappa = 1.0 / 3.0; }
  else if (fr == "constant") { ph.recon = ATH_RECON_CONSTANT; }
  else if (fr == "weno") { ph.recon = ATH_RECON_WENO; }
  else if (fr == "wenoZ") { ph.recon = ATH_RECON_WENOZ; }
  else Fail("unsupported faceReconstruction " + fr);

  const auto lim = get("limiter", "none");
  ph.limiter = lim == "none" ? ATH_LIMITER_NONE
               : lim == "minmod" ? ATH_LIMITER_MINMOD
               : lim == "vanAlbada" ? ATH_LIMITER_VANALBADA
               : (Fail("unsupported limiter " + lim), 0);
  const auto flux = get("inviscidFlux", "roe");
  ph.flux = flux == "roe" ? ATH_FLUX_ROE : flux == "ausm" ? ATH_FLUX_AUSM
            : (Fail("unsupported inviscidFlux " + flux), 0);

  const auto ms = get("matrixSolver", "lusgs");
  ph.solver = ms == "lusgs" ? ATH_SOLVER_LUSGS : ms == "blusgs" ? ATH_SOLVER_BLUSGS
              : ms == "dplur" ? ATH_SOLVER_DPLUR : ms == "bdplur" ? ATH_SOLVER_BDPLUR
              : (Fail("unsupported matrixSolver " + ms), 0);
  ph.sweeps = (int)getd("matrixSweeps", 1);
  if (ph.sweeps < 1) Fail("matrixSweeps must be at least 1");
  ph.relax = getd("matrixRelaxation", 1.0);
  ph.cfl_start = getd("cflStart", 1.0);
  ph.cfl_step = getd("cflStep", 0.0);
  ph.cfl_max = getd("cflMax", 1.0);
  if (get("inviscidFluxJacobian", "rusanov") != "rusanov")
    Fail("only the rusanov inviscid flux jacobian is supported");
  // physics models this build implements: one calorically perfect ideal gas
  // with Sutherland transport, frozen chemistry, central viscous face values
  // (the reference's defaults, src/input.cpp:59-95); anything else would
  // silently change the arithmetic, so it is refused
  for (const auto &kd : {std::make_pair("thermodynamicModel", "caloricallyPerfect"),
                         std::make_pair("equationOfState", "idealGas"),
                         std::make_pair("transportModel", "sutherland"),
                         std::make_pair("diffusionModel", "none"),
                         std::make_pair("chemistryModel", "frozen"),
                         std::make_pair("viscousFaceReconstruction", "central")})
    if (get(kd.first, kd.second) != kd.second)
      Fail(std::string("only ") + kd.first + " " + kd.second + " is supported");
  // multigrid (input::ReadInput src/input.cpp:437-455, CheckMultigrid
  // :1042): grid levels and the cycle (input::MultigridCycleIndex,
  // include/input.hpp:281: W visits each coarser level twice per visit of
  // its finer one, V once)
  ph.mg_levels = (int)getd("multigridLevels", 1);
  if (ph.mg_levels < 1) Fail("multigridLevels must be >= 1");
  {
    const auto cyc = get("multigridCycle", "V");
    if (cyc != "V" && cyc != "W") Fail("multigridCycle must be 'V' or 'W'");
    ph.mg_cycle = cyc == "W" ? 2 : 1;
  }
  const auto tm = get("turbulenceModel", "none");
  if (tm != "none" && ph.eqn != ATH_EQN_RANS) Fail("turbulence model needs equationSet rans");
  ph.turb = ATH_TURB_NONE;
  if (ph.eqn == ATH_EQN_RANS) {
    // input::AssignTurbulenceModel (src/input.cpp): sst2003, kOmegaWilcox2006
    if (tm == "sst2003") ph.turb = ATH_TURB_SST2003;
    else if (tm == "kOmegaWilcox2006") ph.turb = ATH_TURB_KW2006;
    else Fail("only turbulenceModel sst2003 and kOmegaWilcox2006 are supported");
  }
  ph.nv = ph.eqn == ATH_EQN_RANS ? 7 : 5;
  // input::NumberGhostLayers (src/input.cpp:1127): 1 constant, 2 MUSCL, 3 WENO
  ph.ng = ph.recon == ATH_RECON_CONSTANT ? 1 : (ph.recon == ATH_RECON_MUSCL ? 2 : 3);

  // fluid and references
  Fluid fl;
  {
    const auto dir = DirName(path);
    const std::string file = sv.species + ".dat";
    if (!ReadFluidFile(dir + "/" + file, fl)) {
      const char *inst = std::getenv("AITHER_INSTALL_DIRECTORY");
      if (inst) ReadFluidFile(std::string(inst) + "/fluidDatabase/" + file, fl);
    }
  }
  const double tref = getd("referenceTemperature", -1.0);
  const double rref = getd("referenceDensity", -1.0);
  const double lref = getd("referenceLength", 1.0);
  if (!(tref > 0) || !(rref > 0)) Fail("reference temperature and density are required");
  const double ru = 8.3144598;  // J/mol-K
  const double gas_const_dim = ru / fl.molar_mass;
  double aref = 0.0;
  {
    const double gamma = (fl.n + 1) / fl.n;
    aref += 1.0 * gamma * gas_const_dim * tref;
    aref = std::sqrt(aref);
  }
  const double hf_nd = fl.hf / (fl.molar_mass * (aref * aref));
  const double mm_nd = fl.molar_mass / (rref / std::pow(lref, 3.0));
  const double ru_nd = ru / (aref * aref * rref / (tref * std::pow(lref, 3.0)));
  ph.gas_r = ru_nd / mm_nd;
  ph.gas_n = fl.n;
  ph.gas_hf = hf_nd;
  ph.mu_c1 = fl.mu_c1;
  ph.mu_s = fl.mu_s;
  ph.k_c1 = fl.k_c1;
  ph.k_s = fl.k_s;
  ph.t_ref = tref;
  // sutherland ctor (src/transport.cpp:31): mixture reference viscosity,
  // conductivity reference, and transport::SetScaling mu/(rho a l)
  ph.mu_ref = fl.mu_c1 * std::pow(tref, 1.5) / (tref + fl.mu_s);
  ph.k_ref = (aref * aref * ph.mu_ref) / tref;
  ph.r_ref = rref;
  ph.a_ref = aref;
  ph.l_ref = lref;
  ph.visc_scale = ph.mu_ref / (rref * aref * lref);
  // global time step, nondimensional (procBlock::CalcBlockTimeStep,
  // src/procBlock.cpp:808)
  ph.dt_global = getd("timeStep", -1.0) > 0.0 ? getd("timeStep", -1.0) * aref / lref : 0.0;
  sv.time_step = getd("timeStep", -1.0);
  ph.visc_cfl_coeff = ph.kappa == 1.0 ? 4.0 : (ph.kappa == -2.0 ? 2.0 : 1.0);

  // boundary states
  const double pscale = rref * aref * aref;
  for (auto &call : SplitList(get("boundaryStates", "<>"))) {
    auto pc = ParseCall(call);
    BCStateIn si;
    auto &s = si.s;
    const auto &name = pc.first;
    auto &m = pc.second;
    auto num = [&](const char *k, double def) {
      auto it = m.find(k);
      return it == m.end() ? def : std::stod(it->second);
    };
    if (name == "periodic") {
      s.type = ATH_BC_PERIODIC;
      si.start_tag = (int)num("startTag", -1);
      si.end_tag = (int)num("endTag", -1);
      if (m.count("translation")) {
        ParseVec3(m["translation"], si.translation);
        for (auto &t : si.translation) t = t / lref;
      } else {
        Fail("only translational periodic boundaries are supported");
      }
      s.tag = si.start_tag;
    } else {
      s.type = BCType(name);
      s.tag = (int)num("tag", -1);
      // DEFAULT_TURB_INTENSITY / DEFAULT_EDDY_VISC_RATIO (include/inputStates.hpp:41)
      s.turb_intensity = 0.01;
      s.eddy_visc_ratio = 0.01;
      if (m.count("density")) s.rho = std::stod(m["density"]) / rref;
      if (m.count("pressure")) {
        s.p = std::stod(m["pressure"]) / pscale;
        s.p_out = s.p;
      }
      if (m.count("velocity")) {
        double v[3];
        ParseVec3(m["velocity"], v);
        if (s.type == ATH_BC_VISCOUS_WALL) {
          s.wall_u = v[0] / aref; s.wall_v = v[1] / aref; s.wall_w = v[2] / aref;
        } else {
          s.u = v[0] / aref; s.v = v[1] / aref; s.w = v[2] / aref;
        }
      }
      if (m.count("p0")) s.p0 = std::stod(m["p0"]) / pscale;
      if (m.count("t0")) s.t0 = std::stod(m["t0"]) / tref;
      if (m.count("direction")) {
        ParseVec3(m["direction"], s.dir);
        const double mg = std::sqrt(s.dir[0] * s.dir[0] + s.dir[1] * s.dir[1] +
                                    s.dir[2] * s.dir[2]);
        for (auto &x : s.dir) x = x / mg;
      }
      if (m.count("temperature")) {
        s.isothermal = 1;
        s.wall_t = std::stod(m["temperature"]) / tref;
      }
      if (m.count("heatFlux")) {
        // viscousWall::Nondimensionalize (src/inputStates.cpp:775)
        s.heat_flux = 1;
        s.wall_q = std::stod(m["heatFlux"]) / std::pow(aref / lref, 3.0);
      }
      // inlet / pressureOutlet: nonreflecting=true with lengthScale
      // (inlet::AssignExtraData, pressureOutlet ctor src/inputStates.cpp:475,
      // 615; the length is divided by the reference length)
      if (m.count("nonreflecting")) {
        if (name != "inlet" && name != "pressureOutlet")
          Fail("nonreflecting is an inlet / pressureOutlet parameter");
        s.nonreflecting = m["nonreflecting"] == "true" ? 1 : 0;
      }
      if (m.count("lengthScale")) s.length_scale = std::stod(m["lengthScale"]) / lref;
      if (s.nonreflecting && !m.count("lengthScale"))
        Fail("lengthScale must be specified with nonreflecting");
      if (m.count("wallTreatment") && m["wallTreatment"] != "lowRe")
        Fail("wall laws are not supported");
      if (m.count("turbulenceIntensity")) s.turb_intensity = num("turbulenceIntensity", 0);
      if (m.count("eddyViscosityRatio")) s.eddy_visc_ratio = num("eddyViscosityRatio", 0);
    }
    sv.states_in.push_back(si);
    sv.states.push_back(s);
  }

  // initial conditions: uniform icStates, one per block tag or a default
  // (tag -1) for the others (input::ICStateForBlock src/input.cpp:1146:
  // an exact tag match wins over the default)
  struct IcIn {
    int tag;
    double w[7];
  };
  std::vector<IcIn> ics;
  for (auto &call : SplitList(get("initialConditions", "<>"))) {
    auto pc = ParseCall(call);
    auto &m = pc.second;
    if (m.count("file")) continue;  // point clouds: state set by caller
    IcIn x{};
    x.tag = m.count("tag") ? std::stoi(m["tag"]) : -1;
    double v[3] = {0, 0, 0};
    if (m.count("velocity")) ParseVec3(m["velocity"], v);
    x.w[0] = std::stod(m["density"]) / rref;
    x.w[1] = v[0] / aref;
    x.w[2] = v[1] / aref;
    x.w[3] = v[2] / aref;
    x.w[4] = std::stod(m["pressure"]) / pscale;
    const double tint = m.count("turbulenceIntensity") ? std::stod(m["turbulenceIntensity"]) : 0.01;
    const double vrat = m.count("eddyViscosityRatio") ? std::stod(m["eddyViscosityRatio"]) : 0.01;
    if (ph.nv == 7) FarfieldTurbulence(x.w, tint, vrat, ph);
    ics.push_back(x);
  }
  auto ic_for_block = [&](int blk) -> const IcIn * {
    const IcIn *pick = nullptr;
    for (auto &x : ics) {
      if (x.tag == blk) return &x;
      if (x.tag == -1 && !pick) pick = &x;
    }
    return pick;
  };
  IcIn ic_none{};
  ic_none.w[0] = 1.0;
  ic_none.w[4] = 1.0 / 1.4;
  if (ph.nv == 7) FarfieldTurbulence(ic_none.w, 0.01, 0.01, ph);

  // grid
  const auto grid = DirName(path) + "/" + get("gridName", "") + ".xyz";
  auto blocks = ReadPlot3d(grid, lref);

  // boundary conditions table: number of blocks, then per block a line
  // with the surface counts (i, j, k) followed by the surfaces
  {
    size_t li = 0;
    const int nbc = std::stoi(kv["boundaryConditions"]);
    if (nbc != (int)blocks.size())
      Fail("boundaryConditions block count does not match the grid");
    for (int b = 0; b < nbc; ++b) {
      if (li >= bc_lines.size()) Fail("truncated boundaryConditions");
      std::istringstream cnt(bc_lines[li++]);
      int ci = 0, cj = 0, ck = 0;
      cnt >> ci >> cj >> ck;
      for (int s = 0; s < ci + cj + ck; ++s) {
        if (li >= bc_lines.size()) Fail("truncated boundaryConditions");
        std::istringstream is(bc_lines[li++]);
        Surface sf;
        is >> sf.name >> sf.i1 >> sf.i2 >> sf.j1 >> sf.j2 >> sf.k1 >> sf.k2 >> sf.tag;
        if (!is) Fail("bad boundary surface line");
        sf.type = BCType(sf.name);
        blocks[b].surfs.push_back(sf);
      }
    }
  }

  const int solve = (int)st.solves.size();
  const int first = (int)st.blocks.size();
  int bidx = 0;
  for (auto &b : blocks) {
    const IcIn *icb = ics.empty() ? &ic_none : ic_for_block(bidx);
    if (!icb)
      Fail("no initial condition for block " + std::to_string(bidx) +
           " (neither its tag nor a default, tag -1)");
    const double *ic = icb->w;
    ++bidx;
    b.ng = ph.ng;
    b.nv = ph.nv;
    b.solve = solve;
    BuildGeometry(b, st.geom_device);
    BuildGhostGeometry(b);
    BuildHyperplanes(b);
    b.state0.assign((size_t)b.NCell() * b.nv, 0.0);
    for (int k = 0; k < b.nk; ++k)
      for (int j = 0; j < b.nj; ++j)
        for (int i = 0; i < b.ni; ++i)
          for (int v = 0; v < b.nv; ++v)
            b.state0[(size_t)b.Cell(i, j, k) * b.nv + v] = ic[v];
    sv.blocks.push_back((int)st.blocks.size());
    st.blocks.push_back(std::move(b));
  }
  (void)first;
  st.solves.push_back(std::move(sv));
  BuildGhostOps(st, solve);
  BuildEdgeOps(st, solve);
  // widths from the face centres of the assembled geometry, ghosts included
  // (gridLevel::AuxillaryAndWidths src/gridLevel.cpp:431, after the
  // connection swaps)
  for (int bi : st.solves[solve].blocks) BuildCellWidths(st.blocks[bi]);
  // procBlock::CalcWallDistance (src/procBlock.cpp:6030) runs for every case
  // with viscous walls (src/main.cpp:200); without walls the distance keeps
  // its default of 1e10
  if (st.solves[solve].phys.eqn != ATH_EQN_EULER) BuildWallDistance(st, solve);
  if (ph.mg_levels > 1) {
    // the coarse levels' forcing enters the mean-flow equations of steady
    // solves here: turbulence equations, time-accurate terms and the
    // nonreflecting boundaries' time levels are not carried to them
    const auto &p = st.solves[solve].phys;
    if (p.eqn == ATH_EQN_RANS) Fail("multigrid with the turbulence equations is not supported");
    if (p.multilevel || p.nl_iters > 1)
      Fail("multigrid is supported for steady solves (one nonlinear iteration per step)");
    for (const auto &bs : st.solves[solve].states)
      if (bs.nonreflecting) Fail("multigrid with nonreflecting boundaries is not supported");
    BuildCoarseLevels(st, solve);
  }
}

}  // namespace ath
