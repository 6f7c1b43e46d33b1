// Setup on the device: the geometry of a block's physical cells and faces
// (procBlock constructor, src/procBlock.cpp:59 -> plot3dBlock::Volume,
// Centroid, FaceAreaI/J/K, FaceCenterI/J/K, src/plot3d.cpp:60-360) and the
// wall distance of its physical cells (procBlock::CalcWallDistance,
// src/procBlock.cpp:6030), computed by kernels instead of host loops.
//
// The arithmetic is the host setup's (setup.cpp BuildGeometry /
// BuildWallDistance) operation for operation; this unit is built with
// --fmad=false and the host with -ffp-contract=off, so every value is the
// same bit for bit.  The wall distance is the square root of the smallest
// squared distance to a viscous-wall face centre: the host finds it with a
// k-d tree, the device by comparing every centre, and both take the
// minimum of the same set of values.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "cuda_check.hpp"
#include "errors.hpp"
#include "setup.hpp"

namespace ath {
namespace {

struct DV3 {
  double x, y, z;
};
__device__ __forceinline__ DV3 Add(DV3 a, DV3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ DV3 Sub(DV3 a, DV3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ DV3 Scale(double s, DV3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double Dot(DV3 a, DV3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ DV3 Cross(DV3 a, DV3 b) {
  return {a.y * b.z - a.z * b.y, -1.0 * (a.x * b.z - a.z * b.x), a.x * b.y - a.y * b.x};
}

struct NodesDev {
  const double *x;  // [3][(ni+1)(nj+1)(nk+1)]
  int ni, nj, nk;
  __device__ DV3 At(int i, int j, int k) const {
    const size_t n = (size_t)(ni + 1) * (nj + 1) * (nk + 1);
    const size_t q = (size_t)i + (size_t)(ni + 1) * (j + (size_t)(nj + 1) * k);
    return {x[q], x[n + q], x[2 * n + q]};
  }
};

struct PadDev {
  int ng, NI, NJ, NK;
  __device__ int64_t Cell(int i, int j, int k) const {
    return (int64_t)(i + ng) + (int64_t)NI * ((j + ng) + (int64_t)NJ * (k + ng));
  }
  __device__ int64_t Face(int d, int i, int j, int k) const {
    const int fi = NI + (d == 0), fj = NJ + (d == 1);
    return (int64_t)(i + ng) + (int64_t)fi * ((j + ng) + (int64_t)fj * (k + ng));
  }
  __device__ int64_t NFace(int d) const {
    return (int64_t)(NI + (d == 0)) * (NJ + (d == 1)) * (NK + (d == 2));
  }
  __device__ int64_t NCell() const { return (int64_t)NI * NJ * NK; }
};

__device__ __forceinline__ double Pyramid(DV3 p, DV3 a, DV3 b, DV3 c, DV3 d) {
  const DV3 xp = Scale(0.25, Add(Add(Add(Sub(a, p), Sub(b, p)), Sub(c, p)), Sub(d, p)));
  const DV3 xac = Sub(c, a);
  const DV3 xbd = Sub(d, b);
  return 1.0 / 6.0 * Dot(xp, Cross(xac, xbd));
}

// volume (six pyramids about the centroid) and centroid (mean of the eight
// nodes) of every physical cell; *bad counts non-positive volumes
__global__ void k_geom_cells(NodesDev N, PadDev B, double *vol, double *cen, int *bad) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)N.ni * N.nj * N.nk) return;
  const int i = (int)(t % N.ni), j = (int)((t / N.ni) % N.nj),
            k = (int)(t / ((int64_t)N.ni * N.nj));
  const DV3 c0 = N.At(i, j, k), c1 = N.At(i + 1, j, k), c2 = N.At(i, j + 1, k),
            c3 = N.At(i + 1, j + 1, k), c4 = N.At(i, j, k + 1), c5 = N.At(i + 1, j, k + 1),
            c6 = N.At(i, j + 1, k + 1), c7 = N.At(i + 1, j + 1, k + 1);
  const DV3 ce =
      Scale(0.125, Add(Add(Add(Add(Add(Add(Add(c0, c1), c2), c3), c4), c5), c6), c7));
  double v = 0.0;
  v += Pyramid(ce, c0, c4, c6, c2);
  v += Pyramid(ce, c1, c3, c7, c5);
  v += Pyramid(ce, c0, c1, c5, c4);
  v += Pyramid(ce, c2, c6, c7, c3);
  v += Pyramid(ce, c0, c2, c3, c1);
  v += Pyramid(ce, c4, c5, c7, c6);
  if (!(v > 0)) atomicAdd(bad, 1);
  const int64_t id = B.Cell(i, j, k), nc = B.NCell();
  vol[id] = v;
  cen[id] = ce.x;
  cen[nc + id] = ce.y;
  cen[2 * nc + id] = ce.z;
}

// area vector (half the cross product of the diagonals; unit normal and
// magnitude) and centre (mean of the four nodes) of every face of
// direction D between and around the physical cells
template <int D>
__global__ void k_geom_faces(NodesDev N, PadDev B, double *fa, double *fc) {
  const int ei = N.ni + (D == 0), ej = N.nj + (D == 1), ek = N.nk + (D == 2);
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)ei * ej * ek) return;
  const int i = (int)(t % ei), j = (int)((t / ei) % ej), k = (int)(t / ((int64_t)ei * ej));
  DV3 xac, xbd, n0, n1, n2, n3;
  if (D == 0) {
    xac = Sub(N.At(i, j + 1, k + 1), N.At(i, j, k));
    xbd = Sub(N.At(i, j + 1, k), N.At(i, j, k + 1));
    n0 = N.At(i, j, k), n1 = N.At(i, j + 1, k), n2 = N.At(i, j, k + 1), n3 = N.At(i, j + 1, k + 1);
  } else if (D == 1) {
    xac = Sub(N.At(i, j, k + 1), N.At(i + 1, j, k));
    xbd = Sub(N.At(i, j, k), N.At(i + 1, j, k + 1));
    n0 = N.At(i, j, k), n1 = N.At(i + 1, j, k), n2 = N.At(i, j, k + 1), n3 = N.At(i + 1, j, k + 1);
  } else {
    xac = Sub(N.At(i, j + 1, k), N.At(i + 1, j, k));
    xbd = Sub(N.At(i + 1, j + 1, k), N.At(i, j, k));
    n0 = N.At(i, j, k), n1 = N.At(i + 1, j, k), n2 = N.At(i, j + 1, k), n3 = N.At(i + 1, j + 1, k);
  }
  const DV3 a = Scale(0.5, Cross(xbd, xac));
  const double m = sqrt(Dot(a, a));
  const int64_t id = B.Face(D, i, j, k), nf = B.NFace(D);
  fa[id] = a.x / m;
  fa[nf + id] = a.y / m;
  fa[2 * nf + id] = a.z / m;
  fa[3 * nf + id] = m;
  const DV3 c = Scale(0.25, Add(Add(Add(n0, n1), n2), n3));
  fc[id] = c.x;
  fc[nf + id] = c.y;
  fc[2 * nf + id] = c.z;
}

// wall distance of every physical cell: the square root of the smallest
// squared distance to a wall-face centre (the centres are staged through
// shared memory tile by tile)
constexpr int kWallTile = 256;
__global__ void __launch_bounds__(kWallTile) k_wall_dist(const double *wf, int nw, PadDev B,
                                                         int ni, int nj, int nk,
                                                         const double *cen, double *wd) {
  __shared__ double tile[3 * kWallTile];
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = t < (int64_t)ni * nj * nk;
  double x = 0.0, y = 0.0, z = 0.0;
  int64_t id = 0;
  if (live) {
    const int i = (int)(t % ni), j = (int)((t / ni) % nj), k = (int)(t / ((int64_t)ni * nj));
    id = B.Cell(i, j, k);
    const int64_t nc = B.NCell();
    x = cen[id];
    y = cen[nc + id];
    z = cen[2 * nc + id];
  }
  double best = 1.7976931348623157e308;
  for (int w0 = 0; w0 < nw; w0 += kWallTile) {
    const int cnt = min(kWallTile, nw - w0);
    __syncthreads();
    for (int q = threadIdx.x; q < 3 * cnt; q += blockDim.x) tile[q] = wf[3 * (int64_t)w0 + q];
    __syncthreads();
    for (int q = 0; q < cnt; ++q) {
      const double dx = x - tile[3 * q], dy = y - tile[3 * q + 1], dz = z - tile[3 * q + 2];
      const double d2 = dx * dx + dy * dy + dz * dz;
      if (d2 < best) best = d2;
    }
  }
  if (live) wd[id] = sqrt(best);
}

// Device copies of host vectors for one setup step on a private stream,
// stream-ordered from a per-device pool that keeps freed memory: a setup
// that runs while solves iterate on the same GPU (a served request being
// parsed) neither synchronises the device nor waits for their streams.
struct DevBuf {
  cudaStream_t s = nullptr;
  std::vector<void *> ptrs;
  explicit DevBuf(int device) {
    Check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
    Check(cudaMemPoolSetAttribute(Pool(device), cudaMemPoolAttrReleaseThreshold, &keep_),
          "pool attribute");
  }
  ~DevBuf() {
    for (void *p : ptrs) cudaFreeAsync(p, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  static cudaMemPool_t Pool(int device) {
    static cudaMemPool_t pools[64] = {};
    static std::mutex mu;
    if (device < 0 || device >= 64) throw Error(ATH_ERR_ARG, "device id out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (!pools[device]) {
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = device;
      Check(cudaMemPoolCreate(&pools[device], &props), "cudaMemPoolCreate");
    }
    return pools[device];
  }
  uint64_t keep_ = UINT64_MAX;
  template <typename T>
  T *Up(const std::vector<T> &v) {
    int dev = 0;
    Check(cudaGetDevice(&dev), "cudaGetDevice");
    T *p = nullptr;
    Check(cudaMallocFromPoolAsync(reinterpret_cast<void **>(&p),
                                  std::max<size_t>(v.size(), 1) * sizeof(T), Pool(dev), s),
          "cudaMallocFromPoolAsync");
    ptrs.push_back(p);
    if (!v.empty())
      Check(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s),
            "upload");
    Check(cudaStreamSynchronize(s), "upload");
    return p;
  }
  template <typename T>
  void Down(std::vector<T> &v, const T *p) {
    Check(cudaMemcpyAsync(v.data(), p, v.size() * sizeof(T), cudaMemcpyDeviceToHost, s),
          "download");
    Check(cudaStreamSynchronize(s), "download");
  }
};

}  // namespace

void DeviceGeometry(Block &b, int device) {
  Check(cudaSetDevice(device), "cudaSetDevice");
  DevBuf m(device);
  const NodesDev N{m.Up(b.nodes), b.ni, b.nj, b.nk};
  const PadDev B{b.ng, b.NI, b.NJ, b.NK};
  double *vol = m.Up(b.vol), *cen = m.Up(b.center);
  double *fa[3], *fc[3];
  for (int d = 0; d < 3; ++d) {
    fa[d] = m.Up(b.farea[d]);
    fc[d] = m.Up(b.fcenter[d]);
  }
  int *bad = m.Up(std::vector<int>{0});
  const int64_t nc = (int64_t)b.ni * b.nj * b.nk;
  k_geom_cells<<<(unsigned)((nc + 255) / 256), 256, 0, m.s>>>(N, B, vol, cen, bad);
  const int64_t nf[3] = {(int64_t)(b.ni + 1) * b.nj * b.nk, (int64_t)b.ni * (b.nj + 1) * b.nk,
                         (int64_t)b.ni * b.nj * (b.nk + 1)};
  k_geom_faces<0><<<(unsigned)((nf[0] + 255) / 256), 256, 0, m.s>>>(N, B, fa[0], fc[0]);
  k_geom_faces<1><<<(unsigned)((nf[1] + 255) / 256), 256, 0, m.s>>>(N, B, fa[1], fc[1]);
  k_geom_faces<2><<<(unsigned)((nf[2] + 255) / 256), 256, 0, m.s>>>(N, B, fa[2], fc[2]);
  Check(cudaGetLastError(), "geometry kernels");
  std::vector<int> nbad(1);
  m.Down(nbad, bad);
  if (nbad[0] > 0) throw std::runtime_error("non-positive cell volume in grid");
  m.Down(b.vol, vol);
  m.Down(b.center, cen);
  for (int d = 0; d < 3; ++d) {
    m.Down(b.farea[d], fa[d]);
    m.Down(b.fcenter[d], fc[d]);
  }
}

void DeviceWallDistance(const std::vector<double> &wf, Block &b, int device) {
  Check(cudaSetDevice(device), "cudaSetDevice");
  DevBuf m(device);
  const PadDev B{b.ng, b.NI, b.NJ, b.NK};
  const double *w = m.Up(wf);
  const double *cen = m.Up(b.center);
  double *wd = m.Up(b.wall_dist);
  const int64_t nc = (int64_t)b.ni * b.nj * b.nk;
  k_wall_dist<<<(unsigned)((nc + kWallTile - 1) / kWallTile), kWallTile, 0, m.s>>>(
      w, (int)(wf.size() / 3), B, b.ni, b.nj, b.nk, cen, wd);
  Check(cudaGetLastError(), "wall distance kernel");
  m.Down(b.wall_dist, wd);
}

}  // namespace ath
