// Geometry precompute of one grid on the device: partial-solid nodes,
// wetting boundary nodes, wall normals, near-wall distance / weight, the
// top-surface flag, the next-interior node of direct wetting, the node-class
// byte and the penalisation fraction in the compute type.
//
// Bit-exact with the reference's set_solid + ConningtonLeeWetting precompute
// (pytorch-lbm lbm/fe_ac_solver.py:193-237, lbm/fe_wetting.py:122-367), and
// with the host restatement of the same steps (lbm_geometry.cpp, which serves
// lbm_geometry_host): every floating-point operation of the smooth normals and
// of the top-surface test is an explicitly rounded IEEE operation (no
// contraction), in the fraction's own type as numpy evaluates it.
//
// Kernels, in launch order (one thread per node; each reads only inputs or
// the previous kernels' outputs):
//   k_geo_bits     solid / partial / boundary bits of every node, the
//                  near-wall distance seed (0 at boundary nodes, else far)
//   k_geo_smooth   wall normals -grad(frac)/|grad(frac)| times the boundary
//                  mask (np.gradient stencil); off the boundary the signed
//                  zero that product leaves
//   k_geo_discrete wall normals from solid-neighbour counting (no fraction)
//   k_geo_dist_axis one axis of the near-wall distance transform (3 launches)
//   k_geo_final    class byte, top flag, next-interior node, fraction in the
//                  compute type
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "lbm_common.cuh"
#include "lbm_tables.h"

namespace lbm {

namespace {

constexpr uint8_t kBitSolid = 1, kBitPartial = 2, kBitBoundary = 4;
// near-wall distances saturate here: any value above kNearWallPasses reads as far
constexpr int kDistCap = kNearWallPasses + 1;

struct GeoGrid {
  int nx, ny, nz, N;
  bool two_d;
  FastDiv dz, dy;  // division by nz and ny
};

__device__ __forceinline__ int gidx(const GeoGrid& g, int ix, int iy, int iz) { return (ix * g.ny + iy) * g.nz + iz; }
__device__ __forceinline__ int gwrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
__device__ __forceinline__ void gdecode(const GeoGrid& g, int n, int& ix, int& iy, int& iz) {
  const int t = (int)g.dz.div((unsigned)n);
  iz = n - t * g.nz;
  ix = (int)g.dy.div((unsigned)t);
  iy = t - ix * g.ny;
}

// Lattice velocities of the grid's lattice (D3Q19, or D2Q9 with e_z = 0).
__device__ __forceinline__ void evec(bool two_d, int q, int& x, int& y, int& z) {
  if (two_d) {
    // D2Q9 order of lbm/lattice.py:46-55
    constexpr int e2[9][2] = {{0, 0}, {1, 0}, {-1, 0}, {0, 1}, {0, -1}, {1, 1}, {-1, 1}, {-1, -1}, {1, -1}};
    x = e2[q][0];
    y = e2[q][1];
    z = 0;
  } else {
    x = ex(q);
    y = ey(q);
    z = ez(q);
  }
}

// Explicitly rounded arithmetic in the fraction's type.
__device__ __forceinline__ float r_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double r_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float r_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double r_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float r_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double r_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float r_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double r_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float r_sqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double r_sqrt(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float to_f32(float a) { return a; }
__device__ __forceinline__ float to_f32(double a) { return __double2float_rn(a); }

// fraction_dtype 1: float32, 2: float64 (as the C ABI's LBM_DT_* codes)
__device__ __forceinline__ bool is_partial(const void* frac, int fdt, int n) {
  if (fdt == 1) {
    const float v = static_cast<const float*>(frac)[n];
    return v > 0.01f && v < 0.99f;
  }
  if (fdt == 2) {
    const double v = static_cast<const double*>(frac)[n];
    return v > 0.01 && v < 0.99;
  }
  return false;
}

__global__ void __launch_bounds__(kBlock) k_geo_bits(GeoGrid g, const uint8_t* __restrict__ solid,
                                                     const void* __restrict__ frac, int fdt, int wetting,
                                                     uint8_t* __restrict__ bits, uint8_t* __restrict__ dist) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= g.N) return;
  const bool s = solid[n] != 0;
  uint8_t b = s ? kBitSolid : 0;
  if (!s && is_partial(frac, fdt, n)) b |= kBitPartial;
  if (wetting && !s) {
    // a fluid node with a solid periodic neighbour x + e_q for some q (the
    // reference marks the fluid nodes m + e_q of the solid nodes m; D3Q19 and
    // D2Q9 are symmetric, so the two descriptions agree)
    int ix, iy, iz;
    gdecode(g, n, ix, iy, iz);
    // every neighbour's load issued before any is tested (no early exit: a
    // chain of dependent loads per node otherwise)
    const int xm = gwrap(ix - 1, g.nx), xp = gwrap(ix + 1, g.nx), ym = gwrap(iy - 1, g.ny),
              yp = gwrap(iy + 1, g.ny), zm = gwrap(iz - 1, g.nz), zp = gwrap(iz + 1, g.nz);
    const int xs[3] = {xm, ix, xp}, ys[3] = {ym, iy, yp}, zs[3] = {zm, iz, zp};
    bool bnd = false;
    if (g.two_d) {
#pragma unroll
      for (int q = 1; q < kQ2; ++q) {
        int x, y, z;
        evec(true, q, x, y, z);
        bnd |= solid[gidx(g, xs[x + 1], ys[y + 1], iz)] != 0;
      }
    } else {
#pragma unroll
      for (int q = 1; q < Q; ++q) bnd |= solid[gidx(g, xs[ex(q) + 1], ys[ey(q) + 1], zs[ez(q) + 1])] != 0;
    }
    if (bnd) b |= kBitBoundary;
  }
  bits[n] = b;
  dist[n] = (b & kBitBoundary) ? 0 : kDistCap;
}

// np.gradient of frac along one axis at node (ix, iy, iz): central
// differences inside (difference / 2), first-order one-sided at the two ends
// (difference / 1).
template <typename F>
__device__ __forceinline__ F grad_axis(const GeoGrid& g, const F* frac, int ix, int iy, int iz, int axis) {
  const int n_ax = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
  const int i = axis == 0 ? ix : (axis == 1 ? iy : iz);
  auto at = [&](int j) -> F {
    return axis == 0 ? frac[gidx(g, j, iy, iz)] : (axis == 1 ? frac[gidx(g, ix, j, iz)] : frac[gidx(g, ix, iy, j)]);
  };
  // x / 1 is x and x / 2 is x * 0.5 exactly (one rounding of the same real
  // number), without the division's slow float64 path
  if (i == 0) return r_sub(at(1), at(0));
  if (i == n_ax - 1) return r_sub(at(n_ax - 1), at(n_ax - 2));
  return r_mul(r_sub(at(i + 1), at(i - 1)), (F)0.5);
}

// Smooth wall normals, off the boundary: the reference's (-g / |g|) * 0 is a
// zero with the sign of -g there (|g| is clamped positive and the fraction
// has no NaN), i.e. +0 where g carries a sign bit and -0 elsewhere; no
// division.  Boundary nodes are appended to `list` (their order does not
// matter: each node's normal depends on its own inputs only) and normalised
// by k_geo_smooth_bnd, so that the float64 square root and divisions run on
// dense warps instead of on the one or two boundary lanes of a warp.
template <typename F>
__global__ void __launch_bounds__(kBlock) k_geo_smooth(GeoGrid g, const F* __restrict__ frac,
                                                       const uint8_t* __restrict__ bits, float* __restrict__ wn,
                                                       int* __restrict__ list, unsigned* __restrict__ count) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= g.N) return;
  if (bits[n] & kBitBoundary) {
    list[atomicAdd(count, 1u)] = n;
    return;
  }
  int ix, iy, iz;
  gdecode(g, n, ix, iy, iz);
  const size_t N = (size_t)g.N;
  const F g0 = grad_axis(g, frac, ix, iy, iz, 0);
  const F g1 = grad_axis(g, frac, ix, iy, iz, 1);
  const F g2 = g.two_d ? (F)0 : grad_axis(g, frac, ix, iy, iz, 2);
  wn[n] = signbit(g0) ? 0.0f : -0.0f;
  wn[N + n] = signbit(g1) ? 0.0f : -0.0f;
  wn[2 * N + n] = g.two_d ? 0.0f : (signbit(g2) ? 0.0f : -0.0f);
}

// Smooth wall normals of the boundary nodes in `list` (k_geo_smooth):
// -g / max(|g|, 1e-10) times the mask 1, in the fraction's type, then float32.
template <typename F>
__global__ void __launch_bounds__(kBlock) k_geo_smooth_bnd(GeoGrid g, const F* __restrict__ frac,
                                                           const int* __restrict__ list,
                                                           const unsigned* __restrict__ count,
                                                           float* __restrict__ wn) {
  const int cnt = (int)*count;
  const size_t N = (size_t)g.N;
  for (int i = blockIdx.x * kBlock + threadIdx.x; i < cnt; i += gridDim.x * kBlock) {
    const int n = list[i];
    int ix, iy, iz;
    gdecode(g, n, ix, iy, iz);
    const F g0 = grad_axis(g, frac, ix, iy, iz, 0);
    const F g1 = grad_axis(g, frac, ix, iy, iz, 1);
    const F g2 = g.two_d ? (F)0 : grad_axis(g, frac, ix, iy, iz, 2);
    const F mask = (F)1;
    F acc = (F)0;
    acc = r_add(acc, r_mul(g0, g0));
    acc = r_add(acc, r_mul(g1, g1));
    if (!g.two_d) acc = r_add(acc, r_mul(g2, g2));
    F mag = r_sqrt(acc);
    if (mag < (F)1e-10) mag = (F)1e-10;
    wn[n] = to_f32(r_mul(r_div(-g0, mag), mask));
    wn[N + n] = to_f32(r_mul(r_div(-g1, mag), mask));
    wn[2 * N + n] = g.two_d ? 0.0f : to_f32(r_mul(r_div(-g2, mag), mask));
  }
}

// Discrete wall normals (fe_wetting.py:152-203): minus the mean of the solid
// neighbours' directions (non-periodic bounds), normalised, in float64.
__global__ void __launch_bounds__(kBlock) k_geo_discrete(GeoGrid g, const uint8_t* __restrict__ solid,
                                                         const uint8_t* __restrict__ bits, float* __restrict__ wn) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= g.N) return;
  const size_t N = (size_t)g.N;
  double nm[3] = {0.0, 0.0, 0.0};
  if (bits[n] & kBitBoundary) {
    int ix, iy, iz;
    gdecode(g, n, ix, iy, iz);
    const int nq = g.two_d ? kQ2 : Q;
    int count = 0;
    for (int q = 1; q < nq; ++q) {
      int x, y, z;
      evec(g.two_d, q, x, y, z);
      const int jx = ix + x, jy = iy + y, jz = iz + z;
      if (jx >= 0 && jx < g.nx && jy >= 0 && jy < g.ny && jz >= 0 && jz < g.nz && solid[gidx(g, jx, jy, jz)]) {
        nm[0] = __dsub_rn(nm[0], (double)x);
        nm[1] = __dsub_rn(nm[1], (double)y);
        nm[2] = __dsub_rn(nm[2], (double)z);
        ++count;
      }
    }
    if (count > 0) {
      for (int d = 0; d < 3; ++d) nm[d] = __ddiv_rn(nm[d], (double)count);
      const double norm =
          __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(nm[0], nm[0]), __dmul_rn(nm[1], nm[1])), __dmul_rn(nm[2], nm[2])));
      if (norm > 1e-10)
        for (int d = 0; d < 3; ++d) nm[d] = __ddiv_rn(nm[d], norm);
    }
  }
  for (int d = 0; d < 3; ++d) wn[d * N + n] = __double2float_rn(nm[d]);
}

// The near-wall distance (fe_wetting.py:280-292): 11 synchronous passes of
// periodic face-neighbour min-plus from the boundary nodes give the distance
// in the periodic face graph of the grid, i.e. the smallest periodic L1
// distance to a boundary node, where it is at most 11, and 100 (far)
// elsewhere.  The L1 distance is a sum of per-axis ring distances, so it is
// computed as three one-axis transforms, each out(i) = min over |k| <= 11 of
// in(i + k mod L) + |k|, saturated at kDistCap (exact: saturation commutes
// with adding a non-negative offset, and a node farther than 11 only needs
// to read as far).  k_geo_final maps values above 11 to far.
__global__ void __launch_bounds__(kBlock) k_geo_dist_axis(GeoGrid g, const uint8_t* __restrict__ in,
                                                          uint8_t* __restrict__ out, int axis) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= g.N) return;
  int ix, iy, iz;
  gdecode(g, n, ix, iy, iz);
  const int L = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
  const int i = axis == 0 ? ix : (axis == 1 ? iy : iz);
  const int stride = axis == 0 ? g.ny * g.nz : (axis == 1 ? g.nz : 1);
  const uint8_t* line = in + (n - i * stride);
  int best = in[n];
  int jp = i, jm = i;
#pragma unroll
  for (int k = 1; k <= kNearWallPasses; ++k) {
    jp = jp + 1 == L ? 0 : jp + 1;
    jm = jm == 0 ? L - 1 : jm - 1;
    best = min(best, min((int)line[jp * stride], (int)line[jm * stride]) + k);
  }
  out[n] = (uint8_t)min(best, kDistCap);
}

// Node-class byte (lbm_common.cuh), top-surface flag of the boundary-phi
// relaxation (|n_last| / |n| > 1/2 in the solver precision, fe_ac_solver.py:
// 602-606), next-interior node of direct wetting (one step along the wall
// normal rounded half to even, clamped, kept where fluid; fe_wetting.py:
// 313-367), and the penalisation fraction in the compute type T.
template <typename T>
__global__ void __launch_bounds__(kBlock) k_geo_final(GeoGrid g, const uint8_t* __restrict__ bits,
                                                      const uint8_t* __restrict__ dist, const float* __restrict__ wn,
                                                      int wetting, int dbl_precision, const void* __restrict__ frac,
                                                      int fdt, uint8_t* __restrict__ cls, int* __restrict__ nsw,
                                                      T* __restrict__ eps) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= g.N) return;
  const size_t N = (size_t)g.N;
  const uint8_t b = bits[n];
  const bool solid = b & kBitSolid, bnd = b & kBitBoundary;
  bool top = false;
  if (bnd) {
    const float a = wn[n], bb = wn[N + n], c = wn[2 * N + n];
    if (g.two_d) {
      if (dbl_precision) {
        const double x = a, y = bb;
        double m = __dsqrt_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
        if (m < 1e-10) m = 1e-10;
        top = __ddiv_rn(fabs(y), m) > 0.5;
      } else {
        float m = __fsqrt_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(bb, bb)));
        if (m < 1e-10f) m = 1e-10f;
        top = __fdiv_rn(fabsf(bb), m) > 0.5f;
      }
    } else if (dbl_precision) {
      const double x = a, y = bb, z = c;
      double m = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
      if (m < 1e-10) m = 1e-10;
      top = __ddiv_rn(fabs(z), m) > 0.5;
    } else {
      float m = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(bb, bb)), __fmul_rn(c, c)));
      if (m < 1e-10f) m = 1e-10f;
      top = __fdiv_rn(fabsf(c), m) > 0.5f;
    }
    if (nsw) {
      int ix, iy, iz;
      gdecode(g, n, ix, iy, iz);
      const int cc[3] = {ix, iy, iz}, ext[3] = {g.nx, g.ny, g.nz};
      int t[3];
      for (int d = 0; d < 3; ++d) {
        const int sh = __float2int_rn(wn[d * N + n]);
        const int v = cc[d] + sh;
        t[d] = v < 0 ? 0 : (v > ext[d] - 1 ? ext[d] - 1 : v);
      }
      const int m = gidx(g, t[0], t[1], t[2]);
      nsw[n] = (bits[m] & kBitSolid) ? -1 : m;
    }
  } else if (nsw) {
    nsw[n] = -1;
  }
  uint8_t c = 0;
  if (solid) c |= kSolid;
  if (bnd) c |= kBoundary;
  if (b & kBitPartial) c |= kPartial;
  if (top) c |= kTop;
  int code;
  const uint8_t d = dist[n];
  if (solid) code = kWwSolidCode;
  else if (wetting && d <= kNearWallPasses) code = d;
  else code = kWwFarCode;
  cls[n] = (uint8_t)(c | (code << kWwShift));
  if (eps) {
    T e = T(0);
    if (fdt == 1) e = (T) static_cast<const float*>(frac)[n];
    else if (fdt == 2) e = (T) static_cast<const double*>(frac)[n];
    eps[n] = e;
  }
}

}  // namespace

// The device geometry precompute.  solid: N bytes (nonzero = solid); frac:
// N elements of fdt (0 none, 1 float32, 2 float64) or null; scratch: 256-byte
// aligned, three N-byte planes, then at the next 256-byte boundary 256 bytes
// (the boundary-node count) and N ints (the boundary-node list).  Writes cls (N), wn (3 N floats), nsw (N ints, or null when direct
// wetting is off) and eps (N elements of T, zero without a fraction), all on
// the device, asynchronously on `st`.
template <typename T>
cudaError_t launch_geometry(int nx, int ny, int nz, const uint8_t* solid, const void* frac, int fdt, bool wetting,
                            bool dbl_precision, uint8_t* scratch, uint8_t* cls, float* wn, int* nsw, T* eps,
                            cudaStream_t st) {
  GeoGrid g{nx, ny, nz, nx * ny * nz, nz == 1, make_fastdiv((unsigned)nz), make_fastdiv((unsigned)ny)};
  const int grid = (g.N + kBlock - 1) / kBlock;
  uint8_t* bits = scratch;
  uint8_t* dist = scratch + g.N;
  k_geo_bits<<<grid, kBlock, 0, st>>>(g, solid, frac, fdt, wetting ? 1 : 0, bits, dist);
  if (wetting) {
    if (fdt != 0) {
      // boundary list (N ints) and its length after the three distance bytes of scratch
      const size_t off = (3 * (size_t)g.N + 255) & ~(size_t)255;
      unsigned* count = reinterpret_cast<unsigned*>(scratch + off);
      int* list = reinterpret_cast<int*>(scratch + off + 256);
      cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned), st);
      if (e != cudaSuccess) return e;
      int dev = 0, nsm = 0;
      e = cudaGetDevice(&dev);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      const int bgrid = std::min(grid, 4 * nsm);
      if (fdt == 1) {
        k_geo_smooth<float><<<grid, kBlock, 0, st>>>(g, static_cast<const float*>(frac), bits, wn, list, count);
        k_geo_smooth_bnd<float><<<bgrid, kBlock, 0, st>>>(g, static_cast<const float*>(frac), list, count, wn);
      } else {
        k_geo_smooth<double><<<grid, kBlock, 0, st>>>(g, static_cast<const double*>(frac), bits, wn, list, count);
        k_geo_smooth_bnd<double><<<bgrid, kBlock, 0, st>>>(g, static_cast<const double*>(frac), list, count, wn);
      }
    } else {
      k_geo_discrete<<<grid, kBlock, 0, st>>>(g, solid, bits, wn);
    }
    // z, y, x transforms (2-D grids: y, x): dist -> tmp -> dist -> tmp
    uint8_t* tmp = scratch + 2 * (size_t)g.N;
    uint8_t* src = dist;
    uint8_t* dst = tmp;
    for (int axis = g.two_d ? 1 : 2; axis >= 0; --axis) {
      k_geo_dist_axis<<<grid, kBlock, 0, st>>>(g, src, dst, axis);
      uint8_t* t = src;
      src = dst;
      dst = t;
    }
    dist = src;
  } else {
    cudaError_t e = cudaMemsetAsync(wn, 0, 3 * (size_t)g.N * sizeof(float), st);
    if (e != cudaSuccess) return e;
  }
  k_geo_final<T><<<grid, kBlock, 0, st>>>(g, bits, dist, wn, wetting ? 1 : 0, dbl_precision ? 1 : 0, frac, fdt, cls,
                                          wetting ? nsw : nullptr, eps);
  return cudaGetLastError();
}

template cudaError_t launch_geometry<float>(int, int, int, const uint8_t*, const void*, int, bool, bool, uint8_t*,
                                            uint8_t*, float*, int*, float*, cudaStream_t);
template cudaError_t launch_geometry<double>(int, int, int, const uint8_t*, const void*, int, bool, bool, uint8_t*,
                                             uint8_t*, float*, int*, double*, cudaStream_t);

}  // namespace lbm
