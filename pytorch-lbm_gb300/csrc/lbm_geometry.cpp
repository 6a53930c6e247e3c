// Host-side geometry precompute of one grid: partial-solid nodes, wetting
// boundary nodes, wall normals, near-wall distance / weight and the node-class
// byte read by the kernels.
//
// Bit-exact with the reference's set_solid + ConningtonLeeWetting precompute
// (pytorch-lbm lbm/fe_ac_solver.py:193-237, lbm/fe_wetting.py:122-311).  Must
// be compiled with floating-point contraction off: the smooth normals repeat
// numpy's float32/float64 operation sequence exactly.
#include "lbm_geometry.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "lbm_tables.h"

namespace lbm {

namespace {

inline int64_t idx(int64_t ix, int64_t iy, int64_t iz, int64_t ny, int64_t nz) {
  return (ix * ny + iy) * nz + iz;
}

inline int64_t wrap(int64_t i, int64_t n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// fn(begin, end) over [0, n) split into contiguous ranges on the host's
// cores.  Every loop it runs computes each index independently, so the
// result does not depend on the split.
template <typename Fn>
void parallel_for(int64_t n, Fn fn) {
  const unsigned hw = std::thread::hardware_concurrency();
  int64_t nt = std::min<int64_t>(hw ? hw : 1, 32);
  if (n < 4096 || nt < 2) {
    fn((int64_t)0, n);
    return;
  }
  nt = std::min<int64_t>(nt, n);
  std::vector<std::thread> th;
  for (int64_t t = 1; t < nt; ++t) th.emplace_back(fn, n * t / nt, n * (t + 1) / nt);
  fn((int64_t)0, n / nt);
  for (auto& x : th) x.join();
}

// Smooth wall normals -grad(frac)/|grad(frac)| times the boundary mask, with
// np.gradient's stencil (central inside, one-sided first order at the edges)
// evaluated in the fraction's own type F (fe_wetting.py:242-267).  Every node
// is computed: off the boundary the product with the mask is a signed zero
// (-0 where -grad/|grad| is negative or -0), as in the reference's array.
// A 2-D grid (nz == 1) has two axes; its third component is 0.
template <typename F>
void smooth_normals(const F* frac, const HostVec<uint8_t>& bnd, int64_t nx, int64_t ny, int64_t nz,
                    HostVec<float>& wn) {
  const int64_t N = nx * ny * nz;
  const bool two_d = nz == 1;
  auto grad_axis = [&](int64_t ix, int64_t iy, int64_t iz, int axis) -> F {
    int64_t n_ax = axis == 0 ? nx : (axis == 1 ? ny : nz);
    int64_t i = axis == 0 ? ix : (axis == 1 ? iy : iz);
    auto at = [&](int64_t j) -> F {
      return axis == 0 ? frac[idx(j, iy, iz, ny, nz)]
           : (axis == 1 ? frac[idx(ix, j, iz, ny, nz)] : frac[idx(ix, iy, j, ny, nz)]);
    };
    if (i == 0) return (F)(at(1) - at(0)) / (F)1.0;
    if (i == n_ax - 1) return (F)(at(n_ax - 1) - at(n_ax - 2)) / (F)1.0;
    return (F)(at(i + 1) - at(i - 1)) / (F)2.0;
  };
  parallel_for(nx, [&](int64_t x0, int64_t x1) {
  for (int64_t ix = x0; ix < x1; ++ix)
    for (int64_t iy = 0; iy < ny; ++iy)
      for (int64_t iz = 0; iz < nz; ++iz) {
        const int64_t n = idx(ix, iy, iz, ny, nz);
        const F mask = bnd[n] ? (F)1 : (F)0;
        const F g0 = grad_axis(ix, iy, iz, 0);
        const F g1 = grad_axis(ix, iy, iz, 1);
        const F g2 = two_d ? (F)0 : grad_axis(ix, iy, iz, 2);
        F acc = (F)0;
        acc = acc + g0 * g0;
        acc = acc + g1 * g1;
        if (!two_d) acc = acc + g2 * g2;
        F mag = std::sqrt(acc);
        if (mag < (F)1e-10) mag = (F)1e-10;
        wn[n] = (float)(((-g0) / mag) * mask);
        wn[N + n] = (float)(((-g1) / mag) * mask);
        wn[2 * N + n] = two_d ? 0.0f : (float)(((-g2) / mag) * mask);
      }
  });
}

}  // namespace

int compute_geometry(int64_t nx, int64_t ny, int64_t nz, const uint8_t* solid_in, const void* fraction,
                     int fraction_dtype, bool wetting, bool dbl_precision, Geometry& g) {
  const int64_t N = nx * ny * nz;
  // nz == 1: a 2-D grid on D2Q9 (its velocities as 3-D vectors with e_z = 0;
  // the z neighbours of the near-wall search are then the node itself)
  const bool two_d = nz == 1;
  const int nq = two_d ? kQ2 : kQ;
  const int(*E)[3] = two_d ? kE2 : kE;
  for (auto* v : {&g.solid, &g.partial, &g.boundary, &g.near_wall, &g.top, &g.cls, &g.dist}) v->resize(N);
  g.wall_normal.resize(3 * N);
  g.wall_weight.resize(N);
  g.nsw.resize(N);
  g.has_fraction = fraction_dtype != 0;
  g.n_boundary = 0;
  // every table's initial value, in parallel (this also touches the pages first)
  parallel_for(N, [&](int64_t n0, int64_t n1) {
    for (int64_t n = n0; n < n1; ++n) {
      g.solid[n] = solid_in[n] ? 1 : 0;
      bool part = false;
      if (fraction_dtype == 1) {
        const float v = static_cast<const float*>(fraction)[n];
        part = v > 0.01f && v < 0.99f;
      } else if (fraction_dtype == 2) {
        const double v = static_cast<const double*>(fraction)[n];
        part = v > 0.01 && v < 0.99;
      }
      g.partial[n] = (part && !g.solid[n]) ? 1 : 0;
      g.boundary[n] = g.near_wall[n] = g.top[n] = 0;
      g.dist[n] = 100;
      g.wall_weight[n] = 0.0f;
      g.nsw[n] = -1;
      g.wall_normal[n] = g.wall_normal[N + n] = g.wall_normal[2 * N + n] = 0.0f;
    }
  });

  if (wetting) {
    // boundary: fluid node whose periodic neighbour x - e_q is solid for some
    // q, found from the solid side (solid nodes are the smaller set): every
    // fluid x = m + e_q of a solid m.  Threads take slabs of x; a target in a
    // neighbouring slab may be marked by two threads, so the marks are relaxed
    // atomic stores of the same value.
    parallel_for(nx, [&](int64_t x0, int64_t x1) {
      for (int64_t ix = x0; ix < x1; ++ix)
        for (int64_t iy = 0; iy < ny; ++iy)
          for (int64_t iz = 0; iz < nz; ++iz) {
            if (!g.solid[idx(ix, iy, iz, ny, nz)]) continue;
            for (int q = 1; q < nq; ++q) {
              const int64_t n =
                  idx(wrap(ix + E[q][0], nx), wrap(iy + E[q][1], ny), wrap(iz + E[q][2], nz), ny, nz);
              if (!g.solid[n]) __atomic_store_n(&g.boundary[n], (uint8_t)1, __ATOMIC_RELAXED);
            }
          }
    });
    for (int64_t n = 0; n < N; ++n) g.n_boundary += g.boundary[n];
    // wall normals
    if (fraction_dtype == 1) {
      smooth_normals(static_cast<const float*>(fraction), g.boundary, nx, ny, nz, g.wall_normal);
    } else if (fraction_dtype == 2) {
      smooth_normals(static_cast<const double*>(fraction), g.boundary, nx, ny, nz, g.wall_normal);
    } else {
      // discrete neighbour counting with non-periodic bounds (fe_wetting.py:152-203)
      parallel_for(nx, [&](int64_t x0, int64_t x1) {
      for (int64_t ix = x0; ix < x1; ++ix)
        for (int64_t iy = 0; iy < ny; ++iy)
          for (int64_t iz = 0; iz < nz; ++iz) {
            const int64_t n = idx(ix, iy, iz, ny, nz);
            if (!g.boundary[n]) continue;
            double nm[3] = {0.0, 0.0, 0.0};
            int count = 0;
            for (int q = 1; q < nq; ++q) {
              const int64_t jx = ix + E[q][0], jy = iy + E[q][1], jz = iz + E[q][2];
              if (jx >= 0 && jx < nx && jy >= 0 && jy < ny && jz >= 0 && jz < nz &&
                  g.solid[idx(jx, jy, jz, ny, nz)]) {
                nm[0] -= E[q][0];
                nm[1] -= E[q][1];
                nm[2] -= E[q][2];
                ++count;
              }
            }
            if (count > 0) {
              for (int d = 0; d < 3; ++d) nm[d] /= count;
              const double norm = std::sqrt(nm[0] * nm[0] + nm[1] * nm[1] + nm[2] * nm[2]);
              if (norm > 1e-10)
                for (int d = 0; d < 3; ++d) nm[d] /= norm;
            }
            for (int d = 0; d < 3; ++d) g.wall_normal[d * N + n] = (float)nm[d];
          }
      });
    }
    // Near-wall distance: 11 synchronous passes of periodic face-neighbour
    // min-plus from the boundary nodes (fe_wetting.py:280-292) equal the
    // face-graph distance capped at 11 (else 100); computed by breadth-first
    // search from all boundary nodes at once.
    std::vector<int64_t> frontier, next;
    for (int64_t n = 0; n < N; ++n)
      if (g.boundary[n]) {
        g.dist[n] = 0;
        frontier.push_back(n);
      }
    for (int pass = 1; pass <= kNearWallPasses && !frontier.empty(); ++pass) {
      next.clear();
      for (int64_t n : frontier) {
        const int64_t iz = n % nz, t = n / nz, iy = t % ny, ix = t / ny;
        const int64_t nb[6] = {idx(wrap(ix - 1, nx), iy, iz, ny, nz), idx(wrap(ix + 1, nx), iy, iz, ny, nz),
                               idx(ix, wrap(iy - 1, ny), iz, ny, nz), idx(ix, wrap(iy + 1, ny), iz, ny, nz),
                               idx(ix, iy, wrap(iz - 1, nz), ny, nz), idx(ix, iy, wrap(iz + 1, nz), ny, nz)};
        for (int64_t m : nb)
          if (g.dist[m] == 100) {
            g.dist[m] = (uint8_t)pass;
            next.push_back(m);
          }
      }
      frontier.swap(next);
    }
    // wall weight exp(-dist / (xi/2)) in float32, 0 in solid (fe_wetting.py:295-303)
    float lut[kWwCodes];
    near_wall_weights(lut);
    parallel_for(N, [&](int64_t n0, int64_t n1) {
      for (int64_t n = n0; n < n1; ++n) {
        if (g.solid[n]) {
          g.dist[n] = 100;
          g.wall_weight[n] = 0.0f;
        } else {
          g.wall_weight[n] = lut[g.dist[n] <= kNearWallPasses ? g.dist[n] : kWwFarCode];
          g.near_wall[n] = g.dist[n] < 10 ? 1 : 0;  // dist < 2 xi
        }
      }
    });
    // top-surface flag of the boundary-phi relaxation, |n_last| / |n| > 1/2
    // in the solver precision, n_last the component along the last axis (z,
    // or y on a 2-D grid) (fe_ac_solver.py:602-606)
    parallel_for(N, [&](int64_t n0, int64_t n1) {
    for (int64_t n = n0; n < n1; ++n) {
      if (!g.boundary[n]) continue;
      const float a = g.wall_normal[n], b = g.wall_normal[N + n], c = g.wall_normal[2 * N + n];
      bool top;
      if (two_d) {
        if (dbl_precision) {
          const double x = a, y = b;
          double m = std::sqrt(x * x + y * y);
          if (m < 1e-10) m = 1e-10;
          top = std::fabs(y) / m > 0.5;
        } else {
          float m = std::sqrt(a * a + b * b);
          if (m < 1e-10f) m = 1e-10f;
          top = std::fabs(b) / m > 0.5f;
        }
      } else if (dbl_precision) {
        const double x = a, y = b, z = c;
        double m = std::sqrt((x * x + y * y) + z * z);
        if (m < 1e-10) m = 1e-10;
        top = std::fabs(z) / m > 0.5;
      } else {
        float m = std::sqrt((a * a + b * b) + c * c);
        if (m < 1e-10f) m = 1e-10f;
        top = std::fabs(c) / m > 0.5f;
      }
      g.top[n] = top ? 1 : 0;
    }
    });
    // next-interior node of each boundary node for the cubic-wall-energy
    // boundary phi: one step along the wall normal rounded half to even,
    // clamped to the grid (not periodic); kept only where that node is fluid
    // (fe_wetting.py:313-367)
    parallel_for(nx, [&](int64_t x0, int64_t x1) {
    for (int64_t ix = x0; ix < x1; ++ix)
      for (int64_t iy = 0; iy < ny; ++iy)
        for (int64_t iz = 0; iz < nz; ++iz) {
          const int64_t n = idx(ix, iy, iz, ny, nz);
          if (!g.boundary[n]) continue;
          const int64_t c[3] = {ix, iy, iz}, ext[3] = {nx, ny, nz};
          int64_t t[3];
          for (int d = 0; d < 3; ++d) {
            const int64_t sh = (int64_t)std::nearbyint(g.wall_normal[d * N + n]);
            t[d] = std::min<int64_t>(std::max<int64_t>(c[d] + sh, 0), ext[d] - 1);
          }
          const int64_t m = idx(t[0], t[1], t[2], ny, nz);
          if (!g.solid[m]) g.nsw[n] = (int32_t)m;
        }
    });
  }
  // node-class byte
  parallel_for(N, [&](int64_t n0, int64_t n1) {
  for (int64_t n = n0; n < n1; ++n) {
    uint8_t c = 0;
    if (g.solid[n]) c |= 1;
    if (g.boundary[n]) c |= 2;
    if (g.partial[n]) c |= 4;
    if (g.top[n]) c |= 8;
    int code;
    if (g.solid[n]) code = kWwSolidCode;
    else if (wetting && g.dist[n] <= kNearWallPasses) code = g.dist[n];
    else code = kWwFarCode;
    c |= (uint8_t)(code << 4);
    g.cls[n] = c;
  }
  });
  return 0;
}

void near_wall_weights(float* lut) {
  // exp(-d / 2.5) in float32 for d = 0..11, d = 100 (code 12) and 0 for solid
  // (code 13).  float32 exp of torch is correctly rounded on these inputs;
  // the double exp rounded once to float reproduces it.
  for (int d = 0; d <= kNearWallPasses; ++d) {
    const float x = (-(float)d) / 2.5f;
    lut[d] = (float)std::exp((double)x);
  }
  lut[kWwFarCode] = (float)std::exp((double)((-100.0f) / 2.5f));
  lut[kWwSolidCode] = 0.0f;
  lut[14] = 0.0f;
  lut[15] = 0.0f;
}

}  // namespace lbm
