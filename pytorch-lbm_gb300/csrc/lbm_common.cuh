// Shared definitions of the GB300 Allen-Cahn LBM kernels: D3Q19 tables, node
// classes, per-step constants and device-state pointers.
#pragma once
#include <cstddef>
#include <cstdint>

namespace lbm {

constexpr int Q = 19;
constexpr int kBlock = 256;  // threads per block of the node-parallel kernels
// Threads per block of the paired update kernel (lbm_pair.cuh): blocks of 128
// threads at 128 registers (4 per SM) leave fewer SM slots idle behind a
// block's last warp than blocks of 256 (2 per SM).
constexpr int kPairUpdBlock = 128;

// D3Q19 velocity set in the population order of the reference
// (pytorch-lbm lbm/lattice.py:70-95).  Written as constexpr functions so that
// fully unrolled loops fold every component to an immediate.
__host__ __device__ constexpr int ex(int q) {
  return (q == 1 || q == 7 || q == 10 || q == 11 || q == 14) ? 1
       : (q == 2 || q == 8 || q == 9 || q == 12 || q == 13) ? -1 : 0;
}
__host__ __device__ constexpr int ey(int q) {
  return (q == 3 || q == 7 || q == 8 || q == 15 || q == 18) ? 1
       : (q == 4 || q == 9 || q == 10 || q == 16 || q == 17) ? -1 : 0;
}
__host__ __device__ constexpr int ez(int q) {
  return (q == 5 || q == 11 || q == 12 || q == 15 || q == 16) ? 1
       : (q == 6 || q == 13 || q == 14 || q == 17 || q == 18) ? -1 : 0;
}
__host__ __device__ constexpr int opp(int q) {
  return q == 0 ? 0 : (q <= 6 ? ((q & 1) ? q + 1 : q - 1)
                              : (q <= 10 ? (q <= 8 ? q + 2 : q - 2)
                                         : (q <= 14 ? (q <= 12 ? q + 2 : q - 2)
                                                    : (q <= 16 ? q + 2 : q - 2))));
}
__host__ __device__ constexpr int ecomp(int q, int d) { return d == 0 ? ex(q) : (d == 1 ? ey(q) : ez(q)); }

// D3Q19 lattice constants as compile-time values in the compute type T: the
// float32 weights of the reference (lbm/lattice.py:82-88, float32 even in
// float64 runs) widened to T, c_s^2 = 1/3 rounded to T, and the products the
// step uses.  Each is the same single rounding the host applies when it fills
// Consts (checked when a grid's constants are built), so kernels may use either;
// as immediates they cost no loads.
template <typename T>
struct Lat {
  __host__ __device__ static constexpr T w(int q) {
    return q == 0 ? T(float(1.0 / 3.0)) : (q <= 6 ? T(float(1.0 / 18.0)) : T(float(1.0 / 36.0)));
  }
  __host__ __device__ static constexpr T cs2() { return T(1.0 / 3.0); }
  __host__ __device__ static constexpr T inv_cs2() { return T(1) / cs2(); }
  __host__ __device__ static constexpr T two_cs2() { return T(2.0 * (1.0 / 3.0)); }
  __host__ __device__ static constexpr T inv_two_cs2() { return T(1) / two_cs2(); }
  __host__ __device__ static constexpr T wc(int q) { return w(q) / cs2(); }       // w_q / cs2
  __host__ __device__ static constexpr T w2c(int q) { return T(2) * wc(q); }      // 2 w_q / cs2
  __host__ __device__ static constexpr T inv_w(int q) { return T(1) / w(q); }     // 1 / w_q
};

// Node class byte.
constexpr uint8_t kSolid = 1;     // solid node (bounce-back)
constexpr uint8_t kBoundary = 2;  // fluid node with a solid D3Q19 neighbour (wetting)
constexpr uint8_t kPartial = 4;   // volume-penalised partial-solid node
constexpr uint8_t kTop = 8;       // boundary node with |n_z|/|n| > 0.5 (boundary-phi relaxation)
constexpr int kWwShift = 4;       // bits 4..7: near-wall weight code (0..11 distance, 12 far, 13 solid)
constexpr int kWwFar = 12;
constexpr int kWwSolid = 13;

// Periodic neighbour offsets of one node: o?[d + 1] is the flat-index offset
// of a step d in {-1, 0, +1} along that axis, wrapped at the domain edge.
struct Nbr {
  int ox[3], oy[3], oz[3];
  __device__ __forceinline__ int at(int n, int dx, int dy, int dz) const {
    return n + ox[dx + 1] + oy[dy + 1] + oz[dz + 1];
  }
};

__device__ __forceinline__ Nbr make_nbr_xyz(int ix, int iy, int iz, int nx, int ny, int nz) {
  const int sx = ny * nz, sy = nz;
  Nbr b;
  b.ox[0] = ix == 0 ? (nx - 1) * sx : -sx;
  b.ox[1] = 0;
  b.ox[2] = ix == nx - 1 ? -(nx - 1) * sx : sx;
  b.oy[0] = iy == 0 ? (ny - 1) * sy : -sy;
  b.oy[1] = 0;
  b.oy[2] = iy == ny - 1 ? -(ny - 1) * sy : sy;
  b.oz[0] = iz == 0 ? nz - 1 : -1;
  b.oz[1] = 0;
  b.oz[2] = iz == nz - 1 ? -(nz - 1) : 1;
  return b;
}

__device__ __forceinline__ Nbr make_nbr(int n, int nx, int ny, int nz, int* ix_out, int* iy_out,
                                        int* iz_out) {
  const int iz = n % nz;
  const int t = n / nz;
  const int iy = t % ny;
  const int ix = t / ny;
  const int sx = ny * nz, sy = nz;
  Nbr b;
  b.ox[0] = ix == 0 ? (nx - 1) * sx : -sx;
  b.ox[1] = 0;
  b.ox[2] = ix == nx - 1 ? -(nx - 1) * sx : sx;
  b.oy[0] = iy == 0 ? (ny - 1) * sy : -sy;
  b.oy[1] = 0;
  b.oy[2] = iy == ny - 1 ? -(ny - 1) * sy : sy;
  b.oz[0] = iz == 0 ? nz - 1 : -1;
  b.oz[1] = 0;
  b.oz[2] = iz == nz - 1 ? -(nz - 1) : 1;
  *ix_out = ix;
  *iy_out = iy;
  *iz_out = iz;
  return b;
}

// Exact n / d for 0 <= n < 2^31 and 1 <= d < 2^31 by a multiply-high and a
// shift (division by an invariant integer, Granlund & Montgomery 1994):
// with l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1,
// n / d = (umulhi(n, m) + n) >> l.
struct FastDiv {
  unsigned d, m, l;
  __device__ __forceinline__ unsigned div(unsigned n) const { return (__umulhi(n, m) + n) >> l; }
};
inline FastDiv make_fastdiv(unsigned d) {
  FastDiv f;
  f.d = d;
  f.l = 0;
  while ((1ull << f.l) < d) ++f.l;
  f.m = (unsigned)((((1ull << f.l) - d) << 32) / d + 1ull);
  return f;
}

// Storage element of node n (see Consts::nh): n in the linear layout, 2n or
// 2(n - nh) + 1 in the paired layout.
template <typename K>
__host__ __device__ __forceinline__ unsigned sidx(const K& k, int n) {
  const unsigned nh = (unsigned)k.nh, un = (unsigned)n;
  if (nh == 0u) return un;
  return un < nh ? 2u * un : 2u * (un - nh) + 1u;
}

// Population arrays (f, g), u and phi store component j of node n at
// j * Np + sidx(n), Np = N rounded up to a multiple of kAlignNodes, so that every component
// array starts on a 128-byte line and a warp's 32 consecutive nodes of one
// component fill whole lines.  Caller-facing arrays are dense (j * N + n).
constexpr int kAlignNodes = 32;

// Constants of one grid's time step in the compute type T.  Every value is
// the reference's python-double expression rounded once to T at the point the
// reference mixes it into a T tensor.
template <typename T>
struct Consts {
  int nx, ny, nz, N;
  int Np;             // component stride of f, g and u (N rounded up to kAlignNodes)
  FastDiv dz, dy;     // division by nz and by ny
  // Paired layout (3-D grids with even nx): nodes x and x + nx/2 of the same
  // (y, z) share one pair p = ((x mod nx/2) ny + y) nz + z; the populations,
  // u and phi of the pair's lower node sit at element 2p of their component
  // array and the upper node's at 2p + 1, so one 8-byte (float) or 4-byte
  // (half) word holds both.  nh = N / 2 pairs, hx = nx / 2; nh == 0 selects
  // the linear layout (element n).  Node-indexed arrays (class byte, wall
  // normal, fraction, amplification, mu) keep node order n: the lower node of
  // pair p is node p, the upper node p + nh.
  int nh, hx;
  T w[Q];      // lattice weights (float32 table, widened)
  T wc[Q];     // w_i / cs2                      (stencil weights)
  T w2c[Q];    // 2 w_i / cs2                    (laplacian weights)
  T wac[Q];    // (1 - 1/(2 tau_f)) w_i          (Allen-Cahn source)
  T wac3[Q];   // wac_i / cs2
  T inv_w[Q];  // 1 / w_i (deviation storage)
  T cs2, two_cs2, inv_cs2, inv_two_cs2, inv_W;
  T beta4, kappa, phi_c, W;
  T rho_l, rho_g, rho_floor, drho;
  T visc;      // (1/2 - tau_g) / tau_g
  T omega_f;   // 1 / tau_f
  T omega_g;   // 1 / tau_l (tau_l == tau_g)
  T tau_l, tl_m, tg_m;  // tau_l, tau_l - 1/2, tau_g - 1/2
  int tau_const;        // tau_l == tau_g
  T gforce[3];
  int has_gforce;
  int stab_mode;
  T ac_scale, sharpen_reduce;
  int wetting, linear, geometric, amp_active, relax_on;
  float h_over_kappa_f;  // ghost offset factor (linear), float32 like n.e_i
  float pcok_f;          // phi_c / kappa (quadratic), float32 like n.e_i
  T mu_wall_add;         // mu_wall * mu_wall_scale (linear)
  T cos_t, sin_t, amp;
  T relax_r, relax_target;
  T ww[16];              // near-wall weight by code (float32 values)
  // chemical-potential gradient terms of the interface source
  // (lbm/fe_ac_solver.py:457-486): 0 none, kGmuCH Cahn-Hilliard, kGmuDrive mu_drive
  int gmu_mode;
  T mob, guo, mu_drive_a;  // mobility cs2 (tau_f - 1/2), tau_f / (tau_f - 1/2), mu_drive * mobility
};
constexpr int kGmuCH = 1;
constexpr int kGmuDrive = 2;

// Device state of one grid.  T is the compute type, S the population
// storage type (T itself, or half for the deviation-storage form).
template <typename T, typename S = T>
struct State {
  const S* fin;   // populations read this step (post-collision of the last step, or raw)
  const S* gin;
  S* fout;        // post-collision populations written this step
  S* gout;
  T* u;           // velocity [3][N], in place
  const T* phi_in;  // phi recovered by the last step (before its mass correction)
  T* phi_out;       // phi recovered by this step (written by the phi kernel in the two-kernel step)
  const uint8_t* cls;
  const float* wn;  // wall normal [3][N] (non-zero at boundary nodes only)
  const T* eps;     // solid fraction (read at partial nodes only)
  const T* amp;     // per-node geometric amplification (read at boundary nodes only; null: the scalar k.amp)
  T* mu;            // chemical potential of this step [Np] (k_mu; the gradient-of-mu modes only)
  T* gmu;           // its isotropic gradient [3][Np] (k_gradmu; the gradient-of-mu modes only)
  const int* nsw;   // next-interior fluid node of a boundary node or -1 [N] (direct wetting only)
  // direct wetting (cubic wall energy, fe_wetting.py:369-416), null when off:
  // (1 - a)^2, 4 a, -(1 - a), 2 a with a = 6 sigma cos(theta) / kappa (2 a = 0: no cubic root).
  // Kept out of Consts: the step kernels' register allocation is sensitive to its size.
  const T* cubic;
  double* partials; // one per block
  unsigned* counter;
  T* cbuf;          // mass-correction factor of the last two steps
  double* scal;     // [0] phi_mass_init, [1] last sum(phi)
  unsigned* status;
  int c_prev, c_cur;  // cbuf slots: factor applied to fin, factor produced this step
};

// Droplet to inject mid-run (lbm/fe_ac_solver.py:645-732): centre, radius,
// interface width, impact velocity; obs_init: the attributes phi, u, P are
// those of init_fields (no step since init or the last injection).
struct InjectParams {
  double c[3], radius, xi, u[3];
  int obs_init;
};

// Tiling of the fused step kernel: one CTA per tile of TX x TY x TZ nodes
// (z fastest), tiles clipped at the domain edge.
struct Tiling {
  int tx, ty, tz;     // tile extents
  int ntx, nty, ntz;  // tiles per axis
  int hmax;           // (tx + 2)(ty + 2)(tz + 2): halo-tile nodes
};

}  // namespace lbm
