// The 2-D (nz == 1) D2Q9 form of the Allen-Cahn phase-field step
// (pytorch-lbm lbm/fe_ac_solver.py:380-639 with lbm/lattice.py:36-57): the
// same pull-form state, node classes, correction factors and step sequencing
// as the 3-D kernels, with the D2Q9 velocity set and two velocity components.
//
// Layout: node n = ix * ny + iy (y fastest), populations and u at
// j * Np + n like the 3-D form.  One thread per node; a step is
//   k2_phi     phi of every node from the pulled f (bounce-back, volume
//              penalisation, last step's mass correction and boundary-phi
//              relaxation) and the grid sum of phi -> this step's correction;
//   k2_mu, k2_gradmu  (Cahn-Hilliard and mu-drive modes only) mu of every
//              node, then its isotropic gradient;
//   k2_update  stencils, wetting, forces, velocity, both BGK collisions.
// Besides: k2_init (init_fields), k2_inject (inject_droplet), k2_observe and
// k2_populations (attribute read-out).
// These kernels keep the reference's operation order (divisions, per-
// population non-equilibrium stress) instead of the restructured moment and
// collision algebra of the 3-D kernels, and are compiled without FMA
// contraction: float32 parity on the 2-D cases needed both.
#include <cuda_runtime.h>

#include "lbm_common.cuh"

namespace lbm {
namespace d2 {

constexpr int Q9 = 9;

// D2Q9 in the reference's population order: rest, E, W, N, S, NE, NW, SW, SE.
__host__ __device__ constexpr int ex(int q) { return (q == 1 || q == 5 || q == 8) ? 1 : (q == 2 || q == 6 || q == 7) ? -1 : 0; }
__host__ __device__ constexpr int ey(int q) { return (q == 3 || q == 5 || q == 6) ? 1 : (q == 4 || q == 7 || q == 8) ? -1 : 0; }
__host__ __device__ constexpr int opp(int q) {
  return q == 0 ? 0 : q == 1 ? 2 : q == 2 ? 1 : q == 3 ? 4 : q == 4 ? 3 : q == 5 ? 7 : q == 6 ? 8 : q == 7 ? 5 : 6;
}
// float32 weights widened to T (lbm/lattice.py:51-55; float32 in float64 runs too)
template <typename T>
__host__ __device__ constexpr T w(int q) {
  return q == 0 ? T(float(4.0 / 9.0)) : (q <= 4 ? T(float(1.0 / 9.0)) : T(float(1.0 / 36.0)));
}
template <typename T>
__host__ __device__ constexpr T cs2() { return T(1.0 / 3.0); }

template <typename T>
__device__ __forceinline__ T clamp01(T v) {
  return v < T(0) ? T(0) : (v > T(1) ? T(1) : v);
}

// Periodic neighbour n + (dx, dy) of node (ix, iy).
struct Nb2 {
  int ox[3], oy[3];
  __device__ __forceinline__ int at(int n, int dx, int dy) const { return n + ox[dx + 1] + oy[dy + 1]; }
};
__device__ __forceinline__ Nb2 make_nb2(int n, int nx, int ny) {
  const int ix = n / ny, iy = n - (n / ny) * ny;
  Nb2 b;
  b.ox[0] = ix == 0 ? (nx - 1) * ny : -ny;
  b.ox[1] = 0;
  b.ox[2] = ix == nx - 1 ? -(nx - 1) * ny : ny;
  b.oy[0] = iy == 0 ? ny - 1 : -1;
  b.oy[1] = 0;
  b.oy[2] = iy == ny - 1 ? -(ny - 1) : 1;
  return b;
}

template <typename T>
__device__ __forceinline__ T seqsum(const T (&v)[Q9]) {
  T s = v[0];
#pragma unroll
  for (int q = 1; q < Q9; ++q) s = s + v[q];
  return s;
}

// Populations of node n as the reference holds them at the start of the step:
// pulled from x - e_q, the node's own opposite values at solid nodes
// (bounce-back), blended with them at partial nodes (volume penalisation),
// times corr (the last step's mass correction; 1 for the raw state).
template <typename T, bool RAW>
__device__ __forceinline__ void fetch9(T (&v)[Q9], const T* __restrict__ F, int Np, int n, const Nb2& nb,
                                       uint8_t c, T eps, T corr) {
  if (RAW) {
#pragma unroll
    for (int q = 0; q < Q9; ++q) v[q] = F[q * Np + n];
    return;
  }
  if (c & kSolid) {
#pragma unroll
    for (int q = 0; q < Q9; ++q) v[q] = F[opp(q) * Np + n];
  } else {
#pragma unroll
    for (int q = 0; q < Q9; ++q) v[q] = F[q * Np + nb.at(n, -ex(q), -ey(q))];
    if (c & kPartial) {
      const T one_m = T(1) - eps;
#pragma unroll
      for (int q = 0; q < Q9; ++q) v[q] = one_m * v[q] + eps * F[opp(q) * Np + n];
    }
  }
  if (corr != T(1)) {
#pragma unroll
    for (int q = 0; q < Q9; ++q) v[q] = v[q] * corr;
  }
}

// Boundary-phi relaxation target of a top-surface boundary node
// (lbm/fe_ac_solver.py:594-624; direct wetting fe_wetting.py:369-416), or
// negative when the node is not active: as the 3-D form.
template <typename T>
__device__ __forceinline__ T relax_target(const Consts<T>& k, const T* __restrict__ phi_arr,
                                          const int* __restrict__ nsw, const T* __restrict__ cubic, int n, T phi_prev,
                                          T corr) {
  const T pb = clamp01(phi_prev * corr);
  if (!(pb > T(0.15) && pb < T(0.85))) return T(-1);
  T target = k.relax_target;
  if (cubic) {
    target = pb;
    const int m = nsw[n];
    if (m >= 0 && cubic[3] != T(0) && pb > T(0.01) && pb < T(0.99)) {
      const T pn = clamp01(phi_arr[m] * corr);
      T disc = cubic[0] + cubic[1] * pn;
      disc = disc < T(0) ? T(0) : disc;
      target = clamp01((cubic[2] + sqrt(disc)) / cubic[3]);
    }
  }
  return clamp01(pb + k.relax_r * (target - pb));
}

template <typename T>
__device__ __forceinline__ T relax_scale(T target, T sum_f) {
  const T safe = sum_f < T(1e-10) ? T(1e-10) : sum_f;
  const T s = target / safe;
  return s < T(0.5) ? T(0.5) : (s > T(2.0) ? T(2.0) : s);
}

// f of node n at the start of the step (pull, correction, relaxation).
template <typename T, bool RAW>
__device__ __forceinline__ void fetch_f9(T (&v)[Q9], const Consts<T>& k, const State<T, T>& s, int n,
                                         const Nb2& nb, uint8_t c, T eps) {
  const T corr = RAW ? T(1) : s.cbuf[s.c_prev];
  fetch9<T, RAW>(v, s.fin, k.Np, n, nb, c, eps, corr);
  if (!RAW && k.relax_on && (c & kTop)) {
    const T r = relax_target(k, s.phi_in, s.nsw, s.cubic, n, s.phi_in[n], corr);
    if (r >= T(0)) {
      const T sc = relax_scale(r, seqsum(v));
#pragma unroll
      for (int q = 0; q < Q9; ++q) v[q] = v[q] * sc;
    }
  }
}

// Ghost value of a boundary node's solid neighbour in direction q
// (fe_wetting.py:418-446): n.e_q in float32, then the linear or quadratic form.
template <typename T>
__device__ __forceinline__ T ghost(const Consts<T>& k, float n0, float n1, int q, T v) {
  float nde = 0.0f;
  nde = __fadd_rn(nde, __fmul_rn(n0, (float)ex(q)));
  nde = __fadd_rn(nde, __fmul_rn(n1, (float)ey(q)));
  return k.linear ? v - (T)__fmul_rn(nde, k.h_over_kappa_f) : v + (T)__fmul_rn(nde, k.pcok_f) * v * (T(1) - v);
}

// Fused isotropic gradient and laplacian of phi (lbm/fe_ac_solver.py:296-320),
// or the unfused laplacian of init_fields (:282-294) when !FUSED.
template <typename T, bool FUSED>
__device__ __forceinline__ void grad_lap(const Consts<T>& k, const State<T, T>& s, int n, const Nb2& nb, uint8_t c,
                                         T phi, const T* __restrict__ field, T& gx, T& gy, T& lap) {
  const bool gh = k.wetting && (c & kBoundary);
  float n0 = 0.0f, n1 = 0.0f;
  if (gh) {
    n0 = s.wn[n];
    n1 = s.wn[k.N + n];
  }
  gx = gy = lap = T(0);
#pragma unroll
  for (int q = 1; q < Q9; ++q) {
    const int m = nb.at(n, ex(q), ey(q));
    T ps = field[m];
    if (gh && (s.cls[m] & kSolid)) ps = ghost(k, n0, n1, q, phi);
    if (FUSED) {
      const T wi = w<T>(q) / cs2<T>();
      if (ex(q) != 0) gx = gx + (ex(q) > 0 ? wi : -wi) * ps;
      if (ey(q) != 0) gy = gy + (ey(q) > 0 ? wi : -wi) * ps;
      lap = lap + (T(2) * wi) * (ps - phi);
    } else {
      lap = lap + (T(2) * w<T>(q)) * (ps - phi) / cs2<T>();
    }
  }
}

// Chemical potential (lbm/fe_ac_solver.py:326-340).
template <typename T>
__device__ __forceinline__ T chem_pot(const Consts<T>& k, uint8_t c, T phi, T lap) {
  T mu = k.beta4 * phi * (phi - T(1)) * (phi - T(0.5)) - k.kappa * lap;
  if (k.wetting && (c & kBoundary)) {
    if (k.linear) mu = mu + k.mu_wall_add;
    else mu = mu + k.phi_c * phi * (T(1) - phi);
  }
  return mu;
}

// e_q . (a0, a1) with the reference's two-term sums.
template <typename T>
__device__ __forceinline__ T edot(int q, T a0, T a1) {
  if (ex(q) != 0 && ey(q) != 0) return (ex(q) > 0 ? a0 : -a0) + (ey(q) > 0 ? a1 : -a1);
  if (ex(q) != 0) return ex(q) > 0 ? a0 : -a0;
  if (ey(q) != 0) return ey(q) > 0 ? a1 : -a1;
  return T(0);
}

// t[q] = (c e_q . (a0, a1)) / d for every q, with one division per opposite
// pair (q, opp q): e_opp(q) . a = -(e_q . a) exactly, and (c (-x)) / d =
// -((c x) / d) in IEEE arithmetic, so the opposite's value is the negation.
// c and d depend on the weight class (cw: per q); the rest value is
// (c 0) / d.  Same values as the per-q expression of the reference.
template <typename T, typename CW>
__device__ __forceinline__ void pair_div(T (&t)[Q9], T a0, T a1, CW cw, T d) {
  t[0] = (cw(0) * edot(0, a0, a1)) / d;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int q = i < 2 ? 1 + 2 * i : 5 + (i - 2);  // 1, 3, 5, 6
    t[q] = (cw(q) * edot(q, a0, a1)) / d;
    t[opp(q)] = -t[q];
  }
}

// Block total published; the last block to finish adds the block totals
// (each of its threads a fixed strided subset, then a fixed shuffle tree, so
// the float64 total is the same on every run) and returns true in thread 0
// with the grid total (exact for float phi: unsigned 64-bit fixed point with
// 31 fraction bits; NaN carried by a flag).
constexpr unsigned long long kNaN = ~0ull;
template <typename T>
__device__ __forceinline__ bool grid_total(double part_d, unsigned long long part_u, bool nan, double* partials,
                                           unsigned* counter, double* total) {
  __shared__ unsigned long long su[kBlock / 32];
  __shared__ double sd[kBlock / 32];
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    part_u += __shfl_down_sync(0xffffffffu, part_u, o);
    part_d += __shfl_down_sync(0xffffffffu, part_d, o);
  }
  const bool any_nan = __syncthreads_or(nan) != 0;
  if (lane == 0) {
    su[wid] = part_u;
    sd[wid] = part_d;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long r = 0ull;
    double d = 0.0;
    for (int i = 0; i < kBlock / 32; ++i) {
      r += su[i];
      d += sd[i];
    }
    if (sizeof(T) == 8) partials[blockIdx.x] = d;
    else reinterpret_cast<unsigned long long*>(partials)[blockIdx.x] = any_nan ? kNaN : r;
    __threadfence();
    s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  double td = 0.0;
  unsigned long long tu = 0ull;
  bool nn = false;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += kBlock) {
    if (sizeof(T) == 8) {
      td += ((const volatile double*)partials)[b];
    } else {
      const unsigned long long v = ((const volatile unsigned long long*)partials)[b];
      if (v == kNaN) nn = true;
      else tu += v;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    td += __shfl_down_sync(0xffffffffu, td, o);
    tu += __shfl_down_sync(0xffffffffu, tu, o);
  }
  nn = __syncthreads_or(nn) != 0;
  if (lane == 0) {
    su[wid] = tu;
    sd[wid] = td;
  }
  __syncthreads();
  if (threadIdx.x != 0) return false;
  double d = 0.0;
  unsigned long long r = 0ull;
  for (int i = 0; i < kBlock / 32; ++i) {
    r += su[i];
    d += sd[i];
  }
  if (sizeof(T) == 8) *total = d;
  else *total = nn ? __longlong_as_double(0x7ff8000000000000ll) : (double)r / 2147483648.0;
  *counter = 0u;
  return true;
}

template <typename T>
__device__ __forceinline__ void add_phi(T phi, double& d, unsigned long long& u, bool& nan) {
  if (sizeof(T) == 8) {
    d += (double)phi;
  } else {
    u += (unsigned long long)__float2uint_rn((float)phi * 2147483648.0f);
    nan |= !(phi == phi);
  }
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
// init_fields (lbm/fe_ac_solver.py:239-261): phi = clamp(phi0), f = f_eq,
// g = g_eq(0, u), phi-mass reference.
template <typename T, typename Src>
__global__ void __launch_bounds__(kBlock) k2_init(Consts<T> k, State<T, T> s, const Src* phi0, const Src* u0) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  double part = 0.0;
  if (n < k.N) {
    const T phi = clamp01((T)phi0[n]);
    const T v0 = u0 ? (T)u0[n] : T(0), v1 = u0 ? (T)u0[k.N + n] : T(0);
    const T usq = v0 * v0 + v1 * v1;
    const T b = usq / (T(2) * cs2<T>());
    T* f = const_cast<T*>(s.fin);
    T* g = const_cast<T*>(s.gin);
#pragma unroll
    for (int q = 0; q < Q9; ++q) {
      const T ec = edot(q, v0, v1) / cs2<T>();
      f[q * k.Np + n] = phi * (w<T>(q) * (((T(1) + ec) + ec * ec / T(2)) - b));
      g[q * k.Np + n] = T(0) * w<T>(q) + w<T>(q) * ((ec + ec * ec / T(2)) - b);
    }
    s.u[n] = v0;
    s.u[k.Np + n] = v1;
    s.u[2 * k.Np + n] = T(0);
    s.phi_out[n] = phi;
    part = (double)phi;
  }
  // phi_mass_init = sum(phi).item() in T (float64 partials in block order)
  double total;
  if (grid_total<double>(part, 0ull, false, s.partials, s.counter, &total)) {
    s.scal[0] = (double)(T)total;
    s.scal[1] = total;
    s.cbuf[0] = T(1);
    s.cbuf[1] = T(1);
  }
}

// phi of every node of this step, its grid sum and the mass-correction factor
// (lbm/fe_ac_solver.py:385-389, 582-589).
// Persistent: a grid of about one wave strides over the nodes, so that few
// blocks publish partial sums.
template <typename T, bool RAW>
__global__ void __launch_bounds__(kBlock) k2_phi(Consts<T> k, State<T, T> s) {
  double pd = 0.0;
  unsigned long long pu = 0ull;
  bool nan = false;
  for (int n = blockIdx.x * kBlock + threadIdx.x; n < k.N; n += gridDim.x * kBlock) {
    const uint8_t c = s.cls[n];
    T phi = T(0);
    if (!(c & kSolid)) {
      const Nb2 nb = make_nb2(n, k.nx, k.ny);
      const T eps = (c & kPartial) ? s.eps[n] : T(0);
      T v[Q9];
      fetch_f9<T, RAW>(v, k, s, n, nb, c, eps);
      phi = clamp01(seqsum(v));
    }
    s.phi_out[n] = phi;
    add_phi(phi, pd, pu, nan);
  }
  double total;
  if (grid_total<T>(pd, pu, nan, s.partials, s.counter, &total)) {
    const T sum = (T)total;
    T corr = T(1);
    if (sum > T(1e-6)) {
      const T safe = sum < T(1e-6) ? T(1e-6) : sum;
      corr = (T(1) / safe) * (T)s.scal[0];
    } else {
      atomicOr(s.status, 2u);
    }
    if (!(total == total) || total - total != 0.0) atomicOr(s.status, 1u);
    s.cbuf[s.c_cur] = corr;
    s.scal[1] = total;
  }
}

// mu of every node from this step's phi (the update kernel's arithmetic).
template <typename T>
__global__ void __launch_bounds__(kBlock) k2_mu(Consts<T> k, State<T, T> s) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  const uint8_t c = s.cls[n];
  const Nb2 nb = make_nb2(n, k.nx, k.ny);
  const T phi = s.phi_out[n];
  T gx, gy, lap;
  grad_lap<T, true>(k, s, n, nb, c, phi, s.phi_out, gx, gy, lap);
  s.mu[n] = chem_pot(k, c, phi, lap);
}

// Isotropic gradient of mu with the ghost correction applied to mu itself
// (lbm/fe_ac_solver.py:267-280): grad_d += ((w_q e_qd) mu(x + e_q)) / cs2.
template <typename T>
__global__ void __launch_bounds__(kBlock) k2_gradmu(Consts<T> k, State<T, T> s) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  const uint8_t c = s.cls[n];
  const Nb2 nb = make_nb2(n, k.nx, k.ny);
  const T mu = s.mu[n];
  const bool gh = k.wetting && (c & kBoundary);
  const float n0 = gh ? s.wn[n] : 0.0f, n1 = gh ? s.wn[k.N + n] : 0.0f;
  T gx = T(0), gy = T(0);
#pragma unroll
  for (int q = 1; q < Q9; ++q) {
    const int m = nb.at(n, ex(q), ey(q));
    T v = s.mu[m];
    if (gh && (s.cls[m] & kSolid)) v = ghost(k, n0, n1, q, mu);
    if (ex(q) != 0) gx = gx + ((w<T>(q) * T(ex(q))) * v) / cs2<T>();
    if (ey(q) != 0) gy = gy + ((w<T>(q) * T(ey(q))) * v) / cs2<T>();
  }
  s.gmu[n] = gx;
  s.gmu[k.Np + n] = gy;
}

// The rest of the step for every node (lbm/fe_ac_solver.py:392-530): phi
// stencil -> gradient, laplacian, chemical potential, geometric wetting
// correction; pressure, non-equilibrium stress (new P, old u), forces,
// velocity, Allen-Cahn source, both BGK collisions; writes fout, gout, u.
// ac: the python-double Allen-Cahn source coefficient 1 - 1 / (2 tau_f).
// OMEGA1: tau_f == 1 (the reference's default tau_h), where the phase-field
// collision f - (f - f_eq) + src is taken as f_eq + src and f is not read
// again (the two differ by at most an ulp of f where f and f_eq are more
// than a factor of two apart).
template <typename T, bool RAW, bool FIRST, bool GMU, bool OMEGA1 = false>
__global__ void __launch_bounds__(kBlock) k2_update(Consts<T> k, State<T, T> s, double ac) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  const int Np = k.Np;
  const uint8_t c = s.cls[n];
  const Nb2 nb = make_nb2(n, k.nx, k.ny);
  const T phi = s.phi_out[n];
  T gx, gy, lap;
  grad_lap<T, true>(k, s, n, nb, c, phi, s.phi_out, gx, gy, lap);
  const T rho = phi * k.rho_l + (T(1) - phi) * k.rho_g;
  const T rho_eff = rho < k.rho_floor ? k.rho_floor : rho;
  const T mu = GMU ? s.mu[n] : chem_pot(k, c, phi, lap);

  // geometric contact-angle gradient correction (fe_wetting.py:448-539); the
  // identity where the wall normal is zero, so boundary nodes only
  if (k.geometric && (c & kBoundary)) {
    const T n0 = (T)s.wn[n], n1 = (T)s.wn[k.N + n];
    const T gn = n0 * gx + n1 * gy;
    const T tx = gx - gn * n0, ty = gy - gn * n1;
    T tm = sqrt(tx * tx + ty * ty);
    tm = tm < T(1e-10) ? T(1e-10) : tm;
    T gd = (-tm * k.cos_t) / k.sin_t;
    T a = k.amp;
    bool amp_on = k.amp_active;
    if (s.amp) {
      a = s.amp[n];
      amp_on = a > T(1);
    }
    if (amp_on) gd = gn + (gd - gn) * a;
    const T cx = tx + gd * n0, cy = ty + gd * n1;
    const T gm = sqrt(gx * gx + gy * gy);
    if (gm > T(1e-6)) {
      const T bl = k.ww[c >> kWwShift];
      gx = gx + bl * (cx - gx);
      gy = gy + bl * (cy - gy);
    }
  }

  // g as the reference holds it at the step start, u and phi of the last step
  const T eps = (c & kPartial) ? s.eps[n] : T(0);
  T g[Q9];
  fetch9<T, RAW>(g, s.gin, Np, n, nb, c, eps, T(1));
  const T uo0 = s.u[n], uo1 = s.u[Np + n];
  const T pp = FIRST ? T(0) : s.phi_in[n];

  // 3.-4. pressure and the non-equilibrium stress with the new P, old u
  const T P = seqsum(g);
  T sxx = T(0), syy = T(0), sxy = T(0);
  {
    const T usq = uo0 * uo0 + uo1 * uo1;
    const T b = usq / (T(2) * cs2<T>());
    T ecs[Q9];
    pair_div(ecs, uo0, uo1, [](int) { return T(1); }, cs2<T>());
#pragma unroll
    for (int q = 1; q < Q9; ++q) {
      const T ec = ecs[q];
      const T geq = P * w<T>(q) + w<T>(q) * ((ec + ec * ec / T(2)) - b);
      const T d = g[q] - geq;
      if (ex(q) != 0) sxx = sxx + d;
      if (ey(q) != 0) syy = syy + d;
      if (ex(q) * ey(q) != 0) sxy = sxy + (ex(q) * ey(q) > 0 ? d : -d);
    }
  }

  // 5. forces (Fakhari 2017, :416-439)
  T F0 = mu * gx, F1 = mu * gy;
  if (k.stab_mode <= 1) {
    const T fp = ((-P) * k.drho) * k.cs2;
    F0 = F0 + fp * gx;
    F1 = F1 + fp * gy;
  }
  if (k.stab_mode == 0) {
    F0 = F0 + (k.visc * (sxx * gx + sxy * gy)) * k.drho;
    F1 = F1 + (k.visc * (sxy * gx + syy * gy)) * k.drho;
  }
  if (k.has_gforce) {
    F0 = F0 + k.gforce[0] * rho;
    F1 = F1 + k.gforce[1] * rho;
  }

  // 6. velocity (:442-447)
  T ux = T(0), uy = T(0);
  bool fx = true, fy = true;
#pragma unroll
  for (int q = 1; q < Q9; ++q) {
    if (ex(q) != 0) {
      const T t = ex(q) > 0 ? g[q] : -g[q];
      ux = fx ? t : ux + t;
      fx = false;
    }
    if (ey(q) != 0) {
      const T t = ey(q) > 0 ? g[q] : -g[q];
      uy = fy ? t : uy + t;
      fy = false;
    }
  }
  T u0 = ux + (T(0.5) * F0) / rho_eff, u1 = uy + (T(0.5) * F1) / rho_eff;
  if (c & kSolid) u0 = u1 = T(0);

  // 7. interface source (:450-494)
  T S0 = FIRST ? T(0) : phi * u0 - pp * uo0;
  T S1 = FIRST ? T(0) : phi * u1 - pp * uo1;
  T mx = T(0), my = T(0);
  if (GMU) {
    mx = s.gmu[n];
    my = s.gmu[Np + n];
  }
  if (GMU && k.gmu_mode == kGmuCH) {
    S0 = S0 + (k.mob * (mx - gx)) * k.guo;
    S1 = S1 + (k.mob * (my - gy)) * k.guo;
  } else {
    T gm = sqrt(gx * gx + gy * gy);
    gm = gm < T(1e-10) ? T(1e-10) : gm;
    const T lam = ((T(4) * phi) * (T(1) - phi)) / k.W;
    T sx = ((k.cs2 * lam) * (gx / gm)) * k.ac_scale, sy = ((k.cs2 * lam) * (gy / gm)) * k.ac_scale;
    if (k.wetting) {
      const T red = T(1) - k.sharpen_reduce * k.ww[c >> kWwShift];
      sx = sx * red;
      sy = sy * red;
    }
    S0 = S0 + sx;
    S1 = S1 + sy;
    if (GMU) {
      S0 = S0 + k.mu_drive_a * mx;
      S1 = S1 + k.mu_drive_a * my;
    }
  }

  // 8. collisions (:496-530); the pre-collision f is this step's pulled f
  T f[Q9];
  if (!OMEGA1) fetch_f9<T, RAW>(f, k, s, n, nb, c, eps);
  T om, ns;
  if (k.tau_const) {
    om = k.omega_g;
  } else {
    const T eta = phi * k.rho_l * k.tl_m + (T(1) - phi) * k.rho_g * k.tg_m;
    const T rden = phi * k.rho_l + (T(1) - phi) * k.rho_g;
    om = T(1) / (T(0.5) + eta / rden);
  }
  ns = T(1) - om * T(0.5);
  const T usq = u0 * u0 + u1 * u1;
  const T b = usq / (T(2) * cs2<T>());
  const T acT = (T)ac;
  T ecs[Q9], src[Q9], G[Q9];
  pair_div(ecs, u0, u1, [](int) { return T(1); }, cs2<T>());
  pair_div(src, S0, S1, [&](int q) { return acT * w<T>(q); }, cs2<T>());
  pair_div(G, F0, F1, [&](int q) { return ns * w<T>(q); }, rho_eff * cs2<T>());
#pragma unroll
  for (int q = 0; q < Q9; ++q) {
    const T ec = ecs[q];
    const T sq = ec * ec / T(2);
    const T feq = phi * (w<T>(q) * (((T(1) + ec) + sq) - b));
    s.fout[q * Np + n] = OMEGA1 ? feq + src[q] : (f[q] - k.omega_f * (f[q] - feq)) + src[q];
    const T geq = P * w<T>(q) + w<T>(q) * ((ec + sq) - b);
    s.gout[q * Np + n] = (g[q] - om * (g[q] - geq)) + G[q];
  }
  s.u[n] = u0;
  s.u[Np + n] = u1;
}

// Field read-out after the last step (the reference's attribute values):
// s.phi_out holds the last recovered phi, s.cbuf[s.c_cur] its correction;
// mode 0 reads the state init_fields left.
template <typename T, bool RAW_IN>
__global__ void __launch_bounds__(kBlock) k2_observe(Consts<T> k, State<T, T> s, unsigned mask, int mode, T* phi_o,
                                                     T* rho_o, T* u_o, T* P_o, T* p_o, T* mu_o) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  const uint8_t c = s.cls[n];
  const T phi = s.phi_out[n];
  const T rho = phi * k.rho_l + (T(1) - phi) * k.rho_g;
  const Nb2 nb = make_nb2(n, k.nx, k.ny);
  if (mask & 1u) {
    T v = phi;
    if (mode == 1) {
      const T corr = s.cbuf[s.c_cur];
      v = clamp01(phi * corr);
      if (k.relax_on && (c & kTop)) {
        const T r = relax_target(k, (const T*)s.phi_out, s.nsw, s.cubic, n, phi, corr);
        if (r >= T(0)) v = r;
      }
    }
    phi_o[n] = v;
  }
  if (mask & 2u) rho_o[n] = rho;
  if (mask & 4u) {
    u_o[n] = s.u[n];
    u_o[k.N + n] = s.u[k.Np + n];
  }
  if (mask & (8u | 16u)) {
    T P = T(0);
    if (mode == 1) {
      const T eps = (c & kPartial) ? s.eps[n] : T(0);
      T g[Q9];
      fetch9<T, RAW_IN>(g, s.gin, k.Np, n, nb, c, eps, T(1));
      P = seqsum(g);
    }
    if (mask & 8u) P_o[n] = P;
    if (mask & 16u) p_o[n] = mode == 1 ? P * k.cs2 : rho * k.cs2;
  }
  if (mask & 32u) {
    T gx, gy, lap;
    if (mode == 1) grad_lap<T, true>(k, s, n, nb, c, phi, s.phi_out, gx, gy, lap);
    else grad_lap<T, false>(k, s, n, nb, c, phi, s.phi_out, gx, gy, lap);
    mu_o[n] = chem_pot(k, c, phi, lap);
  }
}

// Current populations in the reference layout [9][N].
template <typename T, bool RAW>
__global__ void __launch_bounds__(kBlock) k2_populations(Consts<T> k, State<T, T> s, T* f_o, T* g_o) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  const uint8_t c = s.cls[n];
  const Nb2 nb = make_nb2(n, k.nx, k.ny);
  const T eps = (c & kPartial) ? s.eps[n] : T(0);
  T v[Q9];
  if (f_o) {
    fetch_f9<T, RAW>(v, k, s, n, nb, c, eps);
#pragma unroll
    for (int q = 0; q < Q9; ++q) f_o[q * k.N + n] = v[q];
  }
  if (g_o) {
    fetch9<T, RAW>(v, s.gin, k.Np, n, nb, c, eps, T(1));
#pragma unroll
    for (int q = 0; q < Q9; ++q) g_o[q * k.N + n] = v[q];
  }
}

// Mid-run droplet injection (lbm/fe_ac_solver.py:645-732) on a 2-D grid: the
// 3-D k_inject's steps with D2Q9 and two velocity components.  Reads the
// state as the reference holds it between steps (phi / u / P attributes,
// populations as k2_populations rebuilds them), blends the droplet in and
// writes the raw state init_fields leaves: f, g to the other population
// buffer, phi to the other phi buffer, u in place.  Sums the new phi (the new
// phi-mass reference) and counts the core nodes.
template <typename T, bool RAW>
__global__ void __launch_bounds__(kBlock) k2_inject(Consts<T> k, State<T, T> s, InjectParams ip,
                                                    const T* __restrict__ P_attr, unsigned* core_count) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  double part = 0.0;
  bool core = false;
  if (n < k.N) {
    const int Np = k.Np;
    const uint8_t c = s.cls[n];
    const Nb2 nb = make_nb2(n, k.nx, k.ny);
    const int ix = n / k.ny, iy = n - (n / k.ny) * k.ny;
    // the droplet as the reference builds it: float64 profile, stored as float32
    const double dx = ix - ip.c[0], dy = iy - ip.c[1];
    const double dist = sqrt(dx * dx + dy * dy);
    double Cd = 0.5 + 0.5 * tanh(2.0 * (ip.radius - dist) / ip.xi);
    Cd = Cd < 0.0 ? 0.0 : (Cd > 1.0 ? 1.0 : Cd);
    const T C = (T)(float)Cd;
    core = C > T(0.1);
    // the attributes phi, u, P the reference holds now
    const T corr = s.cbuf[s.c_prev];
    T phi = s.phi_in[n];
    if (!ip.obs_init) {
      const T pr = phi;
      phi = clamp01(pr * corr);
      if (k.relax_on && (c & kTop)) {
        const T r = relax_target(k, s.phi_in, s.nsw, s.cubic, n, pr, corr);
        if (r >= T(0)) phi = r;
      }
    }
    T u0 = s.u[n], u1 = s.u[Np + n];
    const T P = ip.obs_init ? T(0) : P_attr[n];
    const T eps = (c & kPartial) ? s.eps[n] : T(0);
    T fv[Q9], gv[Q9];
    fetch_f9<T, RAW>(fv, k, s, n, nb, c, eps);
    fetch9<T, RAW>(gv, s.gin, Np, n, nb, c, eps, T(1));
    // new phi: the maximum with the droplet in its core, clamped, zero in solid
    T pn = core ? (phi > C ? phi : C) : phi;
    pn = clamp01(pn);
    if (c & kSolid) pn = T(0);
    // new u: (1 - C) u + C u_impact everywhere, zero in solid
    u0 = (T(1) - C) * u0 + C * (T)ip.u[0];
    u1 = (T(1) - C) * u1 + C * (T)ip.u[1];
    if (c & kSolid) u0 = u1 = T(0);
    if (core) {
      const T b = (u0 * u0 + u1 * u1) / (T(2) * cs2<T>());
#pragma unroll
      for (int q = 0; q < Q9; ++q) {
        const T ec = edot(q, u0, u1) / cs2<T>();
        fv[q] = pn * (w<T>(q) * (((T(1) + ec) + ec * ec / T(2)) - b));
        gv[q] = P * w<T>(q) + w<T>(q) * ((ec + ec * ec / T(2)) - b);
      }
    }
#pragma unroll
    for (int q = 0; q < Q9; ++q) {
      s.fout[q * Np + n] = fv[q];
      s.gout[q * Np + n] = gv[q];
    }
    s.u[n] = u0;
    s.u[Np + n] = u1;
    s.phi_out[n] = pn;
    part = (double)pn;
  }
  const int cnt = __syncthreads_count(core);
  if (threadIdx.x == 0 && cnt) atomicAdd(core_count, (unsigned)cnt);
  double total;
  if (grid_total<double>(part, 0ull, false, s.partials, s.counter, &total)) {
    s.scal[0] = (double)(T)total;  // phi_mass_init = phi.sum().item() in T
    s.scal[1] = total;
  }
}

inline int blocks_of(int N) { return (N + kBlock - 1) / kBlock; }

// Blocks of the persistent phi kernel: at most one wave of the device (8
// resident 256-thread blocks per SM at its 32 registers).
inline int phi_blocks_of(int N) {
  static const int wave = [] {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 1;
    return 8 * (sms > 0 ? sms : 1);
  }();
  const int b = blocks_of(N);
  return b < wave ? b : wave;
}

}  // namespace d2

// ---------------------------------------------------------------------------
// Host-side launchers (called from lbm_capi.cu)
// ---------------------------------------------------------------------------
template <typename T, typename Src>
cudaError_t launch_init2d(const Consts<T>& k, const State<T, T>& s, const Src* phi0, const Src* u0, cudaStream_t st) {
  d2::k2_init<T, Src><<<d2::blocks_of(k.N), kBlock, 0, st>>>(k, s, phi0, u0);
  return cudaGetLastError();
}

// One step: k2_phi, [k2_mu, k2_gradmu], k2_update.  `mid` (may be null) is
// recorded between the phi kernel and the rest.
template <typename T>
cudaError_t launch_step2d(const Consts<T>& k, const State<T, T>& s, bool raw, bool first, double ac, cudaStream_t st,
                          cudaEvent_t mid) {
  const int nb = d2::blocks_of(k.N), np = d2::phi_blocks_of(k.N);
  if (raw) d2::k2_phi<T, true><<<np, kBlock, 0, st>>>(k, s);
  else d2::k2_phi<T, false><<<np, kBlock, 0, st>>>(k, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (mid) {
    e = cudaEventRecord(mid, st);
    if (e != cudaSuccess) return e;
  }
  const bool gmu = s.mu != nullptr;
  if (gmu) {
    d2::k2_mu<T><<<nb, kBlock, 0, st>>>(k, s);
    d2::k2_gradmu<T><<<nb, kBlock, 0, st>>>(k, s);
  }
#define LBM_UPD2(R, F)                                                      \
  if (gmu) d2::k2_update<T, R, F, true><<<nb, kBlock, 0, st>>>(k, s, ac);  \
  else d2::k2_update<T, R, F, false><<<nb, kBlock, 0, st>>>(k, s, ac);
  if (raw && first) {
    LBM_UPD2(true, true)
  } else if (raw) {
    LBM_UPD2(true, false)
  } else if (first) {
    LBM_UPD2(false, true)
  } else if (!gmu && k.omega_f == T(1)) {
    d2::k2_update<T, false, false, false, true><<<nb, kBlock, 0, st>>>(k, s, ac);
  } else {
    LBM_UPD2(false, false)
  }
#undef LBM_UPD2
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_observe2d(const Consts<T>& k, const State<T, T>& s, bool raw_in, unsigned mask, int mode, T* phi,
                             T* rho, T* u, T* P, T* p, T* mu, cudaStream_t st) {
  const int nb = d2::blocks_of(k.N);
  if (raw_in) d2::k2_observe<T, true><<<nb, kBlock, 0, st>>>(k, s, mask, mode, phi, rho, u, P, p, mu);
  else d2::k2_observe<T, false><<<nb, kBlock, 0, st>>>(k, s, mask, mode, phi, rho, u, P, p, mu);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_populations2d(const Consts<T>& k, const State<T, T>& s, bool raw, T* f, T* g, cudaStream_t st) {
  const int nb = d2::blocks_of(k.N);
  if (raw) d2::k2_populations<T, true><<<nb, kBlock, 0, st>>>(k, s, f, g);
  else d2::k2_populations<T, false><<<nb, kBlock, 0, st>>>(k, s, f, g);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_inject2d(const Consts<T>& k, const State<T, T>& s, bool raw, const InjectParams& ip,
                            const T* P_attr, unsigned* core_count, cudaStream_t st) {
  const int nb = d2::blocks_of(k.N);
  if (raw) d2::k2_inject<T, true><<<nb, kBlock, 0, st>>>(k, s, ip, P_attr, core_count);
  else d2::k2_inject<T, false><<<nb, kBlock, 0, st>>>(k, s, ip, P_attr, core_count);
  return cudaGetLastError();
}

#define LBM_INST2D(T)                                                                                               \
  template cudaError_t launch_init2d<T, float>(const Consts<T>&, const State<T, T>&, const float*, const float*,    \
                                               cudaStream_t);                                                       \
  template cudaError_t launch_init2d<T, double>(const Consts<T>&, const State<T, T>&, const double*, const double*, \
                                                cudaStream_t);                                                      \
  template cudaError_t launch_step2d<T>(const Consts<T>&, const State<T, T>&, bool, bool, double, cudaStream_t,     \
                                        cudaEvent_t);                                                               \
  template cudaError_t launch_observe2d<T>(const Consts<T>&, const State<T, T>&, bool, unsigned, int, T*, T*, T*,   \
                                           T*, T*, T*, cudaStream_t);                                               \
  template cudaError_t launch_populations2d<T>(const Consts<T>&, const State<T, T>&, bool, T*, T*, cudaStream_t);  \
  template cudaError_t launch_inject2d<T>(const Consts<T>&, const State<T, T>&, bool, const InjectParams&, const T*, \
                                          unsigned*, cudaStream_t);
LBM_INST2D(float)
LBM_INST2D(double)
#undef LBM_INST2D

}  // namespace lbm
