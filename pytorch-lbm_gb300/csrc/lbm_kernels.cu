// Device kernels of the GB300 Allen-Cahn phase-field LBM step.
//
// State convention ("pull" form).  Between steps the population buffers hold
// POST-COLLISION values F(x, q) of every node, solid and partial nodes
// included.  The reference's state at the start of a step (pytorch-lbm
// lbm/fe_ac_solver.py:548-636: streamed, bounced back at solid nodes,
// volume-penalised at partial nodes, scaled by the global phi-mass correction
// c, then boundary-phi relaxed at active boundary nodes) is reconstructed on
// read:
//   fluid x    f(x,q) = c F(x - e_q, q)                               (periodic)
//   solid x    f(x,q) = c F(x, opp q)                                  (:556-566)
//   partial x  f(x,q) = c ((1 - eps) F(x - e_q, q) + eps F(x, opp q))  (:569-578)
//   relaxed x  f(x,q) *= clamp(phi_new / max(sum_q f(x,q), 1e-10), 1/2, 2)   (:594-636)
// where the relaxation target phi_new is recomputed from the previous step's
// phi and c (it depends on nothing else).  g is reconstructed the same way
// without c and without relaxation.  Right after init (RAW) the buffers hold
// the reference state itself.
//
// One step = two launches (k_phi_batch, k_update_batch; the first step after
// init: k_phi, k_update).  k_phi recovers phi of every node (pulling f) into
// the phi buffer and reduces the grid's sum of phi, an exact fixed-point sum,
// into the next mass-correction factor; k_update reads the phi stencil from
// L2 and runs the stencils, wetting, forces, velocity, Allen-Cahn source and
// both BGK collisions of every node (pulling g).  The batched kernels serve
// many grids per launch through a case table and single grids through a
// one-entry table.  An alternative fused kernel (k_step) does a whole step in
// one launch per tile of nodes, recomputing phi on a one-node halo in shared
// memory.  Arithmetic follows the reference's operation order where it
// matters for parity; the isotropic gradient is accumulated without FMA
// contraction.  (Measured and dropped for k_phi: runs of four consecutive
// nodes per thread -- 43 -> 58 us, the per-thread runs break coalescing.)
#include <cooperative_groups.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "lbm_common.cuh"

namespace lbm {

template <typename T>
__device__ __forceinline__ T clamp01(T v) {
  // torch.clamp(v, 0, 1): NaN propagates.
  return v < T(0) ? T(0) : (v > T(1) ? T(1) : v);
}

template <typename T>
__device__ __forceinline__ T ldg(const T* p) {
  return __ldg(p);
}

// L2 cache policies.  KEEP (evict_last) marks the populations that phase A of
// the step kernel reads and phase B reads again; ONCE (evict_first) marks
// data touched once per step (g, u, phi, every store), so that it does not
// displace them.
struct Pol {
  unsigned long long keep, once, same;
  __device__ __forceinline__ static Pol make() {
    Pol p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p.keep));
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p.once));
    asm("createpolicy.fractional.L2::evict_unchanged.b64 %0, 1.0;" : "=l"(p.same));
    return p;
  }
};
__device__ __forceinline__ float ld_pol(const float* p, unsigned long long pol) {
  float v;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ double ld_pol(const double* p, unsigned long long pol) {
  double v;
  asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ void st_pol(float* p, float v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(pol));
}
__device__ __forceinline__ void st_pol(double* p, double v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(p), "d"(v), "l"(pol));
}
__device__ __forceinline__ __half ld_pol(const __half* p, unsigned long long pol) {
  unsigned short v;
  asm("ld.global.nc.L2::cache_hint.b16 %0, [%1], %2;" : "=h"(v) : "l"(p), "l"(pol));
  return __ushort_as_half(v);
}
__device__ __forceinline__ void st_pol(__half* p, __half v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.b16 [%0], %1, %2;" ::"l"(p), "h"(__half_as_ushort(v)), "l"(pol));
}

// Asynchronous global -> shared copies of one 4- or 8-byte element (no
// register holds the value in flight), with an L2 policy.
template <typename T>
__device__ __forceinline__ void cp_async(T* sdst, const T* gsrc, unsigned long long pol) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "cp.async copies 4, 8 or 16 bytes");
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], %2, %3;" ::"r"(sa), "l"(gsrc),
               "n"(sizeof(T)), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory");
}

// Population storage.  S == T stores the population itself.  S == half (the
// deviation-storage form) stores f as its normalised deviation from the
// rest-state equilibrium w_q phi, d = F / w_q - phi_ref, where phi_ref is the
// phi of the node that will read the value (its own phi of the previous step,
// known to the reader without a load), and g as G / w_q (its rest-state
// equilibrium w_q P has P ~ 0).  Arithmetic is always in T.
template <typename T, typename S>
struct PopIO {
  static constexpr bool kDev = false;
  __device__ __forceinline__ static T ld_f(S raw, int, T, const Consts<T>&) { return raw; }
  __device__ __forceinline__ static S st_f(T v, int, T, const Consts<T>&) { return v; }
  __device__ __forceinline__ static T ld_g(S raw, int, const Consts<T>&) { return raw; }
  __device__ __forceinline__ static S st_g(T v, int, const Consts<T>&) { return v; }
};
template <>
struct PopIO<float, __half> {
  static constexpr bool kDev = true;
  __device__ __forceinline__ static float ld_f(__half raw, int q, float ref, const Consts<float>& k) {
    return Lat<float>::w(q) * (__half2float(raw) + ref);
  }
  __device__ __forceinline__ static __half st_f(float v, int q, float ref, const Consts<float>& k) {
    return __float2half_rn(v * Lat<float>::inv_w(q) - ref);
  }
  __device__ __forceinline__ static float ld_g(__half raw, int q, const Consts<float>& k) {
    return Lat<float>::w(q) * __half2float(raw);
  }
  __device__ __forceinline__ static __half st_g(float v, int q, const Consts<float>& k) {
    return __float2half_rn(v * Lat<float>::inv_w(q));
  }
};

// sqrt(x) for the magnitudes of the step, taken only where it can matter:
// below 1e-21 (sqrt < 3.2e-11) every caller clamps the magnitude to 1e-10 or
// compares it with 1e-6, so 0 is returned there.  A zero gradient (most of the
// domain away from the interface) then never enters the square root's
// special-case path.  Same results as sqrt(x) after the callers' clamp or
// comparison; NaN still propagates.
// GUARD selects it; the float32 update keeps the plain sqrt (measured on the
// 150x150x107 case: the guard makes the half form 0.1791 -> 0.1759 ms per
// step but the float32 form 0.1699 -> 0.1790, its register allocation shifting).
template <bool GUARD, typename T>
__device__ __forceinline__ T sqrt_mag(T x) {
  if constexpr (GUARD) return (x >= T(1e-21) || x != x) ? sqrt(x) : T(0);
  else return sqrt(x);
}

// Separately rounded multiply and add (never contracted into an FMA).  The
// isotropic gradient is accumulated with these so that mirror-symmetric
// neighbour pairs cancel to exactly zero, as in the reference: the
// sharpening normal grad/|grad| is otherwise set by an FMA's rounding residue
// at the points where the gradient vanishes.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rcp(float a) { return 1.0f / a; }
// Fused multiply-add, written out where the step relies on it.
template <typename T>
__device__ __forceinline__ T fma_(T a, T b, T c) { return fma(a, b, c); }
__device__ __forceinline__ double rcp(double a) { return 1.0 / a; }

// q = floor(t / d) for 0 <= t < 2^22 via a float reciprocal: the relative
// error of (t + 1/2) * (1/d) is below 2^-23, inside the 1/(2d) margin.
__device__ __forceinline__ int fdiv(int t, float inv_d) { return (int)(((float)t + 0.5f) * inv_d); }

// Block-wide sum of a double; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double s_warp[kBlock / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) s_warp[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < kBlock / 32; ++i) r += s_warp[i];
  }
  return r;
}

// Publishes this block's partial sum; the last block to finish sums all
// partials in block order (deterministic) and returns true in thread 0 with
// the total in *total.  Resets the counter for the next launch.
__device__ __forceinline__ bool last_block_total(double part, double* partials, unsigned* counter,
                                                 double* total, int blk = -1, int nblk = -1) {
  __shared__ bool s_last;
  if (blk < 0) {
    blk = blockIdx.x;
    nblk = gridDim.x;
  }
  if (threadIdx.x == 0) {
    partials[blk] = part;
    __threadfence();
    const unsigned done = atomicAdd(counter, 1u);
    s_last = (done == (unsigned)nblk - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  double acc = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) acc += ((volatile double*)partials)[i];
  acc = block_sum(acc);
  if (threadIdx.x == 0) {
    *total = acc;
    *counter = 0u;
  }
  return threadIdx.x == 0;
}

// ---------------------------------------------------------------------------
// Population reconstruction (pull form -> reference state at step start)
// ---------------------------------------------------------------------------
// Loads of the step kernel carry an L2 policy; the read-out kernels (no
// policy) use plain read-only loads.
template <bool USE_POL, typename S>
__device__ __forceinline__ S ld_sel(const S* p, unsigned long long pol) {
  if constexpr (USE_POL) return ld_pol(p, pol);
  else return ldg(p);
}
__device__ __forceinline__ __half ldg(const __half* p) { return __ldg(p); }

// Populations of node n as the reference holds them at the start of the step
// (before the mass correction, which WITH_C applies).  IS_F selects the
// f encoding of PopIO; phi_in (the previous step's phi) supplies the deviation
// references of the half form: the node's own phi for pulled values, the
// neighbour x - e_q's phi for the node's own opposite slot (bounce-back, VP).
// MAP: the state arrays use the layout of k (sidx); without it the linear
// layout is assumed (the batched single-node kernels, which serve linear grids).
template <typename T, typename S, bool RAW, bool WITH_C, bool IS_F, bool USE_POL = false, bool MAP = false>
__device__ __forceinline__ void fetch_pop(T (&v)[Q], const Consts<T>& k, const S* __restrict__ F,
                                          const T* __restrict__ phi_in, int n, size_t N, const Nbr& nb,
                                          uint8_t c, T eps, T corr, unsigned long long pol = 0ull) {
  using IO = PopIO<T, S>;
  auto I = [&](int m) -> unsigned { return MAP ? sidx(k, m) : (unsigned)m; };
  // element offsets q Np + m stay below 2^31 (checked when the grid is created)
  const unsigned Nu = (unsigned)k.Np, nu = I(n);
  (void)N;
  const T ref_self = (IO::kDev && IS_F) ? ldg(phi_in + nu) : T(0);
  auto ld = [&](int q, unsigned idx, T ref) -> T {
    const S raw = ld_sel<USE_POL>(F + idx, pol);
    return IS_F ? IO::ld_f(raw, q, ref, k) : IO::ld_g(raw, q, k);
  };
  auto ref_nb = [&](int q) -> T {
    return (IO::kDev && IS_F) ? ldg(phi_in + I(nb.at(n, -ex(q), -ey(q), -ez(q)))) : T(0);
  };
  if (RAW) {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = ld(q, q * Nu + nu, ref_self);
    return;
  }
  if (c & kSolid) {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = ld(opp(q), opp(q) * Nu + nu, ref_nb(q));
  } else {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = ld(q, q * Nu + I(nb.at(n, -ex(q), -ey(q), -ez(q))), ref_self);
    if (c & kPartial) {
      const T one_m = T(1) - eps;
#pragma unroll
      for (int q = 0; q < Q; ++q) v[q] = one_m * v[q] + eps * ld(opp(q), opp(q) * Nu + nu, ref_nb(q));
    }
  }
  if (WITH_C) {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = v[q] * corr;
  }
}

template <typename T>
__device__ __forceinline__ T seqsum(const T (&v)[Q]) {
  T s = v[0];
#pragma unroll
  for (int q = 1; q < Q; ++q) s = s + v[q];
  return s;
}

// Boundary-phi relaxation target of top-surface boundary node n from the
// previous step's phi (phi_prev = phi_arr[n]) and mass correction
// (lbm/fe_ac_solver.py:594-624); negative when the node is not active.  With
// direct wetting the target is the cubic-wall-energy boundary phi from the
// corrected phi of the node's next-interior node (fe_wetting.py:369-416), or
// the node's own phi where that does not apply.
template <typename T, bool MAP = false>
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
      const T pn = clamp01(phi_arr[MAP ? sidx(k, m) : (unsigned)m] * corr);
      T disc = cubic[0] + cubic[1] * pn;
      disc = disc < T(0) ? T(0) : disc;
      target = clamp01((cubic[2] + sqrt(disc)) / cubic[3]);
    }
  }
  return clamp01(pb + k.relax_r * (target - pb));
}

// Relaxation scale of lbm/fe_ac_solver.py:626-629.
template <typename T>
__device__ __forceinline__ T relax_scale(T target, T sum_f) {
  const T safe = sum_f < T(1e-10) ? T(1e-10) : sum_f;
  const T s = target / safe;
  return s < T(0.5) ? T(0.5) : (s > T(2.0) ? T(2.0) : s);
}

// f at node n as the reference holds it at the start of the step.
template <typename T, typename S, bool RAW, bool USE_POL = false, bool MAP = false>
__device__ __forceinline__ void fetch_f(T (&v)[Q], const Consts<T>& k, const State<T, S>& s, int n, size_t N,
                                        const Nbr& nb, uint8_t c, T eps, unsigned long long pol = 0ull) {
  const T corr = RAW ? T(1) : s.cbuf[s.c_prev];
  fetch_pop<T, S, RAW, !RAW, true, USE_POL, MAP>(v, k, s.fin, s.phi_in, n, N, nb, c, eps, corr, pol);
  if (!RAW && k.relax_on && (c & kTop)) {
    const T r = relax_target<T, MAP>(k, s.phi_in, s.nsw, s.cubic, n,
                                     ldg(s.phi_in + (MAP ? sidx(k, n) : (unsigned)n)), corr);
    if (r >= T(0)) {
      const T sc = relax_scale(r, seqsum(v));
#pragma unroll
      for (int q = 0; q < Q; ++q) v[q] = v[q] * sc;
    }
  }
}

// Lattice constants as the step kernels read them: compile-time immediates
// (IMM) or the grid's constant table.  Both hold the same values (the table is
// checked against the immediates when it is built); which is faster depends
// on the kernel's register allocation (measured on the 150x150x107 case:
// immediates for the half-storage form, 0.1829 -> 0.1797 ms per step; the
// table for float storage, 0.1746 -> 0.1698).
template <typename T, bool IMM>
struct LatK {
  const Consts<T>& k;
  __device__ __forceinline__ T w(int q) const { return IMM ? Lat<T>::w(q) : k.w[q]; }
  __device__ __forceinline__ T wc(int q) const { return IMM ? Lat<T>::wc(q) : k.wc[q]; }
  __device__ __forceinline__ T w2c(int q) const { return IMM ? Lat<T>::w2c(q) : k.w2c[q]; }
  __device__ __forceinline__ T cs2() const { return IMM ? Lat<T>::cs2() : k.cs2; }
  __device__ __forceinline__ T inv_cs2() const { return IMM ? Lat<T>::inv_cs2() : k.inv_cs2; }
  __device__ __forceinline__ T inv_two_cs2() const { return IMM ? Lat<T>::inv_two_cs2() : k.inv_two_cs2; }
};

// ---------------------------------------------------------------------------
// Isotropic gradient / laplacian with the ghost-node wetting correction
// (lbm/fe_ac_solver.py:296-320 fused, :282-294 unfused; fe_wetting.py:418-446).
// ps[q] holds phi(x + e_q); nsolid(q) tells whether that neighbour is solid.
// ---------------------------------------------------------------------------
// PAIR: the gradient from opposite-pair differences t_q = (w_q / cs2)
// (phi(x + e_q) - phi(x - e_q)), nine products instead of thirty, with
// mirror partners summed first so that a mirror-symmetric phi still gives
// an exactly zero component (the sharpening normal grad / |grad| depends on
// it where the gradient vanishes).
template <typename T, bool FUSED, typename St, typename SolidFn, bool PAIR = false, bool IMM = false>
__device__ __forceinline__ void grad_lap(const Consts<T>& k, const St& s, int n, uint8_t c, T phi,
                                         T (&ps)[Q], SolidFn nsolid, T& gx, T& gy, T& gz, T& lap) {
  const LatK<T, IMM> L{k};
  if (k.wetting && (c & kBoundary)) {
    const size_t N = (size_t)k.N;
    const float n0 = s.wn[n], n1 = s.wn[N + n], n2 = s.wn[2 * N + n];
#pragma unroll
    for (int q = 1; q < Q; ++q) {
      if (nsolid(q)) {
        float nde = 0.0f;
        nde = __fadd_rn(nde, __fmul_rn(n0, (float)ex(q)));
        nde = __fadd_rn(nde, __fmul_rn(n1, (float)ey(q)));
        nde = __fadd_rn(nde, __fmul_rn(n2, (float)ez(q)));
        if (k.linear) {
          ps[q] = phi - (T)__fmul_rn(nde, k.h_over_kappa_f);
        } else {
          ps[q] = phi + (T)__fmul_rn(nde, k.pcok_f) * phi * (T(1) - phi);
        }
      }
    }
  }
  gx = gy = gz = lap = T(0);
  if constexpr (PAIR) {
    auto t = [&](int q) { return mul_rn(L.wc(q), ps[q] - ps[opp(q)]); };
    const T t1 = t(1), t3 = t(3), t5 = t(5), t7 = t(7), t8 = t(8), t11 = t(11), t12 = t(12), t15 = t(15),
            t16 = t(16);
    gx = add_rn(add_rn(t1, t7 - t8), t11 - t12);  // e_x: q 1, 7, -8, 11, -12 (and their opposites)
    gy = add_rn(add_rn(t3, t7 + t8), t15 - t16);  // e_y: q 3, 7, 8, 15, -16
    gz = add_rn(add_rn(t5, t11 + t12), t15 + t16);  // e_z: q 5, 11, 12, 15, 16
  }
#pragma unroll
  for (int q = 1; q < Q; ++q) {
    if (!PAIR) {
      if (ex(q) != 0) gx = add_rn(gx, mul_rn(ex(q) > 0 ? L.wc(q) : -L.wc(q), ps[q]));
      if (ey(q) != 0) gy = add_rn(gy, mul_rn(ey(q) > 0 ? L.wc(q) : -L.wc(q), ps[q]));
      if (ez(q) != 0) gz = add_rn(gz, mul_rn(ez(q) > 0 ? L.wc(q) : -L.wc(q), ps[q]));
    }
    if (FUSED) {
      lap = fma_(L.w2c(q), ps[q] - phi, lap);
    } else {
      lap = lap + (T(2) * L.w(q)) * (ps[q] - phi) / L.cs2();
    }
  }
}

// Chemical potential (lbm/fe_ac_solver.py:326-340).
template <typename T>
__device__ __forceinline__ T chem_pot(const Consts<T>& k, uint8_t c, T phi, T lap) {
  T mu = fma_(-k.kappa, lap, k.beta4 * phi * (phi - T(1)) * (phi - T(0.5)));
  if (k.wetting && (c & kBoundary)) {
    if (k.linear) mu = mu + k.mu_wall_add;
    else mu = mu + k.phi_c * phi * (T(1) - phi);
  }
  return mu;
}

// Isotropic gradient of the chemical potential (the reference's unfused
// _lattice_gradient(mu_phi), lbm/fe_ac_solver.py:267-280), with the ghost
// correction of fe_wetting.py:418-446 applied to mu itself at a boundary
// node's solid neighbours: per direction q in order, per axis with
// e_q != 0, grad += (w_q e_q / cs2) mu(x + e_q).  (The reference divides each
// term by cs2; multiplying by the folded weight differs by an ulp per term and
// avoids 30 divisions per node.)
template <typename T, typename St, typename MuAt, typename SolidFn>
__device__ __forceinline__ void grad_mu(const Consts<T>& k, const St& s, int n, uint8_t c, T mu, MuAt mu_at,
                                        SolidFn nsolid, T& gx, T& gy, T& gz) {
  const bool ghost = k.wetting && (c & kBoundary);
  float n0 = 0.0f, n1 = 0.0f, n2 = 0.0f;
  if (ghost) {
    const size_t N = (size_t)k.N;
    n0 = s.wn[n];
    n1 = s.wn[N + n];
    n2 = s.wn[2 * N + n];
  }
  gx = gy = gz = T(0);
#pragma unroll
  for (int q = 1; q < Q; ++q) {
    T v = mu_at(q);
    if (ghost && nsolid(q)) {
      float nde = 0.0f;
      nde = __fadd_rn(nde, __fmul_rn(n0, (float)ex(q)));
      nde = __fadd_rn(nde, __fmul_rn(n1, (float)ey(q)));
      nde = __fadd_rn(nde, __fmul_rn(n2, (float)ez(q)));
      v = k.linear ? mu - (T)__fmul_rn(nde, k.h_over_kappa_f) : mu + (T)__fmul_rn(nde, k.pcok_f) * mu * (T(1) - mu);
    }
    const T w = Lat<T>::wc(q);
    if (ex(q) != 0) gx = add_rn(gx, mul_rn(ex(q) > 0 ? w : -w, v));
    if (ey(q) != 0) gy = add_rn(gy, mul_rn(ey(q) > 0 ? w : -w, v));
    if (ez(q) != 0) gz = add_rn(gz, mul_rn(ez(q) > 0 ? w : -w, v));
  }
}

// e_q . (a0, a1, a2) with the reference's exact two-term sums.
template <typename T>
__device__ __forceinline__ T edot(int q, T a0, T a1, T a2) {
  T r = T(0);
  bool any = false;
  if (ex(q) != 0) { r = ex(q) > 0 ? a0 : -a0; any = true; }
  if (ey(q) != 0) { const T t = ey(q) > 0 ? a1 : -a1; r = any ? r + t : t; any = true; }
  if (ez(q) != 0) { const T t = ez(q) > 0 ? a2 : -a2; r = any ? r + t : t; }
  return r;
}

// ---------------------------------------------------------------------------
// The update of one node (lbm/fe_ac_solver.py:392-530): stencils, chemical
// potential, wetting, pressure, stress, forces, velocity, Allen-Cahn source
// and both BGK collisions; writes fout, gout, u, phi_out.
// ---------------------------------------------------------------------------
// First population of each opposite pair (q, opp q) of D3Q19.
__host__ __device__ constexpr int pair_first(int i) {
  return i == 0 ? 1 : i == 1 ? 3 : i == 2 ? 5 : i == 3 ? 7 : i == 4 ? 8 : i == 5 ? 11 : i == 6 ? 12 : i == 7 ? 15 : 16;
}

// OMEGA1: tau_f == 1 (the reference's default tau_h = 1.0), where the
// phase-field BGK collision f - (f - f_eq) + src is f_eq + src and the
// pre-collision f is not read.  PhiAt(q) gives phi(x + e_q) of this step,
// SolidAt(q) whether x + e_q is solid.
// Words of one node's staging slot: the 19 streamed g, u of the last step, phi
// of the last step.
constexpr int kStage = Q + 4;

// Start the asynchronous copies of the g pulled from the neighbours (the
// streamed values of a fluid node; solid and partial nodes patch them with
// their own values when used, so no node class is needed here), u and the
// previous phi of node n into a staging slot (word j at st[j * kBlock]).
template <typename T, bool RAW, bool FIRST>
__device__ __forceinline__ void stage_node(const Consts<T>& k, const State<T, T>& s, int n, const Nbr& nb,
                                           T* st, unsigned long long pol) {
  const unsigned Nu = (unsigned)k.Np, nu = sidx(k, n);
  if (RAW) {
#pragma unroll
    for (int q = 0; q < Q; ++q) cp_async(st + q * kBlock, s.gin + (q * Nu + nu), pol);
  } else {
#pragma unroll
    for (int q = 0; q < Q; ++q)
      cp_async(st + q * kBlock, s.gin + (q * Nu + sidx(k, nb.at(n, -ex(q), -ey(q), -ez(q)))), pol);
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) cp_async(st + (Q + d) * kBlock, s.u + (d * Nu + nu), pol);
  if (!FIRST) cp_async(st + (Q + 3) * kBlock, s.phi_in + nu, pol);
}

// STAGED: g, u and the previous phi come from the node's cp.async staging
// slot `st` (word j at st[j * kBlock]); otherwise they are loaded here.
template <typename T, typename S, bool RAW, bool FIRST, bool OMEGA1, bool STAGED, bool STORE_PHI, bool GMU,
          bool MAP, typename PhiAt, typename SolidAt, typename RefAt>
__device__ __forceinline__ void update_node(const Consts<T>& k, const State<T, S>& s, int n, const Nbr& nb,
                                            uint8_t c, T phi, PhiAt phi_at, SolidAt solid_at, RefAt ref_at,
                                            const Pol& pol, const T* st) {
  using IO = PopIO<T, S>;
  constexpr bool IMM = IO::kDev;
  const LatK<T, IMM> L{k};
  const size_t N = (size_t)k.N;
  // nu: the node's storage element (f, g, u, phi); nn: its node index (node-order arrays)
  const unsigned Nu = (unsigned)k.Np, nu = MAP ? sidx(k, n) : (unsigned)n, nn = (unsigned)n;

  // 2. first the stencil: gradient and laplacian with the ghost-node wetting values
  T ps[Q];
#pragma unroll
  for (int q = 1; q < Q; ++q) ps[q] = phi_at(q);
  T gx, gy, gz, lap;
  grad_lap<T, true, State<T, S>, SolidAt, true, IMM>(k, s, n, c, phi, ps, solid_at, gx, gy, gz, lap);

  // then g (pulled), u and phi of the last step.  Loading them after the
  // stencil keeps the 18 stencil values and the 19 populations from being
  // live at once (fewer registers, no spills; measured 157 -> 137 us per
  // update launch on the 150x150x107 case; moving the density, chemical
  // potential and wall correction ahead of these loads as well measured 143).
  const T eps = (c & kPartial) ? s.eps[n] : T(0);
  T g[Q];
  T uo0, uo1, uo2, pp;
  if constexpr (STAGED) {
    const T* gin = reinterpret_cast<const T*>(s.gin);
    if (!RAW && (c & kSolid)) {
      // bounce-back: the node's own opposite values, not the staged pulled ones
#pragma unroll
      for (int q = 0; q < Q; ++q) g[q] = ldg(gin + (opp(q) * Nu + nu));
    } else {
#pragma unroll
      for (int q = 0; q < Q; ++q) g[q] = st[q * kBlock];
    }
    if (!RAW && (c & kPartial)) {
      const T one_m = T(1) - eps;
#pragma unroll
      for (int q = 0; q < Q; ++q) g[q] = one_m * g[q] + eps * ldg(gin + (opp(q) * Nu + nu));
    }
    uo0 = st[Q * kBlock];
    uo1 = st[(Q + 1) * kBlock];
    uo2 = st[(Q + 2) * kBlock];
    pp = FIRST ? T(0) : st[(Q + 3) * kBlock];
  } else {
    fetch_pop<T, S, RAW, false, false, true, MAP>(g, k, s.gin, s.phi_in, n, N, nb, c, eps, T(1), pol.once);
    uo0 = ld_pol(s.u + nu, pol.once);
    uo1 = ld_pol(s.u + (Nu + nu), pol.once);
    uo2 = ld_pol(s.u + (2 * Nu + nu), pol.once);
    pp = FIRST ? T(0) : ld_pol(s.phi_in + nu, pol.once);
  }

  const T rho = fma_(phi, k.rho_l, (T(1) - phi) * k.rho_g);
  const T rho_eff = rho < k.rho_floor ? k.rho_floor : rho;
  // with a chemical-potential gradient term, mu of every node comes from k_mu
  // (the same arithmetic), so that the node's own mu and its neighbours' agree
  const T mu = GMU ? ld_pol(s.mu + n, pol.keep) : chem_pot(k, c, phi, lap);

  // geometric contact-angle gradient correction (fe_wetting.py:448-539).  The
  // wall normal is zero away from boundary nodes, where the correction is the
  // identity, so only boundary nodes are visited.
  if (k.geometric && (c & kBoundary)) {
    const T n0 = (T)s.wn[n], n1 = (T)s.wn[N + n], n2 = (T)s.wn[2 * N + n];
    const T gn = add_rn(add_rn(mul_rn(n0, gx), mul_rn(n1, gy)), mul_rn(n2, gz));
    const T tx = gx - mul_rn(gn, n0), ty = gy - mul_rn(gn, n1), tz = gz - mul_rn(gn, n2);
    T tm = sqrt_mag<IMM>(add_rn(add_rn(mul_rn(tx, tx), mul_rn(ty, ty)), mul_rn(tz, tz)));
    tm = tm < T(1e-10) ? T(1e-10) : tm;
    T gd = mul_rn(-tm, k.cos_t) / k.sin_t;
    // scalar amplification, or a per-node field active where alpha > 1 (fe_wetting.py:503-512)
    T a = k.amp;
    bool amp_on = k.amp_active;
    if (s.amp) {
      a = s.amp[n];
      amp_on = a > T(1);
    }
    if (amp_on) gd = add_rn(gn, mul_rn(gd - gn, a));
    const T cx = add_rn(tx, mul_rn(gd, n0)), cy = add_rn(ty, mul_rn(gd, n1)), cz = add_rn(tz, mul_rn(gd, n2));
    const T gm = sqrt_mag<IMM>(add_rn(add_rn(mul_rn(gx, gx), mul_rn(gy, gy)), mul_rn(gz, gz)));
    if (gm > T(1e-6)) {
      const T bl = k.ww[c >> kWwShift];
      gx = add_rn(gx, mul_rn(bl, cx - gx));
      gy = add_rn(gy, mul_rn(bl, cy - gy));
      gz = add_rn(gz, mul_rn(bl, cz - gz));
    }
  }

  // 3.-4. moments of g from opposite-pair sums s_i = g_q + g_opp q and
  // differences d_i = g_q - g_opp q (pairs i = 0..8: q = 1, 3, 5, 7, 8, 11,
  // 12, 15, 16): pressure P = sum g, momentum sum e g, and the second moment
  // Pi = sum e e g, from which the non-equilibrium stress with the new P and
  // the old u (:409-413) is Pi_ab - P cs2 delta_ab - u_a u_b, since the D3Q19
  // weights satisfy sum w e_a e_b = cs2 delta_ab and
  // sum w e_a e_b e_c e_d = cs2^2 (delta_ab delta_cd + delta_ac delta_bd + delta_ad delta_bc).
  T sp[9], dp[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    sp[i] = g[pair_first(i)] + g[opp(pair_first(i))];
    dp[i] = g[pair_first(i)] - g[opp(pair_first(i))];
  }
  T P = g[0];
#pragma unroll
  for (int i = 0; i < 9; ++i) P = P + sp[i];
  T sxx, syy, szz, sxy, sxz, syz;
  {
    const T pc = P * L.cs2();
    sxx = fma_(-uo0, uo0, (sp[0] + (sp[3] + sp[4]) + (sp[5] + sp[6])) - pc);
    syy = fma_(-uo1, uo1, (sp[1] + (sp[3] + sp[4]) + (sp[7] + sp[8])) - pc);
    szz = fma_(-uo2, uo2, (sp[2] + (sp[5] + sp[6]) + (sp[7] + sp[8])) - pc);
    sxy = fma_(-uo0, uo1, sp[3] - sp[4]);
    sxz = fma_(-uo0, uo2, sp[5] - sp[6]);
    syz = fma_(-uo1, uo2, sp[7] - sp[8]);
  }

  // 5. forces (Fakhari 2017, :416-439)
  T F0 = mu * gx, F1 = mu * gy, F2 = mu * gz;
  if (k.stab_mode <= 1) {
    const T fp = ((-P) * k.drho) * L.cs2();
    F0 = fma_(fp, gx, F0);
    F1 = fma_(fp, gy, F1);
    F2 = fma_(fp, gz, F2);
  }
  if (k.stab_mode == 0) {
    F0 = fma_(k.visc * fma_(sxz, gz, fma_(sxy, gy, sxx * gx)), k.drho, F0);
    F1 = fma_(k.visc * fma_(syz, gz, fma_(syy, gy, sxy * gx)), k.drho, F1);
    F2 = fma_(k.visc * fma_(szz, gz, fma_(syz, gy, sxz * gx)), k.drho, F2);
  }
  if (k.has_gforce) {
    F0 = fma_(k.gforce[0], rho, F0);
    F1 = fma_(k.gforce[1], rho, F1);
    F2 = fma_(k.gforce[2], rho, F2);
  }

  // 6. velocity (:442-447)
  T u0, u1, u2;
  {
    const T hr = T(0.5) * rcp(rho_eff);
    u0 = fma_(F0, hr, dp[0] + (dp[3] - dp[4]) + (dp[5] - dp[6]));
    u1 = fma_(F1, hr, dp[1] + (dp[3] + dp[4]) + (dp[7] - dp[8]));
    u2 = fma_(F2, hr, dp[2] + (dp[5] + dp[6]) + (dp[7] + dp[8]));
    if (c & kSolid) u0 = u1 = u2 = T(0);
  }
  const T b = fma_(u2, u2, fma_(u1, u1, u0 * u0)) * L.inv_two_cs2();

  // 7. Allen-Cahn source (:450-494)
  T S0, S1, S2;
  {
    T d0 = T(0), d1 = T(0), d2 = T(0);
    if (!FIRST) {
      d0 = fma_(phi, u0, -pp * uo0);
      d1 = fma_(phi, u1, -pp * uo1);
      d2 = fma_(phi, u2, -pp * uo2);
    }
    T gm = sqrt_mag<IMM>(fma_(gz, gz, fma_(gy, gy, gx * gx)));
    gm = gm < T(1e-10) ? T(1e-10) : gm;
    const T lam = ((T(4) * phi) * (T(1) - phi)) * k.inv_W;
    T cl = L.cs2() * lam * k.ac_scale * rcp(gm);
    if (k.wetting) cl = cl * (T(1) - k.sharpen_reduce * k.ww[c >> kWwShift]);
    if constexpr (GMU) {
      // grad mu of this node (k_gradmu)
      const T mx = ld_pol(s.gmu + nn, pol.once), my = ld_pol(s.gmu + (Nu + nn), pol.once),
              mz = ld_pol(s.gmu + (2 * Nu + nn), pol.once);
      if (k.gmu_mode == kGmuCH) {
        // Cahn-Hilliard: d(phi u) + M (grad mu - grad phi) tau_f / (tau_f - 1/2)  (:457-461)
        S0 = d0 + (k.mob * (mx - gx)) * k.guo;
        S1 = d1 + (k.mob * (my - gy)) * k.guo;
        S2 = d2 + (k.mob * (mz - gz)) * k.guo;
      } else {
        // Allen-Cahn with the mu drive: sharpening + d(phi u) + mu_drive M grad mu  (:484-486)
        S0 = fma_(cl, gx, d0) + k.mu_drive_a * mx;
        S1 = fma_(cl, gy, d1) + k.mu_drive_a * my;
        S2 = fma_(cl, gz, d2) + k.mu_drive_a * mz;
      }
    } else {
      S0 = fma_(cl, gx, d0);
      S1 = fma_(cl, gy, d1);
      S2 = fma_(cl, gz, d2);
    }
  }

  // 8. both BGK collisions (:496-530) one opposite pair (q, opp q) at a time.
  // With ec = e_q.u / cs2 (odd in q) the equilibria split into a part even in
  // q and a part odd in q:
  //   g_eq_q = w (P - b + ec^2/2) + w ec,   f_eq_q = phi w (1 - b + ec^2/2) + phi w ec,
  // and the forcing and Allen-Cahn source terms are odd, so each pair costs
  // one even and one odd term per lattice.
  T om;
  if (k.tau_const) {
    om = k.omega_g;
  } else {
    const T eta = phi * k.rho_l * k.tl_m + (T(1) - phi) * k.rho_g * k.tg_m;
    const T rden = phi * k.rho_l + (T(1) - phi) * k.rho_g;
    om = rcp(T(0.5) + eta / rden);
  }
  const T omo = T(1) - om;
  const T nsd = (T(1) - om * T(0.5)) * rcp(rho_eff * L.cs2());
  const T Pb = P - b;
  const T omb = T(1) - b;
  const T pf = OMEGA1 ? phi : k.omega_f * phi;  // omega_f phi
  const T u3x = u0 * L.inv_cs2(), u3y = u1 * L.inv_cs2(), u3z = u2 * L.inv_cs2();
  T f[Q];
  if (!OMEGA1) fetch_f<T, S, RAW, true, MAP>(f, k, s, n, N, nb, c, eps, pol.same);
  auto store_g = [&](int q, T v) { st_pol(s.gout + (q * Nu + nu), IO::st_g(v, q, k), pol.once); };
  auto store_f = [&](int q, T v) {
    st_pol(s.fout + (q * Nu + nu), IO::st_f(v, q, IO::kDev ? ref_at(q) : T(0), k), pol.once);
  };
  {
    const T ow = om * L.w(0);
    store_g(0, fma_(omo, g[0], ow * Pb));
    const T pw = pf * L.w(0);
    const T f0 = pw * omb;
    store_f(0, OMEGA1 ? f0 : fma_(T(1) - k.omega_f, f[0], f0));
  }
  // per weight class (axis pairs i < 3, diagonal pairs i >= 3): omega w,
  // omega w / 2, omega w (P - b), nsd w; omega_f phi w, its half, omega_f phi w (1 - b)
  const T wa = L.w(1), wd = L.w(7);
  const T owa = om * wa, owd = om * wd;
  const T howa = T(0.5) * owa, howd = T(0.5) * owd;
  const T obpa = owa * Pb, obpd = owd * Pb;
  const T nwa = nsd * wa, nwd = nsd * wd;
  const T pwa = pf * wa, pwd = pf * wd;
  const T hpwa = T(0.5) * pwa, hpwd = T(0.5) * pwd;
  const T pwba = pwa * omb, pwbd = pwd * omb;
  const T aca = k.wac3[1], acd = k.wac3[7];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const int q = pair_first(i), p = opp(q);
    const bool ax = i < 3;
    const T ec = edot(q, u3x, u3y, u3z);
    // hydrodynamic pair
    const T ge = fma_((ax ? howa : howd) * ec, ec, ax ? obpa : obpd);
    const T go = fma_(ax ? owa : owd, ec, (ax ? nwa : nwd) * edot(q, F0, F1, F2));
    store_g(q, fma_(omo, g[q], ge + go));
    store_g(p, fma_(omo, g[p], ge - go));
    // phase-field pair
    const T fe = fma_((ax ? hpwa : hpwd) * ec, ec, ax ? pwba : pwbd);
    const T fo = fma_(ax ? pwa : pwd, ec, (ax ? aca : acd) * edot(q, S0, S1, S2));
    if (OMEGA1) {
      store_f(q, fe + fo);
      store_f(p, fe - fo);
    } else {
      const T omf = T(1) - k.omega_f;
      store_f(q, fma_(omf, f[q], fe + fo));
      store_f(p, fma_(omf, f[p], fe - fo));
    }
  }
  st_pol(s.u + nu, u0, pol.once);
  st_pol(s.u + (Nu + nu), u1, pol.once);
  st_pol(s.u + (2 * Nu + nu), u2, pol.once);
  if (STORE_PHI) st_pol(s.phi_out + nu, phi, pol.once);
}

// ---------------------------------------------------------------------------
// Tile sums of phi.  Float phi in [0, 1] is summed as unsigned 64-bit fixed
// point with 31 fraction bits: exact, so the total does not depend on the
// order of summation or on the tiling, and free of the (slow on this part)
// float64 pipe; NaN is carried by a flag.  Double phi is summed in double.
// ---------------------------------------------------------------------------
constexpr unsigned long long kSumNaN = ~0ull;
constexpr double kFix = 2147483648.0;  // 2^31

template <typename T>
struct TileSum {
  double a = 0.0;
  __device__ __forceinline__ void add(T phi) { a += (double)phi; }
};
template <>
struct TileSum<float> {
  unsigned long long a = 0ull;
  bool nan = false;
  __device__ __forceinline__ void add(float phi) {
    a += (unsigned long long)__float2uint_rn(phi * 2147483648.0f);
    nan |= !(phi == phi);
  }
};

// Block total of the tile sums, published; the last block to finish adds the
// block totals in block order and returns true in thread 0 with the grid
// total in *total (NaN if any phi was NaN).  Resets the counter.  blk / nblk:
// this block's index among the blocks that share the sum and their number
// (default: the launch grid).
template <typename T>
__device__ __forceinline__ bool grid_phi_total(TileSum<T>& ts, double* partials, unsigned* counter,
                                               double* total, int blk = -1, int nblk = -1) {
  if (blk < 0) {
    blk = blockIdx.x;
    nblk = gridDim.x;
  }
  if constexpr (sizeof(T) == 8) {
    return last_block_total(block_sum(ts.a), partials, counter, total, blk, nblk);
  } else {
    __shared__ unsigned long long s_warp[kBlock / 32];
    __shared__ bool s_last;
    unsigned long long v = ts.a;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const bool nan = __syncthreads_or(ts.nan) != 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) s_warp[wid] = v;
    __syncthreads();
    unsigned long long* up = reinterpret_cast<unsigned long long*>(partials);
    if (threadIdx.x == 0) {
      unsigned long long r = 0ull;
#pragma unroll
      for (int i = 0; i < kBlock / 32; ++i) r += s_warp[i];
      up[blk] = nan ? kSumNaN : r;
      __threadfence();
      s_last = (atomicAdd(counter, 1u) == (unsigned)nblk - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    unsigned long long acc = 0ull;
    bool any_nan = false;
    for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
      const unsigned long long p = ((volatile unsigned long long*)up)[i];
      if (p == kSumNaN) any_nan = true;
      else acc += p;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    any_nan = __syncthreads_or(any_nan) != 0;
    if (lane == 0) s_warp[wid] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long r = 0ull;
#pragma unroll
      for (int i = 0; i < kBlock / 32; ++i) r += s_warp[i];
      *total = any_nan ? __longlong_as_double(0x7ff8000000000000ll) : (double)r / kFix;
      *counter = 0u;
    }
    return threadIdx.x == 0;
  }
}

// ---------------------------------------------------------------------------
// The fused time step
// ---------------------------------------------------------------------------
// Resident blocks per SM the step kernel is compiled for: three for float
// populations (80 registers), two for half populations (the deviation
// decoding needs more registers; half the bytes need less parallelism), one
// for double.
template <typename T, typename S>
struct StepOccupancy {
  static constexpr int blocks = sizeof(T) == 8 ? 1 : (sizeof(S) == 2 ? 2 : 3);
};

// Shared memory of the step kernel: phi and class of the halo tile, then (for
// float and double populations) the staging slots, 16-byte aligned.
template <typename T>
__host__ __device__ __forceinline__ size_t stage_offset(const Tiling& tl) {
  return ((size_t)tl.hmax * (sizeof(T) + 1) + 15) & ~(size_t)15;
}
template <typename T, typename S>
size_t step_smem_bytes(const Tiling& tl) {
  const bool staged = sizeof(S) == sizeof(T);
  return stage_offset<T>(tl) + (staged ? (size_t)2 * kStage * kBlock * sizeof(T) : 0);
}

template <typename T, typename S, bool RAW, bool FIRST, bool OMEGA1>
__global__ void __launch_bounds__(kBlock, StepOccupancy<T, S>::blocks) k_step(Consts<T> k, State<T, S> s, Tiling tl) {
  // shared memory: phi and node class of the tile and its halo
  extern __shared__ __align__(16) unsigned char smem[];
  T* sphi = reinterpret_cast<T*>(smem);
  uint8_t* scls = reinterpret_cast<uint8_t*>(sphi + tl.hmax);
  // staging slots of phase B (float and double populations): 2 x kStage words per thread
  constexpr bool STAGED = std::is_same<S, T>::value;
  T* stage = reinterpret_cast<T*>(smem + stage_offset<T>(tl));
  const size_t N = (size_t)k.N;
  const Pol pol = Pol::make();

  // tile of this CTA, clipped at the domain edge
  const int b = blockIdx.x;
  const int bz = b % tl.ntz, byx = b / tl.ntz;
  const int by = byx % tl.nty, bx = byx / tl.nty;
  const int x0 = bx * tl.tx, y0 = by * tl.ty, z0 = bz * tl.tz;
  const int ex_ = min(tl.tx, k.nx - x0), ey_ = min(tl.ty, k.ny - y0), ez_ = min(tl.tz, k.nz - z0);
  const int HY = ey_ + 2, HZ = ez_ + 2;
  const int H = (ex_ + 2) * HY * HZ;
  const int E = ex_ * ey_ * ez_;
  const float inv_hz = 1.0f / (float)HZ, inv_hy = 1.0f / (float)HY;
  const float inv_ez = 1.0f / (float)ez_, inv_ey = 1.0f / (float)ey_;

  // phase B's first chunk of g, u and previous phi does not depend on phi:
  // its copies fly during phase A
  auto stage_chunk = [&](int t, int slot) {
    if constexpr (STAGED) {
      if (t < E) {
        const int r = fdiv(t, inv_ez);
        const int lz = t - r * ez_;
        const int lx = fdiv(r, inv_ey);
        const int ly = r - lx * ey_;
        const int n = ((x0 + lx) * k.ny + (y0 + ly)) * k.nz + (z0 + lz);
        const Nbr nb = make_nbr_xyz(x0 + lx, y0 + ly, z0 + lz, k.nx, k.ny, k.nz);
        stage_node<T, RAW, FIRST>(k, s, n, nb, stage + slot * kStage * kBlock + threadIdx.x, pol.once);
      }
      cp_async_commit();
    }
  };
  stage_chunk(threadIdx.x, 0);

  // phase A: phi on the tile and its halo, and the tile's sum of phi
  TileSum<T> part;
  // no periodic wrap anywhere in the halo or its pull sources: constant offsets
  const bool inner = x0 >= 2 && x0 + ex_ + 2 <= k.nx && y0 >= 2 && y0 + ey_ + 2 <= k.ny && z0 >= 2 &&
                     z0 + ez_ + 2 <= k.nz;
  if (inner) {
    Nbr nbc;
    nbc.ox[0] = -k.ny * k.nz; nbc.ox[1] = 0; nbc.ox[2] = k.ny * k.nz;
    nbc.oy[0] = -k.nz; nbc.oy[1] = 0; nbc.oy[2] = k.nz;
    nbc.oz[0] = -1; nbc.oz[1] = 0; nbc.oz[2] = 1;
    const int n00 = ((x0 - 1) * k.ny + (y0 - 1)) * k.nz + (z0 - 1);
    for (int h = threadIdx.x; h < H; h += kBlock) {
      const int r = fdiv(h, inv_hz);
      const int hz = h - r * HZ;
      const int hx = fdiv(r, inv_hy);
      const int hy = r - hx * HY;
      const int n = n00 + (hx * k.ny + hy) * k.nz + hz;
      const uint8_t c = s.cls[n];
      const bool own = hx >= 1 && hx <= ex_ && hy >= 1 && hy <= ey_ && hz >= 1 && hz <= ez_;
      T phi = T(0);
      if (!(c & kSolid)) {
        const T eps = (c & kPartial) ? s.eps[n] : T(0);
        T v[Q];
        fetch_f<T, S, RAW, true, true>(v, k, s, n, N, nbc, c, eps, pol.keep);
        phi = clamp01(seqsum(v));
      }
      sphi[h] = phi;
      scls[h] = c;
      if (own) part.add(phi);
    }
  } else {
    for (int h = threadIdx.x; h < H; h += kBlock) {
      const int r = fdiv(h, inv_hz);
      const int hz = h - r * HZ;
      const int hx = fdiv(r, inv_hy);
      const int hy = r - hx * HY;
      int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
      gx = gx < 0 ? gx + k.nx : (gx >= k.nx ? gx - k.nx : gx);
      gy = gy < 0 ? gy + k.ny : (gy >= k.ny ? gy - k.ny : gy);
      gz = gz < 0 ? gz + k.nz : (gz >= k.nz ? gz - k.nz : gz);
      const int n = (gx * k.ny + gy) * k.nz + gz;
      const uint8_t c = s.cls[n];
      const bool own = hx >= 1 && hx <= ex_ && hy >= 1 && hy <= ey_ && hz >= 1 && hz <= ez_;
      T phi = T(0);
      if (!(c & kSolid)) {
        const Nbr nb = make_nbr_xyz(gx, gy, gz, k.nx, k.ny, k.nz);
        const T eps = (c & kPartial) ? s.eps[n] : T(0);
        T v[Q];
        fetch_f<T, S, RAW, true, true>(v, k, s, n, N, nb, c, eps, pol.keep);
        phi = clamp01(seqsum(v));
      }
      sphi[h] = phi;
      scls[h] = c;
      if (own) part.add(phi);
    }
  }
  __syncthreads();

  // sum(phi) of the grid -> mass-correction factor of this step (:582-589)
  double total;
  if (grid_phi_total<T>(part, s.partials, s.counter, &total)) {
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

  // phase B: the tile's nodes, one chunk of kBlock nodes at a time; the next
  // chunk's copies are started before this chunk is computed
  const int sx = HY * HZ;
  const int nch = (E + kBlock - 1) / kBlock;
  for (int j = 0; j < nch; ++j) {
    const int t = j * kBlock + threadIdx.x;
    if constexpr (STAGED) {
      stage_chunk(t + kBlock, (j + 1) & 1);
      cp_async_wait<1>();
    }
    if (t < E) {
      const int r = fdiv(t, inv_ez);
      const int lz = t - r * ez_;
      const int lx = fdiv(r, inv_ey);
      const int ly = r - lx * ey_;
      const int h = ((lx + 1) * HY + (ly + 1)) * HZ + (lz + 1);
      const int n = ((x0 + lx) * k.ny + (y0 + ly)) * k.nz + (z0 + lz);
      const Nbr nb = make_nbr_xyz(x0 + lx, y0 + ly, z0 + lz, k.nx, k.ny, k.nz);
      // phi of this step at x + e_q (also the deviation reference, in the half
      // form, of the next step's reader of slot (x, q))
      update_node<T, S, RAW, FIRST, OMEGA1, STAGED, true, false, true>(
          k, s, n, nb, scls[h], sphi[h], [&](int q) { return sphi[h + ex(q) * sx + ey(q) * HZ + ez(q)]; },
          [&](int q) { return (scls[h + ex(q) * sx + ey(q) * HZ + ez(q)] & kSolid) != 0; },
          [&](int q) { return sphi[h + ex(q) * sx + ey(q) * HZ + ez(q)]; }, pol,
          stage + (j & 1) * kStage * kBlock + threadIdx.x);
    }
  }
  if constexpr (STAGED) cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// The two-kernel time step: k_phi recovers phi of every node (one thread per
// node, linear order) and the grid sum of phi; k_update then runs the rest of
// the step for every node, reading the phi stencil from L2.  Both stream their
// arrays in z-fastest order, so warps move whole 128-byte lines.  With
// omega_f == 1 f is read by k_phi only, and the pair moves the algorithmic
// bytes of the step plus the phi stencil's L2 traffic.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void decode(const FastDiv& dz, const FastDiv& dy, int n, int nz, int ny, int& ix,
                                       int& iy, int& iz) {
  const int t = (int)dz.div((unsigned)n);
  iz = n - t * nz;
  ix = (int)dy.div((unsigned)t);
  iy = t - ix * ny;
}

// Persistent: a grid of about one wave strides over the nodes, so that the
// per-block publication of the partial sum happens once per block.
// phi of node n (written to phi_out) added to the block's sum.
template <typename T, typename S, bool RAW, bool MAP = false>
__device__ __forceinline__ void phi_node(const Consts<T>& k, const State<T, S>& s, int n, uint8_t c, const Pol& pol,
                                         TileSum<T>& part) {
  T phi = T(0);
  if (!(c & kSolid)) {
    int ix, iy, iz;
    decode(k.dz, k.dy, n, k.nz, k.ny, ix, iy, iz);
    const Nbr nb = make_nbr_xyz(ix, iy, iz, k.nx, k.ny, k.nz);
    const T eps = (c & kPartial) ? s.eps[n] : T(0);
    T v[Q];
    // f is read again by k_update only when omega_f != 1
    fetch_f<T, S, RAW, true, MAP>(v, k, s, n, (size_t)k.N, nb, c, eps, k.omega_f == T(1) ? pol.once : pol.keep);
    phi = clamp01(seqsum(v));
  }
  st_pol(s.phi_out + (MAP ? sidx(k, n) : (unsigned)n), phi, pol.keep);  // read back (stencil) by k_update
  part.add(phi);
}

// sum(phi) of the grid -> mass-correction factor of this step (:582-589),
// computed by the last of the grid's nblk blocks to finish.
template <typename T, typename S>
__device__ __forceinline__ void phi_finish(const State<T, S>& s, TileSum<T>& part, int blk, int nblk) {
  double total;
  if (grid_phi_total<T>(part, s.partials, s.counter, &total, blk, nblk)) {
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

template <typename T, typename S, bool RAW>
__global__ void __launch_bounds__(kBlock) k_phi(Consts<T> k, State<T, S> s) {
  const Pol pol = Pol::make();
  TileSum<T> part;
  for (int n = blockIdx.x * kBlock + threadIdx.x; n < k.N; n += gridDim.x * kBlock)
    phi_node<T, S, RAW, true>(k, s, n, s.cls[n], pol, part);
  phi_finish(s, part, blockIdx.x, gridDim.x);
}

// Blocks per SM the update kernels are compiled for (256 threads each).  The
// half form also runs 4 (64 registers, 40 bytes of spills): measured on the
// 150x150x107 case 141 -> 127 us per update launch against 3 blocks without spills.
template <typename T, typename S, bool GMU = false>
struct UpdateOccupancy {
  static constexpr int blocks = sizeof(T) == 8 ? 1 : 4;
};

template <typename T, typename S, bool RAW, bool FIRST, bool OMEGA1, bool GMU, bool MAP = false>
__device__ __forceinline__ void update_one(const Consts<T>& k, const State<T, S>& s, int n, const Pol& pol) {
  int ix, iy, iz;
  decode(k.dz, k.dy, n, k.nz, k.ny, ix, iy, iz);
  const Nbr nb = make_nbr_xyz(ix, iy, iz, k.nx, k.ny, k.nz);
  const T* __restrict__ pc = s.phi_out;  // phi of this step (k_phi)
  const uint8_t c = s.cls[n];
  auto I = [&](int m) -> unsigned { return MAP ? sidx(k, m) : (unsigned)m; };
  const T phi = ld_pol(pc + I(n), pol.keep);
  update_node<T, S, RAW, FIRST, OMEGA1, false, false, GMU, MAP>(
      k, s, n, nb, c, phi, [&](int q) { return ld_pol(pc + I(nb.at(n, ex(q), ey(q), ez(q))), pol.keep); },
      [&](int q) { return (s.cls[nb.at(n, ex(q), ey(q), ez(q))] & kSolid) != 0; },
      [&](int q) { return ld_pol(pc + I(nb.at(n, ex(q), ey(q), ez(q))), pol.keep); }, pol, (const T*)nullptr);
}

// One thread per node, linear order.  (Measured slower on the 150x150x107
// case: a persistent grid-stride form, and forms that stage the next node's
// g, u and previous phi in shared memory with cp.async or with bulk copies
// per chunk of nodes -- the copies, the smaller L1 and the block-wide waits
// cost more than the latency they hide.)
template <typename T, typename S, bool RAW, bool FIRST, bool OMEGA1, bool GMU = false>
__global__ void __launch_bounds__(kBlock, UpdateOccupancy<T, S, GMU>::blocks) k_update(Consts<T> k, State<T, S> s) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n < k.N) update_one<T, S, RAW, FIRST, OMEGA1, GMU, true>(k, s, n, Pol::make());
}

// Gradient of the chemical potential of every node (mu from k_mu), for the
// modes whose interface source needs it; read by the update kernel.
template <typename T, typename S>
__global__ void __launch_bounds__(kBlock) k_gradmu(Consts<T> k, State<T, S> s) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  int ix, iy, iz;
  decode(k.dz, k.dy, n, k.nz, k.ny, ix, iy, iz);
  const Nbr nb = make_nbr_xyz(ix, iy, iz, k.nx, k.ny, k.nz);
  const Pol pol = Pol::make();
  const uint8_t c = s.cls[n];
  const T mu = ld_pol(s.mu + n, pol.keep);
  T mx, my, mz;
  grad_mu(k, s, n, c, mu, [&](int q) { return ld_pol(s.mu + nb.at(n, ex(q), ey(q), ez(q)), pol.keep); },
          [&](int q) { return (s.cls[nb.at(n, ex(q), ey(q), ez(q))] & kSolid) != 0; }, mx, my, mz);
  const unsigned Nu = (unsigned)k.Np, nu = (unsigned)n;
  st_pol(s.gmu + nu, mx, pol.keep);
  st_pol(s.gmu + (Nu + nu), my, pol.keep);
  st_pol(s.gmu + (2 * Nu + nu), mz, pol.keep);
}

// Chemical potential of every node of this step (phi from the phi kernel),
// for the modes whose interface source needs its gradient; the same
// stencil and arithmetic as the update kernel's.
template <typename T, typename S>
__global__ void __launch_bounds__(kBlock) k_mu(Consts<T> k, State<T, S> s) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  int ix, iy, iz;
  decode(k.dz, k.dy, n, k.nz, k.ny, ix, iy, iz);
  const Nbr nb = make_nbr_xyz(ix, iy, iz, k.nx, k.ny, k.nz);
  const Pol pol = Pol::make();
  const T* __restrict__ pc = s.phi_out;
  const uint8_t c = s.cls[n];
  const T phi = ld_pol(pc + sidx(k, n), pol.keep);
  T ps[Q];
#pragma unroll
  for (int q = 1; q < Q; ++q) ps[q] = ld_pol(pc + sidx(k, nb.at(n, ex(q), ey(q), ez(q))), pol.keep);
  auto solid_at = [&](int q) { return (s.cls[nb.at(n, ex(q), ey(q), ez(q))] & kSolid) != 0; };
  T gx, gy, gz, lap;
  grad_lap<T, true, State<T, S>, decltype(solid_at), true>(k, s, n, c, phi, ps, solid_at, gx, gy, gz, lap);
  st_pol(s.mu + n, chem_pot(k, c, phi, lap), pol.keep);
}

// ---------------------------------------------------------------------------
// Batched step: many independent grids advance in one launch of each kernel
// (a single grid uses the same kernels with a one-case table and no block ->
// case table, so that it gives the same results alone and in a batch).
// A block finds its case in a block -> case table and copies the case's
// constants and state pointers (CaseDesc) into shared memory; the arithmetic
// per node is the single-grid step's, and each case's sum of phi is reduced
// over that case's blocks only, so a case gives bit-identical results alone
// and in a batch.  Cases in their first step after init are not batched.
// ---------------------------------------------------------------------------
template <typename T, typename S>
struct CaseDesc {
  Consts<T> k;
  State<T, S> s;
  int phi_blk0, phi_nblk;  // the case's blocks in the k_phi_batch grid
  int upd_blk0, upd_nblk;  // and in the k_update_batch grid
};

// Programmatic dependent launch between the step kernels: a kernel launched
// with the programmatic-serialization attribute may start while the kernel
// before it drains; it reads its descriptor, lets the next kernel be
// scheduled (each block triggers on entry, so the next grid starts during
// this grid's last wave), and waits for the previous grid to complete and
// flush its memory before it reads anything that grid wrote.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename D>
__device__ __forceinline__ void load_desc(D& dst, const D* src) {
  static_assert(sizeof(D) % 4 == 0, "descriptor copied as 32-bit words");
  const unsigned* a = reinterpret_cast<const unsigned*>(src);
  unsigned* b = reinterpret_cast<unsigned*>(&dst);
  for (int i = threadIdx.x; i < (int)(sizeof(D) / 4); i += blockDim.x) b[i] = __ldg(a + i);
  __syncthreads();
}

template <typename T, typename S>
__global__ void __launch_bounds__(kBlock, sizeof(T) == 8 ? 3 : 4) k_phi_batch(const CaseDesc<T, S>* __restrict__ cases,
                                                     const unsigned short* __restrict__ blk2case) {
  __shared__ CaseDesc<T, S> d;
  load_desc(d, cases + (blk2case ? blk2case[blockIdx.x] : 0));
  pdl_trigger();
  pdl_wait();  // f of the previous update kernel
  const Pol pol = Pol::make();
  const int b = blockIdx.x - d.phi_blk0, nb = d.phi_nblk;
  TileSum<T> part;
  // the class byte of the thread's next node is loaded one node ahead, so
  // that the pulled loads of a node do not wait for its class load
  const int N = d.k.N, stride = nb * kBlock;
  int n = b * kBlock + threadIdx.x;
  uint8_t c = n < N ? d.s.cls[n] : 0;
  for (; n < N; n += stride) {
    const uint8_t c_next = n + stride < N ? d.s.cls[n + stride] : 0;
    phi_node<T, S, false>(d.k, d.s, n, c, pol, part);
    c = c_next;
  }
  phi_finish(d.s, part, b, nb);
}

// BS threads per block (the autotuners choose 128 or 256), compiled for the
// same registers per thread at either size.
template <typename T, typename S, bool OMEGA1, bool GMU = false, int BS = kBlock>
__global__ void __launch_bounds__(BS, UpdateOccupancy<T, S, GMU>::blocks * kBlock / BS) k_update_batch(
    const CaseDesc<T, S>* __restrict__ cases, const unsigned short* __restrict__ blk2case) {
  __shared__ CaseDesc<T, S> d;
  load_desc(d, cases + (blk2case ? blk2case[blockIdx.x] : 0));
  pdl_trigger();
  pdl_wait();  // phi of the phi kernel (mu of k_mu with GMU)
  const int n = (blockIdx.x - d.upd_blk0) * BS + threadIdx.x;
  if (n < d.k.N) update_one<T, S, false, false, OMEGA1, GMU>(d.k, d.s, n, Pol::make());
}

// ---------------------------------------------------------------------------
// The batched step as ONE cooperative launch: a grid of resident blocks runs
// the phi kernel's virtual blocks (the block -> case table's phi part), a
// grid-wide barrier (cooperative groups: every block of a cooperative launch
// is resident, so the barrier ends), then the update kernel's virtual blocks.
// Each virtual block does exactly what the block of the same index does in
// k_phi_batch / k_update_batch (same descriptor, same nodes, same arithmetic,
// the same last-block reduction per case), so the results are those of the
// two-launch step bit for bit.  Linear-layout cases only.
// ---------------------------------------------------------------------------
template <typename T, typename S>
__global__ void __launch_bounds__(kBlock, UpdateOccupancy<T, S>::blocks) k_batch_coop(
    const CaseDesc<T, S>* __restrict__ cases, const unsigned short* __restrict__ b2c, int phi_blocks,
    int upd_blocks_om1, int upd_blocks_other) {
  __shared__ CaseDesc<T, S> d;
  const Pol pol = Pol::make();
  for (int vb = blockIdx.x; vb < phi_blocks; vb += gridDim.x) {
    __syncthreads();  // the previous virtual block is done with d
    load_desc(d, cases + b2c[vb]);
    const int b = vb - d.phi_blk0, nb = d.phi_nblk;
    TileSum<T> part;
    const int N = d.k.N, stride = nb * kBlock;
    int n = b * kBlock + threadIdx.x;
    uint8_t c = n < N ? d.s.cls[n] : 0;
    for (; n < N; n += stride) {
      const uint8_t c_next = n + stride < N ? d.s.cls[n + stride] : 0;
      phi_node<T, S, false>(d.k, d.s, n, c, pol, part);
      c = c_next;
    }
    phi_finish(d.s, part, b, nb);
  }
  cooperative_groups::this_grid().sync();
  const int upd_blocks = upd_blocks_om1 + upd_blocks_other;
  for (int vb = blockIdx.x; vb < upd_blocks; vb += gridDim.x) {
    __syncthreads();
    load_desc(d, cases + b2c[phi_blocks + vb]);
    const int n = (vb - (vb < upd_blocks_om1 ? 0 : upd_blocks_om1) - d.upd_blk0) * kBlock + threadIdx.x;
    if (n < d.k.N) {
      if (vb < upd_blocks_om1) update_one<T, S, false, false, true, false>(d.k, d.s, n, pol);
      else update_one<T, S, false, false, false, false>(d.k, d.s, n, pol);
    }
  }
}

}  // namespace lbm

#include "lbm_pair.cuh"

namespace lbm {

// Grid of a persistent kernel: resident blocks per SM x SMs (one wave), at
// most one block per kBlock nodes.  The occupancy lookup runs once per kernel
// and device; host threads may launch concurrently (the serving loop sets up
// cases on a second thread), so the cache is guarded.
template <typename Kern>
static cudaError_t resident_grid(Kern fn, int nodes, int* grid) {
  static std::mutex mu;
  static int cached_dev = -1, cached = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int waves;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (cached_dev != dev) {
      int nsm = 0, b = 0;
      e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, kBlock, 0);
      if (e != cudaSuccess) return e;
      cached = nsm * (b > 0 ? b : 1);
      cached_dev = dev;
    }
    waves = cached;
  }
  const int full = (nodes + kBlock - 1) / kBlock;
  *grid = waves < full ? waves : full;
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// init_fields (lbm/fe_ac_solver.py:239-261): phi = clamp(phi0), f = f_eq,
// g = g_eq(0, u), phi-mass reference.
// ---------------------------------------------------------------------------
template <typename T, typename S, typename Src>
__global__ void __launch_bounds__(kBlock) k_init(Consts<T> k, State<T, S> s, const Src* phi0, const Src* u0) {
  using IO = PopIO<T, S>;
  const int n = blockIdx.x * kBlock + threadIdx.x;
  const size_t N = (size_t)k.N;
  double part = 0.0;
  if (n < k.N) {
    const T phi = clamp01((T)phi0[n]);
    const T v0 = u0 ? (T)u0[n] : T(0), v1 = u0 ? (T)u0[N + n] : T(0), v2 = u0 ? (T)u0[2 * N + n] : T(0);
    const T b = ((v0 * v0 + v1 * v1) + v2 * v2) / k.two_cs2;
    S* f = const_cast<S*>(s.fin);
    S* g = const_cast<S*>(s.gin);
    const unsigned e = sidx(k, n);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const T ec = edot(q, v0, v1, v2) / k.cs2;
      // the state right after init is read in place (RAW): deviation reference = own phi
      f[(size_t)q * k.Np + e] = IO::st_f(phi * (k.w[q] * (((T(1) + ec) + ec * ec / T(2)) - b)), q, phi, k);
      g[(size_t)q * k.Np + e] = IO::st_g(T(0) * k.w[q] + k.w[q] * ((ec + ec * ec / T(2)) - b), q, k);
    }
    s.u[e] = v0;
    s.u[k.Np + e] = v1;
    s.u[2 * (size_t)k.Np + e] = v2;
    s.phi_out[e] = phi;
    part = (double)phi;
  }
  part = block_sum(part);
  double total;
  if (last_block_total(part, s.partials, s.counter, &total)) {
    s.scal[0] = (double)(T)total;  // phi_mass_init = sum(phi).item() in T
    s.scal[1] = total;
    s.cbuf[0] = T(1);
    s.cbuf[1] = T(1);
  }
}

// ---------------------------------------------------------------------------
// Mid-run droplet injection (lbm/fe_ac_solver.py:645-732).  Reads the state
// the reference holds between steps (populations as k_populations rebuilds
// them, phi / u / P as the attributes), blends the new droplet in and writes
// the result in the raw form init_fields leaves (populations as the reference
// holds them): f, g to the other population buffer, phi to the other phi
// buffer, u in place.  Sums the new phi (the new phi-mass reference) and
// counts the core nodes.
// ---------------------------------------------------------------------------
template <typename T, typename S, bool RAW>
__global__ void __launch_bounds__(kBlock) k_inject(Consts<T> k, State<T, S> s, InjectParams ip,
                                                   const T* __restrict__ P_attr, unsigned* core_count) {
  using IO = PopIO<T, S>;
  const int n = blockIdx.x * kBlock + threadIdx.x;
  double part = 0.0;
  bool core = false;
  if (n < k.N) {
    const size_t N = (size_t)k.N;
    const unsigned Nu = (unsigned)k.Np, nu = sidx(k, n);
    const uint8_t c = s.cls[n];
    int ix, iy, iz;
    const Nbr nb = make_nbr(n, k.nx, k.ny, k.nz, &ix, &iy, &iz);
    // the droplet as the reference builds it: float64 profile, stored as float32
    const double dx = ix - ip.c[0], dy = iy - ip.c[1], dz = iz - ip.c[2];
    const double dist = sqrt((dx * dx + dy * dy) + dz * dz);
    double Cd = 0.5 + 0.5 * tanh(2.0 * (ip.radius - dist) / ip.xi);
    Cd = Cd < 0.0 ? 0.0 : (Cd > 1.0 ? 1.0 : Cd);
    const T C = (T)(float)Cd;
    core = C > T(0.1);
    // the attributes phi, u, P the reference holds now
    const T corr = s.cbuf[s.c_prev];
    T phi = s.phi_in[nu];
    if (!ip.obs_init) {
      const T pr = phi;
      phi = clamp01(pr * corr);
      if (k.relax_on && (c & kTop)) {
        const T r = relax_target<T, true>(k, s.phi_in, s.nsw, s.cubic, n, pr, corr);
        if (r >= T(0)) phi = r;
      }
    }
    T u[3] = {s.u[nu], s.u[Nu + nu], s.u[2 * Nu + nu]};
    const T P = ip.obs_init ? T(0) : P_attr[n];
    // the populations the reference holds now
    const T eps = (c & kPartial) ? s.eps[n] : T(0);
    T fv[Q], gv[Q];
    fetch_f<T, S, RAW, false, true>(fv, k, s, n, N, nb, c, eps);
    fetch_pop<T, S, RAW, false, false, false, true>(gv, k, s.gin, s.phi_in, n, N, nb, c, eps, T(1));
    // new phi: the maximum with the droplet in its core, clamped, zero in solid
    T pn = core ? (phi > C ? phi : C) : phi;
    pn = clamp01(pn);
    if (c & kSolid) pn = T(0);
    // new u: (1 - C) u + C u_impact everywhere, zero in solid
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      u[d] = add_rn(mul_rn(T(1) - C, u[d]), mul_rn(C, (T)ip.u[d]));
      if (c & kSolid) u[d] = T(0);
    }
    if (core) {
      const T b = ((u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]) / k.two_cs2;
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const T ec = edot(q, u[0], u[1], u[2]) / k.cs2;
        fv[q] = pn * (k.w[q] * (((T(1) + ec) + ec * ec / T(2)) - b));
        gv[q] = P * k.w[q] + k.w[q] * ((ec + ec * ec / T(2)) - b);
      }
    }
    // raw form: the next step reads these in place (deviation reference: own phi)
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      s.fout[q * Nu + nu] = IO::st_f(fv[q], q, pn, k);
      s.gout[q * Nu + nu] = IO::st_g(gv[q], q, k);
    }
    s.u[nu] = u[0];
    s.u[Nu + nu] = u[1];
    s.u[2 * Nu + nu] = u[2];
    s.phi_out[nu] = pn;
    part = (double)pn;
  }
  const int cnt = __syncthreads_count(core);
  if (threadIdx.x == 0 && cnt) atomicAdd(core_count, (unsigned)cnt);
  part = block_sum(part);
  double total;
  if (last_block_total(part, s.partials, s.counter, &total)) {
    s.scal[0] = (double)(T)total;  // phi_mass_init = phi.sum().item() in T
    s.scal[1] = total;
  }
}

// ---------------------------------------------------------------------------
// Field read-out (the reference's attribute values after the last step).
// s.phi_out holds the last recovered phi, s.cbuf[s.c_cur] its correction.
// ---------------------------------------------------------------------------
enum ObserveMode { kObsInit = 0, kObsStep = 1 };

template <typename T, typename S, bool RAW_IN>
__global__ void __launch_bounds__(kBlock) k_observe(Consts<T> k, State<T, S> s, unsigned mask, int mode,
                                                    T* phi_o, T* rho_o, T* u_o, T* P_o, T* p_o, T* mu_o) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  const size_t N = (size_t)k.N;
  const uint8_t c = s.cls[n];
  const unsigned e = sidx(k, n);
  const T phi = s.phi_out[e];
  const T rho = phi * k.rho_l + (T(1) - phi) * k.rho_g;
  if (mask & 1u) {
    T v = phi;
    if (mode == kObsStep) {
      const T corr = s.cbuf[s.c_cur];
      v = clamp01(phi * corr);
      if (k.relax_on && (c & kTop)) {
        const T r = relax_target<T, true>(k, (const T*)s.phi_out, s.nsw, s.cubic, n, phi, corr);
        if (r >= T(0)) v = r;
      }
    }
    phi_o[n] = v;
  }
  if (mask & 2u) rho_o[n] = rho;
  if (mask & 4u) {
    u_o[n] = s.u[e];
    u_o[N + n] = s.u[k.Np + e];
    u_o[2 * N + n] = s.u[2 * (size_t)k.Np + e];
  }
  if (mask & (8u | 16u | 32u)) {
    int ix, iy, iz;
    const Nbr nb = make_nbr(n, k.nx, k.ny, k.nz, &ix, &iy, &iz);
    if (mask & (8u | 16u)) {
      T P = T(0);
      if (mode == kObsStep) {
        const T eps = (c & kPartial) ? s.eps[n] : T(0);
        T g[Q];
        fetch_pop<T, S, RAW_IN, false, false, false, true>(g, k, s.gin, s.phi_in, n, N, nb, c, eps, T(1));
        P = seqsum(g);
      }
      if (mask & 8u) P_o[n] = P;
      if (mask & 16u) p_o[n] = mode == kObsStep ? P * k.cs2 : rho * k.cs2;
    }
    if (mask & 32u) {
      T ps[Q];
#pragma unroll
      for (int q = 1; q < Q; ++q) ps[q] = ldg(s.phi_out + sidx(k, nb.at(n, ex(q), ey(q), ez(q))));
      auto nsolid = [&](int q) { return (s.cls[nb.at(n, ex(q), ey(q), ez(q))] & kSolid) != 0; };
      T gx, gy, gz, lap;
      if (mode == kObsStep) grad_lap<T, true>(k, s, n, c, phi, ps, nsolid, gx, gy, gz, lap);
      else grad_lap<T, false>(k, s, n, c, phi, ps, nsolid, gx, gy, gz, lap);
      mu_o[n] = chem_pot(k, c, phi, lap);
    }
  }
}

// Current populations in the reference layout: s.fin/s.gin hold the last
// step's output, s.phi_in that step's phi and s.c_prev its correction.
template <typename T, typename S, bool RAW>
__global__ void __launch_bounds__(kBlock) k_populations(Consts<T> k, State<T, S> s, T* f_o, T* g_o) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  const size_t N = (size_t)k.N;
  const uint8_t c = s.cls[n];
  int ix, iy, iz;
  const Nbr nb = make_nbr(n, k.nx, k.ny, k.nz, &ix, &iy, &iz);
  const T eps = (c & kPartial) ? s.eps[n] : T(0);
  T v[Q];
  if (f_o) {
    fetch_f<T, S, RAW, false, true>(v, k, s, n, N, nb, c, eps);
#pragma unroll
    for (int q = 0; q < Q; ++q) f_o[(size_t)q * N + n] = v[q];
  }
  if (g_o) {
    fetch_pop<T, S, RAW, false, false, false, true>(v, k, s.gin, s.phi_in, n, N, nb, c, eps, T(1));
#pragma unroll
    for (int q = 0; q < Q; ++q) g_o[(size_t)q * N + n] = v[q];
  }
}

// ---------------------------------------------------------------------------
// Spread diagnostics over a phi field (fe_measure.py:11-82 + sweep z_com):
// volume, C_max, extents of phi > 0.5 (solid excluded), z centre, count, NaN.
// Partials per block: [sum, max, minx, maxx, miny, maxy, minz, maxz, sumz, count, nan]
// ---------------------------------------------------------------------------
constexpr int kMeasVals = 11;

// r <- merge(r, q): sum, max, (min, max) x 3 axes, sum, sum, max
template <typename A, typename B>
__device__ __forceinline__ void meas_merge(A& r, const B& q) {
  r[0] += q[0];
  r[1] = fmax(r[1], (double)q[1]);
#pragma unroll
  for (int j = 2; j < 8; j += 2) {
    r[j] = fmin(r[j], (double)q[j]);
    r[j + 1] = fmax(r[j + 1], (double)q[j + 1]);
  }
  r[8] += q[8];
  r[9] += q[9];
  r[10] = fmax(r[10], (double)q[10]);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_measure(int nx, int ny, int nz, const T* __restrict__ phi,
                                                   const uint8_t* __restrict__ cls, double* partials,
                                                   unsigned* counter, double* out, double* ext6) {
  const int N = nx * ny * nz;
  double v[kMeasVals] = {0.0, -1e300, 1e300, -1e300, 1e300, -1e300, 1e300, -1e300, 0.0, 0.0, 0.0};
  for (int n = blockIdx.x * kBlock + threadIdx.x; n < N; n += gridDim.x * kBlock) {
    T p = phi[n];
    if (cls[n] & kSolid) p = T(0);
    const double d = (double)p;
    if (!(d == d)) v[10] = 1.0;
    v[0] += d;
    v[1] = d > v[1] ? d : v[1];
    if (p > T(0.5)) {
      const int iz = n % nz, t = n / nz, iy = t % ny, ix = t / ny;
      v[2] = fmin(v[2], (double)ix); v[3] = fmax(v[3], (double)ix);
      v[4] = fmin(v[4], (double)iy); v[5] = fmax(v[5], (double)iy);
      v[6] = fmin(v[6], (double)iz); v[7] = fmax(v[7], (double)iz);
      v[8] += (double)iz;
      v[9] += 1.0;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double q[kMeasVals];
#pragma unroll
    for (int j = 0; j < kMeasVals; ++j) q[j] = __shfl_down_sync(0xffffffffu, v[j], o);
    meas_merge(v, q);
  }
  __shared__ double sw[kBlock / 32][kMeasVals];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
    for (int j = 0; j < kMeasVals; ++j) sw[wid][j] = v[j];
  __syncthreads();
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    for (int w = 1; w < kBlock / 32; ++w) meas_merge(v, sw[w]);
    for (int j = 0; j < kMeasVals; ++j) partials[(size_t)blockIdx.x * kMeasVals + j] = v[j];
    __threadfence();
    s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // last block: every thread merges a strided subset of the block partials,
  // then warps and finally thread 0 merge (a fixed, deterministic order)
  double r[kMeasVals] = {0.0, -1e300, 1e300, -1e300, 1e300, -1e300, 1e300, -1e300, 0.0, 0.0, 0.0};
  const volatile double* pp = partials;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += kBlock) {
    double q[kMeasVals];
    for (int j = 0; j < kMeasVals; ++j) q[j] = pp[(size_t)b * kMeasVals + j];
    meas_merge(r, q);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double q[kMeasVals];
#pragma unroll
    for (int j = 0; j < kMeasVals; ++j) q[j] = __shfl_down_sync(0xffffffffu, r[j], o);
    meas_merge(r, q);
  }
  __syncthreads();
  if (lane == 0)
    for (int j = 0; j < kMeasVals; ++j) sw[wid][j] = r[j];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kBlock / 32; ++w) meas_merge(r, sw[w]);
    const bool any = r[9] > 0.0;
    const double Dx = any ? r[3] - r[2] + 1.0 : 0.0;
    const double Dy = any ? r[5] - r[4] + 1.0 : 0.0;
    const double Dz = any ? r[7] - r[6] + 1.0 : 0.0;
    out[0] = r[0];
    out[1] = r[1];
    out[2] = Dx;
    out[3] = Dy;
    out[4] = Dz;
    out[5] = Dy > 0.0 ? Dx / Dy : 0.0;
    out[6] = any ? r[8] / r[9] : 0.0;
    out[7] = r[9];
    out[8] = r[10];
    if (ext6) {
      // first and last index of the phi > 0.5 set along x, y, z (-1 when empty)
#pragma unroll
      for (int j = 0; j < 6; ++j) ext6[j] = any ? r[2 + j] : -1.0;
    }
    *counter = 0u;
  }
}

// Total momentum sum_x rho(phi) u of a field pair (phi dense [N], u with
// component stride us), rho = phi rho_l + (1 - phi) rho_g, accumulated in
// float64 per node in a fixed order (block partials, then the last block
// sums them in block order).  Writes out3.
// u in the state's layout: nh pairs (paired layout) or 0 (linear).
struct NhOnly {
  int nh;
};
template <typename T>
__global__ void __launch_bounds__(kBlock) k_momentum(int N, const T* __restrict__ phi, const T* __restrict__ u,
                                                    int us, int nh, double rho_l, double rho_g, double* partials,
                                                    unsigned* counter, double* out3) {
  double m[3] = {0.0, 0.0, 0.0};
  const NhOnly lay{nh};
  for (int n = blockIdx.x * kBlock + threadIdx.x; n < N; n += gridDim.x * kBlock) {
    const double p = (double)phi[n];
    const double rho = p * rho_l + (1.0 - p) * rho_g;
    const unsigned e = sidx(lay, n);
#pragma unroll
    for (int d = 0; d < 3; ++d) m[d] += rho * (double)u[(size_t)d * us + e];
  }
  __shared__ double sw[kBlock / 32][3];
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double v = m[d];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sw[wid][d] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int d = 0; d < 3; ++d) {
      double v = 0.0;
      for (int w = 0; w < kBlock / 32; ++w) v += sw[w][d];
      partials[(size_t)blockIdx.x * 3 + d] = v;
    }
    __threadfence();
    s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  __threadfence();
  const volatile double* pp = partials;
  for (int d = 0; d < 3; ++d) {
    double v = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) v += pp[(size_t)b * 3 + d];
    out3[d] = v;
  }
  *counter = 0u;
}

// ---------------------------------------------------------------------------
// Host-side launchers (called from lbm_capi.cu)
// ---------------------------------------------------------------------------
template <typename T, typename S, bool RAW, bool FIRST, bool OMEGA1>
static cudaError_t launch_step_t(const Consts<T>& k, const State<T, S>& s, const Tiling& tl, cudaStream_t st) {
  const size_t sm = step_smem_bytes<T, S>(tl);
  auto fn = k_step<T, S, RAW, FIRST, OMEGA1>;
  if (sm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  fn<<<tl.ntx * tl.nty * tl.ntz, kBlock, sm, st>>>(k, s, tl);
  return cudaGetLastError();
}

template <typename T, typename S, bool RAW, bool FIRST, bool OMEGA1>
static cudaError_t launch_two_t(const Consts<T>& k, const State<T, S>& s, cudaStream_t st, cudaEvent_t mid) {
  int gphi = 0;
  cudaError_t e = resident_grid(k_phi<T, S, RAW>, k.N, &gphi);
  if (e != cudaSuccess) return e;
  k_phi<T, S, RAW><<<gphi, kBlock, 0, st>>>(k, s);
  if (mid) {
    e = cudaEventRecord(mid, st);
    if (e != cudaSuccess) return e;
  }
  const int blocks = (k.N + kBlock - 1) / kBlock;
  if (k.gmu_mode) {
    // the gradient-of-mu modes: float and double storage, first step here
    // (later steps run the batched kernels)
    if constexpr (RAW && FIRST && sizeof(S) != 2) {
      k_mu<T, S><<<blocks, kBlock, 0, st>>>(k, s);
      k_gradmu<T, S><<<blocks, kBlock, 0, st>>>(k, s);
      k_update<T, S, RAW, FIRST, OMEGA1, true><<<blocks, kBlock, 0, st>>>(k, s);
      return cudaGetLastError();
    } else {
      return cudaErrorNotSupported;
    }
  }
  k_update<T, S, RAW, FIRST, OMEGA1><<<blocks, kBlock, 0, st>>>(k, s);
  return cudaGetLastError();
}

// The first step after init reads the reference state in place (RAW) and has
// no phi u of a previous step (FIRST); every later step is neither.  A tiling
// with tx == 0 selects the two-kernel step, else the fused tiled kernel.
// `mid` (may be null) is recorded between k_phi and k_update, or before the
// fused kernel.
template <typename T, typename S>
cudaError_t launch_step(const Consts<T>& k, const State<T, S>& s, const Tiling& tl, bool raw, bool first,
                        cudaStream_t st, cudaEvent_t mid) {
  if (raw != first) return cudaErrorInvalidValue;
  if (k.gmu_mode && tl.tx != 0) return cudaErrorNotSupported;  // no fused-kernel form of these modes
  if (tl.tx == 0) {
    const bool om1 = k.omega_f == T(1);
    if (raw)
      return om1 ? launch_two_t<T, S, true, true, true>(k, s, st, mid)
                 : launch_two_t<T, S, true, true, false>(k, s, st, mid);
    return om1 ? launch_two_t<T, S, false, false, true>(k, s, st, mid)
               : launch_two_t<T, S, false, false, false>(k, s, st, mid);
  }
  if (mid) {
    cudaError_t e = cudaEventRecord(mid, st);
    if (e != cudaSuccess) return e;
  }
  const bool om1 = k.omega_f == T(1);
  if (raw)
    return om1 ? launch_step_t<T, S, true, true, true>(k, s, tl, st) : launch_step_t<T, S, true, true, false>(k, s, tl, st);
  return om1 ? launch_step_t<T, S, false, false, true>(k, s, tl, st)
             : launch_step_t<T, S, false, false, false>(k, s, tl, st);
}

// Launch with programmatic stream serialization (see pdl_wait).
constexpr int kPdlOn = 1;  // 0: plain stream serialization
template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl_bs(void (*fn)(KArgs...), int blocks, int threads, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = kPdlOn;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, fn, args...);
}
template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*fn)(KArgs...), int blocks, cudaStream_t st, Args... args) {
  return launch_pdl_bs(fn, blocks, kBlock, st, args...);
}

// Batched step kernels over a device case table; blocks: the grid (the
// length of the block -> case table).
template <typename T, typename S>
cudaError_t launch_phi_batch(const void* cases, const unsigned short* b2c, int blocks, cudaStream_t st) {
  if (blocks <= 0) return cudaSuccess;
  return launch_pdl(k_phi_batch<T, S>, blocks, st, static_cast<const CaseDesc<T, S>*>(cases), b2c);
}
// bs: threads per block of the update kernel, 256 or (without the
// gradient-of-mu modes) 128.
template <typename T, typename S>
cudaError_t launch_update_batch(const void* cases, const unsigned short* b2c, int blocks, bool omega1,
                                cudaStream_t st, bool gmu, int bs) {
  if (blocks <= 0) return cudaSuccess;
  auto c = static_cast<const CaseDesc<T, S>*>(cases);
  if (gmu) {
    if constexpr (sizeof(S) != 2) {
      if (bs != kBlock) return cudaErrorInvalidValue;
      if (omega1) return launch_pdl(k_update_batch<T, S, true, true>, blocks, st, c, b2c);
      return launch_pdl(k_update_batch<T, S, false, true>, blocks, st, c, b2c);
    } else {
      return cudaErrorNotSupported;
    }
  }
  if (bs == 128) {
    if (omega1) return launch_pdl_bs(k_update_batch<T, S, true, false, 128>, blocks, 128, st, c, b2c);
    return launch_pdl_bs(k_update_batch<T, S, false, false, 128>, blocks, 128, st, c, b2c);
  }
  if (bs != kBlock) return cudaErrorInvalidValue;
  if (omega1) return launch_pdl(k_update_batch<T, S, true>, blocks, st, c, b2c);
  return launch_pdl(k_update_batch<T, S, false>, blocks, st, c, b2c);
}
// The paired-layout step kernels over a device case table of paired grids.
// (float compute only: float64 grids keep the linear layout)
template <typename T, typename S>
cudaError_t launch_phi_pair(const void* cases, const unsigned short* b2c, int blocks, cudaStream_t st) {
  if constexpr (sizeof(T) == 8) {
    return cudaErrorNotSupported;
  } else {
    if (blocks <= 0) return cudaSuccess;
    return launch_pdl(k_phi_pair<T, S>, blocks, st, static_cast<const CaseDesc<T, S>*>(cases), b2c);
  }
}
template <typename T, typename S>
cudaError_t launch_update_pair(const void* cases, const unsigned short* b2c, int blocks, bool omega1,
                               cudaStream_t st, bool gmu) {
  if constexpr (sizeof(T) == 8) {
    return cudaErrorNotSupported;
  } else {
    if (blocks <= 0) return cudaSuccess;
    auto c = static_cast<const CaseDesc<T, S>*>(cases);
    constexpr int bs = kPairUpdBlock;
    if (gmu) {
      if constexpr (sizeof(S) != 2) {
        if (omega1) return launch_pdl_bs(k_update_pair<T, S, true, true>, blocks, bs, st, c, b2c);
        return launch_pdl_bs(k_update_pair<T, S, false, true>, blocks, bs, st, c, b2c);
      } else {
        return cudaErrorNotSupported;
      }
    }
    if (omega1) return launch_pdl_bs(k_update_pair<T, S, true, false>, blocks, bs, st, c, b2c);
    return launch_pdl_bs(k_update_pair<T, S, false, false>, blocks, bs, st, c, b2c);
  }
}
// The cooperative single-launch batched step (k_batch_coop) over a table
// whose update blocks run 256 threads; grid: resident blocks of the kernel.
template <typename T, typename S>
cudaError_t launch_batch_coop(const void* cases, const unsigned short* b2c, int phi_blocks, int upd_om1,
                              int upd_other, cudaStream_t st) {
  static std::mutex mu;
  static int cached_dev = -1, cached = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int grid;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (cached_dev != dev) {
      int nsm = 0, b = 0;
      e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_coop<T, S>, kBlock, 0);
      if (e != cudaSuccess) return e;
      cached = nsm * b;
      cached_dev = dev;
    }
    grid = cached;
  }
  const int work = std::max(phi_blocks, upd_om1 + upd_other);
  if (work <= 0) return cudaSuccess;
  if (grid > work) grid = work;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kBlock);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_batch_coop<T, S>, static_cast<const CaseDesc<T, S>*>(cases), b2c, phi_blocks,
                            upd_om1, upd_other);
}

// k_mu and k_gradmu of one grid (plain stream order: they wait for the phi kernel, and the
// next update kernel waits for it).
template <typename T, typename S>
cudaError_t launch_mu(const Consts<T>& k, const State<T, S>& s, cudaStream_t st) {
  const int blocks = (k.N + kBlock - 1) / kBlock;
  k_mu<T, S><<<blocks, kBlock, 0, st>>>(k, s);
  k_gradmu<T, S><<<blocks, kBlock, 0, st>>>(k, s);
  return cudaGetLastError();
}
template <typename T, typename S>
size_t case_desc_bytes() {
  return sizeof(CaseDesc<T, S>);
}
// Fills one descriptor in host memory.
template <typename T, typename S>
void fill_case_desc(void* dst, const Consts<T>& k, const State<T, S>& s, int phi_blk0, int phi_nblk, int upd_blk0,
                    int upd_nblk) {
  CaseDesc<T, S> d;
  std::memset(&d, 0, sizeof(d));
  d.k = k;
  d.s = s;
  d.phi_blk0 = phi_blk0;
  d.phi_nblk = phi_nblk;
  d.upd_blk0 = upd_blk0;
  d.upd_nblk = upd_nblk;
  std::memcpy(dst, &d, sizeof(d));
}

template <typename T, typename S>
cudaError_t launch_inject(const Consts<T>& k, const State<T, S>& s, bool raw, const InjectParams& ip,
                          const T* P_attr, unsigned* core_count, cudaStream_t st) {
  const int grid = (k.N + kBlock - 1) / kBlock;
  if (raw)
    k_inject<T, S, true><<<grid, kBlock, 0, st>>>(k, s, ip, P_attr, core_count);
  else
    k_inject<T, S, false><<<grid, kBlock, 0, st>>>(k, s, ip, P_attr, core_count);
  return cudaGetLastError();
}

template <typename T, typename S, typename Src>
cudaError_t launch_init(const Consts<T>& k, const State<T, S>& s, const Src* phi0, const Src* u0, cudaStream_t st) {
  const int grid = (k.N + kBlock - 1) / kBlock;
  k_init<T, S, Src><<<grid, kBlock, 0, st>>>(k, s, phi0, u0);
  return cudaGetLastError();
}

template <typename T, typename S>
cudaError_t launch_observe(const Consts<T>& k, const State<T, S>& s, bool raw_in, unsigned mask, int mode,
                           T* phi, T* rho, T* u, T* P, T* p, T* mu, cudaStream_t st) {
  const int grid = (k.N + kBlock - 1) / kBlock;
  if (raw_in) k_observe<T, S, true><<<grid, kBlock, 0, st>>>(k, s, mask, mode, phi, rho, u, P, p, mu);
  else k_observe<T, S, false><<<grid, kBlock, 0, st>>>(k, s, mask, mode, phi, rho, u, P, p, mu);
  return cudaGetLastError();
}

template <typename T, typename S>
cudaError_t launch_populations(const Consts<T>& k, const State<T, S>& s, bool raw, T* f, T* g, cudaStream_t st) {
  const int grid = (k.N + kBlock - 1) / kBlock;
  if (raw) k_populations<T, S, true><<<grid, kBlock, 0, st>>>(k, s, f, g);
  else k_populations<T, S, false><<<grid, kBlock, 0, st>>>(k, s, f, g);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_measure(int nx, int ny, int nz, const T* phi, const uint8_t* cls, double* partials,
                           int max_blocks, unsigned* counter, double* out, cudaStream_t st, double* ext6) {
  const int N = nx * ny * nz;
  int grid = (N + kBlock - 1) / kBlock;
  if (grid > max_blocks) grid = max_blocks;
  k_measure<T><<<grid, kBlock, 0, st>>>(nx, ny, nz, phi, cls, partials, counter, out, ext6);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_momentum(int N, const T* phi, const T* u, int us, int nh, double rho_l, double rho_g,
                            double* partials, int max_blocks, unsigned* counter, double* out3, cudaStream_t st) {
  int grid = (N + kBlock - 1) / kBlock;
  if (grid > max_blocks) grid = max_blocks;
  k_momentum<T><<<grid, kBlock, 0, st>>>(N, phi, u, us, nh, rho_l, rho_g, partials, counter, out3);
  return cudaGetLastError();
}
template cudaError_t launch_momentum<float>(int, const float*, const float*, int, int, double, double, double*, int,
                                            unsigned*, double*, cudaStream_t);
template cudaError_t launch_momentum<double>(int, const double*, const double*, int, int, double, double, double*,
                                             int, unsigned*, double*, cudaStream_t);

// ---------------------------------------------------------------------------
// Allocation-free spread diagnostics.  Some callers cannot allocate device
// memory: code that runs inside a memory pool handed out by another runtime,
// host code under a driver that forbids cudaMalloc after start-up, or a
// measurement hook that must not perturb the allocator it observes.  For them
// the block partials and the completion counter of k_measure live in this
// file-scope scratch, which every GPU that loads the library holds until the
// process exits.  Calls share it and it keeps the last call's contents, so
// calls that overlap on the GPU (different streams, or different host
// threads on one device) race and must be serialised by the caller.
// ---------------------------------------------------------------------------
constexpr int kStaticMeasBlocks = 1024;  // 1024 x 11 doubles = 90,112 bytes of partials
static __device__ __align__(256) double g_static_meas_partials[kStaticMeasBlocks * kMeasVals];
static __device__ __align__(256) unsigned g_static_meas_counter;

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
double* g_static_partials_dev[kMaxDevices] = {};
unsigned* g_static_counter_dev[kMaxDevices] = {};
}  // namespace

// Device addresses of the static scratch on the current device.  In host
// code the two arrays' names only denote host-side shadows; the device
// addresses come from cudaGetSymbolAddress, looked up once per device with
// that device current (which may load this module onto the device, so the
// first call on a device should come before any stream capture).
static cudaError_t static_meas_scratch(double** partials, unsigned** counter) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_partials_dev[dev]) {
    void* p = nullptr;
    void* c = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_meas_partials);
    if (e != cudaSuccess) return e;
    e = cudaGetSymbolAddress(&c, g_static_meas_counter);
    if (e != cudaSuccess) return e;
    g_static_counter_dev[dev] = static_cast<unsigned*>(c);
    g_static_partials_dev[dev] = static_cast<double*>(p);
  }
  *partials = g_static_partials_dev[dev];
  *counter = g_static_counter_dev[dev];
  return cudaSuccess;
}

// k_measure over a caller's phi and 0/1 solid mask with the static scratch;
// writes the 9 outputs to `out` (device).  No allocation.
template <typename T>
cudaError_t launch_measure_static(int nx, int ny, int nz, const T* phi, const uint8_t* solid, double* out,
                                  cudaStream_t st) {
  double* partials = nullptr;
  unsigned* counter = nullptr;
  cudaError_t e = static_meas_scratch(&partials, &counter);
  if (e != cudaSuccess) return e;
  // the counter must start at zero: a launch that failed part-way leaves it set
  e = cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  return launch_measure<T>(nx, ny, nz, phi, solid, partials, kStaticMeasBlocks, counter, out, st, nullptr);
}
template cudaError_t launch_measure_static<float>(int, int, int, const float*, const uint8_t*, double*, cudaStream_t);
template cudaError_t launch_measure_static<double>(int, int, int, const double*, const uint8_t*, double*,
                                                   cudaStream_t);

template size_t step_smem_bytes<float, float>(const Tiling&);
template size_t step_smem_bytes<double, double>(const Tiling&);
template size_t step_smem_bytes<float, __half>(const Tiling&);

#define LBM_INSTANTIATE(T, S)                                                                                   \
  template cudaError_t launch_step<T, S>(const Consts<T>&, const State<T, S>&, const Tiling&, bool, bool,        \
                                         cudaStream_t, cudaEvent_t);                                             \
  template cudaError_t launch_init<T, S, float>(const Consts<T>&, const State<T, S>&, const float*, const float*,  \
                                                cudaStream_t);                                                   \
  template cudaError_t launch_init<T, S, double>(const Consts<T>&, const State<T, S>&, const double*,             \
                                                 const double*, cudaStream_t);                                    \
  template cudaError_t launch_observe<T, S>(const Consts<T>&, const State<T, S>&, bool, unsigned, int, T*, T*, T*, \
                                            T*, T*, T*, cudaStream_t);                                           \
  template cudaError_t launch_populations<T, S>(const Consts<T>&, const State<T, S>&, bool, T*, T*, cudaStream_t);  \
  template cudaError_t launch_inject<T, S>(const Consts<T>&, const State<T, S>&, bool, const InjectParams&,        \
                                           const T*, unsigned*, cudaStream_t);

LBM_INSTANTIATE(float, float)
LBM_INSTANTIATE(double, double)
LBM_INSTANTIATE(float, __half)
#undef LBM_INSTANTIATE

#define LBM_INSTANTIATE_BATCH(T, S)                                                                             \
  template cudaError_t launch_phi_batch<T, S>(const void*, const unsigned short*, int, cudaStream_t);           \
  template cudaError_t launch_update_batch<T, S>(const void*, const unsigned short*, int, bool, cudaStream_t,    \
                                                 bool, int);                                                     \
  template cudaError_t launch_mu<T, S>(const Consts<T>&, const State<T, S>&, cudaStream_t);                     \
  template cudaError_t launch_phi_pair<T, S>(const void*, const unsigned short*, int, cudaStream_t);            \
  template cudaError_t launch_batch_coop<T, S>(const void*, const unsigned short*, int, int, int, cudaStream_t);  \
  template cudaError_t launch_update_pair<T, S>(const void*, const unsigned short*, int, bool, cudaStream_t,     \
                                                bool);                                                          \
  template size_t case_desc_bytes<T, S>();                                                                      \
  template void fill_case_desc<T, S>(void*, const Consts<T>&, const State<T, S>&, int, int, int, int);
LBM_INSTANTIATE_BATCH(float, float)
LBM_INSTANTIATE_BATCH(double, double)
LBM_INSTANTIATE_BATCH(float, __half)
#undef LBM_INSTANTIATE_BATCH

template cudaError_t launch_measure<float>(int, int, int, const float*, const uint8_t*, double*, int, unsigned*,
                                           double*, cudaStream_t, double*);
template cudaError_t launch_measure<double>(int, int, int, const double*, const uint8_t*, double*, int, unsigned*,
                                            double*, cudaStream_t, double*);

}  // namespace lbm
