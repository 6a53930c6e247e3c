// Device kernels of the GB300 Allen-Cahn phase-field LBM step.
//
// State convention ("pull" form).  Between steps the population buffers hold
// POST-COLLISION values F(x, q) of every node, solid and partial nodes
// included.  The reference's state at the start of a step (pytorch-lbm
// lbm/fe_ac_solver.py:548-591: streamed, bounced back at solid nodes,
// volume-penalised at partial nodes, scaled by the global phi-mass correction
// c, then boundary-phi relaxed at active boundary nodes) is reconstructed on
// read:
//   fluid x    f(x,q) = c F(x - e_q, q)                       (periodic)
//   solid x    f(x,q) = c F(x, opp q)                          (:556-566)
//   partial x  f(x,q) = c ((1 - eps) F(x - e_q, q) + eps F(x, opp q))  (:569-578)
//   relaxed x  f(x,q) *= clamp(phi_new / max(sum_q f(x,q), 1e-10), 1/2, 2)  (:620-636)
// g is reconstructed the same way without c and without relaxation.  Right
// after init (RAW) the buffers hold the reference state itself.
//
// One step = two launches: k_phi (phi recovery + deterministic global sum ->
// c) and k_collide (stencils, wetting, forces, velocity, Allen-Cahn source,
// both BGK collisions, relaxation bookkeeping).  Arithmetic follows the
// reference's operation order; sums run in population order.
#include <cuda_runtime.h>

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

// Block-wide sum of a double; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double s_warp[kBlock / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
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
                                                 double* total) {
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = part;
    __threadfence();
    const unsigned done = atomicAdd(counter, 1u);
    s_last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  // The last block reduces the partials with all its threads, in a fixed order.
  double acc = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) acc += ((volatile double*)partials)[i];
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
template <typename T, bool RAW, bool WITH_C>
__device__ __forceinline__ void fetch_pop(T (&v)[Q], const T* __restrict__ F, int n, size_t N,
                                          const Nbr& nb, uint8_t c, T eps, T corr) {
  if (RAW) {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = ldg(F + (size_t)q * N + n);
    return;
  }
  if (c & kSolid) {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = ldg(F + (size_t)opp(q) * N + n);
  } else {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = ldg(F + (size_t)q * N + nb.at(n, -ex(q), -ey(q), -ez(q)));
    if (c & kPartial) {
      const T one_m = T(1) - eps;
#pragma unroll
      for (int q = 0; q < Q; ++q) v[q] = one_m * v[q] + eps * ldg(F + (size_t)opp(q) * N + n);
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

// Relaxation scale of lbm/fe_ac_solver.py:626-629.
template <typename T>
__device__ __forceinline__ T relax_scale(T target, T sum_f) {
  const T safe = sum_f < T(1e-10) ? T(1e-10) : sum_f;
  const T s = target / safe;
  return s < T(0.5) ? T(0.5) : (s > T(2.0) ? T(2.0) : s);
}

// ---------------------------------------------------------------------------
// K1: phi recovery, sum(phi) and the mass-correction factor
// ---------------------------------------------------------------------------
template <typename T, bool RAW>
__global__ void __launch_bounds__(kBlock) k_phi(Consts<T> k, State<T> s) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  const size_t N = (size_t)k.N;
  double part = 0.0;
  if (n < k.N) {
    const uint8_t c = s.cls[n];
    T phi = T(0);
    if (!(c & kSolid)) {
      int ix, iy, iz;
      const Nbr nb = make_nbr(n, k.nx, k.ny, k.nz, &ix, &iy, &iz);
      const T eps = (c & kPartial) ? s.eps[n] : T(0);
      T v[Q];
      fetch_pop<T, RAW, !RAW>(v, s.fin, n, N, nb, c, eps, RAW ? T(1) : s.cbuf[s.c_prev]);
      if (!RAW && (c & kTop)) {
        const T r = s.relax[n];
        if (r >= T(0)) {
          const T sc = relax_scale(r, seqsum(v));
#pragma unroll
          for (int q = 0; q < Q; ++q) v[q] = v[q] * sc;
          s.relax[n] = sc;  // k_collide applies the same scale
        }
      }
      phi = clamp01(seqsum(v));
    }
    s.phi[n] = phi;
    part = (double)phi;
  }
  part = block_sum(part);
  double total;
  if (last_block_total(part, s.partials, s.counter, &total)) {
    // lbm/fe_ac_solver.py:582-589, in T: c = (1/max(S,1e-6)) * M0 if S > 1e-6 else 1
    const T S = (T)total;
    T corr = T(1);
    if (S > T(1e-6)) {
      const T safe = S < T(1e-6) ? T(1e-6) : S;
      corr = (T(1) / safe) * (T)s.scal[0];
    } else {
      atomicOr(s.status, 2u);
    }
    if (!(total == total) || total - total != 0.0) atomicOr(s.status, 1u);
    s.cbuf[s.c_cur] = corr;
    s.scal[1] = total;
  }
}

// ---------------------------------------------------------------------------
// Isotropic gradient / laplacian with the ghost-node wetting correction
// (lbm/fe_ac_solver.py:296-320 fused, :282-294 unfused; fe_wetting.py:418-446)
// ---------------------------------------------------------------------------
template <typename T, bool FUSED>
__device__ __forceinline__ void stencil(const Consts<T>& k, const State<T>& s, int n, const Nbr& nb,
                                        uint8_t c, T phi, T& gx, T& gy, T& gz, T& lap) {
  T ps[Q];
#pragma unroll
  for (int q = 1; q < Q; ++q) ps[q] = ldg(s.phi + nb.at(n, ex(q), ey(q), ez(q)));
  if (k.wetting && (c & kBoundary)) {
    const size_t N = (size_t)k.N;
    const float n0 = s.wn[n], n1 = s.wn[N + n], n2 = s.wn[2 * N + n];
#pragma unroll
    for (int q = 1; q < Q; ++q) {
      if (s.cls[nb.at(n, ex(q), ey(q), ez(q))] & kSolid) {
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
#pragma unroll
  for (int q = 1; q < Q; ++q) {
    if (ex(q) != 0) gx = gx + (ex(q) > 0 ? k.wc[q] : -k.wc[q]) * ps[q];
    if (ey(q) != 0) gy = gy + (ey(q) > 0 ? k.wc[q] : -k.wc[q]) * ps[q];
    if (ez(q) != 0) gz = gz + (ez(q) > 0 ? k.wc[q] : -k.wc[q]) * ps[q];
    if (FUSED) {
      lap = lap + k.w2c[q] * (ps[q] - phi);
    } else {
      lap = lap + (T(2) * k.w[q]) * (ps[q] - phi) / k.cs2;
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

// ---------------------------------------------------------------------------
// K2: fused stencil + wetting + forces + velocity + source + collisions
// ---------------------------------------------------------------------------
template <typename T, bool RAW, bool FIRST>
__global__ void __launch_bounds__(kBlock) k_collide(Consts<T> k, State<T> s) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  const size_t N = (size_t)k.N;
  const uint8_t c = s.cls[n];
  int ix, iy, iz;
  const Nbr nb = make_nbr(n, k.nx, k.ny, k.nz, &ix, &iy, &iz);
  const T phi = s.phi[n];  // clamped, 0 in solid; phi_safe == phi

  // 2. density
  const T rho = phi * k.rho_l + (T(1) - phi) * k.rho_g;
  const T rho_eff = rho < k.rho_floor ? k.rho_floor : rho;

  // gradient, laplacian, chemical potential
  T gx, gy, gz, lap;
  stencil<T, true>(k, s, n, nb, c, phi, gx, gy, gz, lap);
  const T mu = chem_pot(k, c, phi, lap);

  // geometric contact-angle gradient correction (fe_wetting.py:448-539).  The
  // wall normal is zero away from boundary nodes, where the correction is the
  // identity, so only boundary nodes are visited.
  if (k.geometric && (c & kBoundary)) {
    const T n0 = (T)s.wn[n], n1 = (T)s.wn[N + n], n2 = (T)s.wn[2 * N + n];
    const T gn = (n0 * gx + n1 * gy) + n2 * gz;
    const T tx = gx - gn * n0, ty = gy - gn * n1, tz = gz - gn * n2;
    T tm = sqrt((tx * tx + ty * ty) + tz * tz);
    tm = tm < T(1e-10) ? T(1e-10) : tm;
    T gd = ((-tm) * k.cos_t) / k.sin_t;
    if (k.amp_active) {
      const T delta = gd - gn;
      gd = gn + delta * k.amp;
    }
    const T cx = tx + gd * n0, cy = ty + gd * n1, cz = tz + gd * n2;
    const T gm = sqrt((gx * gx + gy * gy) + gz * gz);
    if (gm > T(1e-6)) {
      const T bl = k.ww[c >> kWwShift];
      gx = gx + bl * (cx - gx);
      gy = gy + bl * (cy - gy);
      gz = gz + bl * (cz - gz);
    }
  }

  // 3. pressure from the hydrodynamic populations
  const T eps = (c & kPartial) ? s.eps[n] : T(0);
  T g[Q];
  fetch_pop<T, RAW, false>(g, s.gin, n, N, nb, c, eps, T(1));
  const T P = seqsum(g);

  // 4. non-equilibrium stress with the new P and the old u (:409-413)
  const T uo0 = s.u[n], uo1 = s.u[N + n], uo2 = s.u[2 * N + n];
  T sxx, syy, szz, sxy, sxz, syz;
  {
    const T usq = (uo0 * uo0 + uo1 * uo1) + uo2 * uo2;
    const T b = usq / k.two_cs2;
    bool fxx = true, fyy = true, fzz = true, fxy = true, fxz = true, fyz = true;
    sxx = syy = szz = sxy = sxz = syz = T(0);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      T eu = T(0);
      bool any = false;
      if (ex(q) != 0) { eu = ex(q) > 0 ? uo0 : -uo0; any = true; }
      if (ey(q) != 0) { const T t = ey(q) > 0 ? uo1 : -uo1; eu = any ? eu + t : t; any = true; }
      if (ez(q) != 0) { const T t = ez(q) > 0 ? uo2 : -uo2; eu = any ? eu + t : t; any = true; }
      const T ec = eu / k.cs2;
      const T sq = k.w[q] * ((ec + ec * ec / T(2)) - b);
      const T gneq = g[q] - (P * k.w[q] + sq);
      if (ex(q) != 0) { sxx = fxx ? gneq : sxx + gneq; fxx = false; }
      if (ey(q) != 0) { syy = fyy ? gneq : syy + gneq; fyy = false; }
      if (ez(q) != 0) { szz = fzz ? gneq : szz + gneq; fzz = false; }
      if (ex(q) * ey(q) != 0) { const T t = ex(q) * ey(q) > 0 ? gneq : -gneq; sxy = fxy ? t : sxy + t; fxy = false; }
      if (ex(q) * ez(q) != 0) { const T t = ex(q) * ez(q) > 0 ? gneq : -gneq; sxz = fxz ? t : sxz + t; fxz = false; }
      if (ey(q) * ez(q) != 0) { const T t = ey(q) * ez(q) > 0 ? gneq : -gneq; syz = fyz ? t : syz + t; fyz = false; }
    }
  }

  // 5. forces (Fakhari 2017, :416-439)
  T F0, F1, F2;
  {
    const T fp = ((-P) * k.drho) * k.cs2;
    const T m0 = (sxx * gx + sxy * gy) + sxz * gz;
    const T m1 = (sxy * gx + syy * gy) + syz * gz;
    const T m2 = (sxz * gx + syz * gy) + szz * gz;
    F0 = mu * gx;
    F1 = mu * gy;
    F2 = mu * gz;
    if (k.stab_mode <= 1) {
      F0 = F0 + fp * gx;
      F1 = F1 + fp * gy;
      F2 = F2 + fp * gz;
    }
    if (k.stab_mode == 0) {
      F0 = F0 + (k.visc * m0) * k.drho;
      F1 = F1 + (k.visc * m1) * k.drho;
      F2 = F2 + (k.visc * m2) * k.drho;
    }
    if (k.has_gforce) {
      F0 = F0 + k.gforce[0] * rho;
      F1 = F1 + k.gforce[1] * rho;
      F2 = F2 + k.gforce[2] * rho;
    }
  }

  // 6. velocity (:442-447)
  T u0, u1, u2;
  {
    bool f0 = true, f1 = true, f2 = true;
    u0 = u1 = u2 = T(0);
#pragma unroll
    for (int q = 1; q < Q; ++q) {
      if (ex(q) != 0) { const T t = ex(q) > 0 ? g[q] : -g[q]; u0 = f0 ? t : u0 + t; f0 = false; }
      if (ey(q) != 0) { const T t = ey(q) > 0 ? g[q] : -g[q]; u1 = f1 ? t : u1 + t; f1 = false; }
      if (ez(q) != 0) { const T t = ez(q) > 0 ? g[q] : -g[q]; u2 = f2 ? t : u2 + t; f2 = false; }
    }
    u0 = u0 + (T(0.5) * F0) / rho_eff;
    u1 = u1 + (T(0.5) * F1) / rho_eff;
    u2 = u2 + (T(0.5) * F2) / rho_eff;
    if (c & kSolid) u0 = u1 = u2 = T(0);
  }

  // 7. Allen-Cahn source (:450-494)
  T S0, S1, S2;
  {
    T d0 = T(0), d1 = T(0), d2 = T(0);
    if (!FIRST) {
      const T pp = s.phi_prev[n];
      d0 = phi * u0 - pp * uo0;
      d1 = phi * u1 - pp * uo1;
      d2 = phi * u2 - pp * uo2;
    }
    T gm = sqrt((gx * gx + gy * gy) + gz * gz);
    gm = gm < T(1e-10) ? T(1e-10) : gm;
    const T lam = ((T(4) * phi) * (T(1) - phi)) / k.W;
    const T cl = k.cs2 * lam;
    T sh0 = ((cl * (gx / gm)) * k.ac_scale);
    T sh1 = ((cl * (gy / gm)) * k.ac_scale);
    T sh2 = ((cl * (gz / gm)) * k.ac_scale);
    if (k.wetting) {
      const T fac = T(1) - k.sharpen_reduce * k.ww[c >> kWwShift];
      sh0 = sh0 * fac;
      sh1 = sh1 * fac;
      sh2 = sh2 * fac;
    }
    S0 = d0 + sh0;
    S1 = d1 + sh1;
    S2 = d2 + sh2;
  }

  // 8. collisions (:496-530)
  const T usq = (u0 * u0 + u1 * u1) + u2 * u2;
  const T b = usq / k.two_cs2;
  {
    T f[Q];
    fetch_pop<T, RAW, !RAW>(f, s.fin, n, N, nb, c, eps, RAW ? T(1) : s.cbuf[s.c_prev]);
    if (!RAW && (c & kTop)) {
      const T sc = s.relax[n];
      if (sc >= T(0)) {
#pragma unroll
        for (int q = 0; q < Q; ++q) f[q] = f[q] * sc;
      }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      T eu = T(0), es = T(0);
      bool any = false;
      if (ex(q) != 0) { eu = ex(q) > 0 ? u0 : -u0; es = ex(q) > 0 ? S0 : -S0; any = true; }
      if (ey(q) != 0) {
        const T t = ey(q) > 0 ? u1 : -u1, ts = ey(q) > 0 ? S1 : -S1;
        eu = any ? eu + t : t; es = any ? es + ts : ts; any = true;
      }
      if (ez(q) != 0) {
        const T t = ez(q) > 0 ? u2 : -u2, ts = ez(q) > 0 ? S2 : -S2;
        eu = any ? eu + t : t; es = any ? es + ts : ts; any = true;
      }
      const T ec = eu / k.cs2;
      const T feq = phi * (k.w[q] * (((T(1) + ec) + ec * ec / T(2)) - b));
      const T src = (k.wac[q] * es) / k.cs2;
      s.fout[(size_t)q * N + n] = (f[q] - k.omega_f * (f[q] - feq)) + src;
    }
  }
  {
    T tau;
    if (k.tau_const) {
      tau = k.tau_l;
    } else {
      const T eta = phi * k.rho_l * k.tl_m + (T(1) - phi) * k.rho_g * k.tg_m;
      const T rden = phi * k.rho_l + (T(1) - phi) * k.rho_g;
      tau = T(0.5) + eta / rden;
    }
    const T rcp = T(1) / tau;
    const T ns = T(1) - rcp * T(0.5);
    const T den = rho_eff * k.cs2;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      T eu = T(0), eF = T(0);
      bool any = false;
      if (ex(q) != 0) { eu = ex(q) > 0 ? u0 : -u0; eF = ex(q) > 0 ? F0 : -F0; any = true; }
      if (ey(q) != 0) {
        const T t = ey(q) > 0 ? u1 : -u1, tf = ey(q) > 0 ? F1 : -F1;
        eu = any ? eu + t : t; eF = any ? eF + tf : tf; any = true;
      }
      if (ez(q) != 0) {
        const T t = ez(q) > 0 ? u2 : -u2, tf = ez(q) > 0 ? F2 : -F2;
        eu = any ? eu + t : t; eF = any ? eF + tf : tf; any = true;
      }
      const T ec = eu / k.cs2;
      const T sq = k.w[q] * ((ec + ec * ec / T(2)) - b);
      const T geq = P * k.w[q] + sq;
      const T G = ((ns * k.w[q]) * eF) / den;
      s.gout[(size_t)q * N + n] = (g[q] - rcp * (g[q] - geq)) + G;
    }
  }
  s.u[n] = u0;
  s.u[N + n] = u1;
  s.u[2 * N + n] = u2;
  s.phi_prev[n] = phi;

  // 12. boundary-phi relaxation target for the next step (:594-624)
  if (k.relax_on && (c & kTop)) {
    const T pb = clamp01(phi * s.cbuf[s.c_cur]);
    T r = T(-1);
    if (pb > T(0.15) && pb < T(0.85)) r = clamp01(pb + k.relax_r * (k.relax_target - pb));
    s.relax[n] = r;
  }
}

// ---------------------------------------------------------------------------
// init_fields (lbm/fe_ac_solver.py:239-261): phi = clamp(phi0), f = f_eq,
// g = g_eq(0, u), phi-mass reference.
// ---------------------------------------------------------------------------
template <typename T, typename S>
__global__ void __launch_bounds__(kBlock) k_init(Consts<T> k, State<T> s, const S* phi0, const S* u0) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  const size_t N = (size_t)k.N;
  double part = 0.0;
  if (n < k.N) {
    const T phi = clamp01((T)phi0[n]);
    const T v0 = u0 ? (T)u0[n] : T(0), v1 = u0 ? (T)u0[N + n] : T(0), v2 = u0 ? (T)u0[2 * N + n] : T(0);
    const T usq = (v0 * v0 + v1 * v1) + v2 * v2;
    const T b = usq / k.two_cs2;
    T* f = const_cast<T*>(s.fin);
    T* g = const_cast<T*>(s.gin);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      T eu = T(0);
      bool any = false;
      if (ex(q) != 0) { eu = ex(q) > 0 ? v0 : -v0; any = true; }
      if (ey(q) != 0) { const T t = ey(q) > 0 ? v1 : -v1; eu = any ? eu + t : t; any = true; }
      if (ez(q) != 0) { const T t = ez(q) > 0 ? v2 : -v2; eu = any ? eu + t : t; any = true; }
      const T ec = eu / k.cs2;
      f[(size_t)q * N + n] = phi * (k.w[q] * (((T(1) + ec) + ec * ec / T(2)) - b));
      g[(size_t)q * N + n] = T(0) * k.w[q] + k.w[q] * ((ec + ec * ec / T(2)) - b);
    }
    s.u[n] = v0;
    s.u[N + n] = v1;
    s.u[2 * N + n] = v2;
    s.phi[n] = phi;
    s.phi_prev[n] = phi;
    s.relax[n] = T(-1);
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
// Field read-out (the reference's attribute values after the last step)
// ---------------------------------------------------------------------------
enum ObserveMode { kObsInit = 0, kObsStep = 1 };

template <typename T, bool RAW_IN>
__global__ void __launch_bounds__(kBlock) k_observe(Consts<T> k, State<T> s, unsigned mask, int mode,
                                                    T* phi_o, T* rho_o, T* u_o, T* P_o, T* p_o, T* mu_o) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  const size_t N = (size_t)k.N;
  const uint8_t c = s.cls[n];
  const T phi = s.phi[n];
  const T rho = phi * k.rho_l + (T(1) - phi) * k.rho_g;
  if (mask & 1u) {
    T v = phi;
    if (mode == kObsStep) {
      v = clamp01(phi * s.cbuf[s.c_cur]);
      if (k.relax_on && (c & kTop)) {
        const T r = s.relax[n];
        if (r >= T(0)) v = r;
      }
    }
    phi_o[n] = v;
  }
  if (mask & 2u) rho_o[n] = rho;
  if (mask & 4u) {
    u_o[n] = s.u[n];
    u_o[N + n] = s.u[N + n];
    u_o[2 * N + n] = s.u[2 * N + n];
  }
  if (mask & (8u | 16u | 32u)) {
    int ix, iy, iz;
    const Nbr nb = make_nbr(n, k.nx, k.ny, k.nz, &ix, &iy, &iz);
    if (mask & (8u | 16u)) {
      T P = T(0);
      if (mode == kObsStep) {
        const T eps = (c & kPartial) ? s.eps[n] : T(0);
        T g[Q];
        fetch_pop<T, RAW_IN, false>(g, s.gin, n, N, nb, c, eps, T(1));
        P = seqsum(g);
      }
      if (mask & 8u) P_o[n] = P;
      if (mask & 16u) p_o[n] = mode == kObsStep ? P * k.cs2 : rho * k.cs2;
    }
    if (mask & 32u) {
      T gx, gy, gz, lap;
      if (mode == kObsStep) stencil<T, true>(k, s, n, nb, c, phi, gx, gy, gz, lap);
      else stencil<T, false>(k, s, n, nb, c, phi, gx, gy, gz, lap);
      mu_o[n] = chem_pot(k, c, phi, lap);
    }
  }
}

// Current populations in the reference layout.
template <typename T, bool RAW>
__global__ void __launch_bounds__(kBlock) k_populations(Consts<T> k, State<T> s, T* f_o, T* g_o) {
  const int n = blockIdx.x * kBlock + threadIdx.x;
  if (n >= k.N) return;
  const size_t N = (size_t)k.N;
  const uint8_t c = s.cls[n];
  int ix, iy, iz;
  const Nbr nb = make_nbr(n, k.nx, k.ny, k.nz, &ix, &iy, &iz);
  const T eps = (c & kPartial) ? s.eps[n] : T(0);
  T v[Q];
  if (f_o) {
    fetch_pop<T, RAW, !RAW>(v, s.fin, n, N, nb, c, eps, RAW ? T(1) : s.cbuf[s.c_cur]);
    if (!RAW && k.relax_on && (c & kTop)) {
      const T r = s.relax[n];
      if (r >= T(0)) {
        const T sc = relax_scale(r, seqsum(v));
#pragma unroll
        for (int q = 0; q < Q; ++q) v[q] = v[q] * sc;
      }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) f_o[(size_t)q * N + n] = v[q];
  }
  if (g_o) {
    fetch_pop<T, RAW, false>(v, s.gin, n, N, nb, c, eps, T(1));
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

template <typename T>
__global__ void __launch_bounds__(kBlock) k_measure(int nx, int ny, int nz, const T* __restrict__ phi,
                                                   const uint8_t* __restrict__ cls, double* partials,
                                                   unsigned* counter, double* out) {
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
  // warp reduce
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v[0] += __shfl_down_sync(0xffffffffu, v[0], o);
    v[1] = fmax(v[1], __shfl_down_sync(0xffffffffu, v[1], o));
#pragma unroll
    for (int j = 2; j < 8; j += 2) {
      v[j] = fmin(v[j], __shfl_down_sync(0xffffffffu, v[j], o));
      v[j + 1] = fmax(v[j + 1], __shfl_down_sync(0xffffffffu, v[j + 1], o));
    }
    v[8] += __shfl_down_sync(0xffffffffu, v[8], o);
    v[9] += __shfl_down_sync(0xffffffffu, v[9], o);
    v[10] = fmax(v[10], __shfl_down_sync(0xffffffffu, v[10], o));
  }
  __shared__ double sw[kBlock / 32][kMeasVals];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
    for (int j = 0; j < kMeasVals; ++j) sw[wid][j] = v[j];
  __syncthreads();
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    for (int w = 1; w < kBlock / 32; ++w) {
      v[0] += sw[w][0];
      v[1] = fmax(v[1], sw[w][1]);
      for (int j = 2; j < 8; j += 2) { v[j] = fmin(v[j], sw[w][j]); v[j + 1] = fmax(v[j + 1], sw[w][j + 1]); }
      v[8] += sw[w][8];
      v[9] += sw[w][9];
      v[10] = fmax(v[10], sw[w][10]);
    }
    for (int j = 0; j < kMeasVals; ++j) partials[(size_t)blockIdx.x * kMeasVals + j] = v[j];
    __threadfence();
    s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    volatile double* pp = partials;
    double r[kMeasVals];
    for (int j = 0; j < kMeasVals; ++j) r[j] = pp[j];
    for (unsigned b = 1; b < gridDim.x; ++b) {
      const volatile double* q = pp + (size_t)b * kMeasVals;
      r[0] += q[0];
      r[1] = fmax(r[1], q[1]);
      for (int j = 2; j < 8; j += 2) { r[j] = fmin(r[j], q[j]); r[j + 1] = fmax(r[j + 1], q[j + 1]); }
      r[8] += q[8];
      r[9] += q[9];
      r[10] = fmax(r[10], q[10]);
    }
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
    *counter = 0u;
  }
}

// ---------------------------------------------------------------------------
// Host-side launchers (called from lbm_capi.cu)
// ---------------------------------------------------------------------------
template <typename T>
cudaError_t launch_step(const Consts<T>& k, const State<T>& s, bool raw, bool first, cudaStream_t st,
                        cudaEvent_t mid) {
  const int grid = (k.N + kBlock - 1) / kBlock;
  if (raw) k_phi<T, true><<<grid, kBlock, 0, st>>>(k, s);
  else k_phi<T, false><<<grid, kBlock, 0, st>>>(k, s);
  if (mid) cudaEventRecord(mid, st);
  if (raw && first) k_collide<T, true, true><<<grid, kBlock, 0, st>>>(k, s);
  else if (raw) k_collide<T, true, false><<<grid, kBlock, 0, st>>>(k, s);
  else if (first) k_collide<T, false, true><<<grid, kBlock, 0, st>>>(k, s);
  else k_collide<T, false, false><<<grid, kBlock, 0, st>>>(k, s);
  return cudaGetLastError();
}

template <typename T, typename S>
cudaError_t launch_init(const Consts<T>& k, const State<T>& s, const S* phi0, const S* u0, cudaStream_t st) {
  const int grid = (k.N + kBlock - 1) / kBlock;
  k_init<T, S><<<grid, kBlock, 0, st>>>(k, s, phi0, u0);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_observe(const Consts<T>& k, const State<T>& s, bool raw_in, unsigned mask, int mode,
                           T* phi, T* rho, T* u, T* P, T* p, T* mu, cudaStream_t st) {
  const int grid = (k.N + kBlock - 1) / kBlock;
  if (raw_in) k_observe<T, true><<<grid, kBlock, 0, st>>>(k, s, mask, mode, phi, rho, u, P, p, mu);
  else k_observe<T, false><<<grid, kBlock, 0, st>>>(k, s, mask, mode, phi, rho, u, P, p, mu);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_populations(const Consts<T>& k, const State<T>& s, bool raw, T* f, T* g, cudaStream_t st) {
  const int grid = (k.N + kBlock - 1) / kBlock;
  if (raw) k_populations<T, true><<<grid, kBlock, 0, st>>>(k, s, f, g);
  else k_populations<T, false><<<grid, kBlock, 0, st>>>(k, s, f, g);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_measure(int nx, int ny, int nz, const T* phi, const uint8_t* cls, double* partials,
                           int max_blocks, unsigned* counter, double* out, cudaStream_t st) {
  const int N = nx * ny * nz;
  int grid = (N + kBlock - 1) / kBlock;
  if (grid > max_blocks) grid = max_blocks;
  k_measure<T><<<grid, kBlock, 0, st>>>(nx, ny, nz, phi, cls, partials, counter, out);
  return cudaGetLastError();
}

template cudaError_t launch_step<float>(const Consts<float>&, const State<float>&, bool, bool, cudaStream_t, cudaEvent_t);
template cudaError_t launch_step<double>(const Consts<double>&, const State<double>&, bool, bool, cudaStream_t, cudaEvent_t);
template cudaError_t launch_init<float, float>(const Consts<float>&, const State<float>&, const float*, const float*, cudaStream_t);
template cudaError_t launch_init<float, double>(const Consts<float>&, const State<float>&, const double*, const double*, cudaStream_t);
template cudaError_t launch_init<double, float>(const Consts<double>&, const State<double>&, const float*, const float*, cudaStream_t);
template cudaError_t launch_init<double, double>(const Consts<double>&, const State<double>&, const double*, const double*, cudaStream_t);
template cudaError_t launch_observe<float>(const Consts<float>&, const State<float>&, bool, unsigned, int, float*, float*, float*, float*, float*, float*, cudaStream_t);
template cudaError_t launch_observe<double>(const Consts<double>&, const State<double>&, bool, unsigned, int, double*, double*, double*, double*, double*, double*, cudaStream_t);
template cudaError_t launch_populations<float>(const Consts<float>&, const State<float>&, bool, float*, float*, cudaStream_t);
template cudaError_t launch_populations<double>(const Consts<double>&, const State<double>&, bool, double*, double*, cudaStream_t);
template cudaError_t launch_measure<float>(int, int, int, const float*, const uint8_t*, double*, int, unsigned*, double*, cudaStream_t);
template cudaError_t launch_measure<double>(int, int, int, const double*, const uint8_t*, double*, int, unsigned*, double*, cudaStream_t);

}  // namespace lbm
