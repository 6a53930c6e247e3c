// Step kernels of the paired layout (Consts::nh > 0): one thread per pair of
// nodes x and x + nx/2 (same y, z).  Both nodes of a pair sit in one 8-byte
// (float), 16-byte (double) or 4-byte (half) word of every population, u and
// phi array, so one load or store moves both, pulled neighbours of both
// nodes sit in one word as well (the pair of x - e_q is the pair of the two
// nodes' neighbours), and float arithmetic runs as packed f32x2 operations
// (FADD2 / FMUL2 / FFMA2) on the pair.  Only a pull across the x-half
// boundary (x' = 0 or x' = nx/2 - 1) swaps the two halves of a word: node x
// = 0 pulls from x = nx - 1, the upper node of pair x' = nx/2 - 1, and node
// x = nx/2 from x = nx/2 - 1, its lower node.
//
// The arithmetic per node is the single-node kernels' (lbm_kernels.cu:
// fetch_pop, update_node): pull streaming with bounce-back and partial-node
// blending rebuilt on read, the mass-correction factor, boundary-phi
// relaxation, the isotropic stencils with the ghost wetting values, chemical
// potential, geometric correction, moments, forces, velocity, Allen-Cahn
// source and both BGK collisions (pytorch-lbm lbm/fe_ac_solver.py:380-639).
// Node-class dependent work (solid, partial, boundary, top-surface nodes) is
// done per half of the pair on the lanes that need it; everything else on the
// pair at once.  Included by lbm_kernels.cu.
#pragma once

namespace lbm {

template <typename T>
struct VecOf;
template <>
struct VecOf<float> {
  using type = float2;
};
template <>
struct VecOf<double> {
  using type = double2;
};
template <typename T>
using V2 = typename VecOf<T>::type;

// Storage word of a pair: two populations of type S.
template <typename S>
struct PairWord;
template <>
struct PairWord<float> {
  using type = float2;
};
template <>
struct PairWord<double> {
  using type = double2;
};
template <>
struct PairWord<__half> {
  using type = __half2;
};

__device__ __forceinline__ float2 vs(float a) { return make_float2(a, a); }
__device__ __forceinline__ double2 vs(double a) { return make_double2(a, a); }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 vmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b as one packed fused operation, exact like a subtraction: (-1) b + a
__device__ __forceinline__ float2 vsub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ double2 vadd(double2 a, double2 b) { return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y)); }
__device__ __forceinline__ double2 vmul(double2 a, double2 b) { return make_double2(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)); }
__device__ __forceinline__ double2 vfma(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}
__device__ __forceinline__ double2 vsub(double2 a, double2 b) { return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y)); }
template <typename V>
__device__ __forceinline__ V vneg(V a) {
  a.x = -a.x;
  a.y = -a.y;
  return a;
}
template <typename V>
__device__ __forceinline__ V vswap(V a) {
  const auto t = a.x;
  a.x = a.y;
  a.y = t;
  return a;
}
template <typename T>
__device__ __forceinline__ T& lane(V2<T>& v, int l) { return l ? v.y : v.x; }
template <typename T>
__device__ __forceinline__ T lane(const V2<T>& v, int l) { return l ? v.y : v.x; }

// Loads and stores of one pair word with an L2 policy.
__device__ __forceinline__ float2 ld2_pol(const float* p, unsigned long long pol) {
  float2 v;
  asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ double2 ld2_pol(const double* p, unsigned long long pol) {
  double2 v;
  asm("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ __half2 ld2_pol(const __half* p, unsigned long long pol) {
  unsigned r;
  asm("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
  __half2 h;
  memcpy(&h, &r, 4);
  return h;
}
__device__ __forceinline__ void st2_pol(float* p, float2 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol));
}
__device__ __forceinline__ void st2_pol(double* p, double2 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(p), "d"(v.x), "d"(v.y), "l"(pol));
}
__device__ __forceinline__ void st2_pol(__half* p, __half2 v, unsigned long long pol) {
  unsigned r;
  memcpy(&r, &v, 4);
  asm volatile("st.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(p), "r"(r), "l"(pol));
}

// Population words in the compute type: PopIO of both halves at once.
template <typename T, typename S>
struct PairIO {
  using V = V2<T>;
  using W = typename PairWord<S>::type;
  __device__ __forceinline__ static V ld_f(W raw, int, V) { return raw; }
  __device__ __forceinline__ static W st_f(V v, int, V) { return v; }
  __device__ __forceinline__ static V ld_g(W raw, int) { return raw; }
  __device__ __forceinline__ static W st_g(V v, int) { return v; }
};
template <>
struct PairIO<float, __half> {
  using V = float2;
  using W = __half2;
  __device__ __forceinline__ static V ld_f(W raw, int q, V ref) {
    return vmul(vs(Lat<float>::w(q)), vadd(__half22float2(raw), ref));
  }
  __device__ __forceinline__ static W st_f(V v, int q, V ref) {
    return __float22half2_rn(vfma(v, vs(Lat<float>::inv_w(q)), vneg(ref)));
  }
  __device__ __forceinline__ static V ld_g(W raw, int q) { return vmul(vs(Lat<float>::w(q)), __half22float2(raw)); }
  __device__ __forceinline__ static W st_g(V v, int q) { return __float22half2_rn(vmul(v, vs(Lat<float>::inv_w(q)))); }
};

// Periodic neighbours of pair p in pair units: the offset of a step
// (dx, dy, dz) and whether it crosses the x-half boundary (swapped halves).
struct PNbr {
  int ox[3], oy[3], oz[3];
  bool sw_lo, sw_hi;  // x' == 0 (a step -1 in x swaps), x' == nx/2 - 1 (a step +1 swaps)
  __device__ __forceinline__ int at(int p, int dx, int dy, int dz) const {
    return p + ox[dx + 1] + oy[dy + 1] + oz[dz + 1];
  }
  __device__ __forceinline__ bool swaps(int dx) const { return dx < 0 ? sw_lo : (dx > 0 ? sw_hi : false); }
};

template <typename T>
__device__ __forceinline__ PNbr make_pnbr(const Consts<T>& k, int p) {
  int ix, iy, iz;
  // p = (x' ny + y) nz + z with x' < nx / 2
  const int t = (int)k.dz.div((unsigned)p);
  iz = p - t * k.nz;
  ix = (int)k.dy.div((unsigned)t);
  iy = t - ix * k.ny;
  const int sx = k.ny * k.nz, sy = k.nz, H = k.hx;
  PNbr b;
  b.ox[0] = ix == 0 ? (H - 1) * sx : -sx;
  b.ox[1] = 0;
  b.ox[2] = ix == H - 1 ? -(H - 1) * sx : sx;
  b.oy[0] = iy == 0 ? (k.ny - 1) * sy : -sy;
  b.oy[1] = 0;
  b.oy[2] = iy == k.ny - 1 ? -(k.ny - 1) * sy : sy;
  b.oz[0] = iz == 0 ? k.nz - 1 : -1;
  b.oz[1] = 0;
  b.oz[2] = iz == k.nz - 1 ? -(k.nz - 1) : 1;
  b.sw_lo = ix == 0;
  b.sw_hi = ix == H - 1;
  return b;
}

// Node index of the neighbour (dx, dy, dz) of half l of pair p.
__device__ __forceinline__ int pair_nbr_node(const PNbr& nb, int p, int l, int nh, int dx, int dy, int dz) {
  const int lp = l ^ (nb.swaps(dx) ? 1 : 0);
  return nb.at(p, dx, dy, dz) + lp * nh;
}

// The word of array A (pair elements) at the neighbour (dx, dy, dz) of pair
// p, halves in the order of the two nodes of p.
template <typename S>
__device__ __forceinline__ typename PairWord<S>::type ld_nbr(const S* __restrict__ A, const PNbr& nb, int p, int dx,
                                                             int dy, int dz, unsigned long long pol) {
  auto w = ld2_pol(A + 2u * (unsigned)nb.at(p, dx, dy, dz), pol);
  return nb.swaps(dx) ? vswap(w) : w;
}

template <typename T>
__device__ __forceinline__ V2<T> clamp01v(V2<T> v) {
  v.x = clamp01(v.x);
  v.y = clamp01(v.y);
  return v;
}

template <typename V>
__device__ __forceinline__ V seqsumv(const V (&v)[Q]) {
  V s = v[0];
#pragma unroll
  for (int q = 1; q < Q; ++q) s = vadd(s, v[q]);
  return s;
}

// Populations of pair p as the reference holds them at the start of the step
// (fetch_pop of both nodes): pulled from x - e_q, the node's own opposite
// slots at solid nodes, blended at partial nodes, times corr (WITH_C).
template <typename T, typename S, bool WITH_C, bool IS_F>
__device__ __forceinline__ void fetch_pop_pair(V2<T> (&v)[Q], const Consts<T>& k, const S* __restrict__ F,
                                               const T* __restrict__ phi_in, int p, const PNbr& nb, uint8_t c0,
                                               uint8_t c1, T eps0, T eps1, T corr, unsigned long long pol) {
  using IO = PairIO<T, S>;
  constexpr bool DEV = PopIO<T, S>::kDev && IS_F;
  using V = V2<T>;
  const unsigned Nu = (unsigned)k.Np, e = 2u * (unsigned)p;
  const V ref_self = DEV ? ld2_pol(phi_in + e, pol) : vs(T(0));
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const auto w = ld_nbr(F + q * Nu, nb, p, -ex(q), -ey(q), -ez(q), pol);
    v[q] = IS_F ? IO::ld_f(w, q, ref_self) : IO::ld_g(w, q);
  }
  if ((c0 | c1) & (kSolid | kPartial)) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      // the node's own slot opp q (bounce-back, penalisation); in the half
      // form its deviation reference is the phi of x - e_q, the slot's writer's pull target
      const V ref = DEV ? ld_nbr(phi_in, nb, p, -ex(q), -ey(q), -ez(q), pol) : vs(T(0));
      const V o = IS_F ? IO::ld_f(ld2_pol(F + opp(q) * Nu + e, pol), opp(q), ref)
                       : IO::ld_g(ld2_pol(F + opp(q) * Nu + e, pol), opp(q));
#pragma unroll
      for (int l = 0; l < 2; ++l) {
        const uint8_t c = l ? c1 : c0;
        const T eps = l ? eps1 : eps0;
        T& x = lane<T>(v[q], l);
        if (c & kSolid) x = lane<T>(o, l);
        else if (c & kPartial) x = (T(1) - eps) * x + eps * lane<T>(o, l);
      }
    }
  }
  if (WITH_C) {
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = vmul(v[q], vs(corr));
  }
}

// f of pair p at the start of the step: fetch_pop_pair with the mass
// correction, then the boundary-phi relaxation of top-surface nodes.
template <typename T, typename S>
__device__ __forceinline__ void fetch_f_pair(V2<T> (&v)[Q], const Consts<T>& k, const State<T, S>& s, int p,
                                             const PNbr& nb, uint8_t c0, uint8_t c1, T eps0, T eps1,
                                             unsigned long long pol) {
  const T corr = s.cbuf[s.c_prev];
  fetch_pop_pair<T, S, true, true>(v, k, s.fin, s.phi_in, p, nb, c0, c1, eps0, eps1, corr, pol);
  if (k.relax_on && ((c0 | c1) & kTop)) {
    const V2<T> sum = seqsumv(v);
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      if (!((l ? c1 : c0) & kTop)) continue;
      const int n = p + l * k.nh;
      const T r = relax_target<T, true>(k, s.phi_in, s.nsw, s.cubic, n, ldg(s.phi_in + 2u * (unsigned)p + l), corr);
      if (r >= T(0)) {
        const T sc = relax_scale(r, lane<T>(sum, l));
#pragma unroll
        for (int q = 0; q < Q; ++q) lane<T>(v[q], l) = lane<T>(v[q], l) * sc;
      }
    }
  }
}

// phi of pair p (written to phi_out) added to the block's sum.  Every pair
// with a fluid half loads its 19 pulled words in one branch-free block, so
// that all of them are in flight at once, and sums them as fetch_f does
// (sequential order); a solid half's phi is 0 whatever it pulled.  A
// top-surface half under boundary-phi relaxation is rescaled from the same
// words (relax_scale of their sum); the rare partial halves (penalisation
// blend with the node's own opposite slots) are recomputed alone by the
// single-node fetch_f.
template <typename T, typename S>
__device__ __forceinline__ void phi_pair(const Consts<T>& k, const State<T, S>& s, int p, uint8_t c0, uint8_t c1,
                                         const Pol& pol, TileSum<T>& part) {
  using IO = PairIO<T, S>;
  using V = V2<T>;
  constexpr bool DEV = PopIO<T, S>::kDev;
  V phi = vs(T(0));
  const uint8_t cor = c0 | c1;
  if (!(c0 & c1 & kSolid)) {
    const PNbr nb = make_pnbr(k, p);
    // f is read again by the update kernel only when omega_f != 1
    const unsigned long long lp = k.omega_f == T(1) ? pol.once : pol.keep;
    const unsigned Nu = (unsigned)k.Np, e = 2u * (unsigned)p;
    const T corr = s.cbuf[s.c_prev];
    const V ref_self = DEV ? ld2_pol(s.phi_in + e, lp) : vs(T(0));
    typename PairWord<S>::type w[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) w[q] = ld_nbr(s.fin + q * Nu, nb, p, -ex(q), -ey(q), -ez(q), lp);
    auto val = [&](int q) { return vmul(IO::ld_f(w[q], q, ref_self), vs(corr)); };
    V sum = val(0);
#pragma unroll
    for (int q = 1; q < Q; ++q) sum = vadd(sum, val(q));
    phi = clamp01v<T>(sum);
    if (k.relax_on && (cor & kTop)) {
#pragma unroll 1
      for (int l = 0; l < 2; ++l) {
        const uint8_t c = l ? c1 : c0;
        if ((c & (kTop | kSolid | kPartial)) != kTop) continue;
        const int n = p + l * k.nh;
        const T r = relax_target<T, true>(k, s.phi_in, s.nsw, s.cubic, n, ldg(s.phi_in + e + l), corr);
        if (r >= T(0)) {
          const T sc = relax_scale(r, lane<T>(sum, l));
          // fetch_f scales each value, then sums: two roundings per term
          T acc = mul_rn(lane<T>(val(0), l), sc);
#pragma unroll
          for (int q = 1; q < Q; ++q) acc = add_rn(acc, mul_rn(lane<T>(val(q), l), sc));
          lane<T>(phi, l) = clamp01(acc);
        }
      }
    }
    if (cor & kPartial) {
      // partial halves through the single-node fetch_f (which reads the paired layout)
#pragma unroll 1
      for (int l = 0; l < 2; ++l) {
        const uint8_t c = l ? c1 : c0;
        if ((c & kSolid) || !(c & kPartial)) continue;
        const int n = p + l * k.nh;
        int ix, iy, iz;
        decode(k.dz, k.dy, n, k.nz, k.ny, ix, iy, iz);
        const Nbr nbs = make_nbr_xyz(ix, iy, iz, k.nx, k.ny, k.nz);
        T v[Q];
        fetch_f<T, S, false, true, true>(v, k, s, n, (size_t)k.N, nbs, c, s.eps[n], lp);
        lane<T>(phi, l) = clamp01(seqsum(v));
      }
    }
    if (c0 & kSolid) phi.x = T(0);
    if (c1 & kSolid) phi.y = T(0);
  }
  st2_pol(s.phi_out + 2u * (unsigned)p, phi, pol.keep);  // read back (stencil) by the update kernel
  part.add(phi.x);
  part.add(phi.y);
}

// Resident blocks per SM of the paired kernels (float compute only: float64
// grids keep the linear layout): the phi kernel at 256 threads (80
// registers: the 19 pulled words stay live for the relaxation), the update
// kernel at kPairUpdBlock (128 registers).
template <typename T, typename S>
struct PairOccupancy {
  static constexpr int phi_blocks = 3;
  static constexpr int upd_blocks = 4;
};

template <typename T, typename S>
__global__ void __launch_bounds__(kBlock, PairOccupancy<T, S>::phi_blocks) k_phi_pair(
    const CaseDesc<T, S>* __restrict__ cases, const unsigned short* __restrict__ blk2case) {
  __shared__ CaseDesc<T, S> d;
  load_desc(d, cases + (blk2case ? blk2case[blockIdx.x] : 0));
  pdl_trigger();
  pdl_wait();  // f of the previous update kernel
  const Pol pol = Pol::make();
  const int b = blockIdx.x - d.phi_blk0, nb = d.phi_nblk;
  TileSum<T> part;
  const int NH = d.k.nh, stride = nb * kBlock;
  int p = b * kBlock + threadIdx.x;
  // class bytes of the thread's next pair loaded one pair ahead
  uint8_t c0 = p < NH ? d.s.cls[p] : 0, c1 = p < NH ? d.s.cls[p + NH] : 0;
  for (; p < NH; p += stride) {
    const bool more = p + stride < NH;
    const uint8_t n0 = more ? d.s.cls[p + stride] : 0, n1 = more ? d.s.cls[p + stride + NH] : 0;
    phi_pair<T, S>(d.k, d.s, p, c0, c1, pol, part);
    c0 = n0;
    c1 = n1;
  }
  phi_finish(d.s, part, b, nb);
}

// The update of pair p (update_node of both nodes).
template <typename T, typename S, bool OMEGA1, bool GMU>
__device__ __forceinline__ void update_pair(const Consts<T>& k, const State<T, S>& s, int p, const Pol& pol) {
  using IO = PairIO<T, S>;
  using V = V2<T>;
  constexpr bool IMM = PopIO<T, S>::kDev;
  const LatK<T, IMM> L{k};
  const size_t N = (size_t)k.N;
  const int nh = k.nh;
  const unsigned Nu = (unsigned)k.Np, e = 2u * (unsigned)p;
  const PNbr nb = make_pnbr(k, p);
  const uint8_t c0 = s.cls[p], c1 = s.cls[p + nh];
  const uint8_t cor = c0 | c1;
  const T* __restrict__ pc = s.phi_out;  // phi of this step (phi kernel)
  const V phi = ld2_pol(pc + e, pol.keep);

  // 2. the stencil: gradient and laplacian with the ghost-node wetting values
  V ps[Q];
#pragma unroll
  for (int q = 1; q < Q; ++q) ps[q] = ld_nbr(pc, nb, p, ex(q), ey(q), ez(q), pol.keep);
  if (k.wetting && (cor & kBoundary)) {
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      if (!((l ? c1 : c0) & kBoundary)) continue;
      const int n = p + l * nh;
      const float n0 = s.wn[n], n1 = s.wn[N + n], n2 = s.wn[2 * N + n];
      const T ph = lane<T>(phi, l);
#pragma unroll
      for (int q = 1; q < Q; ++q) {
        if (s.cls[pair_nbr_node(nb, p, l, nh, ex(q), ey(q), ez(q))] & kSolid) {
          float nde = 0.0f;
          nde = __fadd_rn(nde, __fmul_rn(n0, (float)ex(q)));
          nde = __fadd_rn(nde, __fmul_rn(n1, (float)ey(q)));
          nde = __fadd_rn(nde, __fmul_rn(n2, (float)ez(q)));
          lane<T>(ps[q], l) = k.linear ? ph - (T)__fmul_rn(nde, k.h_over_kappa_f)
                                       : ph + (T)__fmul_rn(nde, k.pcok_f) * ph * (T(1) - ph);
        }
      }
    }
  }
  V gx, gy, gz, lap = vs(T(0));
  {
    // pair differences t_q = (w_q / cs2)(phi(x + e_q) - phi(x - e_q)), mirror
    // partners summed first (exact zeros on symmetry lines)
    auto t = [&](int q) { return vmul(vs(L.wc(q)), vsub(ps[q], ps[opp(q)])); };
    const V t1 = t(1), t3 = t(3), t5 = t(5), t7 = t(7), t8 = t(8), t11 = t(11), t12 = t(12), t15 = t(15),
            t16 = t(16);
    gx = vadd(vadd(t1, vsub(t7, t8)), vsub(t11, t12));
    gy = vadd(vadd(t3, vadd(t7, t8)), vsub(t15, t16));
    gz = vadd(vadd(t5, vadd(t11, t12)), vadd(t15, t16));
#pragma unroll
    for (int q = 1; q < Q; ++q) lap = vfma(vs(L.w2c(q)), vsub(ps[q], phi), lap);
  }

  // then g (pulled), u and phi of the last step (after the stencil: fewer
  // values live at once)
  const T eps0 = (c0 & kPartial) ? s.eps[p] : T(0);
  const T eps1 = (c1 & kPartial) ? s.eps[p + nh] : T(0);
  V g[Q];
  fetch_pop_pair<T, S, false, false>(g, k, s.gin, s.phi_in, p, nb, c0, c1, eps0, eps1, T(1), pol.once);
  const V uo0 = ld2_pol(s.u + e, pol.once);
  const V uo1 = ld2_pol(s.u + (Nu + e), pol.once);
  const V uo2 = ld2_pol(s.u + (2 * Nu + e), pol.once);
  const V pp = ld2_pol(s.phi_in + e, pol.once);


  const V one = vs(T(1));
  const V omphi = vsub(one, phi);
  const V rho = vfma(phi, vs(k.rho_l), vmul(omphi, vs(k.rho_g)));
  V rho_eff = rho;
  rho_eff.x = rho.x < k.rho_floor ? k.rho_floor : rho.x;
  rho_eff.y = rho.y < k.rho_floor ? k.rho_floor : rho.y;
  V mu;
  if constexpr (GMU) {
    mu.x = ld_pol(s.mu + p, pol.keep);
    mu.y = ld_pol(s.mu + (p + nh), pol.keep);
  } else {
    // chemical potential (chem_pot)
    const V cub = vmul(vmul(vmul(vs(k.beta4), phi), vsub(phi, one)), vsub(phi, vs(T(0.5))));
    mu = vfma(vs(-k.kappa), lap, cub);
    if (k.wetting && (cor & kBoundary)) {
#pragma unroll
      for (int l = 0; l < 2; ++l) {
        if (!((l ? c1 : c0) & kBoundary)) continue;
        const T ph = lane<T>(phi, l);
        T& m = lane<T>(mu, l);
        if (k.linear) m = m + k.mu_wall_add;
        else m = m + k.phi_c * ph * (T(1) - ph);
      }
    }
  }

  // geometric contact-angle gradient correction at boundary nodes
  if (k.geometric && (cor & kBoundary)) {
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const uint8_t c = l ? c1 : c0;
      if (!(c & kBoundary)) continue;
      const int n = p + l * nh;
      T ax = lane<T>(gx, l), ay = lane<T>(gy, l), az = lane<T>(gz, l);
      const T n0 = (T)s.wn[n], n1 = (T)s.wn[N + n], n2 = (T)s.wn[2 * N + n];
      const T gn = add_rn(add_rn(mul_rn(n0, ax), mul_rn(n1, ay)), mul_rn(n2, az));
      const T tx = ax - mul_rn(gn, n0), ty = ay - mul_rn(gn, n1), tz = az - mul_rn(gn, n2);
      T tm = sqrt_mag<IMM>(add_rn(add_rn(mul_rn(tx, tx), mul_rn(ty, ty)), mul_rn(tz, tz)));
      tm = tm < T(1e-10) ? T(1e-10) : tm;
      T gd = mul_rn(-tm, k.cos_t) / k.sin_t;
      T a = k.amp;
      bool amp_on = k.amp_active;
      if (s.amp) {
        a = s.amp[n];
        amp_on = a > T(1);
      }
      if (amp_on) gd = add_rn(gn, mul_rn(gd - gn, a));
      const T cx = add_rn(tx, mul_rn(gd, n0)), cy = add_rn(ty, mul_rn(gd, n1)), cz = add_rn(tz, mul_rn(gd, n2));
      const T gm = sqrt_mag<IMM>(add_rn(add_rn(mul_rn(ax, ax), mul_rn(ay, ay)), mul_rn(az, az)));
      if (gm > T(1e-6)) {
        const T bl = k.ww[c >> kWwShift];
        lane<T>(gx, l) = add_rn(ax, mul_rn(bl, cx - ax));
        lane<T>(gy, l) = add_rn(ay, mul_rn(bl, cy - ay));
        lane<T>(gz, l) = add_rn(az, mul_rn(bl, cz - az));
      }
    }
  }

  // 3.-4. moments from opposite-pair sums and differences; stress with the old u
  V sp[9], dp[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    sp[i] = vadd(g[pair_first(i)], g[opp(pair_first(i))]);
    dp[i] = vsub(g[pair_first(i)], g[opp(pair_first(i))]);
  }
  V P = g[0];
#pragma unroll
  for (int i = 0; i < 9; ++i) P = vadd(P, sp[i]);
  V sxx, syy, szz, sxy, sxz, syz;
  {
    const V pc2 = vmul(P, vs(L.cs2()));
    sxx = vfma(vneg(uo0), uo0, vsub(vadd(vadd(sp[0], vadd(sp[3], sp[4])), vadd(sp[5], sp[6])), pc2));
    syy = vfma(vneg(uo1), uo1, vsub(vadd(vadd(sp[1], vadd(sp[3], sp[4])), vadd(sp[7], sp[8])), pc2));
    szz = vfma(vneg(uo2), uo2, vsub(vadd(vadd(sp[2], vadd(sp[5], sp[6])), vadd(sp[7], sp[8])), pc2));
    sxy = vfma(vneg(uo0), uo1, vsub(sp[3], sp[4]));
    sxz = vfma(vneg(uo0), uo2, vsub(sp[5], sp[6]));
    syz = vfma(vneg(uo1), uo2, vsub(sp[7], sp[8]));
  }

  // 5. forces
  V F0 = vmul(mu, gx), F1 = vmul(mu, gy), F2 = vmul(mu, gz);
  if (k.stab_mode <= 1) {
    const V fp = vmul(vmul(vneg(P), vs(k.drho)), vs(L.cs2()));
    F0 = vfma(fp, gx, F0);
    F1 = vfma(fp, gy, F1);
    F2 = vfma(fp, gz, F2);
  }
  if (k.stab_mode == 0) {
    const V vd = vs(k.visc);
    F0 = vfma(vmul(vd, vfma(sxz, gz, vfma(sxy, gy, vmul(sxx, gx)))), vs(k.drho), F0);
    F1 = vfma(vmul(vd, vfma(syz, gz, vfma(syy, gy, vmul(sxy, gx)))), vs(k.drho), F1);
    F2 = vfma(vmul(vd, vfma(szz, gz, vfma(syz, gy, vmul(sxz, gx)))), vs(k.drho), F2);
  }
  if (k.has_gforce) {
    F0 = vfma(vs(k.gforce[0]), rho, F0);
    F1 = vfma(vs(k.gforce[1]), rho, F1);
    F2 = vfma(vs(k.gforce[2]), rho, F2);
  }

  // 6. velocity
  V u0, u1, u2;
  {
    V hr;
    hr.x = T(0.5) * rcp(rho_eff.x);
    hr.y = T(0.5) * rcp(rho_eff.y);
    u0 = vfma(F0, hr, vadd(vadd(dp[0], vsub(dp[3], dp[4])), vsub(dp[5], dp[6])));
    u1 = vfma(F1, hr, vadd(vadd(dp[1], vadd(dp[3], dp[4])), vsub(dp[7], dp[8])));
    u2 = vfma(F2, hr, vadd(vadd(dp[2], vadd(dp[5], dp[6])), vadd(dp[7], dp[8])));
    if (c0 & kSolid) u0.x = u1.x = u2.x = T(0);
    if (c1 & kSolid) u0.y = u1.y = u2.y = T(0);
  }
  const V b = vmul(vfma(u2, u2, vfma(u1, u1, vmul(u0, u0))), vs(L.inv_two_cs2()));

  // 7. Allen-Cahn source
  V S0, S1, S2;
  {
    const V d0 = vfma(phi, u0, vneg(vmul(pp, uo0)));
    const V d1 = vfma(phi, u1, vneg(vmul(pp, uo1)));
    const V d2 = vfma(phi, u2, vneg(vmul(pp, uo2)));
    const V gg = vfma(gz, gz, vfma(gy, gy, vmul(gx, gx)));
    V cl;
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      T gm = sqrt_mag<IMM>(lane<T>(gg, l));
      gm = gm < T(1e-10) ? T(1e-10) : gm;
      const T ph = lane<T>(phi, l);
      const T lam = ((T(4) * ph) * (T(1) - ph)) * k.inv_W;
      T c = L.cs2() * lam * k.ac_scale * rcp(gm);
      if (k.wetting) c = c * (T(1) - k.sharpen_reduce * k.ww[(l ? c1 : c0) >> kWwShift]);
      lane<T>(cl, l) = c;
    }
    if constexpr (GMU) {
      V mx, my, mz;
      mx.x = ld_pol(s.gmu + p, pol.once);
      mx.y = ld_pol(s.gmu + (p + nh), pol.once);
      my.x = ld_pol(s.gmu + (Nu + p), pol.once);
      my.y = ld_pol(s.gmu + (Nu + p + nh), pol.once);
      mz.x = ld_pol(s.gmu + (2 * Nu + p), pol.once);
      mz.y = ld_pol(s.gmu + (2 * Nu + p + nh), pol.once);
      if (k.gmu_mode == kGmuCH) {
        const V mob = vs(k.mob), guo = vs(k.guo);
        S0 = vfma(vmul(mob, vsub(mx, gx)), guo, d0);
        S1 = vfma(vmul(mob, vsub(my, gy)), guo, d1);
        S2 = vfma(vmul(mob, vsub(mz, gz)), guo, d2);
      } else {
        const V a = vs(k.mu_drive_a);
        S0 = vfma(a, mx, vfma(cl, gx, d0));
        S1 = vfma(a, my, vfma(cl, gy, d1));
        S2 = vfma(a, mz, vfma(cl, gz, d2));
      }
    } else {
      S0 = vfma(cl, gx, d0);
      S1 = vfma(cl, gy, d1);
      S2 = vfma(cl, gz, d2);
    }
  }

  // 8. both BGK collisions, one opposite pair (q, opp q) at a time (update_node)
  V om;
  if (k.tau_const) {
    om = vs(k.omega_g);
  } else {
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const T ph = lane<T>(phi, l);
      const T eta = ph * k.rho_l * k.tl_m + (T(1) - ph) * k.rho_g * k.tg_m;
      const T rden = ph * k.rho_l + (T(1) - ph) * k.rho_g;
      lane<T>(om, l) = rcp(T(0.5) + eta / rden);
    }
  }
  const V omo = vsub(one, om);
  V nsd;
#pragma unroll
  for (int l = 0; l < 2; ++l)
    lane<T>(nsd, l) = (T(1) - lane<T>(om, l) * T(0.5)) * rcp(lane<T>(rho_eff, l) * L.cs2());
  const V Pb = vsub(P, b);
  const V omb = vsub(one, b);
  const V pf = OMEGA1 ? phi : vmul(vs(k.omega_f), phi);
  const V ics = vs(L.inv_cs2());
  const V u3x = vmul(u0, ics), u3y = vmul(u1, ics), u3z = vmul(u2, ics);
  V f[Q];
  if (!OMEGA1) fetch_f_pair<T, S>(f, k, s, p, nb, c0, c1, eps0, eps1, pol.same);
  auto store_g = [&](int q, V v) { st2_pol(s.gout + (q * Nu + e), IO::st_g(v, q), pol.once); };
  auto store_f = [&](int q, V v) {
    // half form: deviation from the phi of the node that pulls the slot, x + e_q
    const V ref = PopIO<T, S>::kDev ? V(ld_nbr(pc, nb, p, ex(q), ey(q), ez(q), pol.keep)) : vs(T(0));
    st2_pol(s.fout + (q * Nu + e), IO::st_f(v, q, ref), pol.once);
  };
  const V omf = vs(T(1) - k.omega_f);
  {
    const V ow = vmul(om, vs(L.w(0)));
    store_g(0, vfma(omo, g[0], vmul(ow, Pb)));
    const V pw = vmul(pf, vs(L.w(0)));
    const V f0 = vmul(pw, omb);
    store_f(0, OMEGA1 ? f0 : vfma(omf, f[0], f0));
  }
  const V wa = vs(L.w(1)), wd = vs(L.w(7));
  const V owa = vmul(om, wa), owd = vmul(om, wd);
  const V h = vs(T(0.5));
  const V howa = vmul(h, owa), howd = vmul(h, owd);
  const V obpa = vmul(owa, Pb), obpd = vmul(owd, Pb);
  const V nwa = vmul(nsd, wa), nwd = vmul(nsd, wd);
  const V pwa = vmul(pf, wa), pwd = vmul(pf, wd);
  const V hpwa = vmul(h, pwa), hpwd = vmul(h, pwd);
  const V pwba = vmul(pwa, omb), pwbd = vmul(pwd, omb);
  const V aca = vs(k.wac3[1]), acd = vs(k.wac3[7]);
  auto edotv = [](int q, V a0, V a1, V a2) {
    V r = vs(T(0));
    bool any = false;
    if (ex(q) != 0) { r = ex(q) > 0 ? a0 : vneg(a0); any = true; }
    if (ey(q) != 0) { const V t = ey(q) > 0 ? a1 : vneg(a1); r = any ? vadd(r, t) : t; any = true; }
    if (ez(q) != 0) { const V t = ez(q) > 0 ? a2 : vneg(a2); r = any ? vadd(r, t) : t; }
    return r;
  };
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const int q = pair_first(i), o = opp(q);
    const bool ax = i < 3;
    const V ec = edotv(q, u3x, u3y, u3z);
    const V ge = vfma(vmul(ax ? howa : howd, ec), ec, ax ? obpa : obpd);
    const V go = vfma(ax ? owa : owd, ec, vmul(ax ? nwa : nwd, edotv(q, F0, F1, F2)));
    store_g(q, vfma(omo, g[q], vadd(ge, go)));
    store_g(o, vfma(omo, g[o], vsub(ge, go)));
    const V fe = vfma(vmul(ax ? hpwa : hpwd, ec), ec, ax ? pwba : pwbd);
    const V fo = vfma(ax ? pwa : pwd, ec, vmul(ax ? aca : acd, edotv(q, S0, S1, S2)));
    if (OMEGA1) {
      store_f(q, vadd(fe, fo));
      store_f(o, vsub(fe, fo));
    } else {
      store_f(q, vfma(omf, f[q], vadd(fe, fo)));
      store_f(o, vfma(omf, f[o], vsub(fe, fo)));
    }
  }
  st2_pol(s.u + e, u0, pol.once);
  st2_pol(s.u + (Nu + e), u1, pol.once);
  st2_pol(s.u + (2 * Nu + e), u2, pol.once);
}

template <typename T, typename S, bool OMEGA1, bool GMU>
__global__ void __launch_bounds__(kPairUpdBlock, PairOccupancy<T, S>::upd_blocks) k_update_pair(
    const CaseDesc<T, S>* __restrict__ cases, const unsigned short* __restrict__ blk2case) {
  __shared__ CaseDesc<T, S> d;
  load_desc(d, cases + (blk2case ? blk2case[blockIdx.x] : 0));
  pdl_trigger();
  pdl_wait();  // phi of the phi kernel (mu of k_mu with GMU)
  const int p = (blockIdx.x - d.upd_blk0) * kPairUpdBlock + threadIdx.x;
  if (p < d.k.nh) update_pair<T, S, OMEGA1, GMU>(d.k, d.s, p, Pol::make());
}

}  // namespace lbm
