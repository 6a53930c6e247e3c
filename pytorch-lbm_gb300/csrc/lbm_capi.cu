// C ABI of the GB300 Allen-Cahn phase-field LBM (declarations and the
// reference interface each entry point replaces: include/lbm_gb300.h).
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_common.cuh"
#include "lbm_geometry.h"
#include "lbm_tables.h"

namespace lbm {
template <typename T, typename S>
size_t step_smem_bytes(const Tiling&);
template <typename T, typename S>
cudaError_t launch_step(const Consts<T>&, const State<T, S>&, const Tiling&, bool, bool, cudaStream_t,
                        cudaEvent_t = nullptr);
template <typename T, typename S, typename Src>
cudaError_t launch_init(const Consts<T>&, const State<T, S>&, const Src*, const Src*, cudaStream_t);
template <typename T, typename S>
cudaError_t launch_observe(const Consts<T>&, const State<T, S>&, bool, unsigned, int, T*, T*, T*, T*, T*, T*,
                           cudaStream_t);
template <typename T, typename S>
cudaError_t launch_populations(const Consts<T>&, const State<T, S>&, bool, T*, T*, cudaStream_t);
template <typename T, typename S>
cudaError_t launch_inject(const Consts<T>&, const State<T, S>&, bool, const InjectParams&, const T*, unsigned*,
                          cudaStream_t);
template <typename T>
cudaError_t launch_measure(int, int, int, const T*, const uint8_t*, double*, int, unsigned*, double*,
                           cudaStream_t, double* = nullptr);
template <typename T>
cudaError_t launch_momentum(int, const T*, const T*, int, int, double, double, double*, int, unsigned*, double*,
                            cudaStream_t);
template <typename T>
cudaError_t launch_measure_static(int, int, int, const T*, const uint8_t*, double*, cudaStream_t);
template <typename T, typename S>
cudaError_t launch_phi_batch(const void*, const unsigned short*, int, cudaStream_t);
template <typename T, typename S>
cudaError_t launch_update_batch(const void*, const unsigned short*, int, bool, cudaStream_t, bool, int);
template <typename T, typename S>
cudaError_t launch_mu(const Consts<T>&, const State<T, S>&, cudaStream_t);
template <typename T, typename S>
cudaError_t launch_phi_pair(const void*, const unsigned short*, int, cudaStream_t);
template <typename T, typename S>
cudaError_t launch_update_pair(const void*, const unsigned short*, int, bool, cudaStream_t, bool);
template <typename T, typename S>
cudaError_t launch_batch_coop(const void*, const unsigned short*, int, int, int, cudaStream_t);

// the 2-D (nz == 1, D2Q9) form (lbm_kernels2d.cu)
template <typename T, typename Src>
cudaError_t launch_init2d(const Consts<T>&, const State<T, T>&, const Src*, const Src*, cudaStream_t);
template <typename T>
cudaError_t launch_step2d(const Consts<T>&, const State<T, T>&, bool, bool, double, cudaStream_t, cudaEvent_t);
template <typename T>
cudaError_t launch_observe2d(const Consts<T>&, const State<T, T>&, bool, unsigned, int, T*, T*, T*, T*, T*, T*,
                             cudaStream_t);
template <typename T>
cudaError_t launch_populations2d(const Consts<T>&, const State<T, T>&, bool, T*, T*, cudaStream_t);
template <typename T>
cudaError_t launch_inject2d(const Consts<T>&, const State<T, T>&, bool, const InjectParams&, const T*, unsigned*,
                            cudaStream_t);

template <typename T>
cudaError_t launch_geometry(int, int, int, const uint8_t*, const void*, int, bool, bool, uint8_t*, uint8_t*, float*,
                            int*, T*, cudaStream_t);

template <typename T, typename S>
size_t case_desc_bytes();
template <typename T, typename S>
void fill_case_desc(void*, const Consts<T>&, const State<T, S>&, int, int, int, int);
}  // namespace lbm

using namespace lbm;

static thread_local std::string g_err;

// NVTX range around an entry point, shown by Nsight Systems / ncu --nvtx
// (header-only NVTX: free when no tool is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CUDA_TRY(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(LBM_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
  } while (0)

constexpr int kMeasureBlocks = 1024;
constexpr int kMeasVals = 11;

struct LbmHandle {
  LbmParams prm;
  int prec = LBM_F32;
  int64_t nx = 0, ny = 0, nz = 0, N = 0;
  int64_t Np = 0;  // component stride of f, g, u: N rounded up to kAlignNodes
  bool paired = false;  // paired layout (Consts::nh): 3-D float / half grids with even nx
  int device = 0;
  size_t tsize = 4;  // compute type (u, phi, eps, fields)
  size_t psize = 4;  // population storage type
  // device memory
  void* f[2] = {nullptr, nullptr};
  void* g[2] = {nullptr, nullptr};
  void* u = nullptr;
  void* phi[2] = {nullptr, nullptr};  // phi recovered by the last two steps
  void* eps = nullptr;
  uint8_t* cls = nullptr;
  float* wn = nullptr;
  double* partials = nullptr;
  unsigned* counters = nullptr;  // [0] step/init reductions, [1] measure, [2] status, [3] inject, [4] momentum
  void* cbuf = nullptr;          // 2 x T
  double* scal = nullptr;        // [0] phi_mass_init [1] last sum [2..10] measure output [16..21] extents [24..26] momentum
  void* meas_phi = nullptr;      // N x T scratch for lbm_measure
  void* amp = nullptr;           // N x T per-node geometric amplification (lbm_set_amplification), or null
  void* mu = nullptr;            // Np x T chemical potential of the step (gradient-of-mu modes only)
  void* gmu = nullptr;           // 3 Np x T its gradient (gradient-of-mu modes only)
  int* nsw = nullptr;            // N next-interior node indices (direct wetting only)
  void* cubic = nullptr;         // 4 x T cubic-wall-energy constants (direct wetting only)
  // derived
  bool wetting = false;
  Consts<float> kf{};
  Consts<double> kd{};
  std::vector<uint8_t> cls_host;  // node-class table on the host (lazily fetched; empty = not fetched)
  // sequencing
  bool geometry_set = false, initialized = false;
  Tiling tiling{};
  int cur = 0;            // buffer index holding the current state
  int pc = 0;             // phi buffer holding the latest recovered phi
  bool raw = true;        // current state is the reference state itself (after init)
  bool first = true;      // phi*u of the previous step does not exist yet
  int c_last = 0;         // cbuf slot of the last step's correction
  int64_t steps = 0;
  bool last_raw_in = true;  // mode of the last step's input (for P read-out)
  bool obs_init = true;     // fields read as after init_fields (no step since init or an injection)
  // the two-kernel step runs the batched kernels on a one-case table: device
  // descriptors for the two step parities, valid while desc_ok
  void* desc = nullptr;
  bool desc_ok = false;
  int desc_cur0 = 0;        // cur when the descriptors were filled (parity 0)
  int phi_per_thread = 16;  // nodes per thread of the phi kernel
  int upd_block = kBlock;   // threads per block of the (linear-layout) update kernel: 128 or 256
};

namespace {

template <typename T>
Consts<T> make_consts(const LbmHandle& h, const float* ww_lut) {
  const LbmParams& p = h.prm;
  Consts<T> k;
  std::memset(&k, 0, sizeof(k));
  k.nx = (int)h.nx;
  k.ny = (int)h.ny;
  k.nz = (int)h.nz;
  k.N = (int)h.N;
  k.Np = (int)h.Np;
  k.nh = h.paired ? (int)(h.N / 2) : 0;
  k.hx = h.paired ? (int)(h.nx / 2) : 0;
  k.dz = make_fastdiv((unsigned)h.nz);
  k.dy = make_fastdiv((unsigned)h.ny);
  const double cs2 = 1.0 / 3.0;
  const double tau_f = p.tau_h > 0 ? p.tau_h : p.tau_l;
  const double ac_coeff = 1.0 - 0.5 / tau_f;
  for (int q = 0; q < kQ; ++q) {
    const float wf = q == 0 ? (float)(1.0 / 3.0) : (q <= 6 ? (float)(1.0 / 18.0) : (float)(1.0 / 36.0));
    k.w[q] = (T)wf;
    k.wc[q] = (T)wf / (T)cs2;
    k.w2c[q] = (T)2 * k.wc[q];
    k.wac[q] = (T)ac_coeff * (T)wf;
    k.wac3[q] = k.wac[q] / (T)cs2;
    k.inv_w[q] = (T)1 / (T)wf;
  }
  k.cs2 = (T)cs2;
  k.two_cs2 = (T)(2.0 * cs2);
  k.inv_cs2 = (T)1 / k.cs2;
  k.inv_two_cs2 = (T)1 / k.two_cs2;
  k.inv_W = (T)1 / (T)p.xi;
  k.beta4 = (T)(4.0 * p.beta);
  k.kappa = (T)p.kappa;
  k.phi_c = (T)p.phi_c;
  k.W = (T)p.xi;
  k.rho_l = (T)p.rho_l;
  k.rho_g = (T)p.rho_g;
  k.rho_floor = (T)(0.5 * p.rho_l);
  k.drho = (T)(p.rho_l - p.rho_g);
  k.visc = (T)((0.5 - p.tau_g) / p.tau_g);
  k.omega_f = (T)(1.0 / tau_f);
  k.omega_g = (T)1 / (T)p.tau_l;
  k.tau_l = (T)p.tau_l;
  k.tl_m = (T)(p.tau_l - 0.5);
  k.tg_m = (T)(p.tau_g - 0.5);
  k.tau_const = p.tau_g == p.tau_l;
  k.has_gforce = 0;
  for (int d = 0; d < 3; ++d) {
    k.gforce[d] = (T)p.g_force[d];
    if (p.g_force[d] != 0.0) k.has_gforce = 1;
  }
  k.stab_mode = p.stab_mode;
  k.ac_scale = (T)p.ac_scale;
  k.sharpen_reduce = (T)p.sharpen_reduce;
  k.wetting = h.wetting ? 1 : 0;
  const double deg2rad = M_PI / 180.0;
  const double th = p.theta_eq * deg2rad;
  k.linear = (p.theta_eq > 130.0 || p.theta_eq < 50.0) ? 1 : 0;
  if (k.wetting) {
    if (k.linear) {
      const double hh = p.sigma * std::cos(th);
      double gs = p.ghost_scale;
      if (!(gs > 0.0)) gs = std::fabs(p.theta_eq - 90.0) > 60.0 ? 3.0 : 2.0;
      k.h_over_kappa_f = (float)(hh / p.kappa * gs);
      k.mu_wall_add = (T)((-hh * 2.0) * p.mu_wall_scale);
    } else {
      k.pcok_f = (float)(p.phi_c / p.kappa);
    }
  }
  const double cos_t = std::cos(th), sin_t = std::sin(th);
  k.cos_t = (T)cos_t;
  k.sin_t = (T)sin_t;
  k.geometric = (k.wetting && p.geometric_wetting && std::fabs(sin_t) >= 1e-10) ? 1 : 0;
  k.amp_active = p.geo_amplification > 1.0 ? 1 : 0;
  k.amp = (T)p.geo_amplification;
  // boundary-phi relaxation target (fe_ac_solver.py:165-177, 613-616)
  k.relax_on = 0;
  if (k.wetting && p.boundary_relax > 0 && p.theta_eq != 90.0) {
    const double c = std::cos(th);
    const double disc = 1.0 - 4.0 * (-c / 3.0);
    double target;
    if (disc >= 0) target = 0.5 * (1.0 - std::sqrt(disc));
    else target = 0.5 * (1.0 - std::cos(M_PI - th));
    if (p.direct_wetting) {
      // cubic wall energy (fe_ac_solver.py:609-612); its constants: cubic_consts
      k.relax_on = 1;
      k.relax_r = (T)p.boundary_relax;
    } else if (std::fabs(target - 0.5) > 0.05) {
      k.relax_on = 1;
      k.relax_target = (T)target;
      k.relax_r = (T)p.boundary_relax;
    }
  }
  for (int i = 0; i < 16; ++i) k.ww[i] = (T)ww_lut[i];
  // interface source with grad mu (lbm/fe_ac_solver.py:457-486)
  const double mob = cs2 * (tau_f - 0.5);
  k.gmu_mode = p.interface_mode == LBM_IFACE_CAHN_HILLIARD ? kGmuCH : (p.mu_drive > 0.0 ? kGmuDrive : 0);
  k.mob = (T)mob;
  k.guo = (T)(tau_f / (tau_f - 0.5));
  k.mu_drive_a = (T)(p.mu_drive * mob);
  return k;
}

// Constants of the cubic-wall-energy boundary phi (fe_wetting.py:369-416) in
// the compute type: (1 - a)^2, 4 a, -(1 - a), 2 a, a = 6 sigma cos(theta) /
// kappa; 2 a = 0 when |a| < 1e-10 (no correction).
template <typename T>
void cubic_consts(const LbmParams& p, T* out4) {
  const double a = 6.0 * p.sigma * std::cos(p.theta_eq * M_PI / 180.0) / p.kappa, oma = 1.0 - a;
  out4[0] = (T)(oma * oma);
  out4[1] = (T)(4.0 * a);
  out4[2] = (T)(-oma);
  out4[3] = std::fabs(a) >= 1e-10 ? (T)(2.0 * a) : (T)0;
}

// The constant table holds the same lattice values the kernels may also use
// as compile-time immediates (Lat<T>).
template <typename T>
bool lattice_table_matches(const Consts<T>& k) {
  for (int q = 0; q < kQ; ++q)
    if (k.w[q] != Lat<T>::w(q) || k.wc[q] != Lat<T>::wc(q) || k.w2c[q] != Lat<T>::w2c(q) ||
        k.inv_w[q] != Lat<T>::inv_w(q))
      return false;
  return k.cs2 == Lat<T>::cs2() && k.inv_cs2 == Lat<T>::inv_cs2() && k.two_cs2 == Lat<T>::two_cs2() &&
         k.inv_two_cs2 == Lat<T>::inv_two_cs2();
}

// Compute / storage type pair of a precision: float/float, double/double,
// float/half (deviation-storage form).
template <typename T_, typename S_>
struct Types {
  using T = T_;
  using S = S_;
};
template <typename Fn>
auto with_types(int prec, Fn&& fn) {
  if (prec == LBM_F64) return fn(Types<double, double>{});
  if (prec == LBM_F16) return fn(Types<float, __half>{});
  return fn(Types<float, float>{});
}

// State of a step reading population buffer `in_buf` and phi buffer `phi_in`.
template <typename T, typename S>
State<T, S> make_state(const LbmHandle& h, int in_buf, int phi_in) {
  State<T, S> s;
  std::memset(&s, 0, sizeof(s));
  s.fin = static_cast<const S*>(h.f[in_buf]);
  s.gin = static_cast<const S*>(h.g[in_buf]);
  s.fout = static_cast<S*>(h.f[in_buf ^ 1]);
  s.gout = static_cast<S*>(h.g[in_buf ^ 1]);
  s.u = static_cast<T*>(h.u);
  s.phi_in = static_cast<const T*>(h.phi[phi_in]);
  s.phi_out = static_cast<T*>(h.phi[phi_in ^ 1]);
  s.cls = h.cls;
  s.wn = h.wn;
  s.eps = static_cast<const T*>(h.eps);
  s.amp = static_cast<const T*>(h.amp);
  s.mu = static_cast<T*>(h.mu);
  s.gmu = static_cast<T*>(h.gmu);
  s.nsw = h.nsw;
  s.cubic = static_cast<const T*>(h.cubic);
  s.partials = h.partials;
  s.counter = h.counters;
  s.cbuf = static_cast<T*>(h.cbuf);
  s.scal = h.scal;
  s.status = h.counters + 2;
  return s;
}

// Shared memory the step kernel may use per block: a third of an SM for float
// (three resident blocks), most of one for double.
size_t smem_budget(int prec) { return prec == LBM_F64 ? 200 * 1024 : 70 * 1024; }

Tiling tiling_of(int64_t nx, int64_t ny, int64_t nz, int tx, int ty, int tz) {
  Tiling t;
  tx = std::max(tx, 2);
  ty = std::max(ty, 2);
  tz = std::max(tz, 2);
  t.tx = (int)std::min<int64_t>(tx, nx);
  t.ty = (int)std::min<int64_t>(ty, ny);
  t.tz = (int)std::min<int64_t>(tz, nz);
  t.ntx = (int)((nx + t.tx - 1) / t.tx);
  t.nty = (int)((ny + t.ty - 1) / t.ty);
  t.ntz = (int)((nz + t.tz - 1) / t.tz);
  t.hmax = (t.tx + 2) * (t.ty + 2) * (t.tz + 2);
  return t;
}

size_t tiling_smem(const Tiling& t, int prec) {
  if (t.tx == 0) return 0;
  if (prec == LBM_F64) return step_smem_bytes<double, double>(t);
  if (prec == LBM_F16) return step_smem_bytes<float, __half>(t);
  return step_smem_bytes<float, float>(t);
}

// Step kernels: all extents 0 selects the two-kernel streaming step (the
// default); otherwise the fused tiled kernel, with a z extent balanced over nz
// near 28 and a 6 x 6 x-y cross-section for the extents given as 0.
Tiling make_tiling(int64_t nx, int64_t ny, int64_t nz, int tx, int ty, int tz, int prec) {
  (void)prec;
  if (tx <= 0 && ty <= 0 && tz <= 0) {
    Tiling t;
    std::memset(&t, 0, sizeof(t));
    return t;
  }
  if (tz <= 0) {
    const int ntz = (int)((nz + 27) / 28);
    tz = (int)((nz + ntz - 1) / ntz);
  }
  return tiling_of(nx, ny, nz, tx > 0 ? tx : 6, ty > 0 ? ty : 6, tz);
}

// ---------------------------------------------------------------------------
// Cache of state arrays.  lbm_destroy hands the state arrays of a grid back
// to a per-process cache instead of cudaFree, and lbm_create takes blocks of
// a fitting size (at most 1/8 larger) on the same device from it before it
// calls cudaMalloc: a sweep or a serving loop that opens and closes grids of
// recurring sizes then neither maps nor unmaps device memory per grid.  The
// cache holds at most g_cache_limit bytes (lbm_cache_limit; 0 disables it);
// a cudaMalloc that runs out of memory empties it and retries.  Recycled
// blocks hold old data: every array is written (memset or kernels) before it
// is read, as with fresh cudaMalloc memory, which CUDA does not zero either.
// ---------------------------------------------------------------------------
struct CachedBlock {
  int device;
  size_t bytes;
  void* p;
  unsigned long long seq;  // order of return to the cache (oldest evicted first)
};
std::mutex g_cache_mu;
std::vector<CachedBlock> g_cache;                    // free blocks
std::unordered_map<void*, CachedBlock> g_cache_live; // blocks handed out
size_t g_cache_bytes = 0;
size_t g_cache_limit = (size_t)16 << 30;
unsigned long long g_cache_seq = 0;

// Frees the cached blocks of `device` (every device for -1), each with its
// own device current.
void cache_trim_locked(int device) {
  if (g_cache.empty()) return;
  int cur = -1;
  (void)cudaGetDevice(&cur);
  for (size_t i = 0; i < g_cache.size();) {
    if (device < 0 || g_cache[i].device == device) {
      if (cudaSetDevice(g_cache[i].device) == cudaSuccess) cudaFree(g_cache[i].p);
      g_cache_bytes -= g_cache[i].bytes;
      g_cache[i] = g_cache.back();
      g_cache.pop_back();
    } else {
      ++i;
    }
  }
  if (cur >= 0) (void)cudaSetDevice(cur);
}

cudaError_t cache_alloc(void** p, size_t bytes, int device) {
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    int best = -1;
    for (int i = 0; i < (int)g_cache.size(); ++i) {
      const CachedBlock& b = g_cache[i];
      if (b.device == device && b.bytes >= bytes && b.bytes - bytes <= bytes / 8 &&
          (best < 0 || b.bytes < g_cache[best].bytes))
        best = i;
    }
    if (best >= 0) {
      const CachedBlock b = g_cache[best];
      g_cache[best] = g_cache.back();
      g_cache.pop_back();
      g_cache_bytes -= b.bytes;
      g_cache_live[b.p] = b;
      *p = b.p;
      return cudaSuccess;
    }
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaErrorMemoryAllocation) {
    (void)cudaGetLastError();
    std::lock_guard<std::mutex> lk(g_cache_mu);
    cache_trim_locked(device);
    e = cudaMalloc(p, bytes);
  }
  if (e == cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    g_cache_live[*p] = CachedBlock{device, bytes, *p, 0ull};
  }
  return e;
}

// Returns a block from cache_alloc to the cache, first freeing the blocks
// that have been cached longest while the limit would be exceeded (a block
// larger than the limit is freed); frees anything else.  The caller has
// synchronised the device.
void cache_release(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_cache_mu);
  auto it = g_cache_live.find(p);
  if (it == g_cache_live.end()) {
    cudaFree(p);
    return;
  }
  CachedBlock b = it->second;
  g_cache_live.erase(it);
  if (b.bytes > g_cache_limit) {
    cudaFree(p);
    return;
  }
  while (g_cache_bytes + b.bytes > g_cache_limit && !g_cache.empty()) {
    size_t old = 0;
    for (size_t i = 1; i < g_cache.size(); ++i)
      if (g_cache[i].seq < g_cache[old].seq) old = i;
    int cur = -1;
    (void)cudaGetDevice(&cur);
    if (cudaSetDevice(g_cache[old].device) == cudaSuccess) cudaFree(g_cache[old].p);
    if (cur >= 0) (void)cudaSetDevice(cur);
    g_cache_bytes -= g_cache[old].bytes;
    g_cache[old] = g_cache.back();
    g_cache.pop_back();
  }
  b.seq = ++g_cache_seq;
  g_cache.push_back(b);
  g_cache_bytes += b.bytes;
}

void free_all(LbmHandle* h) {
  void* ptrs[] = {h->f[0], h->f[1], h->g[0], h->g[1], h->u,        h->phi[0], h->phi[1], h->eps,
                  h->cls,  h->wn,   h->partials, h->counters, h->cbuf, h->scal, h->meas_phi, h->desc,
                  h->amp,  h->mu, h->gmu, h->nsw, h->cubic};
  // kernels still queued on any stream may use the arrays (cudaFree would
  // wait for them as well); the handle's device is current while they are
  // released
  int cur = -1;
  (void)cudaGetDevice(&cur);
  const bool on_dev = cudaSetDevice(h->device) == cudaSuccess;
  if (on_dev) cudaDeviceSynchronize();
  for (void* p : ptrs) cache_release(p);
  if (on_dev && cur >= 0) (void)cudaSetDevice(cur);
}

template <typename T>
const Consts<T>& consts_of(const LbmHandle& h);
template <>
const Consts<float>& consts_of<float>(const LbmHandle& h) { return h.kf; }
template <>
const Consts<double>& consts_of<double>(const LbmHandle& h) { return h.kd; }

// A grid with nz == 1 is 2-D: D2Q9 populations, two velocity components.
bool is2d(const LbmHandle* h) { return h->nz == 1; }
int nq_of(int64_t nz) { return nz == 1 ? kQ2 : Q; }
int ndim_of(int64_t nz) { return nz == 1 ? 2 : 3; }

// The 2-D step of the handle's current state (no bookkeeping).
template <typename T>
int launch_next2d(LbmHandle* h, cudaStream_t st, cudaEvent_t mid) {
  State<T, T> s = make_state<T, T>(*h, h->cur, h->pc);
  s.c_prev = h->c_last;
  s.c_cur = h->c_last ^ 1;
  const double tau_f = h->prm.tau_h > 0 ? h->prm.tau_h : h->prm.tau_l;
  CUDA_TRY(launch_step2d<T>(consts_of<T>(*h), s, h->raw, h->first, 1.0 - 0.5 / tau_f, st, mid));
  return LBM_OK;
}

// The spread reduction runs over a 2-D grid as the 1 x nx x ny grid of the
// same memory layout, so that its last-axis centre is the centre along y
// (the wall-normal axis in 2-D); remap_measure2d puts the results back in
// x, y order: Dz = 0 as the reference reports for 2-D fields, and the
// z extents of ext6 (if given) 0 or -1 when the set is empty.
void measure_grid(const LbmHandle* h, int* mx, int* my, int* mz) {
  if (is2d(h)) {
    *mx = 1;
    *my = (int)h->nx;
    *mz = (int)h->ny;
  } else {
    *mx = (int)h->nx;
    *my = (int)h->ny;
    *mz = (int)h->nz;
  }
}
void remap_measure2d(double* out9, double* ext6) {
  const bool any = out9[7] > 0.0;
  out9[2] = out9[3];
  out9[3] = out9[4];
  out9[4] = 0.0;
  out9[5] = out9[3] > 0.0 ? out9[2] / out9[3] : 0.0;
  if (ext6) {
    for (int j = 0; j < 4; ++j) ext6[j] = ext6[j + 2];
    ext6[4] = ext6[5] = any ? 0.0 : -1.0;
  }
}

bool omega1_of(const LbmHandle* h) {
  return h->prec == LBM_F64 ? consts_of<double>(*h).omega_f == 1.0 : consts_of<float>(*h).omega_f == 1.0f;
}

// Blocks of a case in the (batched) phi kernel grid, per_thread nodes per
// thread, and in the update kernel grid (one node per thread).
// (Pairs of nodes in the paired layout.)
int64_t units_of(const LbmHandle* h) { return h->paired ? h->N / 2 : h->N; }
// per_thread counts nodes (a thread of the paired kernel takes per_thread / 2 pairs).
int phi_blocks_of(const LbmHandle* h, int per_thread) {
  const long long per = (long long)kBlock * (h->paired ? std::max(1, per_thread / 2) : per_thread);
  return (int)std::max<long long>(1, (units_of(h) + per - 1) / per);
}
// upd_block: threads per block of the linear-layout update kernel (the
// paired update kernel always runs kPairUpdBlock).
int upd_blocks_of(const LbmHandle* h, int upd_block) {
  const int64_t bs = h->paired ? kPairUpdBlock : upd_block;
  return (int)((units_of(h) + bs - 1) / bs);
}

// The step kernels of a grid's layout over a case table: the paired kernels
// or the single-node kernels.
template <typename T, typename S>
cudaError_t launch_phi_kernel(bool paired, const void* cases, const unsigned short* b2c, int blocks, cudaStream_t st) {
  return paired ? launch_phi_pair<T, S>(cases, b2c, blocks, st) : launch_phi_batch<T, S>(cases, b2c, blocks, st);
}
template <typename T, typename S>
cudaError_t launch_update_kernel(bool paired, const void* cases, const unsigned short* b2c, int blocks, bool omega1,
                                 cudaStream_t st, bool gmu, int upd_block) {
  return paired ? launch_update_pair<T, S>(cases, b2c, blocks, omega1, st, gmu)
                : launch_update_batch<T, S>(cases, b2c, blocks, omega1, st, gmu, upd_block);
}

// The handle's one-case descriptor table for the batched kernels: [0] the
// state as it is now, [1] after one more step.  The descriptor holds device
// pointers that alternate with the step parity, constants and grid extents.
template <typename T, typename S>
int fill_desc(LbmHandle* h, cudaStream_t st) {
  const size_t db = case_desc_bytes<T, S>();
  if (!h->desc) CUDA_TRY(cudaMalloc(&h->desc, 2 * db));
  std::vector<unsigned char> buf(2 * db);
  for (int par = 0; par < 2; ++par) {
    State<T, S> s = make_state<T, S>(*h, h->cur ^ par, h->pc ^ par);
    s.c_prev = h->c_last ^ par;
    s.c_cur = h->c_last ^ par ^ 1;
    fill_case_desc<T, S>(buf.data() + par * db, consts_of<T>(*h), s, 0, phi_blocks_of(h, h->phi_per_thread), 0,
                         upd_blocks_of(h, h->upd_block));
  }
  // earlier steps on `st` may still read the old table
  CUDA_TRY(cudaStreamSynchronize(st));
  CUDA_TRY(cudaMemcpy(h->desc, buf.data(), 2 * db, cudaMemcpyHostToDevice));
  h->desc_ok = true;
  h->desc_cur0 = h->cur;
  return LBM_OK;
}

// Launches the step that would run next (no bookkeeping): the first step
// after init and the fused kernel through launch_step; every other
// two-kernel step through the batched kernels on the handle's one-case table,
// so a grid gives the same results alone and in a batch.  `mid` (may be null)
// is recorded between the two kernels (before the fused kernel).
template <typename T, typename S>
int launch_next(LbmHandle* h, const Tiling& t, cudaStream_t st, cudaEvent_t mid) {
  if (t.tx == 0 && !h->raw && !h->first) {
    if (!h->desc_ok) {
      const int rc = fill_desc<T, S>(h, st);
      if (rc != LBM_OK) return rc;
    }
    const int par = (h->cur ^ h->desc_cur0) & 1;
    const bool gmu = h->mu != nullptr;
    const unsigned char* d = static_cast<const unsigned char*>(h->desc) + par * case_desc_bytes<T, S>();
    CUDA_TRY((launch_phi_kernel<T, S>(h->paired, d, nullptr, phi_blocks_of(h, h->phi_per_thread), st)));
    if (mid) CUDA_TRY(cudaEventRecord(mid, st));
    if (gmu) {
      State<T, S> s = make_state<T, S>(*h, h->cur, h->pc);
      CUDA_TRY((launch_mu<T, S>(consts_of<T>(*h), s, st)));
    }
    CUDA_TRY((launch_update_kernel<T, S>(h->paired, d, nullptr, upd_blocks_of(h, h->upd_block), omega1_of(h), st,
                                         gmu, h->upd_block)));
    return LBM_OK;
  }
  State<T, S> s = make_state<T, S>(*h, h->cur, h->pc);
  s.c_prev = h->c_last;
  s.c_cur = h->c_last ^ 1;
  CUDA_TRY(launch_step<T>(consts_of<T>(*h), s, t, h->raw, h->first, st, mid));
  return LBM_OK;
}

template <typename T, typename S>
int do_step(LbmHandle* h, int nsteps, cudaStream_t st, cudaEvent_t* ev = nullptr) {
  for (int i = 0; i < nsteps; ++i) {
    if (ev) CUDA_TRY(cudaEventRecord(ev[2 * i], st));
    int rc;
    if constexpr (sizeof(S) == sizeof(T)) {
      rc = is2d(h) ? launch_next2d<T>(h, st, ev ? ev[2 * i + 1] : nullptr)
                   : launch_next<T, S>(h, h->tiling, st, ev ? ev[2 * i + 1] : nullptr);
    } else {
      rc = launch_next<T, S>(h, h->tiling, st, ev ? ev[2 * i + 1] : nullptr);
    }
    if (rc != LBM_OK) return rc;
    h->last_raw_in = h->raw;
    h->obs_init = false;
    h->cur ^= 1;
    h->pc ^= 1;
    h->c_last ^= 1;
    h->raw = false;
    h->first = false;
    ++h->steps;
  }
  if (ev) CUDA_TRY(cudaEventRecord(ev[2 * nsteps], st));
  return LBM_OK;
}

}  // namespace

namespace {
// Times `reps` launches of the step kernel that would run next, without
// advancing the state: the same input buffers are read every time and the
// in-place velocity is restored from `u_save` by the caller.
template <typename T, typename S>
int time_tiling(LbmHandle* h, const Tiling& t, int reps, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1,
                float* ms) {
  int rc = launch_next<T, S>(h, t, st, nullptr);  // warm-up (sets smem attributes)
  if (rc != LBM_OK) return rc;
  CUDA_TRY(cudaEventRecord(e0, st));
  for (int i = 0; i < reps && rc == LBM_OK; ++i) rc = launch_next<T, S>(h, t, st, nullptr);
  if (rc != LBM_OK) return rc;
  CUDA_TRY(cudaEventRecord(e1, st));
  CUDA_TRY(cudaEventSynchronize(e1));
  CUDA_TRY(cudaEventElapsedTime(ms, e0, e1));
  return LBM_OK;
}
}  // namespace

namespace {
// Device bytes of one handle's arrays (what lbm_create allocates).
struct Sizes {
  size_t pop, u, phi, eps, cls, wn, partials, counters, cbuf, scal, meas_phi;
  size_t total() const {
    return 4 * pop + u + 2 * phi + eps + cls + wn + partials + counters + cbuf + scal + meas_phi;
  }
};
Sizes sizes_of(int64_t nx, int64_t ny, int64_t nz, int precision) {
  const int64_t N = nx * ny * nz;
  const int64_t Np = (N + kAlignNodes - 1) / kAlignNodes * kAlignNodes;
  const size_t T = precision == LBM_F64 ? 8 : 4;
  const size_t P = precision == LBM_F64 ? 8 : (precision == LBM_F16 ? 2 : 4);
  // per-block partial sums: init (one block per 256 nodes), step (one per
  // tile; tile extents are at least 2) and measure
  const int nblocks = (int)((N + kBlock - 1) / kBlock);
  const size_t max_tiles = (size_t)((nx + 1) / 2) * (size_t)((ny + 1) / 2) * (size_t)((nz + 1) / 2);
  const size_t npart = std::max<size_t>({(size_t)nblocks, max_tiles, (size_t)kMeasureBlocks * kMeasVals});
  Sizes z;
  z.pop = (size_t)nq_of(nz) * Np * P;  // one of f[0], f[1], g[0], g[1]
  z.u = 3 * Np * T;
  z.phi = Np * T;  // phi and class arrays padded to Np like the populations
  z.eps = N * T;
  z.cls = Np;
  z.wn = 3 * N * sizeof(float);
  z.partials = npart * sizeof(double);
  z.counters = 8 * sizeof(unsigned);
  z.cbuf = 2 * T;
  z.scal = 32 * sizeof(double);
  z.meas_phi = N * T;
  return z;
}
}  // namespace

extern "C" {

const char* lbm_last_error(void) { return g_err.c_str(); }

int lbm_footprint(int64_t nx, int64_t ny, int64_t nz, int precision, int64_t* bytes) {
  if (!bytes) return fail(LBM_E_ARG, "lbm_footprint: null argument");
  if (nx < 2 || ny < 2 || nz < 1 || nz == 1 && precision == LBM_F16)
    return fail(LBM_E_UNSUPPORTED, "lbm_footprint: 3-D grids with every extent >= 2, or 2-D grids (nz == 1) in LBM_F32 or LBM_F64");
  if (precision != LBM_F32 && precision != LBM_F64 && precision != LBM_F16)
    return fail(LBM_E_ARG, "lbm_footprint: bad precision");
  *bytes = (int64_t)sizes_of(nx, ny, nz, precision).total();
  return LBM_OK;
}

const char* lbm_version(void) { return "lbm_gb300 0.1 (sm_103a)"; }

int lbm_create(const LbmParams* params, int64_t nx, int64_t ny, int64_t nz, int precision, LbmHandle** out) {
  if (!params || !out) return fail(LBM_E_ARG, "lbm_create: null argument");
  *out = nullptr;
  if (nx < 2 || ny < 2 || nz < 1)
    return fail(LBM_E_UNSUPPORTED, "lbm_create: 3-D grids with every extent >= 2, or 2-D grids (nz == 1) only");
  if (precision != LBM_F32 && precision != LBM_F64 && precision != LBM_F16)
    return fail(LBM_E_ARG, "lbm_create: precision must be LBM_F32, LBM_F64 or LBM_F16");
  if (nz == 1 && precision == LBM_F16)
    return fail(LBM_E_UNSUPPORTED, "lbm_create: 2-D grids (nz == 1) run in LBM_F32 or LBM_F64");
  const int64_t N = nx * ny * nz;
  const int64_t Np = (N + kAlignNodes - 1) / kAlignNodes * kAlignNodes;
  if (Np * Q > (int64_t)0x7fffffff) return fail(LBM_E_ARG, "lbm_create: grid too large (19 N must be < 2^31)");
  if (params->stab_mode < 0 || params->stab_mode > 2) return fail(LBM_E_ARG, "lbm_create: bad stab_mode");
  if (!(params->tau_g > 0.5) || !(params->tau_l > 0.5)) return fail(LBM_E_ARG, "lbm_create: tau_l, tau_g must exceed 0.5");
  if (!(params->xi > 0)) return fail(LBM_E_ARG, "lbm_create: xi must be positive");
  if (params->interface_mode != LBM_IFACE_ALLEN_CAHN && params->interface_mode != LBM_IFACE_CAHN_HILLIARD)
    return fail(LBM_E_ARG, "lbm_create: bad interface_mode");
  if (!(params->mu_drive >= 0.0)) return fail(LBM_E_ARG, "lbm_create: mu_drive must be >= 0");
  const bool gmu = params->interface_mode == LBM_IFACE_CAHN_HILLIARD || params->mu_drive > 0.0;
  if (gmu && precision == LBM_F16)
    return fail(LBM_E_UNSUPPORTED, "lbm_create: interface_mode='cahn-hilliard' and mu_drive > 0 need LBM_F32 or LBM_F64");
  LbmHandle* h = new (std::nothrow) LbmHandle();
  if (!h) return fail(LBM_E_ARG, "lbm_create: out of host memory");
  h->prm = *params;
  h->prec = precision;
  h->nx = nx;
  h->ny = ny;
  h->nz = nz;
  h->N = N;
  h->Np = Np;
  // the linear layout by default: on the 150x150x107 ridge case the paired
  // kernels executed fewer instructions per node but were slower (float32
  // 0.1795 against 0.1699 ms per step, float16 0.1697 against 0.1667)
  h->paired = false;
  h->tsize = precision == LBM_F64 ? 8 : 4;
  h->psize = precision == LBM_F64 ? 8 : (precision == LBM_F16 ? 2 : 4);
  h->wetting = params->theta_eq != 90.0 && params->kappa > 0;
  cudaGetDevice(&h->device);
  const size_t T = h->tsize;
  h->tiling = make_tiling(nx, ny, nz, 0, 0, 0, precision);
  const Sizes z = sizes_of(nx, ny, nz, precision);
  cudaError_t e = cudaSuccess;
  auto A = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cache_alloc(p, bytes, h->device);
  };
  for (int b = 0; b < 2; ++b) {
    A(&h->f[b], z.pop);
    A(&h->g[b], z.pop);
  }
  A(&h->u, z.u);
  A(&h->phi[0], z.phi);
  A(&h->phi[1], z.phi);
  A(&h->eps, z.eps);
  A((void**)&h->cls, z.cls);
  A((void**)&h->wn, z.wn);
  A((void**)&h->partials, z.partials);
  A((void**)&h->counters, z.counters);
  A(&h->cbuf, z.cbuf);
  A((void**)&h->scal, z.scal);
  A(&h->meas_phi, z.meas_phi);
  if (gmu) {
    A(&h->mu, z.phi);
    A(&h->gmu, 3 * z.phi);
  }
  if (e == cudaSuccess) e = cudaMemset(h->counters, 0, 8 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(h->phi[0], 0, Np * T);
  if (e == cudaSuccess) e = cudaMemset(h->phi[1], 0, Np * T);
  if (e == cudaSuccess) e = cudaMemset(h->cls, 0, Np);
  if (e == cudaSuccess) e = cudaMemset(h->scal, 0, 32 * sizeof(double));
  if (e != cudaSuccess) {
    free_all(h);
    delete h;
    return fail(LBM_E_CUDA, std::string("lbm_create: ") + cudaGetErrorString(e));
  }
  *out = h;
  return LBM_OK;
}

int lbm_destroy(LbmHandle* h) {
  if (!h) return LBM_OK;
  free_all(h);
  delete h;
  return LBM_OK;
}

int lbm_cache_limit(uint64_t bytes) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  g_cache_limit = (size_t)bytes;
  if (g_cache_bytes > g_cache_limit) cache_trim_locked(-1);
  return LBM_OK;
}

int lbm_cache_trim(uint64_t* freed_bytes) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  const size_t before = g_cache_bytes;
  cache_trim_locked(-1);
  if (freed_bytes) *freed_bytes = before - g_cache_bytes;
  return LBM_OK;
}

int lbm_cache_bytes(uint64_t* cached_bytes) {
  if (!cached_bytes) return fail(LBM_E_ARG, "lbm_cache_bytes: null argument");
  std::lock_guard<std::mutex> lk(g_cache_mu);
  *cached_bytes = g_cache_bytes;
  return LBM_OK;
}

namespace {
// Scratch of launch_geometry: three N-byte planes (bits, distance, its
// transform), then at the next 256-byte boundary the boundary-node count (256
// bytes reserved) and list (N ints).
size_t geo_scratch_bytes(size_t N) { return ((3 * N + 255) & ~(size_t)255) + 256 + 4 * N; }

// The device geometry precompute of a handle from device copies of the
// solid mask and fraction, then the constant tables; asynchronous on `st`.
// scratch: geo_scratch_bytes(N) device bytes the kernels may use, 256-byte
// aligned.
int set_geometry_device(LbmHandle* h, const uint8_t* solid, const void* fraction, int fraction_dtype,
                        uint8_t* scratch, cudaStream_t st) {
  const int64_t N = h->N;
  const bool direct = h->prm.direct_wetting && h->wetting && h->prm.boundary_relax > 0;
  if (direct && !h->nsw) CUDA_TRY(cudaMalloc(&h->nsw, N * sizeof(int)));
  cudaError_t e;
  if (h->prec == LBM_F64)
    e = launch_geometry<double>((int)h->nx, (int)h->ny, (int)h->nz, solid, fraction, fraction_dtype, h->wetting,
                                true, scratch, h->cls, h->wn, direct ? h->nsw : nullptr,
                                static_cast<double*>(h->eps), st);
  else
    e = launch_geometry<float>((int)h->nx, (int)h->ny, (int)h->nz, solid, fraction, fraction_dtype, h->wetting,
                               false, scratch, h->cls, h->wn, direct ? h->nsw : nullptr, static_cast<float*>(h->eps),
                               st);
  if (e != cudaSuccess) return fail(LBM_E_CUDA, std::string("lbm_set_geometry: ") + cudaGetErrorString(e));
  if (direct) {
    if (!h->cubic) CUDA_TRY(cudaMalloc(&h->cubic, 4 * sizeof(double)));
    if (h->prec == LBM_F64) {
      double c4[4];
      cubic_consts(h->prm, c4);
      CUDA_TRY(cudaMemcpy(h->cubic, c4, sizeof(c4), cudaMemcpyHostToDevice));
    } else {
      float c4[4];
      cubic_consts(h->prm, c4);
      CUDA_TRY(cudaMemcpy(h->cubic, c4, sizeof(c4), cudaMemcpyHostToDevice));
    }
  }
  float lut[kWwCodes];
  near_wall_weights(lut);
  h->kf = make_consts<float>(*h, lut);
  h->kd = make_consts<double>(*h, lut);
  if (!lattice_table_matches(h->kf) || !lattice_table_matches(h->kd))
    return fail(LBM_E_ARG, "lbm_set_geometry: internal error: lattice constant table differs from the kernels' immediates");
  h->cls_host.clear();
  h->geometry_set = true;
  h->desc_ok = false;
  return LBM_OK;
}

// The node-class table on the host (fetched once per geometry).
int class_table_host(LbmHandle* h) {
  if (!h->cls_host.empty()) return LBM_OK;
  h->cls_host.resize((size_t)h->N);
  CUDA_TRY(cudaMemcpy(h->cls_host.data(), h->cls, (size_t)h->N, cudaMemcpyDeviceToHost));
  return LBM_OK;
}
}  // namespace

int lbm_set_geometry(LbmHandle* h, const uint8_t* solid, const void* fraction, int fraction_dtype) {
  NvtxRange range("lbm_set_geometry");
  if (!h || !solid) return fail(LBM_E_ARG, "lbm_set_geometry: null argument");
  if (fraction_dtype < 0 || fraction_dtype > 2 || ((fraction_dtype != 0) != (fraction != nullptr)))
    return fail(LBM_E_ARG, "lbm_set_geometry: fraction and fraction_dtype disagree");
  // the inputs are staged through the population buffer the next step
  // writes (it holds no state between steps): solid (N bytes), the fraction
  // (N elements), then the kernels' scratch
  const size_t N = (size_t)h->N;
  const size_t fb = fraction_dtype == 0 ? 0 : N * (fraction_dtype == 1 ? 4 : 8);
  uint8_t* stage = static_cast<uint8_t*>(h->f[h->cur ^ 1]);
  const size_t off_f = (N + 255) & ~(size_t)255, off_s = (off_f + fb + 255) & ~(size_t)255;
  if (off_s + geo_scratch_bytes(N) > (size_t)nq_of(h->nz) * h->Np * h->psize)
    return fail(LBM_E_ARG, "lbm_set_geometry: internal error: staging exceeds the population buffer");
  CUDA_TRY(cudaMemcpyAsync(stage, solid, N, cudaMemcpyHostToDevice, 0));
  if (fb) CUDA_TRY(cudaMemcpyAsync(stage + off_f, fraction, fb, cudaMemcpyHostToDevice, 0));
  const int rc = set_geometry_device(h, stage, fb ? stage + off_f : nullptr, fraction_dtype, stage + off_s, 0);
  if (rc != LBM_OK) return rc;
  CUDA_TRY(cudaStreamSynchronize(0));
  return LBM_OK;
}

int lbm_set_geometry_device(LbmHandle* h, const uint8_t* solid, const void* fraction, int fraction_dtype,
                            void* stream) {
  NvtxRange range("lbm_set_geometry_device");
  if (!h || !solid) return fail(LBM_E_ARG, "lbm_set_geometry_device: null argument");
  if (fraction_dtype < 0 || fraction_dtype > 2 || ((fraction_dtype != 0) != (fraction != nullptr)))
    return fail(LBM_E_ARG, "lbm_set_geometry_device: fraction and fraction_dtype disagree");
  if (geo_scratch_bytes((size_t)h->N) > (size_t)nq_of(h->nz) * h->Np * h->psize)
    return fail(LBM_E_ARG, "lbm_set_geometry_device: internal error: scratch exceeds the population buffer");
  return set_geometry_device(h, solid, fraction, fraction_dtype, static_cast<uint8_t*>(h->f[h->cur ^ 1]),
                             static_cast<cudaStream_t>(stream));
}

int lbm_set_amplification(LbmHandle* h, const void* alpha, int alpha_dtype) {
  if (!h) return fail(LBM_E_ARG, "lbm_set_amplification: null handle");
  if (!alpha) {
    if (alpha_dtype != LBM_DT_NONE) return fail(LBM_E_ARG, "lbm_set_amplification: alpha and alpha_dtype disagree");
    if (h->amp) {
      // steps already queued may still read the field
      CUDA_TRY(cudaDeviceSynchronize());
      CUDA_TRY(cudaFree(h->amp));
      h->amp = nullptr;
    }
    h->desc_ok = false;
    return LBM_OK;
  }
  if (alpha_dtype != LBM_DT_F32 && alpha_dtype != LBM_DT_F64)
    return fail(LBM_E_ARG, "lbm_set_amplification: alpha_dtype must be LBM_DT_F32 or LBM_DT_F64");
  const int64_t N = h->N;
  // the reference casts the field to the compute type (fe_wetting.py:505)
  std::vector<unsigned char> buf(N * h->tsize);
  for (int64_t n = 0; n < N; ++n) {
    const double a = alpha_dtype == LBM_DT_F32 ? (double)static_cast<const float*>(alpha)[n]
                                               : static_cast<const double*>(alpha)[n];
    if (h->prec == LBM_F64) reinterpret_cast<double*>(buf.data())[n] = a;
    else reinterpret_cast<float*>(buf.data())[n] = (float)a;
  }
  if (!h->amp) CUDA_TRY(cudaMalloc(&h->amp, N * h->tsize));
  else CUDA_TRY(cudaDeviceSynchronize());
  CUDA_TRY(cudaMemcpy(h->amp, buf.data(), N * h->tsize, cudaMemcpyHostToDevice));
  h->desc_ok = false;
  return LBM_OK;
}

namespace {
// Whether kernels on `device` may read pageable host memory in place
// (cudaDevAttrPageableMemoryAccess: a Grace host with address translation
// services reaches it over the chip-to-chip link).  Cached per device.
// LBM_HOST_STAGING=1 in the environment selects the staging copy on every
// device.
bool pageable_direct(int device) {
  static std::mutex mu;
  static std::vector<int> known;  // -1 unknown, 0 no, 1 yes
  static const bool staging = [] {
    const char* v = std::getenv("LBM_HOST_STAGING");
    return v && v[0] == '1';
  }();
  std::lock_guard<std::mutex> lk(mu);
  if (device < 0 || staging) return false;
  if ((int)known.size() <= device) known.resize(device + 1, -1);
  if (known[device] < 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
      (void)cudaGetLastError();
      v = 0;
    }
    known[device] = v ? 1 : 0;
  }
  return known[device] == 1;
}
}  // namespace

int lbm_init_fields(LbmHandle* h, const void* phi, const void* u, int src_dtype, int on_device, void* stream) {
  NvtxRange range("lbm_init_fields");
  if (!h || !phi) return fail(LBM_E_ARG, "lbm_init_fields: null argument");
  if (!h->geometry_set) return fail(LBM_E_STATE, "lbm_init_fields: call lbm_set_geometry first");
  if (src_dtype != LBM_DT_F32 && src_dtype != LBM_DT_F64) return fail(LBM_E_ARG, "lbm_init_fields: bad src_dtype");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t es = src_dtype == LBM_DT_F32 ? 4 : 8;
  const int64_t N = h->N;
  // Host inputs are read by the kernel in place where the device reaches
  // pageable host memory (the call then waits for the kernel, so that the
  // caller may free them on return as after a copy); elsewhere they are
  // staged through the (not yet used) second g buffer: 19 N T-elements hold
  // the 4 N source elements.
  int in = h->cur;
  const void* dphi = phi;
  const void* du = u;
  const bool direct = !on_device && pageable_direct(h->device);
  if (!on_device && !direct) {
    char* stage = static_cast<char*>(h->g[in ^ 1]);
    CUDA_TRY(cudaMemcpyAsync(stage, phi, N * es, cudaMemcpyHostToDevice, st));
    dphi = stage;
    if (u) {
      CUDA_TRY(cudaMemcpyAsync(stage + N * es, u, ndim_of(h->nz) * N * es, cudaMemcpyHostToDevice, st));
      du = stage + N * es;
    }
  }
  cudaError_t e = with_types(h->prec, [&](auto tag) {
    using T = typename decltype(tag)::T;
    using S = typename decltype(tag)::S;
    State<T, S> s = make_state<T, S>(*h, in, h->pc ^ 1);
    if constexpr (sizeof(S) == sizeof(T)) {
      if (is2d(h))
        return src_dtype == LBM_DT_F32
                   ? launch_init2d<T, float>(consts_of<T>(*h), s, (const float*)dphi, (const float*)du, st)
                   : launch_init2d<T, double>(consts_of<T>(*h), s, (const double*)dphi, (const double*)du, st);
    }
    return src_dtype == LBM_DT_F32
               ? launch_init<T, S, float>(consts_of<T>(*h), s, (const float*)dphi, (const float*)du, st)
               : launch_init<T, S, double>(consts_of<T>(*h), s, (const double*)dphi, (const double*)du, st);
  });
  if (e != cudaSuccess) return fail(LBM_E_CUDA, std::string("lbm_init_fields: ") + cudaGetErrorString(e));
  if (direct) CUDA_TRY(cudaStreamSynchronize(st));
  h->initialized = true;
  h->desc_ok = false;
  h->raw = true;
  h->first = true;
  h->c_last = 0;
  h->steps = 0;
  h->last_raw_in = true;
  h->obs_init = true;
  return LBM_OK;
}

int lbm_step(LbmHandle* h, int nsteps, void* stream) {
  NvtxRange range("lbm_step");
  if (!h) return fail(LBM_E_ARG, "lbm_step: null handle");
  if (!h->initialized) return fail(LBM_E_STATE, "lbm_step: call lbm_init_fields first");
  if (nsteps < 0) return fail(LBM_E_ARG, "lbm_step: negative step count");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return with_types(h->prec, [&](auto tag) {
    return do_step<typename decltype(tag)::T, typename decltype(tag)::S>(h, nsteps, st);
  });
}

int lbm_step_profiled(LbmHandle* h, int nsteps, void* stream, float* kernel_ms3) {
  if (!h || !kernel_ms3) return fail(LBM_E_ARG, "lbm_step_profiled: null argument");
  if (!h->initialized) return fail(LBM_E_STATE, "lbm_step_profiled: call lbm_init_fields first");
  if (nsteps <= 0) return fail(LBM_E_ARG, "lbm_step_profiled: nsteps must be positive");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // events: before each step, between its phi and update kernels (before the
  // fused kernel), and after the last step
  std::vector<cudaEvent_t> ev(2 * (size_t)nsteps + 1, nullptr);
  for (auto& e : ev) CUDA_TRY(cudaEventCreate(&e));
  int rc = with_types(h->prec, [&](auto tag) {
    return do_step<typename decltype(tag)::T, typename decltype(tag)::S>(h, nsteps, st, ev.data());
  });
  float tot = 0.f, a = 0.f, b = 0.f;
  if (rc == LBM_OK) {
    cudaError_t e = cudaEventSynchronize(ev.back());
    if (e == cudaSuccess) e = cudaEventElapsedTime(&tot, ev.front(), ev.back());
    for (int i = 0; i < nsteps && e == cudaSuccess; ++i) {
      float x = 0.f, y = 0.f;
      e = cudaEventElapsedTime(&x, ev[2 * i], ev[2 * i + 1]);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&y, ev[2 * i + 1], ev[2 * i + 2]);
      a += x;
      b += y;
    }
    if (e != cudaSuccess) rc = fail(LBM_E_CUDA, std::string("lbm_step_profiled: ") + cudaGetErrorString(e));
  }
  for (auto& e : ev) cudaEventDestroy(e);
  kernel_ms3[0] = a;
  kernel_ms3[1] = b;
  kernel_ms3[2] = tot;
  return rc;
}

int lbm_set_tile(LbmHandle* h, int tx, int ty, int tz) {
  if (!h) return fail(LBM_E_ARG, "lbm_set_tile: null handle");
  if (is2d(h) && (tx || ty || tz)) return fail(LBM_E_UNSUPPORTED, "lbm_set_tile: 2-D grids run the per-node kernels only");
  if (tx == 1 || ty == 1 || tz == 1 || tx < 0 || ty < 0 || tz < 0 || tx > 64 || ty > 64 || tz > 256)
    return fail(LBM_E_ARG, "lbm_set_tile: tile extents must be in [2, 64] x [2, 64] x [2, 256] (0 = automatic)");
  Tiling t = make_tiling(h->nx, h->ny, h->nz, tx, ty, tz, h->prec);
  if (t.tx != 0 && h->mu)
    return fail(LBM_E_UNSUPPORTED, "lbm_set_tile: the gradient-of-mu modes run the two-kernel step only");
  if (tiling_smem(t, h->prec) > 220 * 1024) return fail(LBM_E_ARG, "lbm_set_tile: tile too large for shared memory");
  h->tiling = t;
  return LBM_OK;
}


int lbm_autotune(LbmHandle* h, int reps, void* stream, int* best_txyz3, float* best_ms) {
  if (!h) return fail(LBM_E_ARG, "lbm_autotune: null handle");
  if (is2d(h)) return fail(LBM_E_UNSUPPORTED, "lbm_autotune: 2-D grids have no launch parameters to tune");
  if (!h->initialized) return fail(LBM_E_STATE, "lbm_autotune: call lbm_init_fields first");
  if (reps <= 0) reps = 5;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t ub = 3 * (size_t)h->Np * h->tsize;
  void* u_save = nullptr;
  CUDA_TRY(cudaMalloc(&u_save, ub));
  CUDA_TRY(cudaMemcpyAsync(u_save, h->u, ub, cudaMemcpyDeviceToDevice, st));
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  // candidate tiles: z extents balanced over nz near 32 / 48 / 64, square
  // x-y cross-sections of 4..16 nodes, shared memory within a third of an SM
  std::vector<Tiling> cands;
  cands.push_back(make_tiling(h->nx, h->ny, h->nz, 0, 0, 0, h->prec));  // two-kernel step
  // (the gradient-of-mu modes have no fused-kernel form)
  for (int zt : {24, 32, 48, 64}) {
    if (h->mu) break;
    const int ntz = (int)((h->nz + zt - 1) / zt);
    const int tz = (int)((h->nz + ntz - 1) / ntz);
    for (int sx : {4, 5, 6, 8, 10, 12}) for (int sy : {4, 5, 6, 8, 10, 12}) {
      if (sy < sx - 2 || sy > sx + 2) continue;
      Tiling t = tiling_of(h->nx, h->ny, h->nz, sx, sy, tz);
      if (tiling_smem(t, h->prec) > smem_budget(h->prec)) continue;
      bool dup = false;
      for (const Tiling& c : cands) dup |= (c.tx == t.tx && c.ty == t.ty && c.tz == t.tz);
      if (!dup) cands.push_back(t);
    }
  }
  Tiling best = h->tiling;
  int best_per = h->phi_per_thread, best_bs = h->upd_block;
  float best_t = 1e30f;
  int rc = LBM_OK;
  for (const Tiling& t : cands) {
    // the two-kernel step: also its phi kernel's nodes per thread and the
    // update kernel's threads per block (256 only for the gradient-of-mu modes
    // and the paired layout, whose update kernel has a fixed block)
    const std::vector<int> pers =
        t.tx == 0 ? std::vector<int>{4, 8, 12, 16, 24, 32} : std::vector<int>{h->phi_per_thread};
    const std::vector<int> bss =
        (t.tx == 0 && !h->mu && !h->paired) ? std::vector<int>{128, kBlock} : std::vector<int>{h->upd_block};
    for (int bs : bss) {
      for (int per : pers) {
        if (per != h->phi_per_thread || bs != h->upd_block) {
          h->phi_per_thread = per;
          h->upd_block = bs;
          h->desc_ok = false;
        }
        float ms = 0.f;
        rc = with_types(h->prec, [&](auto tag) {
          return time_tiling<typename decltype(tag)::T, typename decltype(tag)::S>(h, t, reps, st, e0, e1, &ms);
        });
        if (rc != LBM_OK) break;
        if (ms < best_t) {
          best_t = ms;
          best = t;
          best_per = per;
          best_bs = bs;
        }
      }
      if (rc != LBM_OK) break;
    }
    if (rc != LBM_OK) break;
  }
  if (h->phi_per_thread != best_per || h->upd_block != best_bs) {
    h->phi_per_thread = best_per;
    h->upd_block = best_bs;
    h->desc_ok = false;
  }
  cudaMemcpyAsync(h->u, u_save, ub, cudaMemcpyDeviceToDevice, st);
  cudaStreamSynchronize(st);
  cudaFree(u_save);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != LBM_OK) return rc;
  h->tiling = best;
  if (best_txyz3) {
    best_txyz3[0] = best.tx;
    best_txyz3[1] = best.ty;
    best_txyz3[2] = best.tz;
  }
  if (best_ms) *best_ms = best_t / reps;
  return LBM_OK;
}

int lbm_set_layout(LbmHandle* h, int paired) {
  if (!h) return fail(LBM_E_ARG, "lbm_set_layout: null handle");
  if (paired != 0 && paired != 1) return fail(LBM_E_ARG, "lbm_set_layout: paired must be 0 or 1");
  if (h->initialized) return fail(LBM_E_STATE, "lbm_set_layout: call before lbm_init_fields");
  if (paired && (is2d(h) || h->nx % 2 != 0 || h->prec == LBM_F64))
    return fail(LBM_E_UNSUPPORTED, "lbm_set_layout: the paired layout needs a 3-D grid with even nx in LBM_F32 or "
                                   "LBM_F16");
  h->paired = paired != 0;
  h->kf.nh = h->paired ? (int)(h->N / 2) : 0;
  h->kf.hx = h->paired ? (int)(h->nx / 2) : 0;
  h->desc_ok = false;
  return LBM_OK;
}

int lbm_get_layout(LbmHandle* h, int* paired) {
  if (!h || !paired) return fail(LBM_E_ARG, "lbm_get_layout: null argument");
  *paired = h->paired ? 1 : 0;
  return LBM_OK;
}

int lbm_set_launch(LbmHandle* h, int phi_nodes_per_thread, int update_block) {
  if (!h) return fail(LBM_E_ARG, "lbm_set_launch: null handle");
  if (phi_nodes_per_thread < 1 || phi_nodes_per_thread > 64)
    return fail(LBM_E_ARG, "lbm_set_launch: phi_nodes_per_thread must be in [1, 64]");
  if (update_block != 128 && update_block != kBlock)
    return fail(LBM_E_ARG, "lbm_set_launch: update_block must be 128 or 256");
  if (update_block != kBlock && h->mu)
    return fail(LBM_E_UNSUPPORTED, "lbm_set_launch: the gradient-of-mu modes run 256-thread update blocks");
  h->phi_per_thread = phi_nodes_per_thread;
  h->upd_block = update_block;
  h->desc_ok = false;
  return LBM_OK;
}

int lbm_get_launch(LbmHandle* h, int* phi_nodes_per_thread, int* update_block) {
  if (!h) return fail(LBM_E_ARG, "lbm_get_launch: null handle");
  if (phi_nodes_per_thread) *phi_nodes_per_thread = h->phi_per_thread;
  if (update_block) *update_block = h->paired ? kPairUpdBlock : h->upd_block;
  return LBM_OK;
}

int lbm_get_tile(LbmHandle* h, int* txyz3) {
  if (!h || !txyz3) return fail(LBM_E_ARG, "lbm_get_tile: null argument");
  txyz3[0] = h->tiling.tx;
  txyz3[1] = h->tiling.ty;
  txyz3[2] = h->tiling.tz;
  return LBM_OK;
}

int lbm_get_fields(LbmHandle* h, uint32_t mask, void* phi, void* rho, void* u, void* P, void* p, void* mu,
                   void* stream) {
  if (!h) return fail(LBM_E_ARG, "lbm_get_fields: null handle");
  if (!h->initialized) return fail(LBM_E_STATE, "lbm_get_fields: not initialised");
  if (((mask & LBM_FIELD_PHI) && !phi) || ((mask & LBM_FIELD_RHO) && !rho) || ((mask & LBM_FIELD_U) && !u) ||
      ((mask & LBM_FIELD_P) && !P) || ((mask & LBM_FIELD_PRESS) && !p) || ((mask & LBM_FIELD_MU) && !mu))
    return fail(LBM_E_ARG, "lbm_get_fields: selected output is null");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int mode = h->obs_init ? 0 : 1;
  const int in_buf = h->obs_init ? h->cur : (h->cur ^ 1);  // the last step's input buffer
  cudaError_t e;
  // phi_out of the state = the latest recovered phi
  e = with_types(h->prec, [&](auto tag) {
    using T = typename decltype(tag)::T;
    using S = typename decltype(tag)::S;
    State<T, S> s = make_state<T, S>(*h, in_buf, h->pc ^ 1);
    s.c_cur = h->c_last;
    if constexpr (sizeof(S) == sizeof(T)) {
      if (is2d(h))
        return launch_observe2d<T>(consts_of<T>(*h), s, h->last_raw_in, mask, mode, (T*)phi, (T*)rho, (T*)u,
                                   (T*)P, (T*)p, (T*)mu, st);
    }
    return launch_observe<T, S>(consts_of<T>(*h), s, h->last_raw_in, mask, mode, (T*)phi, (T*)rho, (T*)u,
                                (T*)P, (T*)p, (T*)mu, st);
  });
  if (e != cudaSuccess) return fail(LBM_E_CUDA, std::string("lbm_get_fields: ") + cudaGetErrorString(e));
  return LBM_OK;
}

int lbm_inject_droplet(LbmHandle* h, const double* center3, double radius, double xi, const double* u_impact3,
                       int64_t* core_nodes, void* stream) {
  if (!h || !center3) return fail(LBM_E_ARG, "lbm_inject_droplet: null argument");
  if (!h->initialized) return fail(LBM_E_STATE, "lbm_inject_droplet: call lbm_init_fields first");
  if (!(radius >= 0.0) || !(xi > 0.0)) return fail(LBM_E_ARG, "lbm_inject_droplet: radius >= 0 and xi > 0 required");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  InjectParams ip;
  std::memset(&ip, 0, sizeof(ip));
  for (int d = 0; d < 3; ++d) {
    ip.c[d] = center3[d];
    ip.u[d] = u_impact3 ? u_impact3[d] : 0.0;
  }
  ip.radius = radius;
  ip.xi = xi;
  ip.obs_init = h->obs_init ? 1 : 0;
  CUDA_TRY(cudaMemsetAsync(h->counters + 3, 0, sizeof(unsigned), st));
  cudaError_t e = with_types(h->prec, [&](auto tag) {
    using T = typename decltype(tag)::T;
    using S = typename decltype(tag)::S;
    const Consts<T>& k = consts_of<T>(*h);
    cudaError_t r = cudaSuccess;
    if (!h->obs_init) {
      // the P attribute: the pressure of the last step, into the measure scratch
      State<T, S> so = make_state<T, S>(*h, h->cur ^ 1, h->pc ^ 1);
      so.c_cur = h->c_last;
      if constexpr (sizeof(S) == sizeof(T)) {
        if (is2d(h))
          r = launch_observe2d<T>(k, so, h->last_raw_in, LBM_FIELD_P, 1, nullptr, nullptr, nullptr,
                                  static_cast<T*>(h->meas_phi), nullptr, nullptr, st);
        else
          r = launch_observe<T, S>(k, so, h->last_raw_in, LBM_FIELD_P, 1, nullptr, nullptr, nullptr,
                                   static_cast<T*>(h->meas_phi), nullptr, nullptr, st);
      } else {
        r = launch_observe<T, S>(k, so, h->last_raw_in, LBM_FIELD_P, 1, nullptr, nullptr, nullptr,
                                 static_cast<T*>(h->meas_phi), nullptr, nullptr, st);
      }
      if (r != cudaSuccess) return r;
    }
    State<T, S> s = make_state<T, S>(*h, h->cur, h->pc);
    s.c_prev = h->c_last;
    if constexpr (sizeof(S) == sizeof(T)) {
      if (is2d(h))
        return launch_inject2d<T>(k, s, h->raw, ip, static_cast<const T*>(h->meas_phi), h->counters + 3, st);
    }
    return launch_inject<T, S>(k, s, h->raw, ip, static_cast<const T*>(h->meas_phi), h->counters + 3, st);
  });
  if (e != cudaSuccess) return fail(LBM_E_CUDA, std::string("lbm_inject_droplet: ") + cudaGetErrorString(e));
  // the injected state is raw (read in place) and has no previous phi u
  h->cur ^= 1;
  h->pc ^= 1;
  h->raw = true;
  h->first = true;
  h->obs_init = true;
  h->last_raw_in = true;
  h->desc_ok = false;
  if (core_nodes) {
    unsigned cnt = 0;
    CUDA_TRY(cudaMemcpyAsync(&cnt, h->counters + 3, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    *core_nodes = cnt;
  }
  return LBM_OK;
}

int lbm_get_populations(LbmHandle* h, void* f, void* g, void* stream) {
  if (!h) return fail(LBM_E_ARG, "lbm_get_populations: null handle");
  if (!h->initialized) return fail(LBM_E_STATE, "lbm_get_populations: not initialised");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  // fin = the current state, phi_in = the latest phi, c_prev = its correction
  e = with_types(h->prec, [&](auto tag) {
    using T = typename decltype(tag)::T;
    using S = typename decltype(tag)::S;
    State<T, S> s = make_state<T, S>(*h, h->cur, h->pc);
    s.c_prev = h->c_last;
    if constexpr (sizeof(S) == sizeof(T)) {
      if (is2d(h)) return launch_populations2d<T>(consts_of<T>(*h), s, h->raw, (T*)f, (T*)g, st);
    }
    return launch_populations<T, S>(consts_of<T>(*h), s, h->raw, (T*)f, (T*)g, st);
  });
  if (e != cudaSuccess) return fail(LBM_E_CUDA, std::string("lbm_get_populations: ") + cudaGetErrorString(e));
  return LBM_OK;
}

int lbm_get_geometry(LbmHandle* h, uint8_t* node_class, uint8_t* is_boundary, float* wall_normal,
                     float* wall_weight, uint8_t* near_wall, uint8_t* partial) {
  if (!h) return fail(LBM_E_ARG, "lbm_get_geometry: null handle");
  if (!h->geometry_set) return fail(LBM_E_STATE, "lbm_get_geometry: no geometry");
  const size_t N = (size_t)h->N;
  // the device tables: the class byte carries the solid / boundary / partial
  // bits and the near-wall distance code, from which the other tables follow
  CUDA_TRY(cudaDeviceSynchronize());
  const int rc = class_table_host(h);
  if (rc != LBM_OK) return rc;
  const uint8_t* c = h->cls_host.data();
  if (node_class) std::memcpy(node_class, c, N);
  if (wall_normal) CUDA_TRY(cudaMemcpy(wall_normal, h->wn, ndim_of(h->nz) * N * sizeof(float), cudaMemcpyDeviceToHost));
  float lut[kWwCodes];
  near_wall_weights(lut);
  for (size_t n = 0; n < N; ++n) {
    const uint8_t v = c[n];
    const int code = v >> kWwShift;
    if (is_boundary) is_boundary[n] = (v & kBoundary) ? 1 : 0;
    if (partial) partial[n] = (v & kPartial) ? 1 : 0;
    // weight exp(-d / 2.5) of the near-wall distance, 0 in solid and
    // everywhere without wetting; near-wall where d < 10 (fe_wetting.py:295-303)
    if (wall_weight) wall_weight[n] = h->wetting ? lut[code] : 0.0f;
    if (near_wall) near_wall[n] = (!(v & kSolid) && code < 10) ? 1 : 0;
  }
  return LBM_OK;
}

int lbm_geometry_host(int64_t nx, int64_t ny, int64_t nz, const uint8_t* solid, const void* fraction,
                      int fraction_dtype, double theta_eq, double kappa, int precision, uint8_t* node_class,
                      uint8_t* is_boundary, float* wall_normal, float* wall_weight, uint8_t* near_wall,
                      uint8_t* partial) {
  if (!solid) return fail(LBM_E_ARG, "lbm_geometry_host: null solid");
  if (nx < 2 || ny < 2 || nz < 1)
    return fail(LBM_E_UNSUPPORTED, "lbm_geometry_host: 3-D grids with every extent >= 2, or 2-D grids (nz == 1) only");
  if (fraction_dtype < 0 || fraction_dtype > 2 || ((fraction_dtype != 0) != (fraction != nullptr)))
    return fail(LBM_E_ARG, "lbm_geometry_host: fraction and fraction_dtype disagree");
  Geometry g;
  compute_geometry(nx, ny, nz, solid, fraction, fraction_dtype, theta_eq != 90.0 && kappa > 0,
                   precision == LBM_F64, g);
  const size_t N = (size_t)(nx * ny * nz);
  if (node_class) std::memcpy(node_class, g.cls.data(), N);
  if (is_boundary) std::memcpy(is_boundary, g.boundary.data(), N);
  if (wall_normal) std::memcpy(wall_normal, g.wall_normal.data(), ndim_of(nz) * N * sizeof(float));
  if (wall_weight) std::memcpy(wall_weight, g.wall_weight.data(), N * sizeof(float));
  if (near_wall) std::memcpy(near_wall, g.near_wall.data(), N);
  if (partial) std::memcpy(partial, g.partial.data(), N);
  return LBM_OK;
}

int lbm_get_scalars(LbmHandle* h, double* phi_mass_init, double* last_sum_phi, double* last_correction,
                    int64_t* step_count) {
  if (!h) return fail(LBM_E_ARG, "lbm_get_scalars: null handle");
  double sc[2] = {0.0, 0.0};
  if (h->initialized) CUDA_TRY(cudaMemcpy(sc, h->scal, 2 * sizeof(double), cudaMemcpyDeviceToHost));
  if (phi_mass_init) *phi_mass_init = sc[0];
  if (last_sum_phi) *last_sum_phi = sc[1];
  if (last_correction) {
    double c = 1.0;
    if (h->initialized && h->steps > 0) {
      if (h->prec != LBM_F64) {
        float v;
        CUDA_TRY(cudaMemcpy(&v, static_cast<float*>(h->cbuf) + h->c_last, sizeof(float), cudaMemcpyDeviceToHost));
        c = v;
      } else {
        CUDA_TRY(cudaMemcpy(&c, static_cast<double*>(h->cbuf) + h->c_last, sizeof(double), cudaMemcpyDeviceToHost));
      }
    }
    *last_correction = c;
  }
  if (step_count) *step_count = h->steps;
  return LBM_OK;
}

int lbm_measure(LbmHandle* h, double* out9, void* stream) {
  NvtxRange range("lbm_measure");
  if (!h || !out9) return fail(LBM_E_ARG, "lbm_measure: null argument");
  if (!h->initialized) return fail(LBM_E_STATE, "lbm_measure: not initialised");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = lbm_get_fields(h, LBM_FIELD_PHI, h->meas_phi, nullptr, nullptr, nullptr, nullptr, nullptr, stream);
  if (rc) return rc;
  cudaError_t e;
  int mx, my, mz;
  measure_grid(h, &mx, &my, &mz);
  if (h->prec != LBM_F64)
    e = launch_measure<float>(mx, my, mz, (const float*)h->meas_phi, h->cls, h->partials, kMeasureBlocks,
                              h->counters + 1, h->scal + 2, st);
  else
    e = launch_measure<double>(mx, my, mz, (const double*)h->meas_phi, h->cls, h->partials, kMeasureBlocks,
                               h->counters + 1, h->scal + 2, st);
  if (e != cudaSuccess) return fail(LBM_E_CUDA, std::string("lbm_measure: ") + cudaGetErrorString(e));
  CUDA_TRY(cudaMemcpyAsync(out9, h->scal + 2, 9 * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (is2d(h)) remap_measure2d(out9, nullptr);
  return LBM_OK;
}

// ---------------------------------------------------------------------------
// Checkpoints: the complete time-stepping state of a handle as one host blob
// ---------------------------------------------------------------------------
namespace {
constexpr uint32_t kStateMagic = 0x534d424cu;  // "LBMS"
constexpr uint32_t kStateVersion = 1;

struct StateHeader {
  uint32_t magic, version;
  int64_t nx, ny, nz;
  int32_t prec, cur, pc, c_last;
  int32_t raw, first, last_raw_in, obs_init;
  int64_t steps;
  uint64_t geometry_hash;  // FNV-1a of the node-class table (the geometry the state belongs to)
  uint32_t status;
  uint32_t layout;  // 1: paired storage layout, 0: linear
};

uint64_t fnv1a(const uint8_t* p, size_t n) {
  uint64_t x = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) x = (x ^ p[i]) * 1099511628211ull;
  return x;
}

// Device arrays of a checkpoint, in blob order: f and g of the current
// buffer, g of the other buffer, u, both phi buffers, the two
// mass-correction factors, the scalars.
struct StatePart {
  void* dev;
  size_t bytes;
};
std::vector<StatePart> state_parts(LbmHandle* h) {
  const size_t pop = (size_t)nq_of(h->nz) * h->Np * h->psize;
  // g of the last step's input buffer: the pressure read-out after a step sums it
  return {{h->f[h->cur], pop},
          {h->g[h->cur], pop},
          {h->g[h->cur ^ 1], pop},
          {h->u, 3 * (size_t)h->Np * h->tsize},
          {h->phi[0], (size_t)h->Np * h->tsize},
          {h->phi[1], (size_t)h->Np * h->tsize},
          {h->cbuf, 2 * h->tsize},
          {h->scal, 2 * sizeof(double)}};
}
size_t state_bytes(LbmHandle* h) {
  size_t b = sizeof(StateHeader);
  for (const StatePart& p : state_parts(h)) b += p.bytes;
  return b;
}
}  // namespace

int lbm_state_bytes(LbmHandle* h, int64_t* bytes) {
  if (!h || !bytes) return fail(LBM_E_ARG, "lbm_state_bytes: null argument");
  *bytes = (int64_t)state_bytes(h);
  return LBM_OK;
}

int lbm_save_state(LbmHandle* h, void* host, int64_t bytes, void* stream) {
  if (!h || !host) return fail(LBM_E_ARG, "lbm_save_state: null argument");
  if (!h->initialized) return fail(LBM_E_STATE, "lbm_save_state: call lbm_init_fields first");
  if (bytes != (int64_t)state_bytes(h)) return fail(LBM_E_ARG, "lbm_save_state: buffer size is not lbm_state_bytes");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  StateHeader hd;
  std::memset(&hd, 0, sizeof(hd));
  hd.magic = kStateMagic;
  hd.version = kStateVersion;
  hd.nx = h->nx;
  hd.ny = h->ny;
  hd.nz = h->nz;
  hd.prec = h->prec;
  hd.cur = h->cur;
  hd.pc = h->pc;
  hd.c_last = h->c_last;
  hd.raw = h->raw;
  hd.first = h->first;
  hd.last_raw_in = h->last_raw_in;
  hd.obs_init = h->obs_init;
  hd.steps = h->steps;
  {
    const int rc = class_table_host(h);
    if (rc != LBM_OK) return rc;
  }
  hd.geometry_hash = fnv1a(h->cls_host.data(), h->cls_host.size());
  hd.layout = h->paired ? 1u : 0u;
  CUDA_TRY(cudaMemcpyAsync(&hd.status, h->counters + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  char* out = static_cast<char*>(host) + sizeof(StateHeader);
  for (const StatePart& p : state_parts(h)) {
    CUDA_TRY(cudaMemcpyAsync(out, p.dev, p.bytes, cudaMemcpyDeviceToHost, st));
    out += p.bytes;
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  std::memcpy(host, &hd, sizeof(hd));
  return LBM_OK;
}

int lbm_load_state(LbmHandle* h, const void* host, int64_t bytes, void* stream) {
  if (!h || !host) return fail(LBM_E_ARG, "lbm_load_state: null argument");
  if (!h->geometry_set) return fail(LBM_E_STATE, "lbm_load_state: call lbm_set_geometry first");
  if (bytes < (int64_t)sizeof(StateHeader)) return fail(LBM_E_ARG, "lbm_load_state: buffer too small");
  StateHeader hd;
  std::memcpy(&hd, host, sizeof(hd));
  if (hd.magic != kStateMagic || hd.version != kStateVersion)
    return fail(LBM_E_ARG, "lbm_load_state: not a state written by lbm_save_state (bad magic or version)");
  if (hd.nx != h->nx || hd.ny != h->ny || hd.nz != h->nz || hd.prec != h->prec)
    return fail(LBM_E_ARG, "lbm_load_state: the state belongs to a different grid or precision");
  {
    const int rc = class_table_host(h);
    if (rc != LBM_OK) return rc;
  }
  if (hd.geometry_hash != fnv1a(h->cls_host.data(), h->cls_host.size()))
    return fail(LBM_E_ARG, "lbm_load_state: the state belongs to a different geometry");
  if (hd.layout != (h->paired ? 1u : 0u))
    return fail(LBM_E_ARG, "lbm_load_state: the state was written in the other storage layout (lbm_set_layout)");
  if (bytes != (int64_t)state_bytes(h)) return fail(LBM_E_ARG, "lbm_load_state: buffer size is not lbm_state_bytes");
  if ((hd.cur & ~1) || (hd.pc & ~1) || (hd.c_last & ~1) || hd.steps < 0)
    return fail(LBM_E_ARG, "lbm_load_state: corrupt header");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // queued steps may still read the buffers about to be overwritten
  CUDA_TRY(cudaStreamSynchronize(st));
  h->cur = hd.cur;
  h->pc = hd.pc;
  h->c_last = hd.c_last;
  const char* in = static_cast<const char*>(host) + sizeof(StateHeader);
  for (const StatePart& p : state_parts(h)) {
    CUDA_TRY(cudaMemcpyAsync(p.dev, in, p.bytes, cudaMemcpyHostToDevice, st));
    in += p.bytes;
  }
  CUDA_TRY(cudaMemcpyAsync(h->counters + 2, &hd.status, sizeof(unsigned), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  h->raw = hd.raw != 0;
  h->first = hd.first != 0;
  h->last_raw_in = hd.last_raw_in != 0;
  h->obs_init = hd.obs_init != 0;
  h->steps = hd.steps;
  h->initialized = true;
  h->desc_ok = false;
  return LBM_OK;
}

int lbm_reduce(LbmHandle* h, double* sum_phi, double* mom3, int32_t* extents6, float* cmax, void* stream) {
  NvtxRange range("lbm_reduce");
  if (!h) return fail(LBM_E_ARG, "lbm_reduce: null handle");
  if (!h->initialized) return fail(LBM_E_STATE, "lbm_reduce: not initialised");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = lbm_get_fields(h, LBM_FIELD_PHI, h->meas_phi, nullptr, nullptr, nullptr, nullptr, nullptr, stream);
  if (rc) return rc;
  const int N = (int)h->N, us = (int)h->Np;
  int nx, ny, nz;
  measure_grid(h, &nx, &ny, &nz);
  cudaError_t e;
  if (h->prec != LBM_F64) {
    e = launch_measure<float>(nx, ny, nz, (const float*)h->meas_phi, h->cls, h->partials, kMeasureBlocks,
                              h->counters + 1, h->scal + 2, st, h->scal + 16);
    if (e == cudaSuccess)
      e = launch_momentum<float>(N, (const float*)h->meas_phi, (const float*)h->u, us, h->kf.nh, h->prm.rho_l,
                                 h->prm.rho_g, h->partials, kMeasureBlocks, h->counters + 4, h->scal + 24, st);
  } else {
    e = launch_measure<double>(nx, ny, nz, (const double*)h->meas_phi, h->cls, h->partials, kMeasureBlocks,
                               h->counters + 1, h->scal + 2, st, h->scal + 16);
    if (e == cudaSuccess)
      e = launch_momentum<double>(N, (const double*)h->meas_phi, (const double*)h->u, us, h->kd.nh, h->prm.rho_l,
                                  h->prm.rho_g, h->partials, kMeasureBlocks, h->counters + 4, h->scal + 24, st);
  }
  if (e != cudaSuccess) return fail(LBM_E_CUDA, std::string("lbm_reduce: ") + cudaGetErrorString(e));
  double r[25];
  CUDA_TRY(cudaMemcpyAsync(r, h->scal + 2, sizeof(r), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (is2d(h)) remap_measure2d(r, r + 14);
  if (sum_phi) *sum_phi = r[0];
  if (cmax) *cmax = (float)r[1];
  if (extents6)
    for (int j = 0; j < 6; ++j) extents6[j] = (int32_t)r[14 + j];
  if (mom3)
    for (int d = 0; d < 3; ++d) mom3[d] = r[22 + d];
  return LBM_OK;
}

int lbm_status(LbmHandle* h, uint32_t* flags) {
  if (!h || !flags) return fail(LBM_E_ARG, "lbm_status: null argument");
  unsigned v = 0;
  CUDA_TRY(cudaMemcpy(&v, h->counters + 2, sizeof(unsigned), cudaMemcpyDeviceToHost));
  *flags = v;
  return LBM_OK;
}

}  // extern "C"

int lbm_measure_static(int64_t nx, int64_t ny, int64_t nz, const void* phi, int phi_dtype,
                       const uint8_t* solid, double* out9, void* stream) {
  if (!phi || !solid || !out9) return fail(LBM_E_ARG, "lbm_measure_static: null argument");
  if (nx < 1 || ny < 1 || nz < 1) return fail(LBM_E_ARG, "lbm_measure_static: grid extents must be >= 1");
  if (nx > LBM_MEASURE_STATIC_MAX_NODES || ny > LBM_MEASURE_STATIC_MAX_NODES ||
      nz > LBM_MEASURE_STATIC_MAX_NODES || nx * ny > LBM_MEASURE_STATIC_MAX_NODES ||
      nx * ny * nz > LBM_MEASURE_STATIC_MAX_NODES)
    return fail(LBM_E_ARG, "lbm_measure_static: " + std::to_string(nx) + "x" + std::to_string(ny) + "x" +
                               std::to_string(nz) + " exceeds the maximum of " +
                               std::to_string((long long)LBM_MEASURE_STATIC_MAX_NODES) + " nodes");
  if (phi_dtype != LBM_DT_F32 && phi_dtype != LBM_DT_F64)
    return fail(LBM_E_ARG, "lbm_measure_static: phi_dtype must be LBM_DT_F32 or LBM_DT_F64");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (phi_dtype == LBM_DT_F32)
    e = launch_measure_static<float>((int)nx, (int)ny, (int)nz, (const float*)phi, solid, out9, st);
  else
    e = launch_measure_static<double>((int)nx, (int)ny, (int)nz, (const double*)phi, solid, out9, st);
  if (e != cudaSuccess) return fail(LBM_E_CUDA, std::string("lbm_measure_static: ") + cudaGetErrorString(e));
  return LBM_OK;
}

// ---------------------------------------------------------------------------
// Batches of independent grids (one launch per kernel per step for all)
// ---------------------------------------------------------------------------
struct LbmBatch {
  std::vector<LbmHandle*> h;  // launch order: the cases with omega_f == 1 first
  int prec = LBM_F32;
  int device = 0;
  // cases in launch groups: [gstart[g], gstart[g + 1]) for g = 0 linear layout
  // with omega_f == 1, 1 linear other, 2 paired layout with omega_f == 1, 3 paired other
  int gstart[5] = {0, 0, 0, 0, 0};
  int phi_per_thread = 16;  // nodes per phi-kernel thread (half as many pairs in the paired layout)
  int upd_block = kBlock;   // threads per block of the linear-layout update kernel
  bool coop = false;        // one cooperative launch per step (k_batch_coop) instead of two launches
  size_t desc = 0;          // bytes of one case descriptor
  void* table[2] = {nullptr, nullptr};  // device descriptors: [0] this step, [1] the next
  unsigned char* staging = nullptr;     // pinned host copy of both tables
  cudaEvent_t staged = nullptr;         // the last copy out of `staging` has run
  // block -> case: the phi grids of the linear and the paired cases, then the
  // update grids of the four groups
  unsigned short* b2c = nullptr;
  int phi_blocks[2] = {0, 0}, upd_blocks[4] = {0, 0, 0, 0};
  cudaStream_t cap = nullptr;           // stream used to capture the two-step graph
  cudaGraphExec_t graph = nullptr;
};

namespace {

int launch_group(const LbmHandle* h) { return (h->paired ? 2 : 0) + (omega1_of(h) ? 0 : 1); }

// Block -> case tables (device) for the current phi_per_thread; drops the graph.
int batch_layout(LbmBatch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  if (b->b2c) cudaFree(b->b2c);
  b->b2c = nullptr;
  const int n = (int)b->h.size();
  long long pb[2] = {0, 0}, ub[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    pb[b->h[i]->paired ? 1 : 0] += phi_blocks_of(b->h[i], b->phi_per_thread);
    ub[launch_group(b->h[i])] += upd_blocks_of(b->h[i], b->upd_block);
  }
  const long long tot = pb[0] + pb[1] + ub[0] + ub[1] + ub[2] + ub[3];
  if (tot > 0x7fffffff) return fail(LBM_E_ARG, "lbm_batch: grids too large");
  for (int j = 0; j < 2; ++j) b->phi_blocks[j] = (int)pb[j];
  for (int g = 0; g < 4; ++g) b->upd_blocks[g] = (int)ub[g];
  std::vector<unsigned short> t((size_t)tot);
  size_t at[6];
  at[0] = 0;
  at[1] = (size_t)pb[0];
  at[2] = at[1] + (size_t)pb[1];
  for (int g = 0; g < 3; ++g) at[3 + g] = at[2 + g] + (size_t)ub[g];
  for (int i = 0; i < n; ++i) {
    size_t& a = at[b->h[i]->paired ? 1 : 0];
    for (int k = phi_blocks_of(b->h[i], b->phi_per_thread); k > 0; --k) t[a++] = (unsigned short)i;
    size_t& c = at[2 + launch_group(b->h[i])];
    for (int k = upd_blocks_of(b->h[i], b->upd_block); k > 0; --k) t[c++] = (unsigned short)i;
  }
  CUDA_TRY(cudaMalloc(&b->b2c, t.size() * sizeof(unsigned short)));
  CUDA_TRY(cudaMemcpy(b->b2c, t.data(), t.size() * sizeof(unsigned short), cudaMemcpyHostToDevice));
  return LBM_OK;
}

// Descriptors of every case for this step (parity 0) and the next (parity 1).
template <typename T, typename S>
void batch_fill_t(LbmBatch* b) {
  const int n = (int)b->h.size();
  int pb[2] = {0, 0}, ub[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    LbmHandle* h = b->h[i];
    const int phin = phi_blocks_of(h, b->phi_per_thread), updn = upd_blocks_of(h, b->upd_block),
              g = launch_group(h);
    int& pbl = pb[h->paired ? 1 : 0];
    for (int par = 0; par < 2; ++par) {
      State<T, S> s = make_state<T, S>(*h, h->cur ^ par, h->pc ^ par);
      s.c_prev = h->c_last ^ par;
      s.c_cur = h->c_last ^ par ^ 1;
      fill_case_desc<T, S>(b->staging + ((size_t)par * n + i) * b->desc, consts_of<T>(*h), s, pbl, phin, ub[g],
                           updn);
    }
    pbl += phin;
    ub[g] += updn;
  }
}

int batch_fill(LbmBatch* b, cudaStream_t st) {
  // the previous copy out of the staging buffer must have run before it is rewritten
  CUDA_TRY(cudaEventSynchronize(b->staged));
  with_types(b->prec, [&](auto tag) {
    batch_fill_t<typename decltype(tag)::T, typename decltype(tag)::S>(b);
    return 0;
  });
  const size_t bytes = b->h.size() * b->desc;
  CUDA_TRY(cudaMemcpyAsync(b->table[0], b->staging, bytes, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(b->table[1], b->staging + bytes, bytes, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaEventRecord(b->staged, st));
  return LBM_OK;
}

// One batched step reading descriptor table `par`: the phi kernel over every
// linear-layout case and over every paired case, then the update kernel over
// each group (layout x omega_f == 1 or not).  Empty launches are skipped.
template <typename T, typename S>
cudaError_t batch_launch_t(LbmBatch* b, int par, cudaStream_t st) {
  if (b->coop)
    return launch_batch_coop<T, S>(b->table[par], b->b2c, b->phi_blocks[0], b->upd_blocks[0], b->upd_blocks[1], st);
  const unsigned short* t = b->b2c;
  cudaError_t e = cudaSuccess;
  for (int j = 0; j < 2 && e == cudaSuccess; ++j) {
    e = launch_phi_kernel<T, S>(j == 1, b->table[par], t, b->phi_blocks[j], st);
    t += b->phi_blocks[j];
  }
  for (int g = 0; g < 4 && e == cudaSuccess; ++g) {
    e = launch_update_kernel<T, S>(g >= 2, b->table[par], t, b->upd_blocks[g], (g & 1) == 0, st, false,
                                   b->upd_block);
    t += b->upd_blocks[g];
  }
  return e;
}
cudaError_t batch_launch(LbmBatch* b, int par, cudaStream_t st) {
  return with_types(b->prec, [&](auto tag) {
    return batch_launch_t<typename decltype(tag)::T, typename decltype(tag)::S>(b, par, st);
  });
}

// The two-step graph (table 0, then table 1), captured on the batch's own stream.
int batch_graph(LbmBatch* b) {
  if (b->graph) return LBM_OK;
  cudaGraph_t g = nullptr;
  CUDA_TRY(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = batch_launch(b, 0, b->cap);
  if (e == cudaSuccess) e = batch_launch(b, 1, b->cap);
  const cudaError_t e2 = cudaStreamEndCapture(b->cap, &g);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    b->graph = nullptr;
    return fail(LBM_E_CUDA, std::string("lbm_batch: graph capture: ") + cudaGetErrorString(e));
  }
  return LBM_OK;
}

void batch_advance(LbmBatch* b, int nsteps) {
  for (LbmHandle* h : b->h) {
    if (nsteps & 1) {
      h->cur ^= 1;
      h->pc ^= 1;
      h->c_last ^= 1;
    }
    h->steps += nsteps;
    h->last_raw_in = false;
    h->obs_init = false;
  }
}

}  // namespace

extern "C" {

int lbm_batch_create(LbmHandle* const* handles, int n, LbmBatch** out) {
  if (!handles || !out || n < 1) return fail(LBM_E_ARG, "lbm_batch_create: need at least one handle");
  *out = nullptr;
  if (n > 65535) return fail(LBM_E_ARG, "lbm_batch_create: at most 65535 cases");
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  for (int i = 0; i < n; ++i) {
    const LbmHandle* h = handles[i];
    if (!h || h->prec != handles[0]->prec || h->device != dev || !h->geometry_set)
      return fail(LBM_E_ARG, "lbm_batch_create: handles must share the precision and the current device and have "
                             "their geometry set");
    for (int j = 0; j < i; ++j)
      if (handles[j] == h) return fail(LBM_E_ARG, "lbm_batch_create: a handle appears twice");
    if (h->mu)
      return fail(LBM_E_UNSUPPORTED, "lbm_batch_create: the gradient-of-mu modes (cahn-hilliard, mu_drive) step "
                                     "one grid at a time");
    if (is2d(h)) return fail(LBM_E_UNSUPPORTED, "lbm_batch_create: 2-D grids step one grid at a time");
  }
  LbmBatch* b = new (std::nothrow) LbmBatch();
  if (!b) return fail(LBM_E_ARG, "lbm_batch_create: out of host memory");
  b->prec = handles[0]->prec;
  b->device = dev;
  for (int g = 0; g < 4; ++g) {
    b->gstart[g] = (int)b->h.size();
    for (int i = 0; i < n; ++i)
      if (launch_group(handles[i]) == g) b->h.push_back(handles[i]);
  }
  b->gstart[4] = (int)b->h.size();
  b->desc = with_types(b->prec, [&](auto tag) {
    return case_desc_bytes<typename decltype(tag)::T, typename decltype(tag)::S>();
  });
  cudaError_t e = cudaMalloc(&b->table[0], n * b->desc);
  if (e == cudaSuccess) e = cudaMalloc(&b->table[1], n * b->desc);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&b->staging, 2 * n * b->desc);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->staged, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(b->staged, 0);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    lbm_batch_destroy(b);
    return fail(LBM_E_CUDA, std::string("lbm_batch_create: ") + cudaGetErrorString(e));
  }
  const int rc = batch_layout(b);
  if (rc != LBM_OK) {
    lbm_batch_destroy(b);
    return rc;
  }
  *out = b;
  return LBM_OK;
}

int lbm_batch_destroy(LbmBatch* b) {
  if (!b) return LBM_OK;
  if (b->staged) cudaEventSynchronize(b->staged);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->b2c) cudaFree(b->b2c);
  if (b->table[0]) cudaFree(b->table[0]);
  if (b->table[1]) cudaFree(b->table[1]);
  if (b->staging) cudaFreeHost(b->staging);
  if (b->staged) cudaEventDestroy(b->staged);
  if (b->cap) cudaStreamDestroy(b->cap);
  delete b;
  return LBM_OK;
}

int lbm_batch_step(LbmBatch* b, int nsteps, void* stream) {
  NvtxRange range("lbm_batch_step");
  if (!b) return fail(LBM_E_ARG, "lbm_batch_step: null batch");
  if (nsteps < 0) return fail(LBM_E_ARG, "lbm_batch_step: nsteps must be >= 0");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  bool any_first = false;
  for (LbmHandle* h : b->h) {
    if (!h->initialized) return fail(LBM_E_STATE, "lbm_batch_step: a case is not initialised");
    any_first |= h->raw || h->first;
  }
  int rest = nsteps;
  if (any_first && rest > 0) {
    // a case in its first step after init reads its populations in place:
    // every case takes this step through the single-grid kernels (the same
    // arithmetic), the rest run batched
    for (LbmHandle* h : b->h) {
      const int rc = lbm_step(h, 1, stream);
      if (rc != LBM_OK) return rc;
    }
    --rest;
  }
  if (rest == 0) return LBM_OK;
  int rc = batch_fill(b, st);
  if (rc != LBM_OK) return rc;
  if (rest >= 2) {
    rc = batch_graph(b);
    if (rc != LBM_OK) return rc;
    for (int i = 0; i < rest / 2; ++i) CUDA_TRY(cudaGraphLaunch(b->graph, st));
  }
  // after an even number of steps every case is back at the parity of table 0
  if (rest & 1) CUDA_TRY(batch_launch(b, 0, st));
  batch_advance(b, rest);
  return LBM_OK;
}

int lbm_batch_set_cooperative(LbmBatch* b, int on) {
  if (!b) return fail(LBM_E_ARG, "lbm_batch_set_cooperative: null batch");
  if (on != 0 && on != 1) return fail(LBM_E_ARG, "lbm_batch_set_cooperative: on must be 0 or 1");
  if (on) {
    for (LbmHandle* h : b->h)
      if (h->paired)
        return fail(LBM_E_UNSUPPORTED, "lbm_batch_set_cooperative: the single-launch step serves linear-layout cases");
  }
  b->coop = on != 0;
  if (b->coop) b->upd_block = kBlock;
  return batch_layout(b);
}

int lbm_batch_get_launch(LbmBatch* b, int* phi_nodes_per_thread, int* update_block) {
  if (!b) return fail(LBM_E_ARG, "lbm_batch_get_launch: null batch");
  if (phi_nodes_per_thread) *phi_nodes_per_thread = b->phi_per_thread;
  if (update_block) *update_block = b->upd_block;
  return LBM_OK;
}

int lbm_batch_size(LbmBatch* b, int* ncases) {
  if (!b || !ncases) return fail(LBM_E_ARG, "lbm_batch_size: null argument");
  *ncases = (int)b->h.size();
  return LBM_OK;
}

int lbm_batch_autotune(LbmBatch* b, int reps, void* stream, int* best_per_thread, float* best_ms) {
  if (!b) return fail(LBM_E_ARG, "lbm_batch_autotune: null batch");
  if (reps <= 0) reps = 5;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  for (LbmHandle* h : b->h)
    if (!h->initialized || h->raw || h->first)
      return fail(LBM_E_STATE, "lbm_batch_autotune: every case must have taken a step");
  // time batched steps that re-read the current state (u, updated in place, is restored after)
  std::vector<void*> usave(b->h.size(), nullptr);
  for (size_t i = 0; i < b->h.size(); ++i) {
    const size_t ub = 3 * (size_t)b->h[i]->Np * b->h[i]->tsize;
    CUDA_TRY(cudaMalloc(&usave[i], ub));
    CUDA_TRY(cudaMemcpyAsync(usave[i], b->h[i]->u, ub, cudaMemcpyDeviceToDevice, st));
  }
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  int best = b->phi_per_thread, best_bs = b->upd_block, rc = LBM_OK;
  float best_t = 1e30f;
  for (int bs : {128, kBlock})
  for (int per : {1, 2, 4, 8, 12, 16, 24, 32}) {
    if (b->coop && bs != kBlock) continue;  // the cooperative step runs 256-thread update blocks
    b->phi_per_thread = per;
    b->upd_block = bs;
    rc = batch_layout(b);
    if (rc == LBM_OK) rc = batch_fill(b, st);
    if (rc != LBM_OK) break;
    cudaError_t e = batch_launch(b, 0, st);  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) e = batch_launch(b, 0, st);
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess) {
      rc = fail(LBM_E_CUDA, std::string("lbm_batch_autotune: ") + cudaGetErrorString(e));
      break;
    }
    if (ms < best_t) {
      best_t = ms;
      best = per;
      best_bs = bs;
    }
  }
  for (size_t i = 0; i < b->h.size(); ++i) {
    const size_t ub = 3 * (size_t)b->h[i]->Np * b->h[i]->tsize;
    cudaMemcpyAsync(b->h[i]->u, usave[i], ub, cudaMemcpyDeviceToDevice, st);
  }
  cudaStreamSynchronize(st);
  for (void* p : usave) cudaFree(p);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != LBM_OK) return rc;
  b->phi_per_thread = best;
  b->upd_block = best_bs;
  rc = batch_layout(b);
  if (rc != LBM_OK) return rc;
  if (best_per_thread) *best_per_thread = best;
  if (best_ms) *best_ms = best_t / reps;
  return LBM_OK;
}

}  // extern "C"
