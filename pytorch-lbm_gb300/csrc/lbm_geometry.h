// Host geometry precompute (see lbm_geometry.cpp).
#pragma once
#include <cstdint>
#include <memory>
#include <new>
#include <type_traits>
#include <utility>
#include <vector>

namespace lbm {

// Allocator whose resize() leaves new elements default-initialised (no
// zeroing): the geometry tables are filled by parallel loops, which then
// also touch their pages first, instead of one serial zeroing pass.
template <typename T>
struct NoInitAlloc : std::allocator<T> {
  template <typename U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <typename U>
  NoInitAlloc(const NoInitAlloc<U>&) {}
  template <typename U>
  void construct(U* p) noexcept(std::is_nothrow_default_constructible<U>::value) {
    ::new (static_cast<void*>(p)) U;
  }
  template <typename U, typename... A>
  void construct(U* p, A&&... a) {
    ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
  }
};
template <typename T>
using HostVec = std::vector<T, NoInitAlloc<T>>;

struct Geometry {
  HostVec<uint8_t> solid, partial, boundary, near_wall, top, cls;
  HostVec<float> wall_normal;  // [3][N]
  HostVec<float> wall_weight;  // [N]
  HostVec<uint8_t> dist;       // near-wall distance 0..11 (100 = not reached)
  HostVec<int32_t> nsw;        // next-interior fluid node of a boundary node, else -1
  bool has_fraction = false;   // a solid fraction was given
  int64_t n_boundary = 0;
};

// fraction_dtype: 0 none, 1 float32, 2 float64.  wetting: theta != 90 and
// kappa > 0.  dbl_precision selects the precision of the top-surface test.
int compute_geometry(int64_t nx, int64_t ny, int64_t nz, const uint8_t* solid, const void* fraction,
                     int fraction_dtype, bool wetting, bool dbl_precision, Geometry& g);

// Near-wall weight by code (kWwCodes entries).
void near_wall_weights(float* lut);

}  // namespace lbm
