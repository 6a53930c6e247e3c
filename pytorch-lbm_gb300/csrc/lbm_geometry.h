// Host geometry precompute (see lbm_geometry.cpp).
#pragma once
#include <cstdint>
#include <vector>

namespace lbm {

struct Geometry {
  std::vector<uint8_t> solid, partial, boundary, near_wall, top, cls;
  std::vector<float> wall_normal;  // [3][N]
  std::vector<float> wall_weight;  // [N]
  std::vector<int> dist;           // near-wall distance (100 = not reached)
  std::vector<double> fraction;    // solid fraction as given (empty if none)
  std::vector<int32_t> nsw;        // next-interior fluid node of a boundary node, else -1
  int64_t n_boundary = 0;
};

// fraction_dtype: 0 none, 1 float32, 2 float64.  wetting: theta != 90 and
// kappa > 0.  dbl_precision selects the precision of the top-surface test.
int compute_geometry(int64_t nx, int64_t ny, int64_t nz, const uint8_t* solid, const void* fraction,
                     int fraction_dtype, bool wetting, bool dbl_precision, Geometry& g);

// Near-wall weight by code (kWwCodes entries).
void near_wall_weights(float* lut);

}  // namespace lbm
