// Host copies of the D3Q19 tables (population order of pytorch-lbm
// lbm/lattice.py:70-95) and of the near-wall weight coding.
#pragma once

namespace lbm {

constexpr int kQ = 19;
constexpr int kE[kQ][3] = {
    {0, 0, 0},
    {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},   {0, 0, -1},
    {1, 1, 0},  {-1, 1, 0}, {-1, -1, 0}, {1, -1, 0},
    {1, 0, 1},  {-1, 0, 1}, {-1, 0, -1}, {1, 0, -1},
    {0, 1, 1},  {0, -1, 1}, {0, -1, -1}, {0, 1, -1},
};
constexpr int kOpp[kQ] = {0, 2, 1, 4, 3, 6, 5, 9, 10, 7, 8, 13, 14, 11, 12, 17, 18, 15, 16};

// D2Q9 of the 2-D grids (nz == 1; lbm/lattice.py:36-57), as 3-D vectors with
// e_z = 0 so that the 3-D index arithmetic serves both.
constexpr int kQ2 = 9;
constexpr int kE2[kQ2][3] = {
    {0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {1, 1, 0}, {-1, 1, 0}, {-1, -1, 0}, {1, -1, 0},
};
constexpr int kOpp2[kQ2] = {0, 2, 1, 4, 3, 7, 8, 5, 6};

// Near-wall distance propagation passes: int(2 * xi) + 1 with the hard-coded
// xi = 5 of lbm/fe_wetting.py:81,285.
constexpr int kNearWallPasses = 11;
constexpr int kWwCodes = 16;
constexpr int kWwFarCode = 12;    // distance 100 (not reached)
constexpr int kWwSolidCode = 13;  // weight 0

}  // namespace lbm
