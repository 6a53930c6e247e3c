"""D3Q19 velocity set.

The velocity ordering, float32 weights and opposite-direction table are the
population layout of the reference (pytorch-lbm ``lbm/lattice.py:60-96``); the
CUDA kernels hard-code the same table (``csrc/lbm_tables.cuh``).
"""
import numpy as np
import torch

_E = np.array([
    [0, 0, 0],
    [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
    [1, 1, 0], [-1, 1, 0], [-1, -1, 0], [1, -1, 0],
    [1, 0, 1], [-1, 0, 1], [-1, 0, -1], [1, 0, -1],
    [0, 1, 1], [0, -1, 1], [0, -1, -1], [0, 1, -1],
], dtype=np.int32)
_W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, dtype=np.float32)
_OPP = np.array([0, 2, 1, 4, 3, 6, 5, 9, 10, 7, 8, 13, 14, 11, 12, 17, 18, 15, 16],
                dtype=np.int64)


class D3Q19:
    def __init__(self):
        self.dim = 3
        self.q = 19
        self.cs2 = 1.0 / 3.0
        self.e = torch.tensor(_E, dtype=torch.float32)
        self.w = torch.tensor(_W, dtype=torch.float32)
        self.opp = torch.tensor(_OPP, dtype=torch.long)
