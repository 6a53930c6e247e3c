"""Lattice velocity sets: D3Q19 (the GPU path's lattice) and D2Q9.

The velocity ordering, float32 weights and opposite-direction tables are the
population layout of the reference (pytorch-lbm ``lbm/lattice.py:10-96``); the
CUDA kernels hard-code the same tables (D3Q19: ``csrc/lbm_common.cuh``, D2Q9
of the 2-D grids: ``csrc/lbm_kernels2d.cu``).
"""
import numpy as np
import torch


class Lattice:
    """A velocity set: e (Q, dim) and w (Q,) as float32 tensors, opp (Q,) long,
    cs2, and the derived e*w, |e|^2 and pull-streaming shifts -e."""

    def __init__(self, e, w, opp, cs2=1.0 / 3.0):
        self.dim = e.shape[1]
        self.q = e.shape[0]
        self.cs2 = cs2
        self.e = torch.tensor(e, dtype=torch.float32)
        self.w = torch.tensor(w, dtype=torch.float32)
        self.opp = torch.tensor(opp, dtype=torch.long)
        self.ew = self.e * self.w.unsqueeze(1)
        self.e_sq = (self.e ** 2).sum(dim=1)
        self.stream_shifts = -np.asarray(e, dtype=int)


class D2Q9(Lattice):
    def __init__(self):
        e = np.array([[0, 0], [1, 0], [-1, 0], [0, 1], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]], dtype=np.int32)
        w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4, dtype=np.float32)
        opp = np.array([0, 2, 1, 4, 3, 7, 8, 5, 6], dtype=np.int64)
        super().__init__(e, w, opp)


class D3Q19(Lattice):
    def __init__(self):
        e = np.array([
            [0, 0, 0],
            [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
            [1, 1, 0], [-1, 1, 0], [-1, -1, 0], [1, -1, 0],
            [1, 0, 1], [-1, 0, 1], [-1, 0, -1], [1, 0, -1],
            [0, 1, 1], [0, -1, 1], [0, -1, -1], [0, 1, -1],
        ], dtype=np.int32)
        w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, dtype=np.float32)
        opp = np.array([0, 2, 1, 4, 3, 6, 5, 9, 10, 7, 8, 13, 14, 11, 12, 17, 18, 15, 16], dtype=np.int64)
        super().__init__(e, w, opp)
