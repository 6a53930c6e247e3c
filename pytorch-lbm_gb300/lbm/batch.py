"""Batches of independent Allen-Cahn LBM grids on one GPU.

``AllenCahnBatch(solvers)`` advances many ``AllenCahnSolver`` cases together:
each time step is one launch of each step kernel for all cases (the blocks
of one launch are spread over the cases by a block -> case table on the
device), replayed from a captured two-step CUDA graph.  Every case keeps its
own arithmetic, reductions and mass correction, so its fields are
bit-identical to stepping it alone; the solvers remain usable on their own
between batch calls (fields, ``measure()``).

The reference has no batched form: its sweep drivers
(scripts/run_thesis_sweep.py) construct and run one solver per case in turn.
"""
from __future__ import annotations

import ctypes

from . import _native as nat


class AllenCahnBatch:
    def __init__(self, solvers):
        self._solvers = list(solvers)
        if not self._solvers:
            raise ValueError("a batch needs at least one solver")
        for s in self._solvers:
            if not s._initialized:
                raise RuntimeError("every solver of a batch must have called init_fields")
        self._lib = nat.lib()
        arr = (ctypes.c_void_p * len(self._solvers))(*[s._h.value for s in self._solvers])
        h = ctypes.c_void_p()
        nat.check(self._lib.lbm_batch_create(arr, len(self._solvers), ctypes.byref(h)), "lbm_batch_create")
        self._h = h

    def __len__(self):
        return len(self._solvers)

    @property
    def solvers(self):
        return list(self._solvers)

    def run(self, nsteps, stream=None):
        """Advance every case by ``nsteps`` steps (asynchronous)."""
        if self._h is None:
            raise RuntimeError("batch is closed")
        nat.check(self._lib.lbm_batch_step(self._h, int(nsteps), nat.stream_ptr(stream)), "lbm_batch_step")
        for s in self._solvers:
            s.step_count += int(nsteps)
            s.t += float(nsteps)
            s._cache.clear()

    def step(self):
        self.run(1)

    def autotune(self, reps=5, stream=None):
        """Launch shape of the batched step (the phi kernel's nodes per thread
        and the update kernel's threads per block): the fastest candidate on
        the current state (left unchanged).  Returns (nodes per thread, ms per
        step); ``launch_shape()`` gives both choices."""
        best = ctypes.c_int()
        ms = ctypes.c_float()
        nat.check(self._lib.lbm_batch_autotune(self._h, int(reps), nat.stream_ptr(stream), ctypes.byref(best),
                                               ctypes.byref(ms)), "lbm_batch_autotune")
        return int(best.value), float(ms.value)

    def set_cooperative(self, on=True):
        """One cooperative launch per batched step (phi work, grid barrier,
        update work) instead of two launches; same results."""
        nat.check(self._lib.lbm_batch_set_cooperative(self._h, 1 if on else 0), "lbm_batch_set_cooperative")

    def launch_shape(self):
        """(phi-kernel nodes per thread, update-kernel threads per block)."""
        a, b = ctypes.c_int(), ctypes.c_int()
        nat.check(self._lib.lbm_batch_get_launch(self._h, ctypes.byref(a), ctypes.byref(b)), "lbm_batch_get_launch")
        return int(a.value), int(b.value)

    def close(self):
        """Free the batch's tables (not the solvers)."""
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.lbm_batch_destroy(h)
            except Exception:
                pass
        self._h = None

    def __del__(self):
        self.close()


def footprint(shape, dtype):
    """Device bytes of one solver of grid ``shape`` with population ``dtype``
    (torch.float32 / float64 / float16): the admission size of a case."""
    import torch
    prec = {torch.float32: nat.LBM_F32, torch.float64: nat.LBM_F64, torch.float16: nat.LBM_F16}[dtype]
    b = ctypes.c_int64()
    nat.check(nat.lib().lbm_footprint(int(shape[0]), int(shape[1]), int(shape[2]), prec, ctypes.byref(b)),
              "lbm_footprint")
    return int(b.value)
