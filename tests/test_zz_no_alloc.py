"""lbm_measure_static: the spread diagnostics for callers that cannot allocate
device memory (code inside another runtime's memory pool, a driver that forbids
allocation after start-up, a monitoring hook that must not disturb the solve's
allocator).  It keeps its reduction scratch in a static device array of the
library, so the checks here are that it gives what lbm_measure gives, on two
calls in a row (the second one finds the first one's partials and counter
left in the shared array), that calls after the first leave the device's free
memory and the torch allocator's counters unchanged, and that it refuses grids
above its maximum.

Collected last on purpose (the file name sorts after every other test file)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from _cases import CASES, config, inputs  # noqa: E402

# the values lbm_measure returns, in its order
KEYS = ("volume", "C_max", "Dx", "Dy", "Dz", "k", "z_com", "count", "has_nan")
EXACT = ("C_max", "Dx", "Dy", "Dz", "k", "count", "has_nan")


def _static(lib, solver, dn):
    from lbm import _native as nat
    nx, ny, nz = solver.shape
    phi = solver.phi.contiguous()
    solid = solver.solid.contiguous()
    assert solid.dtype == torch.bool and solid.is_cuda and phi.is_cuda
    out = torch.full((9,), -7.0, dtype=torch.float64, device=phi.device)
    dt = nat.LBM_DT_F32 if dn == "float32" else nat.LBM_DT_F64
    rc = lib.lbm_measure_static(nx, ny, nz, nat.ptr(phi), dt, nat.ptr(solid), nat.ptr(out), nat.stream_ptr())
    nat.check(rc, "lbm_measure_static")
    return out.cpu().numpy()


def _handle(lib, solver):
    from lbm import _native as nat
    out = (ctypes.c_double * 9)()
    nat.check(lib.lbm_measure(solver._h, out, nat.stream_ptr()), "lbm_measure")
    return np.array(out[:], dtype=np.float64)


def _compare(a, b):
    for i, key in enumerate(KEYS):
        if key in EXACT:
            assert a[i] == b[i], key
        else:
            assert a[i] == pytest.approx(b[i], rel=1e-12, abs=0), key


@pytest.mark.gpu
@pytest.mark.parametrize("dn", ["float32", "float64"])
def test_measure_static_matches_lbm_measure(built_lib, dn):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from lbm.fe_ac_solver import AllenCahnSolver
    case = CASES["ridge_l162"]
    solid, frac, C, u = inputs(case)
    s = AllenCahnSolver(config(case, "cuda"), dtype=getattr(torch, dn), **case["kw"])
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    for _ in range(2):  # two calls in a row, each after a few more steps
        s.run(5)
        got = _static(built_lib, s, dn)
        ref = _handle(built_lib, s)
        _compare(got, ref)
        assert got[7] > 0 and got[8] == 0.0


@pytest.mark.gpu
def test_measure_static_allocates_nothing(built_lib):
    """After the first call (which may load the module and its static array
    onto the device), further calls change neither cudaMemGetInfo's free
    bytes nor the torch caching allocator's counters."""
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from lbm import _native as nat
    from lbm.fe_ac_solver import AllenCahnSolver
    case = CASES["ridge_l162"]
    solid, frac, C, u = inputs(case)
    s = AllenCahnSolver(config(case, "cuda"), dtype=torch.float32, **case["kw"])
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    s.run(3)
    nx, ny, nz = s.shape
    phi = s.phi.contiguous()
    solid_d = s.solid.contiguous()
    outs = [torch.full((9,), -7.0, dtype=torch.float64, device=phi.device) for _ in range(6)]
    stream = nat.stream_ptr()
    args = (nx, ny, nz, nat.ptr(phi), nat.LBM_DT_F32, nat.ptr(solid_d))
    nat.check(built_lib.lbm_measure_static(*args, nat.ptr(outs[0]), stream), "lbm_measure_static")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    stats0 = torch.cuda.memory_stats()
    for out in outs[1:]:
        nat.check(built_lib.lbm_measure_static(*args, nat.ptr(out), stream), "lbm_measure_static")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    stats1 = torch.cuda.memory_stats()
    assert free1 == free0
    for key in ("allocation.all.allocated", "segment.all.allocated", "reserved_bytes.all.current"):
        assert stats1.get(key, 0) == stats0.get(key, 0), key
    first = outs[0].cpu().numpy()
    for out in outs[1:]:
        assert np.array_equal(out.cpu().numpy(), first)


def test_measure_static_rejects_oversized_grid(built_lib):
    """Argument checks run before any CUDA call, so this needs no GPU."""
    from lbm import _native as nat
    dummy = ctypes.c_void_p(256)
    big = 1 << 11  # 2048^3 = 2^33 nodes > LBM_MEASURE_STATIC_MAX_NODES (2^30)
    rc = built_lib.lbm_measure_static(big, big, big, dummy, nat.LBM_DT_F32, dummy, dummy, None)
    assert rc == -1
    assert b"exceeds the maximum" in built_lib.lbm_last_error()
    rc = built_lib.lbm_measure_static(8, 8, 8, None, nat.LBM_DT_F32, dummy, dummy, None)
    assert rc == -1
