"""The 2-D (nz == 1, D2Q9) form of the step through the C ABI: spread and
global reductions against the oracle, checkpoints, and the options a 2-D
grid refuses.  Parity of the fields against the reference's own 2-D runs is
in test_gpu_parity.py (the *2d* golden cases)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from _cases import CASES, config, golden, inputs  # noqa: E402
from oracle.ac_oracle import measure_spread  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return built_lib


def _solver(name, dtype=torch.float32, init=True):
    from lbm.fe_ac_solver import AllenCahnSolver
    case = CASES[name]
    solid, frac, C, u = inputs(case)
    s = AllenCahnSolver(config(case, "cuda"), dtype=dtype, **case["kw"])
    s.set_solid(solid, frac)
    if init:
        s.init_fields(C, u)
    return s


def test_shapes_and_lattice():
    s = _solver("ridge2d_l162")
    nx, ny, _ = CASES["ridge2d_l162"]["grid"]
    assert s.ndim == 2 and s.lattice.q == 9
    assert s.phi.shape == (nx, ny) and s.u.shape == (2, nx, ny)
    assert s.f.shape == (9, nx, ny) and s.wetting.wall_normal.shape == (2, nx, ny)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_measure_and_reduce_match_host(dtype):
    s = _solver("ridge2d_l162", dtype)
    s.run(5)
    phi = s.phi.cpu().numpy()
    u = s.u.cpu().numpy()
    solid = s.solid.cpu().numpy()
    m = s.measure()
    ref = measure_spread(phi, solid)
    for k in ("Dx", "Dy", "Dz", "k", "count"):
        assert m[k] == ref[k], k
    assert m["Dz"] == 0.0
    assert m["volume"] == pytest.approx(ref["volume"], rel=1e-12)
    assert m["z_com"] == pytest.approx(ref["z_com"], rel=1e-12)  # centre along y
    r = s.reduce()
    assert r["sum_phi"] == pytest.approx(float(phi.astype(np.float64).sum()), rel=1e-12)
    p64 = phi.astype(np.float64)
    rho = p64 * s.config.rho_l + (1.0 - p64) * s.config.rho_g
    mom = [(rho * u[d].astype(np.float64)).sum() for d in range(2)]
    scale = np.abs(rho * np.abs(u).max()).sum() + 1e-300
    assert np.all(np.abs(np.array(r["momentum"][:2]) - mom) <= 1e-10 * scale)
    assert r["momentum"][2] == 0.0
    iface = np.argwhere((phi > 0.5) & ~solid)
    lo, hi = iface.min(0), iface.max(0)
    assert r["extents"] == (lo[0], hi[0], lo[1], hi[1], 0, 0)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_resume_is_bit_identical(dtype):
    a = _solver("direct2d_l150", dtype)
    a.run(3)
    sd = a.state_dict()
    a.run(6)
    b = _solver("direct2d_l150", dtype, init=False)
    b.load_state_dict(sd)
    b.run(6)
    for fa, fb in zip(a.fields("phi", "u", "P", "mu_phi"), b.fields("phi", "u", "P", "mu_phi")):
        assert torch.equal(fa, fb)
    assert a.scalars() == b.scalars()


def test_step_profiled_times_both_kernels():
    import ctypes
    from lbm import _native as nat
    s = _solver("flat2d_q120")
    ms = (ctypes.c_float * 3)()
    nat.check(s._lib.lbm_step_profiled(s._h, 4, nat.stream_ptr(), ms), "lbm_step_profiled")
    assert ms[0] > 0 and ms[1] > 0 and ms[2] > 0
    # the profiled steps are ordinary steps
    b = _solver("flat2d_q120")
    b.run(4)
    assert torch.equal(s.phi, b.phi)


def test_refused_options():
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm import _native as nat
    from lbm.batch import AllenCahnBatch
    case = CASES["flat2d_q120"]
    with pytest.raises(NotImplementedError):
        AllenCahnSolver(config(case, "cuda"), dtype=torch.float16)
    s = _solver("flat2d_q120")
    with pytest.raises(RuntimeError, match="2-D"):
        s.set_tile(4, 4, 4)
    with pytest.raises(RuntimeError, match="2-D"):
        AllenCahnBatch([s])
    s.set_tile(0, 0, 0)  # the per-node kernels: allowed
    s.run(2)
    assert s.status() == 0
