"""The cache of grid state arrays (lbm_destroy keeps them, lbm_create reuses
them): a grid stepped on recycled arrays that hold another grid's state, or
on fresh device memory filled with NaN bytes, gives the bits of the same grid
stepped on its own first allocation (float32, float64, the half storage, a
2-D grid, the gradient-of-mu mode with its extra arrays); the cache's
accounting, its limit and its trim."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from _cases import CASES, config, inputs  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")


def _solver(name, dtype):
    from lbm.fe_ac_solver import AllenCahnSolver
    case = CASES[name]
    solid, frac, C, u = inputs(case)
    s = AllenCahnSolver(config(case, "cuda"), dtype=dtype, **case["kw"])
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    return s


def _run(name, dtype, steps=12):
    s = _solver(name, dtype)
    s.run(steps)
    phi, u = s.fields("phi", "u")
    out = [phi.clone(), u.clone(), s.f.clone(), s.g.clone()]
    torch.cuda.synchronize()
    s.close()
    return out


def _equal(a, b):
    return all(torch.equal(x, y) for x, y in zip(a, b))


# (grid under test, another grid of the same extents whose state fills the recycled arrays)
PAIRS = [("ridge_l162", "direct_ridge_l150", torch.float32),
         ("ridge_l162", "mudrive_ridge_l150", torch.float64),
         ("mudrive_ridge_l150", "ridge_alpha_field", torch.float32),
         ("ridge_l162", "discrete_l162", torch.float16),
         ("ridge2d_l162", "direct2d_l150", torch.float32)]


@pytest.mark.parametrize("name,other,dtype", PAIRS)
def test_recycled_arrays_give_the_same_bits(name, other, dtype):
    from lbm import _native as nat
    nat.cache_trim()
    first = _run(name, dtype)
    assert nat.cache_bytes() > 0
    _run(other, dtype, 20)
    held = nat.cache_bytes()
    s = _solver(name, dtype)
    assert nat.cache_bytes() < held  # the arrays came from the cache
    s.close()
    assert _equal(first, _run(name, dtype))
    nat.cache_trim()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float16])
def test_fresh_memory_filled_with_nan_bytes(dtype):
    """Device memory that held 0xFF bytes (NaN in every float format) before
    the grid's arrays were allocated on it changes nothing."""
    from lbm import _native as nat
    nat.cache_trim()
    first = _run("ridge_l162", dtype)
    nat.cache_trim()
    junk = torch.full((1 << 28,), 255, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    del junk
    torch.cuda.empty_cache()
    assert _equal(first, _run("ridge_l162", dtype))
    nat.cache_trim()


def test_cache_accounting_limit_and_trim():
    from lbm import _native as nat
    from lbm.batch import footprint
    nat.cache_trim()
    assert nat.cache_bytes() == 0
    s = _solver("ridge_l162", torch.float32)
    s.close()
    grid = CASES["ridge_l162"]["grid"]
    held = nat.cache_bytes()
    assert held >= footprint(grid, torch.float32) * 0.9
    free0, _ = torch.cuda.mem_get_info()
    assert nat.cache_trim() == held and nat.cache_bytes() == 0
    free1, _ = torch.cuda.mem_get_info()
    assert free1 > free0
    nat.cache_limit(0)  # caching off: close frees the arrays
    try:
        s = _solver("ridge_l162", torch.float32)
        s.close()
        assert nat.cache_bytes() == 0
    finally:
        nat.cache_limit(16 << 30)
    # a smaller grid does not take a block more than 1/8 larger than it needs
    s = _solver("cfg1_flat64", torch.float32)
    s.close()
    held = nat.cache_bytes()
    s = _solver("flat_q120", torch.float32)
    # only the small arrays of the same size in both grids (counters, scalars,
    # partial sums) are taken
    assert held - nat.cache_bytes() <= 256 << 10 < footprint(CASES["flat_q120"]["grid"], torch.float32)
    s.close()
    nat.cache_trim()


def test_host_inputs_read_in_place_equal_staged_copy(tmp_path):
    """init_fields from host arrays gives the same state whether the kernel
    reads them in place (the default where the device reaches pageable host
    memory) or from a staging copy (LBM_HOST_STAGING=1, in a child process)."""
    import os
    import subprocess
    import sys
    script = tmp_path / "run.py"
    tests = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(tests)
    paths = [root, os.path.join(root, "pytorch-lbm_gb300"), tests, os.path.join(tests, "golden")]
    script.write_text(
        "import sys, numpy as np, torch\n"
        f"sys.path[:0] = {paths!r}\n"
        "import test_gpu_cache as t\n"
        "out = t._run('ridge_l162', torch.float32, 6)\n"
        "np.savez(sys.argv[1], *[x.cpu().numpy() for x in out])\n")
    env = dict(os.environ)
    res = []
    for staging in ("0", "1"):
        env["LBM_HOST_STAGING"] = staging
        path = tmp_path / f"s{staging}.npz"
        subprocess.run([sys.executable, str(script), str(path)], env=env, check=True, timeout=600)
        import numpy as np
        d = np.load(path)
        res.append([d[k] for k in sorted(d.files)])
    for a, b in zip(*res):
        assert a.tobytes() == b.tobytes()


def test_cache_stays_within_its_limit():
    """Past the limit the blocks cached longest make room for the ones just
    returned, and a block larger than the limit is freed: the cache never
    holds more than its limit, whatever the order of grids."""
    from lbm import _native as nat
    from lbm.batch import footprint
    nat.cache_trim()
    try:
        nat.cache_limit(1 << 20)  # below one population array of either grid
        for name in ("ridge_l162", "cfg1_flat64", "ridge_l162"):
            _solver(name, torch.float32).close()
            assert 0 < nat.cache_bytes() <= 1 << 20
        small = footprint(CASES["ridge_l162"]["grid"], torch.float32)
        limit = int(1.5 * small)
        nat.cache_limit(limit)
        for name in ("ridge_l162", "cfg1_flat64", "ridge_l162", "cfg1_flat64"):
            s = _solver(name, torch.float32)
            assert nat.cache_bytes() <= limit
            s.close()
            assert 0 < nat.cache_bytes() <= limit
    finally:
        nat.cache_limit(16 << 30)
        nat.cache_trim()
