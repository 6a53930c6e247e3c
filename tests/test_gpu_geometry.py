"""The device geometry precompute (csrc/lbm_geometry.cu, behind
lbm_set_geometry and lbm_set_geometry_device) against the host restatement
of the same steps (lbm_geometry_host, which tests/test_native_cpu.py pins to
the reference's own tables): node classes, boundary mask, wall normals (the
bytes, so signed zeros count), wall weights, near-wall and partial masks,
for every golden case's geometry in float32 and float64 (the precision of the
top-surface test), 2-D grids included; the host-array and device-array entry
points alike; and the full-size 150x150x107 ridge and a discrete-normal
(no fraction) grid."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from _cases import CASES, config, inputs  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")


def _c(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _tables(N, nd):
    return dict(cls=np.empty(N, np.uint8), bnd=np.empty(N, np.uint8), wn=np.empty((nd, N), np.float32),
                ww=np.empty(N, np.float32), near=np.empty(N, np.uint8), part=np.empty(N, np.uint8))


def _host(lib, grid, solid, frac, theta, kappa, prec):
    nx, ny, nz = grid
    N = nx * ny * nz
    o = _tables(N, 2 if nz == 1 else 3)
    fdt = 0 if frac is None else (1 if frac.dtype == np.float32 else 2)
    rc = lib.lbm_geometry_host(nx, ny, nz, _c(solid.view(np.uint8)), _c(frac) if frac is not None else None, fdt,
                               theta, kappa, prec, _c(o["cls"]), _c(o["bnd"]), _c(o["wn"]), _c(o["ww"]),
                               _c(o["near"]), _c(o["part"]))
    assert rc == 0, lib.lbm_last_error()
    return o


def _device(lib, grid, solid, frac, cfg, prec, on_device):
    from lbm import _native as nat
    nx, ny, nz = grid
    N = nx * ny * nz
    p = nat.LbmParams()
    for k in ("rho_l", "rho_g", "sigma", "xi", "beta", "kappa", "phi_c", "tau_l", "tau_g", "tau_h", "theta_eq"):
        setattr(p, k, float(getattr(cfg, k)))
    p.boundary_relax, p.sharpen_reduce, p.mu_wall_scale, p.geo_amplification, p.ac_scale = 0.3, 0.8, 1.0, 1.0, 1.0
    p.geometric_wetting = 1
    h = ctypes.c_void_p()
    nat.check(lib.lbm_create(ctypes.byref(p), nx, ny, nz, prec, ctypes.byref(h)), "lbm_create")
    try:
        fdt = 0 if frac is None else (1 if frac.dtype == np.float32 else 2)
        if on_device:
            sd = torch.from_numpy(solid.view(np.uint8).copy()).cuda()
            fd = torch.from_numpy(frac).cuda() if frac is not None else None
            nat.check(lib.lbm_set_geometry_device(h, nat.ptr(sd), nat.ptr(fd), fdt, nat.stream_ptr()),
                      "lbm_set_geometry_device")
            torch.cuda.synchronize()
        else:
            nat.check(lib.lbm_set_geometry(h, _c(solid.view(np.uint8)), _c(frac) if frac is not None else None, fdt),
                      "lbm_set_geometry")
        o = _tables(N, 2 if nz == 1 else 3)
        nat.check(lib.lbm_get_geometry(h, _c(o["cls"]), _c(o["bnd"]), _c(o["wn"]), _c(o["ww"]), _c(o["near"]),
                                       _c(o["part"])), "lbm_get_geometry")
        return o
    finally:
        lib.lbm_destroy(h)


def _same(a, b):
    for k in a:
        assert a[k].tobytes() == b[k].tobytes(), k


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("prec", [0, 1])
def test_device_geometry_equals_host(built_lib, name, prec):
    case = CASES[name]
    solid, frac, _, _ = inputs(case)
    solid = np.ascontiguousarray(solid)
    frac = None if frac is None else np.ascontiguousarray(frac)
    cfg = config(case)
    host = _host(built_lib, case["grid"], solid, frac, cfg.theta_eq, cfg.kappa, prec)
    for on_device in (False, True):
        _same(_device(built_lib, case["grid"], solid, frac, cfg, prec, on_device), host)


@pytest.mark.parametrize("frac_dtype", [np.float32, np.float64, None])
def test_device_geometry_full_size_ridge(built_lib, frac_dtype):
    """The drop-in case's 150x150x107 ridge, with its smooth fraction in
    float32 and float64 and without a fraction (discrete normals)."""
    from geometry.substrate import create_substrate_with_fraction
    from lbm.fe_config import FEConfig
    solid, frac = create_substrate_with_fraction(150, 150, 107, "ridge", R_star=1.0, R_d=22.5)
    frac = None if frac_dtype is None else np.ascontiguousarray(frac, dtype=frac_dtype)
    cfg = FEConfig(nx=150, ny=150, nz=107, rho_l=1.0, rho_g=1.0 / 828.0, sigma=0.01424, xi=4.0, tau_l=0.53,
                   tau_g=0.53, theta_eq=162.0)
    solid = np.ascontiguousarray(solid)
    host = _host(built_lib, (150, 150, 107), solid, frac, cfg.theta_eq, cfg.kappa, 0)
    _same(_device(built_lib, (150, 150, 107), solid, frac, cfg, 0, True), host)
    assert int(host["bnd"].sum()) == 51600


def test_solver_geometry_attributes_from_device(built_lib):
    """The facade's wetting attributes after set_solid (device tables) equal
    the host restatement's."""
    from lbm.fe_ac_solver import AllenCahnSolver
    case = CASES["convex_l150"]
    solid, frac, C, u = inputs(case)
    s = AllenCahnSolver(config(case, "cuda"), dtype=torch.float32, **case["kw"])
    s.set_solid(torch.from_numpy(solid), torch.from_numpy(frac))  # tensors are accepted too
    cfg = config(case)
    host = _host(built_lib, case["grid"], np.ascontiguousarray(solid), np.ascontiguousarray(frac), cfg.theta_eq,
                 cfg.kappa, 0)
    shp = case["grid"]
    assert np.array_equal(s.wetting.is_boundary.cpu().numpy().reshape(-1), host["bnd"].astype(bool))
    assert s.wetting.wall_normal.cpu().numpy().tobytes() == host["wn"].tobytes()
    assert np.array_equal(s.wetting.wall_weight.cpu().numpy().reshape(-1), host["ww"])
    assert np.array_equal(s._partial_mask.cpu().numpy().reshape(-1), host["part"].astype(bool))
    assert tuple(s.solid.shape) == tuple(shp) and s.solid.dtype == torch.bool
    s.init_fields(C, u)
    s.run(2)
    assert s.status() == 0
