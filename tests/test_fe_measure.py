"""lbm.fe_measure (the package's measure_spread_factor / measure_contact_angle)
against the reference's own lbm/fe_measure.py outputs on the same fields
(tests/golden/fe_measure_ref.json, made by tests/golden/make_golden_measure.py):
host path bit for bit on CPU; the device reduction of a CUDA field on the GPU
(extents and C_max exact, the float64 volume within float32 summation error)."""
import json
import os

import numpy as np
import pytest

from make_golden_measure import HERE, inputs


@pytest.fixture(scope="module")
def ref():
    with open(os.path.join(HERE, "fe_measure_ref.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("name", sorted(inputs()))
def test_host_measurements_equal_reference(name, ref):
    from lbm.fe_measure import measure_contact_angle, measure_spread_factor
    phi, solid = inputs()[name]
    r = ref[name]
    assert measure_spread_factor(phi, solid) == r["spread"]
    assert measure_spread_factor(phi) == r["spread_nomask"]
    assert measure_contact_angle(phi, solid) == r["contact_angle"]


def test_host_measurements_accept_cpu_tensors(ref):
    torch = pytest.importorskip("torch")
    from lbm.fe_measure import measure_contact_angle, measure_spread_factor
    name = "cap3d_zc2.0"
    phi, solid = inputs()[name]
    assert measure_spread_factor(torch.from_numpy(phi), torch.from_numpy(solid)) == ref[name]["spread"]
    assert measure_contact_angle(torch.from_numpy(phi), torch.from_numpy(solid)) == ref[name]["contact_angle"]


def test_empty_interface():
    from lbm.fe_measure import measure_spread_factor
    phi = np.full((6, 5, 4), 0.25, np.float32)
    assert measure_spread_factor(phi) == {"Dx": 0.0, "Dy": 0.0, "Dz": 0.0, "k": 0.0,
                                          "volume": float(phi.sum()), "C_max": 0.25}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(inputs()))
def test_device_spread_equals_reference(name, ref, built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from lbm.fe_measure import measure_spread_factor
    phi, solid = inputs()[name]
    for mask, key in ((torch.from_numpy(solid).cuda(), "spread"), (None, "spread_nomask")):
        m = measure_spread_factor(torch.from_numpy(phi).cuda(), mask)
        r = ref[name][key]
        for k in ("Dx", "Dy", "Dz", "k", "C_max"):
            assert m[k] == r[k], k
        # float64 sum on the device against numpy's float32 pairwise sum
        assert m["volume"] == pytest.approx(r["volume"], rel=2e-6 if phi.dtype == np.float32 else 1e-12)


def _nan_field():
    phi, solid = inputs()["cap3d_zc2.0"]
    phi = phi.copy()
    # one NaN node in the fluid, away from the wall
    idx = tuple(int(s) // 2 for s in phi.shape)
    phi[idx] = np.nan
    assert not solid[idx]
    return phi, solid


def test_host_nan_field_gives_nan_volume_and_cmax():
    """numpy's sum and max propagate NaN (the reference's volume and C_max)."""
    from lbm.fe_measure import measure_spread_factor
    phi, solid = _nan_field()
    m = measure_spread_factor(phi, solid)
    assert np.isnan(m["volume"]) and np.isnan(m["C_max"])
    assert m["Dx"] > 0


@pytest.mark.gpu
def test_device_nan_field_matches_host(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from lbm.fe_measure import measure_spread_factor
    phi, solid = _nan_field()
    host = measure_spread_factor(phi, solid)
    dev = measure_spread_factor(torch.from_numpy(phi).cuda(), torch.from_numpy(solid).cuda())
    for k in ("Dx", "Dy", "Dz", "k"):
        assert dev[k] == host[k], k
    assert np.isnan(dev["volume"]) and np.isnan(dev["C_max"])


@pytest.mark.gpu
def test_device_measurements_from_concurrent_threads(ref, built_lib):
    """Host threads measuring different fields on their own streams share the
    device scratch of the reduction; the module serialises them, so every
    result equals the reference's."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    import threading
    from lbm.fe_measure import measure_spread_factor
    names = [n for n in sorted(inputs()) if inputs()[n][0].ndim == 3]
    fields = {n: (torch.from_numpy(inputs()[n][0]).cuda(), torch.from_numpy(inputs()[n][1]).cuda())
              for n in names}
    torch.cuda.synchronize()
    errors = []

    def work(offset):
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            for i in range(12):
                n = names[(i + offset) % len(names)]
                m = measure_spread_factor(*fields[n])
                r = ref[n]["spread"]
                if any(m[k] != r[k] for k in ("Dx", "Dy", "Dz", "k", "C_max")):
                    errors.append((n, m, r))

    threads = [threading.Thread(target=work, args=(j,)) for j in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors[:2]


@pytest.mark.parametrize("zc", [-3.0, 2.0, 7.5])
@pytest.mark.parametrize("dim", [2, 3])
def test_wall_contact_angle_of_spherical_caps(built_lib, zc, dim):
    """measure_contact_angle_wall on the spherical caps (radius 12, tanh
    interface of width 4, centre height zc over the wall whose top layer is
    z = 1): within 2 degrees of the cap's analytic angle in the first fluid
    layer z = 2, cos(theta) = (2 - zc) / 12, with the library's own wall
    normals and boundary mask (lbm_geometry_host: discrete normals of the flat
    wall)."""
    import ctypes
    from lbm.fe_measure import measure_contact_angle_wall
    phi, solid = inputs()[f"cap{dim}d_zc{zc}"]
    shape = phi.shape
    nx, ny, nz = shape if dim == 3 else (shape[0], shape[1], 1)
    N = phi.size
    bnd = np.empty(N, np.uint8)
    wn = np.empty((dim, N), np.float32)
    c = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = built_lib.lbm_geometry_host(nx, ny, nz, c(np.ascontiguousarray(solid).view(np.uint8)), None, 0, 120.0, 0.01,
                                     0, None, c(bnd), c(wn), None, None, None)
    assert rc == 0
    theta = measure_contact_angle_wall(phi, solid, wn.reshape((dim,) + shape), bnd.reshape(shape))
    assert theta == pytest.approx(np.degrees(np.arccos((2.0 - zc) / 12.0)), abs=2.0)


def test_wall_contact_angle_without_contact():
    from lbm.fe_measure import measure_contact_angle_wall
    phi, solid = inputs()["cap3d_zc2.0"]
    bnd = np.zeros(phi.shape, bool)
    assert measure_contact_angle_wall(phi, solid, np.zeros((3,) + phi.shape, np.float32), bnd) == 180.0
