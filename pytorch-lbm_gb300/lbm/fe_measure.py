"""Droplet measurements with the reference's functions and return values
(pytorch-lbm ``lbm/fe_measure.py``): spread factors and the wall contact angle.

``measure_spread_factor`` reduces a 2-D or 3-D CUDA field on the device (the library's
allocation-free spread reduction, ``lbm_measure_static``), so a caller that
polls a running solve copies 9 numbers to the host instead of the field;
host arrays and CPU tensors are measured on the host.  ``measure_contact_angle``
scans one wall layer and one column, which the reference does on the host;
it stays there.

The device reduction keeps its block partials in one scratch array per GPU
that every call shares.  This module serialises its own calls (a lock per
device, held from the launch until the 9 results are on the host), so threads
of one process that measure fields on different streams get correct results;
another caller of the C entry point on the same device must not overlap with
it.  The call synchronises with the device, so it cannot be made while a
stream is being captured into a CUDA graph.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover - torch is part of the package's requirements
    torch = None


def _host(x):
    if torch is not None and isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def _empty(volume, c_max):
    return {"Dx": 0.0, "Dy": 0.0, "Dz": 0.0, "k": 0.0, "volume": volume, "C_max": c_max}


_DEVICE_LOCKS: dict = {}
_LOCKS_GUARD = threading.Lock()


def _device_lock(index):
    with _LOCKS_GUARD:
        lk = _DEVICE_LOCKS.get(index)
        if lk is None:
            lk = _DEVICE_LOCKS[index] = threading.Lock()
        return lk


def _spread_device(C, solid_mask):
    from . import _native as nat
    two_d = C.dim() == 2
    # a 2-D field is reduced as the 1 x nx x ny grid of the same memory layout:
    # its "y" and "z" extents are then Dx and Dy
    nx, ny, nz = (1,) + tuple(C.shape) if two_d else tuple(C.shape)
    phi = C.detach().contiguous()
    if phi.dtype not in (torch.float32, torch.float64):
        phi = phi.to(torch.float32)
    if solid_mask is None:
        solid = torch.zeros(C.shape, dtype=torch.uint8, device=C.device)
    else:
        solid = torch.as_tensor(solid_mask, device=C.device).to(torch.bool).contiguous().view(torch.uint8)
    out = torch.empty(9, dtype=torch.float64, device=C.device)
    dt = nat.LBM_DT_F32 if phi.dtype == torch.float32 else nat.LBM_DT_F64
    # the reduction's scratch is shared by every call on the device: one call at a time,
    # from the launch until its results have reached the host
    with torch.cuda.device(C.device), _device_lock(C.device.index):
        nat.check(nat.lib().lbm_measure_static(nx, ny, nz, nat.ptr(phi), dt, ctypes.c_void_p(solid.data_ptr()),
                                               nat.ptr(out), nat.stream_ptr()), "lbm_measure_static")
        v = out.cpu().numpy()
    volume, c_max, count = float(v[0]), float(v[1]), int(v[7])
    if v[8] != 0.0:
        # a NaN node: numpy's max (the reference's C_max) is NaN; the device maximum skips NaN
        c_max = float("nan")
    if count == 0:
        return _empty(volume, c_max)
    Dx, Dy, Dz = (float(v[3]), float(v[4]), 0.0) if two_d else (float(v[2]), float(v[3]), float(v[4]))
    return {"Dx": Dx, "Dy": Dy, "Dz": Dz, "k": Dx / Dy if Dy > 0 else 0.0, "volume": volume, "C_max": c_max}


def measure_spread_factor(C, solid_mask=None) -> dict:
    """Extents Dx, Dy, Dz of the C > 0.5 set (solid nodes excluded), k = Dx / Dy,
    volume = sum of C with solid nodes zeroed, C_max (lbm/fe_measure.py:11-82).

    A 2-D or 3-D CUDA tensor is reduced on its device (the volume summed in
    float64); anything else on the host.  A field with a NaN node gives a NaN
    volume and C_max, as numpy's sum and max do in the reference.

    On the device the reduction uses one scratch array per GPU shared by all
    calls (it allocates no device memory).  Calls from this module are
    serialised per device; they synchronise with the device, so none may be
    made during CUDA graph capture, and a caller of the C entry point
    ``lbm_measure_static`` on the same device must not run concurrently."""
    if torch is not None and isinstance(C, torch.Tensor) and C.is_cuda and C.dim() in (2, 3):
        return _spread_device(C, solid_mask)
    c = np.array(_host(C), copy=True)
    if solid_mask is not None:
        c[_host(solid_mask).astype(bool)] = 0.0
    volume = float(c.sum())
    c_max = float(c.max())
    inside = c > 0.5
    if not inside.any():
        return _empty(volume, c_max)
    ext = []
    for axis in range(c.ndim):
        other = tuple(a for a in range(c.ndim) if a != axis)
        hit = np.flatnonzero(inside.any(axis=other))
        ext.append(float(hit[-1] - hit[0] + 1))
    Dx, Dy = ext[0], ext[1]
    Dz = ext[2] if c.ndim == 3 else 0.0
    return {"Dx": Dx, "Dy": Dy, "Dz": Dz, "k": Dx / Dy if Dy > 0 else 0.0, "volume": volume, "C_max": c_max}


def _contact_angle(c, solid):
    """Contact angle (degrees) from the last axis' first fluid layer above the
    wall, as lbm/fe_measure.py:132-241: the contact-region point farthest from
    the domain's centre axis gives the contact radius r; the height h of the
    C = 0.5 crossing above the wall top in that column (linear interpolation,
    at least 0.5) gives theta = atan2(r, h).  180 when there is no contact."""
    n_last = c.shape[-1]
    wall_top = 0
    for z in range(n_last):
        if not solid[..., z].all():
            wall_top = z
            break
    first = wall_top + 1
    if first >= n_last:
        return 180.0
    layer = c[..., first] > 0.5
    if not layer.any():
        return 180.0
    pts = np.argwhere(layer)
    centre = np.array([s / 2.0 for s in c.shape[:-1]])
    if c.ndim == 2:
        radii = np.abs(pts[:, 0] - centre[0])
    else:
        radii = np.sqrt((pts[:, 0] - centre[0]) ** 2 + (pts[:, 1] - centre[1]) ** 2)
    i = int(np.argmax(radii))
    r = radii[i]
    if r < 1.0:
        return 180.0
    col = c[tuple(pts[i])]
    h = None
    for z in range(first, n_last - 1):
        if col[z] >= 0.5 and col[z + 1] < 0.5:
            h = z + (col[z] - 0.5) / (col[z] - col[z + 1] + 1e-10)
            break
    if h is None:
        return 180.0
    h = h - wall_top
    if h < 0.5:
        h = 0.5
    return float(np.degrees(np.arctan2(r, h)))


def measure_contact_angle(C, solid_mask, axis: str = "z") -> float:
    """Contact angle estimate in degrees (lbm/fe_measure.py:85-241); the wall is
    below the last axis ('z' in 3-D, 'y' in 2-D)."""
    del axis  # the reference also measures along the last axis whatever it is given
    return float(_contact_angle(_host(C), _host(solid_mask).astype(bool)))


def measure_contact_angle_wall(C, solid_mask, wall_normal, is_boundary, band=(0.1, 0.9)) -> float:
    """Contact angle (degrees) against the local wall normal, for curved as
    well as flat substrates.  No counterpart in the reference, whose
    ``measure_contact_angle`` looks for the contact line in one horizontal
    layer and so reports 180 on a droplet sitting on a sphere or a ridge.

    The contact line is the set of wetting boundary nodes (fluid nodes next to
    the solid, ``is_boundary``) with band[0] < C < band[1].  At each of them
    the interface normal is -grad C from central differences along the grid
    axes, or the second-order one-sided difference (-3 C(x) + 4 C(x + e) -
    C(x + 2e)) / 2 into the fluid along an axis with a solid neighbour; with
    the wall normal n (pointing from the solid into the fluid,
    ``wall_normal``: (ndim, ...) as the solver's ``wetting.wall_normal``),
    cos(theta) = -n . grad C / |grad C|, averaged over the contact-line nodes
    with weights |grad C|.  The angle is measured in the first fluid layer,
    about half a node off the wall surface: on a spherical cap of radius R
    that shifts it by about 1 / (2 R) radians.  180 when there is no contact
    line."""
    c = np.asarray(_host(C), dtype=np.float64)
    solid = _host(solid_mask).astype(bool)
    bnd = _host(is_boundary).astype(bool)
    wn = np.asarray(_host(wall_normal), dtype=np.float64)
    lo, hi = band
    idx = np.argwhere(bnd & ~solid & (c > lo) & (c < hi))
    if len(idx) == 0:
        return 180.0
    shape = np.array(c.shape)
    nd = c.ndim
    at = lambda a, ii: a[tuple(ii.T)]
    f0 = at(c, idx)
    grad = np.zeros((len(idx), nd))
    for axis in range(nd):
        e = np.zeros(nd, dtype=np.int64)
        e[axis] = 1
        ip, im = (idx + e) % shape, (idx - e) % shape
        fp, fm = at(c, ip), at(c, im)
        fpp, fmm = at(c, (idx + 2 * e) % shape), at(c, (idx - 2 * e) % shape)
        sp, sm = at(solid, ip), at(solid, im)
        g = 0.5 * (fp - fm)
        g = np.where(sm & ~sp, 0.5 * (-3.0 * f0 + 4.0 * fp - fpp), g)
        g = np.where(sp & ~sm, 0.5 * (3.0 * f0 - 4.0 * fm + fmm), g)
        grad[:, axis] = np.where(sp & sm, 0.0, g)
    n = np.stack([at(wn[d], idx) for d in range(nd)], axis=1)
    gn = np.linalg.norm(grad, axis=1)
    ok = (gn > 1e-8) & (np.linalg.norm(n, axis=1) > 0.5)
    if not ok.any():
        return 180.0
    cos = -(n[ok] * grad[ok]).sum(axis=1) / gn[ok]
    mean = float((gn[ok] * cos).sum() / gn[ok].sum())
    return float(np.degrees(np.arccos(np.clip(mean, -1.0, 1.0))))
