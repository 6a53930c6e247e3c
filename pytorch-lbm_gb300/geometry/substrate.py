"""Substrate solid masks and smooth solid fractions (host numpy).

Shapes and numerics follow pytorch-lbm ``geometry/substrate.py`` so that the
same call gives the same arrays bit for bit: a flat wall at z = 0 (3-D) or
y = 0 (2-D), plus

  ridge   cylinder along y through (nx/2, *, 0), radius R_g, above the floor
  convex  sphere centred at (nx/2, ny/2, R_g), radius R_g
  concave outside of that sphere, below its equator

with R_g = |R*| R_d / dx.  The smooth fraction is clip(signed distance + 1/2,
0, 1) (float32 for a flat wall, float64 otherwise -- the reference's dtype
promotion), and solid = fraction >= 0.5.
"""
import numpy as np


def _radius(R_star, R_d, dx):
    if R_star is None or R_d is None:
        return None
    return abs(R_star) * R_d / dx


def create_substrate(nx, ny, nz=1, substrate_type="flat", R_star=None, R_d=None, dx=1.0):
    """Boolean solid mask (True = solid)."""
    R_g = _radius(R_star, R_d, dx)
    if nz == 1:
        solid = np.zeros((nx, ny), dtype=bool)
        solid[:, 0] = True
        if substrate_type == "flat" or R_g is None:
            return solid
        I, J = np.ogrid[:nx, :ny]
        cx = nx / 2.0
        if substrate_type == "convex":
            solid |= ((I - cx) ** 2 + (J - R_g) ** 2) < R_g ** 2
        elif substrate_type == "concave":
            solid |= (((I - cx) ** 2 + (J - R_g) ** 2) > R_g ** 2) & (J < R_g)
        elif substrate_type == "ridge":
            solid |= (((I - cx) ** 2 + J ** 2) < R_g ** 2) & (J > 0)
        return solid
    solid = np.zeros((nx, ny, nz), dtype=bool)
    solid[:, :, 0] = True
    if substrate_type == "flat" or R_g is None:
        return solid
    i, j, k = np.ogrid[:nx, :ny, :nz]
    cx, cy = nx / 2.0, ny / 2.0
    if substrate_type == "convex":
        solid |= ((i - cx) ** 2 + (j - cy) ** 2 + (k - R_g) ** 2) < R_g ** 2
    elif substrate_type == "concave":
        solid |= (((i - cx) ** 2 + (j - cy) ** 2 + (k - R_g) ** 2) > R_g ** 2) & (k < R_g)
    elif substrate_type == "ridge":
        solid |= (((i - cx) ** 2 + k ** 2) < R_g ** 2) & (k > 0)
    return solid


def _compute_surface_height(solid):
    """Index of the topmost solid node per column along the last axis (-1 if none)."""
    kk = np.arange(solid.shape[-1])
    return np.where(solid, kk, -1).max(axis=-1)


def substrate_surface_height(nx, ny, nz=1, substrate_type="flat", R_star=None, R_d=None,
                             dx=1.0):
    return _compute_surface_height(create_substrate(nx, ny, nz, substrate_type, R_star, R_d, dx))


def create_substrate_with_fraction(nx, ny, nz=1, substrate_type="flat", R_star=None,
                                   R_d=None, dx=1.0):
    """Return (solid, fraction)."""
    R_g = _radius(R_star, R_d, dx)
    if nz == 1:
        frac = np.zeros((nx, ny), dtype=np.float32)
        frac[:, 0] = 1.0
        if substrate_type == "flat" or R_g is None:
            return frac >= 0.5, frac
        I, J = np.ogrid[:nx, :ny]
        cx = nx / 2.0
        if substrate_type == "convex":
            sd = R_g - np.sqrt((I - cx) ** 2.0 + (J - R_g) ** 2.0)
            frac = np.maximum(frac, np.clip(sd + 0.5, 0.0, 1.0))
        elif substrate_type == "concave":
            sd = np.sqrt((I - cx) ** 2.0 + (J - R_g) ** 2.0) - R_g
            frac = np.where(J < R_g, np.maximum(frac, np.clip(sd + 0.5, 0.0, 1.0)), frac)
        elif substrate_type == "ridge":
            sd = R_g - np.sqrt((I - cx) ** 2.0 + J.astype(float) ** 2.0)
            frac = np.where(J > 0, np.maximum(frac, np.clip(sd + 0.5, 0.0, 1.0)), frac)
        return frac >= 0.5, frac
    frac = np.zeros((nx, ny, nz), dtype=np.float32)
    frac[:, :, 0] = 1.0
    if substrate_type == "flat" or R_g is None:
        return frac >= 0.5, frac
    i, j, k = np.ogrid[:nx, :ny, :nz]
    cx, cy = nx / 2.0, ny / 2.0
    if substrate_type == "ridge":
        sd = R_g - np.sqrt((i - cx) ** 2.0 + k.astype(float) ** 2.0)
        frac = np.where(k > 0, np.maximum(frac, np.clip(sd + 0.5, 0.0, 1.0)), frac)
    elif substrate_type == "convex":
        sd = R_g - np.sqrt((i - cx) ** 2.0 + (j - cy) ** 2.0 + (k - R_g) ** 2.0)
        frac = np.maximum(frac, np.clip(sd + 0.5, 0.0, 1.0))
    elif substrate_type == "concave":
        sd = np.sqrt((i - cx) ** 2.0 + (j - cy) ** 2.0 + (k - R_g) ** 2.0) - R_g
        frac = np.where(k < R_g, np.maximum(frac, np.clip(sd + 0.5, 0.0, 1.0)), frac)
    frac = np.broadcast_to(frac, (nx, ny, nz)).copy()
    return frac >= 0.5, frac
