"""Droplet initial conditions (host numpy; inputs to ``init_fields``).

tanh profile C(r) = 1/2 + 1/2 tanh(2 (R - |r - c|) / xi), clipped to [0, 1] and
stored as float32, with impact velocity u = u_impact * C -- the same fields,
dtypes and return values as pytorch-lbm ``lbm/fe_droplet.py:22-112`` so that
seeded inputs are identical bit for bit.
"""
import numpy as np


def _coords(shape):
    return np.ogrid[tuple(slice(0, s) for s in shape)]


def _profile(shape, center, radius, xi):
    r2 = 0
    for ax, c in zip(_coords(shape), center):
        r2 = r2 + (ax - c) ** 2
    C = 0.5 + 0.5 * np.tanh(2.0 * (radius - np.sqrt(r2)) / xi)
    return np.broadcast_to(np.clip(C, 0.0, 1.0), shape).astype(np.float32)


def create_fe_droplet(nx, ny, nz, center=None, radius=None, xi=5.0, rho_l=828.0, rho_g=1.0):
    """Return (C, rho, u) float32; nz == 1 gives the 2-D layout."""
    shape = (nx, ny) if nz == 1 else (nx, ny, nz)
    if radius is None:
        radius = 0.15 * min(shape)
    if center is None:
        center = (nx / 2.0, ny * 0.6) if nz == 1 else (nx / 2.0, ny / 2.0, nz * 0.6)
    C = _profile(shape, center, radius, xi)
    rho = (C * rho_l + (1.0 - C) * rho_g).astype(np.float32)
    u = np.zeros((len(shape),) + shape, dtype=np.float32)
    return C, rho, u


def create_fe_droplet_with_impact(nx, ny, nz, center=None, radius=None, xi=5.0,
                                  rho_l=828.0, rho_g=1.0, u_impact=None):
    """As ``create_fe_droplet`` with u[d] = u_impact[d] * C."""
    C, rho, u = create_fe_droplet(nx, ny, nz, center, radius, xi, rho_l, rho_g)
    if u_impact is None:
        u_impact = (0.0,) * u.shape[0]
    for d in range(u.shape[0]):
        u[d] = u_impact[d] * C
    return C, rho, u


def create_multi_droplet_with_impact(nx, ny, nz, centers, radii, xi=5.0, rho_l=828.0,
                                     rho_g=1.0, u_impacts=None):
    """Several droplets: C = max_k C_k, u = sum_k u_k C_k."""
    shape = (nx, ny) if nz == 1 else (nx, ny, nz)
    ndim = len(shape)
    if u_impacts is None:
        u_impacts = [(0.0,) * ndim] * len(centers)
    C = np.zeros(shape, dtype=np.float32)
    parts = []
    for c, r in zip(centers, radii):
        Ck = _profile(shape, c, r, xi)
        C = np.maximum(C, Ck)
        parts.append(Ck)
    C = np.clip(C, 0.0, 1.0)
    rho = (C * rho_l + (1.0 - C) * rho_g).astype(np.float32)
    u = np.zeros((ndim,) + shape, dtype=np.float32)
    for Ck, ui in zip(parts, u_impacts):
        for d in range(ndim):
            u[d] += ui[d] * Ck
    return C, rho, u
