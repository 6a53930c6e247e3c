"""Legacy-VTK STRUCTURED_POINTS writer with the reference's signature and
output (pytorch-lbm io_utils/vtk_writer.py:10-86).

``write_vtk(filename, rho, u, solid=None, dx=1.0, step=0, t=0.0)`` writes the
same bytes as the reference: the header, then density, velocity and the solid
flags as "%.6e" ASCII values in C order (z fastest).  Fields may be numpy
arrays or torch tensors (device tensors are copied to the host).  The header is
formatted here, with Python's own float formatting; the point data is formatted
by the native library (``lbm_write_vtk``), in parallel, instead of one Python
f-string per value.
"""
import ctypes
import os

import numpy as np


def _host(x, dtype):
    if hasattr(x, "detach"):
        x = x.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(x), dtype=dtype)


def write_vtk(filename, rho, u, solid=None, dx=1.0, step=0, t=0.0):
    """Write density, velocity and the solid mask of one snapshot to ``filename``.

    rho: (nx, ny[, nz]); u: (dim, nx, ny[, nz]); solid: (nx, ny[, nz]) or None.
    2-D fields are written as nz = 1 with a zero z velocity, as the reference does.
    """
    from lbm import _native as nat

    rho_h = _host(rho, np.float64)
    u_h = _host(u, np.float64)
    dim = u_h.shape[0]
    if dim == 2:
        nx, ny = rho_h.shape
        nz = 1
        ux, uy = u_h[0].reshape(-1), u_h[1].reshape(-1)
        uz = np.zeros_like(ux)
    else:
        nx, ny, nz = rho_h.shape
        ux, uy, uz = u_h[0].reshape(-1), u_h[1].reshape(-1), u_h[2].reshape(-1)
    n_points = nx * ny * nz
    sol = None
    if solid is not None:
        # int(val) of each element, as the reference writes it
        s = solid.detach().cpu().numpy() if hasattr(solid, "detach") else np.asarray(solid)
        sol = np.ascontiguousarray(np.trunc(s.astype(np.float64)).astype(np.int32).reshape(-1))
    header = ("# vtk DataFile Version 3.0\n"
              f"LBM output step={step} t={t:.6e}\n"
              "ASCII\n"
              "DATASET STRUCTURED_POINTS\n"
              f"DIMENSIONS {nx} {ny} {nz}\n"
              "ORIGIN 0 0 0\n"
              f"SPACING {dx} {dx} {dx}\n"
              f"POINT_DATA {n_points}\n")
    os.makedirs(os.path.dirname(filename) or ".", exist_ok=True)
    ux, uy, uz = (np.ascontiguousarray(a) for a in (ux, uy, uz))
    rho_flat = np.ascontiguousarray(rho_h.reshape(-1))
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = nat.lib().lbm_write_vtk(os.fsencode(str(filename)), header.encode(), n_points, ptr(rho_flat), ptr(ux),
                                 ptr(uy), ptr(uz), ptr(sol) if sol is not None else None)
    if rc != 0:
        raise OSError(f"write_vtk: cannot write {filename}")
