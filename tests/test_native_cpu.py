"""The C-ABI library without a GPU: it loads, exports every declared entry
point, computes the geometry tables bit-exact, and rejects bad arguments."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from _cases import CASES, config, golden, inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(lbm_\w+)\s*\(", src))
    return names


def test_exports_every_declared_symbol(built_lib):
    from lbm import _native
    declared = _declared()
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(built_lib, name), name
    assert set(_native.EXPORTS) == declared
    out = subprocess.run(["nm", "-D", "--defined-only", _native.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (lbm_\w+)", out))
    assert declared <= exported


def _geometry(lib, case, precision):
    nx, ny, nz = case["grid"]
    N = nx * ny * nz
    solid, frac, _, _ = inputs(case)
    cfg = config(case)
    nd = 2 if nz == 1 else 3  # 2-D grids: D2Q9, two normal components
    o = dict(cls=np.empty(N, np.uint8), bnd=np.empty(N, np.bool_), wn=np.empty((nd, N), np.float32),
             ww=np.empty(N, np.float32), near=np.empty(N, np.bool_), part=np.empty(N, np.bool_))
    c = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    fr = None if frac is None else np.ascontiguousarray(frac)
    fdt = 0 if fr is None else (1 if fr.dtype == np.float32 else 2)
    s8 = np.ascontiguousarray(solid).view(np.uint8)
    rc = lib.lbm_geometry_host(nx, ny, nz, c(s8), c(fr) if fr is not None else None, fdt, cfg.theta_eq,
                               cfg.kappa, precision, c(o["cls"]), c(o["bnd"]), c(o["wn"]), c(o["ww"]),
                               c(o["near"]), c(o["part"]))
    assert rc == 0, lib.lbm_last_error()
    shp = (nx, ny) if nz == 1 else (nx, ny, nz)
    return {k: (v.reshape((nd,) + shp) if k == "wn" else v.reshape(shp)) for k, v in o.items()}


@pytest.mark.parametrize("name,dn", [(n, d) for n, c in CASES.items() for d in c["dtypes"]])
def test_native_geometry_bit_exact(built_lib, name, dn):
    case = CASES[name]
    gd = golden(name, dn)
    o = _geometry(built_lib, case, 0 if dn == "float32" else 1)
    assert np.array_equal(o["cls"] & 1 == 1, gd["solid"])
    if "is_boundary" in gd:
        assert np.array_equal(o["bnd"], gd["is_boundary"])
        # bit for bit, signed zeros included
        assert np.array_equal(o["wn"].view(np.uint32), gd["wall_normal"].view(np.uint32))
        assert np.array_equal(o["ww"].view(np.uint32), gd["wall_weight"].view(np.uint32))
        assert np.array_equal(o["near"], gd["near_wall"])
    else:
        assert not o["bnd"].any()
    if "partial" in gd:
        assert np.array_equal(o["part"], gd["partial"])
    else:
        assert not o["part"].any()
    # class byte consistency
    assert np.array_equal((o["cls"] >> 1) & 1 == 1, o["bnd"])
    assert np.array_equal((o["cls"] >> 2) & 1 == 1, o["part"])
    assert np.all((o["cls"][o["cls"] & 1 == 1] >> 4) == 13)


def test_argument_errors(built_lib):
    from lbm import _native as nat
    p = nat.LbmParams(rho_l=1.0, rho_g=1 / 828.0, sigma=0.01, xi=4.0, beta=0.03, kappa=0.06,
                      tau_l=0.53, tau_g=0.53, tau_h=1.0, theta_eq=120.0)
    h = ctypes.c_void_p()
    assert built_lib.lbm_create(ctypes.byref(p), 8, 8, 0, 0, ctypes.byref(h)) == -4
    assert b"3-D" in built_lib.lbm_last_error()
    # 2-D grids (nz == 1) run in float32 or float64 only
    assert built_lib.lbm_create(ctypes.byref(p), 8, 8, 1, nat.LBM_F16, ctypes.byref(h)) == -4
    assert b"2-D" in built_lib.lbm_last_error()
    assert built_lib.lbm_create(ctypes.byref(p), 8, 8, 8, 7, ctypes.byref(h)) == -1
    assert built_lib.lbm_create(None, 8, 8, 8, 0, ctypes.byref(h)) == -1
    bad = nat.LbmParams(rho_l=1.0, rho_g=1.0, xi=4.0, tau_l=0.5, tau_g=0.53)
    assert built_lib.lbm_create(ctypes.byref(bad), 8, 8, 8, 0, ctypes.byref(h)) == -1
    solid = np.zeros(512, np.uint8)
    assert built_lib.lbm_geometry_host(8, 8, 8, solid.ctypes.data_as(ctypes.c_void_p), None, 1, 120.0, 0.06, 0,
                                       None, None, None, None, None, None) == -1
    assert built_lib.lbm_step(None, 1, None) == -1
    assert built_lib.lbm_destroy(None) == 0


def test_device_tables_match_host_tables(tmp_path):
    """The constexpr D3Q19 functions used in device code equal the host table."""
    src = tmp_path / "t.cu"
    src.write_text(
        '#include <cstdio>\n#include "lbm_common.cuh"\n#include "lbm_tables.h"\n'
        "int main(){int bad=0;for(int q=0;q<19;++q){"
        "if(lbm::ex(q)!=lbm::kE[q][0]||lbm::ey(q)!=lbm::kE[q][1]||lbm::ez(q)!=lbm::kE[q][2]||"
        "lbm::opp(q)!=lbm::kOpp[q])bad++;"
        "if(lbm::kE[lbm::kOpp[q]][0]!=-lbm::kE[q][0]||lbm::kE[lbm::kOpp[q]][1]!=-lbm::kE[q][1]||"
        "lbm::kE[lbm::kOpp[q]][2]!=-lbm::kE[q][2])bad++;}"
        'printf("%d\\n",bad);return bad;}\n')
    exe = tmp_path / "t"
    from lbm._build import CSRC, _nvcc
    r = subprocess.run([_nvcc(), "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "0"


def test_cache_entry_points_without_a_gpu(built_lib):
    """The state-array cache is empty in a process that made no grid: its
    size, trim and limit need no device."""
    from lbm import _native as nat
    assert nat.cache_bytes() == 0
    assert nat.cache_trim() == 0
    nat.cache_limit(0)
    nat.cache_limit(16 << 30)
    assert built_lib.lbm_cache_bytes(None) != 0  # null output pointer rejected
