"""AllenCahnSolver: drop-in front end of the GB300 Allen-Cahn phase-field LBM.

Same constructor, methods and readable attributes as the reference class
(pytorch-lbm ``lbm/fe_ac_solver.py:51-732``): ``FEConfig`` in,
``set_solid(solid_mask, solid_fraction=None)``, ``init_fields(phi, u=None)``,
``step()``, and the fields ``phi, rho, u, P, p, mu_phi, f, g, solid,
step_count, t, phi_mass_init, wetting``.  Every time step runs on the GPU
through the C ABI of ``liblbm_gb300.so`` (two hand-written sm_103a kernels per
step, see csrc/lbm_kernels.cu); there is no CPU path.

Fields are produced on demand: the device keeps only the state the next step
needs (post-collision populations, velocity, the previous phi) and a read of
``solver.phi`` etc. launches a small read-out kernel that reproduces the value
the reference holds after the same step.  Each read returns a new tensor.

``geo_amplification`` may be a scalar or a per-node field of the grid's shape
(torch tensor or numpy array), as in the reference.  ``interface_mode=
'cahn-hilliard'`` and ``mu_drive > 0`` add a chemical-potential pass per step
(float32 / float64); ``direct_wetting`` relaxes top-surface boundary phi towards
the cubic-wall-energy value.  A 2-D grid (``nz == 1``) runs the D2Q9 form
of the same step (csrc/lbm_kernels2d.cu) in float32 or float64, with fields
of shape ``(nx, ny)`` and ``u`` of shape ``(2, nx, ny)``, as the reference's
2-D path; it steps one grid at a time (no batches, no fused tiles, no half
storage).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _native as nat
from .lattice import D2Q9, D3Q19

_STAB = {"fakhari": 0, "liang": 1, "none": 2}


def _host_array(x, dtype):
    if torch.is_tensor(x):
        x = x.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(x), dtype=dtype)


class WettingTables:
    """Read-only view of the wetting precompute (the attributes of the
    reference's ConningtonLeeWetting that callers read:
    lbm/fe_wetting.py:140,147,305-306), as device tensors made on first
    access (the step kernels use the library's own copies; a solve that never
    reads these pays no copy)."""

    def __init__(self, solver, mode, tables_fn):
        self._dev = solver.device
        self._tables_fn = tables_fn
        self._arrays = {}
        self.mode = mode
        cfg = solver.config
        self.theta_deg = cfg.theta_eq
        self.kappa = cfg.kappa
        self.sigma = cfg.sigma
        self.phi_c = cfg.phi_c
        self._geo_amplification = solver._geo_amplification
        if mode == "linear":
            h = cfg.sigma * math.cos(math.radians(cfg.theta_eq))
            gs = solver._ghost_scale
            if gs is None:
                gs = 3.0 if abs(cfg.theta_eq - 90.0) > 60.0 else 2.0
            self._h = h
            self._ghost_scale = gs
            self._h_over_kappa = h / cfg.kappa * gs
            self._mu_wall = -h * 2.0
        else:
            self._phi_c_over_kappa = cfg.phi_c / cfg.kappa
            self._h = self._h_over_kappa = self._mu_wall = 0.0

    def _get(self, key):
        if key not in self._arrays:
            self._arrays[key] = torch.from_numpy(self._tables_fn()[key]).to(self._dev)
        return self._arrays[key]

    @property
    def is_boundary(self):
        return self._get("is_boundary")

    @property
    def wall_normal(self):
        return self._get("wall_normal")

    @property
    def wall_weight(self):
        return self._get("wall_weight")

    @property
    def near_wall_mask(self):
        return self._get("near_wall")


class AllenCahnSolver:
    """Conservative Allen-Cahn + pressure-velocity NS LBM on one GB300."""

    def __init__(self, config, dtype=torch.float64, stab_mode="auto", mu_drive=0.0,
                 boundary_relax=0.3, interface_mode="allen-cahn", ghost_scale=None,
                 sharpen_reduce=0.8, mu_wall_scale=1.0, geometric_wetting=False,
                 direct_wetting=False, ch_wall_blend=0.0, geo_amplification=1.0, ac_scale=1.0):
        if config.nz == 1 and dtype == torch.float16:
            raise NotImplementedError("2-D (D2Q9) grids run in float32 or float64")
        if interface_mode not in ("allen-cahn", "cahn-hilliard"):
            raise ValueError(f"unknown interface_mode {interface_mode!r}")
        if (interface_mode == "cahn-hilliard" or mu_drive > 0.0) and dtype == torch.float16:
            raise NotImplementedError("interface_mode='cahn-hilliard' and mu_drive > 0 need float32 or float64")
        amp_field = None
        if torch.is_tensor(geo_amplification) or isinstance(geo_amplification, np.ndarray):
            # per-node field (lbm/fe_wetting.py:503-512)
            amp_field = _host_array(geo_amplification, np.float64)
            if amp_field.shape != tuple(config.grid_shape):
                raise ValueError(f"geo_amplification field shape {amp_field.shape} != grid {tuple(config.grid_shape)}")
        if dtype not in (torch.float32, torch.float64, torch.float16):
            raise ValueError("dtype must be torch.float32, torch.float64 or torch.float16")
        self.config = config
        dev = torch.device(config.device) if not isinstance(config.device, torch.device) else config.device
        if dev.type != "cuda":
            raise RuntimeError("the GB300 solver runs on a CUDA device only (config.device='cuda')")
        if not torch.cuda.is_available():
            raise RuntimeError("no CUDA device is available; the GB300 solver has no CPU fallback")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        # float16 selects the deviation-storage form: populations in half
        # precision, arithmetic and the exposed fields in float32
        self.population_dtype = dtype
        self.dtype = torch.float32 if dtype == torch.float16 else dtype
        self.step_count = 0
        self.t = 0.0
        self.stab_mode = "fakhari" if stab_mode == "auto" else stab_mode
        if self.stab_mode not in _STAB:
            raise ValueError(f"unknown stab_mode {stab_mode!r}")
        self.mu_drive = mu_drive
        self.boundary_relax = boundary_relax
        self.interface_mode = interface_mode
        self._ghost_scale = ghost_scale
        self._sharpen_reduce = sharpen_reduce
        self._mu_wall_scale = mu_wall_scale
        self.geometric_wetting = geometric_wetting
        self.direct_wetting = direct_wetting
        self.ch_wall_blend = ch_wall_blend
        self._geo_amplification = geo_amplification
        self._ac_scale = ac_scale
        self.shape = tuple(config.grid_shape)
        self.ndim = len(self.shape)
        self.lattice = D2Q9() if self.ndim == 2 else D3Q19()
        self.cs2 = self.lattice.cs2
        self._tau_f = config.tau_h if config.tau_h > 0 else config.tau_l
        self._tau_g = config.tau_g
        self._mobility = self.cs2 * (self._tau_f - 0.5)
        self.solid = torch.zeros(self.shape, dtype=torch.bool, device=dev)
        self.wetting = None
        self.bounce_back = None
        self.solid_fraction = None
        self._tables = None
        self._phi_wall_target = None
        if config.theta_eq != 90.0:
            c = math.cos(math.radians(config.theta_eq))
            disc = 1.0 - 4.0 * (-c / 3.0)
            self._phi_wall_target = (0.5 * (1.0 - math.sqrt(disc)) if disc >= 0 else
                                     0.5 * (1.0 - math.cos(math.pi - math.radians(config.theta_eq))))
        self._prec = {torch.float32: nat.LBM_F32, torch.float64: nat.LBM_F64,
                      torch.float16: nat.LBM_F16}[dtype]
        p = nat.LbmParams()
        for k in ("rho_l", "rho_g", "sigma", "xi", "beta", "kappa", "phi_c", "tau_l", "tau_g",
                  "tau_h", "theta_eq"):
            setattr(p, k, float(getattr(config, k)))
        gf = tuple(config.g_force[:3]) + (0.0,) * (3 - len(config.g_force[:3]))
        p.g_force = (ctypes.c_double * 3)(*[float(x) for x in gf])
        p.boundary_relax = float(boundary_relax)
        p.sharpen_reduce = float(sharpen_reduce)
        p.mu_wall_scale = float(mu_wall_scale)
        p.geo_amplification = 1.0 if amp_field is not None else float(geo_amplification)
        p.ac_scale = float(ac_scale)
        p.ghost_scale = float(ghost_scale) if ghost_scale is not None else 0.0
        p.stab_mode = _STAB[self.stab_mode]
        p.geometric_wetting = 1 if geometric_wetting else 0
        p.interface_mode = nat.IFACE_CAHN_HILLIARD if interface_mode == "cahn-hilliard" else nat.IFACE_ALLEN_CAHN
        p.mu_drive = float(mu_drive)
        p.direct_wetting = 1 if direct_wetting else 0
        self._params = p
        self._lib = nat.lib()
        h = ctypes.c_void_p()
        with torch.cuda.device(dev):
            nat.check(self._lib.lbm_create(ctypes.byref(p), config.nx, config.ny, config.nz,
                                           self._prec, ctypes.byref(h)), "lbm_create")
        self._h = h
        if amp_field is not None:
            nat.check(self._lib.lbm_set_amplification(h, amp_field.ctypes.data_as(ctypes.c_void_p), nat.LBM_DT_F64),
                      "lbm_set_amplification")
        self._geometry_set = False
        self._initialized = False
        self._cache = {}

    def __del__(self):
        self.close()

    def close(self):
        """Free the device state now (the solver is unusable afterwards)."""
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.lbm_destroy(h)
            except Exception:
                pass
        self._h = None
        self._cache = {}

    # -- setup ----------------------------------------------------------------
    def set_solid(self, solid_mask, solid_fraction=None):
        """lbm/fe_ac_solver.py:193-237 (geometry precompute on the device).

        The mask and the fraction (numpy arrays or tensors) are copied to the
        device once; those copies become the ``solid`` and ``solid_fraction``
        attributes and the inputs of the library's geometry kernels."""
        def to_dev(x, dt):
            t = x.detach() if torch.is_tensor(x) else torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=dt)))
            return t.to(device=self.device).contiguous()

        solid_d = to_dev(solid_mask, np.bool_).to(torch.bool)
        if tuple(solid_d.shape) != self.shape:
            raise ValueError(f"solid mask shape {tuple(solid_d.shape)} != grid {self.shape}")
        frac_d = None
        fdt = nat.LBM_DT_NONE
        if solid_fraction is not None:
            fr = solid_fraction if torch.is_tensor(solid_fraction) else np.asarray(solid_fraction)
            is32 = fr.dtype in (np.float32, torch.float32)
            frac_d = to_dev(fr, np.float32 if is32 else np.float64)
            frac_d = frac_d.to(torch.float32 if is32 else torch.float64)
            fdt = nat.LBM_DT_F32 if is32 else nat.LBM_DT_F64
            if tuple(frac_d.shape) != self.shape:
                raise ValueError(f"solid fraction shape {tuple(frac_d.shape)} != grid {self.shape}")
        with torch.cuda.device(self.device):
            nat.check(self._lib.lbm_set_geometry_device(self._h, nat.ptr(solid_d), nat.ptr(frac_d), fdt,
                                                        nat.stream_ptr()), "lbm_set_geometry_device")
        self._geometry_set = True
        self.solid = solid_d
        if frac_d is not None:
            self.solid_fraction = frac_d if frac_d.dtype == self.dtype else frac_d.to(self.dtype)
        # the kernels read these device copies asynchronously: keep them until init_fields
        self._geo_src = (solid_d, frac_d)
        self._tables = None  # the host tables of this geometry, fetched on first use
        cfg = self.config
        if cfg.theta_eq != 90.0 and cfg.kappa > 0:
            mode = "linear" if cfg.theta_eq > 130.0 or cfg.theta_eq < 50.0 else "quadratic"
            self.wetting = WettingTables(self, mode, self._host_tables)
        else:
            self.wetting = None
        self._cache.clear()

    def _host_tables(self):
        if self._tables is None:
            self._tables = self._geometry_tables()
        return self._tables

    @property
    def _partial_mask(self):
        """Partial-solid nodes (the reference's _partial_mask, lbm/fe_ac_solver.py:210)."""
        return torch.from_numpy(self._host_tables()["partial"]).to(self.device)

    @property
    def _has_partial(self):
        return self._geometry_set and bool(self._host_tables()["partial"].any())

    def _geometry_tables(self):
        N = int(np.prod(self.shape))
        out = dict(node_class=np.empty(N, np.uint8), is_boundary=np.empty(N, np.bool_),
                   wall_normal=np.empty((self.ndim, N), np.float32), wall_weight=np.empty(N, np.float32),
                   near_wall=np.empty(N, np.bool_), partial=np.empty(N, np.bool_))
        c = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        nat.check(self._lib.lbm_get_geometry(self._h, c(out["node_class"]), c(out["is_boundary"]),
                                             c(out["wall_normal"]), c(out["wall_weight"]),
                                             c(out["near_wall"]), c(out["partial"])), "lbm_get_geometry")
        return {k: v.reshape((self.ndim,) + self.shape if k == "wall_normal" else self.shape) for k, v in out.items()}

    def init_fields(self, phi_init, u_init=None):
        """lbm/fe_ac_solver.py:239-261."""
        if not self._geometry_set:
            # the reference allows init before set_solid (no solid nodes)
            self.set_solid(np.zeros(self.shape, dtype=bool))
        stream = nat.stream_ptr()
        if torch.is_tensor(phi_init) and phi_init.is_cuda:
            src_dt = torch.float32 if phi_init.dtype == torch.float32 else torch.float64
            phi_d = phi_init.detach().to(device=self.device, dtype=src_dt).contiguous()
            u_d = (u_init.detach().to(device=self.device, dtype=src_dt).contiguous()
                   if u_init is not None else None)
            self._keep = (phi_d, u_d)
            nat.check(self._lib.lbm_init_fields(self._h, nat.ptr(phi_d), nat.ptr(u_d),
                                                nat.LBM_DT_F32 if src_dt == torch.float32 else nat.LBM_DT_F64,
                                                1, stream), "lbm_init_fields")
        else:
            ph = phi_init.detach().cpu().numpy() if torch.is_tensor(phi_init) else np.asarray(phi_init)
            npdt = np.float32 if ph.dtype == np.float32 else np.float64
            ph = np.ascontiguousarray(ph, dtype=npdt)
            if ph.shape != self.shape:
                raise ValueError(f"phi shape {ph.shape} != grid {self.shape}")
            uh = None
            if u_init is not None:
                uh = u_init.detach().cpu().numpy() if torch.is_tensor(u_init) else np.asarray(u_init)
                uh = np.ascontiguousarray(uh, dtype=npdt)
                if uh.shape != (self.ndim,) + self.shape:
                    raise ValueError(f"u shape {uh.shape} != ({self.ndim},) + grid")
            # host sources are copied asynchronously: keep them alive until the copy ran
            self._keep = (ph, uh)
            nat.check(self._lib.lbm_init_fields(
                self._h, ph.ctypes.data_as(ctypes.c_void_p),
                uh.ctypes.data_as(ctypes.c_void_p) if uh is not None else None,
                nat.LBM_DT_F32 if npdt == np.float32 else nat.LBM_DT_F64, 0, stream), "lbm_init_fields")
            torch.cuda.current_stream().synchronize()
        self._keep = None
        self._geo_src = None
        self._initialized = True
        self.step_count = 0
        self.t = 0.0
        self._cache.clear()

    # -- time stepping --------------------------------------------------------
    def step(self):
        """One time step (lbm/fe_ac_solver.py:380-639); asynchronous on the
        current CUDA stream."""
        self.run(1)

    def run(self, nsteps, stream=None):
        """``nsteps`` time steps in one call."""
        if not self._initialized:
            raise RuntimeError("init_fields must be called before step()")
        nat.check(self._lib.lbm_step(self._h, int(nsteps), nat.stream_ptr(stream)), "lbm_step")
        self.step_count += int(nsteps)
        self.t += float(nsteps)
        self._cache.clear()

    # -- mid-run droplet injection --------------------------------------------
    def inject_droplet(self, center, radius, xi, u_impact=None):
        """Inject a droplet at the current time step (lbm/fe_ac_solver.py:645-732):
        phi = max(phi, C) in the droplet core (C > 0.1), u blended towards
        ``u_impact`` with weight C, f and g reset to equilibrium at the core
        nodes, the phi-mass reference re-based, no previous phi u."""
        if not self._initialized:
            raise RuntimeError("init_fields must be called before inject_droplet()")
        if u_impact is None:
            u_impact = (0.0,) * self.ndim
        # the C ABI takes three components; a 2-D grid ignores the third
        pad = lambda v: [float(x) for x in v][:3] + [0.0] * (3 - min(len(v), 3))
        c = (ctypes.c_double * 3)(*pad(center))
        uv = (ctypes.c_double * 3)(*pad(u_impact))
        core = ctypes.c_int64()
        nat.check(self._lib.lbm_inject_droplet(self._h, c, float(radius), float(xi), uv, ctypes.byref(core),
                                               nat.stream_ptr()), "lbm_inject_droplet")
        self._cache.clear()
        center_str = ",".join(f"{x:.0f}" for x in center)
        vel_str = ",".join(f"{x:.3f}" for x in u_impact)
        print(f"  [inject] Droplet at ({center_str}) R={radius:.1f} u=({vel_str}) core_nodes={core.value}")
        return int(core.value)

    # -- fields ---------------------------------------------------------------
    def _fields(self, want):
        missing = [k for k in want if k not in self._cache]
        if missing:
            if not self._initialized:
                raise RuntimeError("fields are defined after init_fields")
            bits = {"phi": nat.FIELD_PHI, "rho": nat.FIELD_RHO, "u": nat.FIELD_U, "P": nat.FIELD_P,
                    "p": nat.FIELD_PRESS, "mu_phi": nat.FIELD_MU}
            mask = 0
            out = {}
            for k in missing:
                shp = (self.ndim,) + self.shape if k == "u" else self.shape
                out[k] = torch.empty(shp, dtype=self.dtype, device=self.device)
                mask |= bits[k]
            nat.check(self._lib.lbm_get_fields(
                self._h, mask, nat.ptr(out.get("phi")), nat.ptr(out.get("rho")), nat.ptr(out.get("u")),
                nat.ptr(out.get("P")), nat.ptr(out.get("p")), nat.ptr(out.get("mu_phi")),
                nat.stream_ptr()), "lbm_get_fields")
            self._cache.update(out)
        return [self._cache[k] for k in want]

    @property
    def phi(self):
        return self._fields(["phi"])[0]

    @property
    def rho(self):
        return self._fields(["rho"])[0]

    @property
    def u(self):
        return self._fields(["u"])[0]

    @property
    def P(self):
        return self._fields(["P"])[0]

    @property
    def p(self):
        return self._fields(["p"])[0]

    @property
    def mu_phi(self):
        return self._fields(["mu_phi"])[0]

    def fields(self, *names):
        """Several fields from one read-out launch, e.g. ``fields('phi', 'u')``."""
        return self._fields(list(names))

    def _populations(self):
        if "f" not in self._cache:
            f = torch.empty((self.lattice.q,) + self.shape, dtype=self.dtype, device=self.device)
            g = torch.empty_like(f)
            nat.check(self._lib.lbm_get_populations(self._h, nat.ptr(f), nat.ptr(g), nat.stream_ptr()),
                      "lbm_get_populations")
            self._cache["f"], self._cache["g"] = f, g
        return self._cache["f"], self._cache["g"]

    @property
    def f(self):
        return self._populations()[0]

    @property
    def g(self):
        return self._populations()[1]

    @property
    def phi_mass_init(self):
        if not self._initialized:
            return None
        m = ctypes.c_double()
        nat.check(self._lib.lbm_get_scalars(self._h, ctypes.byref(m), None, None, None), "lbm_get_scalars")
        return float(m.value)

    def scalars(self):
        """(phi_mass_init, last sum(phi), last mass-correction factor, steps)."""
        a, b, c, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
        nat.check(self._lib.lbm_get_scalars(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                            ctypes.byref(n)), "lbm_get_scalars")
        return a.value, b.value, c.value, n.value

    def measure(self, stream=None):
        """Spread diagnostics of the current phi, reduced on the device:
        volume, C_max, Dx, Dy, Dz, k, z_com, count, has_nan.  On a 2-D grid
        Dz is 0 and z_com is the centre along y (the wall-normal axis)."""
        out = (ctypes.c_double * 9)()
        nat.check(self._lib.lbm_measure(self._h, out, nat.stream_ptr(stream)), "lbm_measure")
        keys = ("volume", "C_max", "Dx", "Dy", "Dz", "k", "z_com", "count", "has_nan")
        d = dict(zip(keys, list(out)))
        d["count"] = int(d["count"])
        d["has_nan"] = bool(d["has_nan"])
        return d

    def reduce(self, stream=None):
        """Global float64 reductions of the current fields on the device:
        sum_phi, momentum (sum rho u, 3 components), extents (first and last
        x, y, z index of phi > 0.5; -1 when empty), C_max.  On a 2-D grid the
        z momentum is 0 and the z extents are 0 (-1 when empty)."""
        sp, cm = ctypes.c_double(), ctypes.c_float()
        mom = (ctypes.c_double * 3)()
        ext = (ctypes.c_int32 * 6)()
        nat.check(self._lib.lbm_reduce(self._h, ctypes.byref(sp), mom, ext, ctypes.byref(cm),
                                       nat.stream_ptr(stream)), "lbm_reduce")
        return {"sum_phi": sp.value, "momentum": tuple(mom), "extents": tuple(ext), "C_max": cm.value}

    def autotune(self, reps=5, stream=None):
        """Pick the fastest step kernel (the two-kernel step or a tile shape of
        the fused kernel) on the current state (the state is left unchanged).
        Returns ((tx, ty, tz), ms per step); (0, 0, 0) is the two-kernel step."""
        t = (ctypes.c_int * 3)()
        ms = ctypes.c_float()
        nat.check(self._lib.lbm_autotune(self._h, int(reps), nat.stream_ptr(stream), t, ctypes.byref(ms)),
                  "lbm_autotune")
        return (t[0], t[1], t[2]), float(ms.value)

    def set_launch_shape(self, phi_nodes_per_thread, update_block):
        """Launch shape of the two-kernel step (results do not depend on it)."""
        nat.check(self._lib.lbm_set_launch(self._h, int(phi_nodes_per_thread), int(update_block)), "lbm_set_launch")

    def launch_shape(self):
        """(phi-kernel nodes per thread, update-kernel threads per block) of the
        two-kernel step, as the autotuner left them."""
        a, b = ctypes.c_int(), ctypes.c_int()
        nat.check(self._lib.lbm_get_launch(self._h, ctypes.byref(a), ctypes.byref(b)), "lbm_get_launch")
        return int(a.value), int(b.value)

    def set_tile(self, tx, ty, tz):
        """Step kernel selection: (0, 0, 0) the two-kernel streaming step (the
        default), else the fused tiled kernel with these tile extents."""
        nat.check(self._lib.lbm_set_tile(self._h, int(tx), int(ty), int(tz)), "lbm_set_tile")

    def get_tile(self):
        """The current step kernel selection ((0, 0, 0) = two-kernel step)."""
        t = (ctypes.c_int * 3)()
        nat.check(self._lib.lbm_get_tile(self._h, t), "lbm_get_tile")
        return tuple(t)

    def set_layout(self, paired):
        """Device storage layout (before ``init_fields``): linear (one element
        per node, the default) or paired (nodes x and x + nx/2 in one word,
        stepped a pair per thread; 3-D float32 / float16 grids with even nx).
        The fields and populations read back are the same in either."""
        nat.check(self._lib.lbm_set_layout(self._h, 1 if paired else 0), "lbm_set_layout")

    @property
    def paired(self):
        """True when the state uses the paired storage layout."""
        v = ctypes.c_int()
        nat.check(self._lib.lbm_get_layout(self._h, ctypes.byref(v)), "lbm_get_layout")
        return bool(v.value)

    # -- checkpoints and snapshots ---------------------------------------------
    def state_dict(self):
        """The complete time-stepping state as host data: resuming from it
        (``load_state_dict`` on a solver built with the same config, options,
        precision and geometry) continues bit-identically.  The reference has
        no counterpart; this is what its long runs lacked for restarts."""
        if not self._initialized:
            raise RuntimeError("state_dict is defined after init_fields")
        n = ctypes.c_int64()
        nat.check(self._lib.lbm_state_bytes(self._h, ctypes.byref(n)), "lbm_state_bytes")
        buf = np.empty(n.value, dtype=np.uint8)
        nat.check(self._lib.lbm_save_state(self._h, buf.ctypes.data_as(ctypes.c_void_p), n.value, nat.stream_ptr()),
                  "lbm_save_state")
        return {"format": "lbm_gb300.state.v1", "grid": tuple(self.shape),
                "precision": str(self.population_dtype).replace("torch.", ""),
                "step_count": int(self.step_count), "t": float(self.t), "state": buf}

    def load_state_dict(self, state):
        """Restore a ``state_dict`` (after ``set_solid`` with the same geometry)."""
        if not self._geometry_set:
            raise RuntimeError("call set_solid (the same geometry) before load_state_dict")
        if str(state["format"]) != "lbm_gb300.state.v1":
            raise ValueError(f"unknown state format {state['format']!r}")
        buf = np.ascontiguousarray(state["state"], dtype=np.uint8)
        nat.check(self._lib.lbm_load_state(self._h, buf.ctypes.data_as(ctypes.c_void_p), buf.size, nat.stream_ptr()),
                  "lbm_load_state")
        self.step_count = int(state["step_count"])
        self.t = float(state["t"])
        self._initialized = True
        self._cache.clear()

    def save_checkpoint(self, path):
        """``state_dict`` to an ``.npz`` file."""
        sd = self.state_dict()
        np.savez(path, format=np.array(sd["format"]), grid=np.array(sd["grid"]), precision=np.array(sd["precision"]),
                 step_count=np.array(sd["step_count"]), t=np.array(sd["t"]), state=sd["state"])

    def load_checkpoint(self, path):
        """Restore a checkpoint written by ``save_checkpoint``."""
        with np.load(path) as z:
            grid = tuple(int(x) for x in z["grid"])
            if grid != tuple(self.shape):
                raise ValueError(f"checkpoint grid {grid} != solver grid {tuple(self.shape)}")
            self.load_state_dict({"format": str(z["format"]), "step_count": int(z["step_count"]),
                                  "t": float(z["t"]), "state": z["state"]})

    def save_snapshot(self, path, step=None):
        """Compressed ``.npz`` snapshot of phi, u and the solid mask with the
        mid-plane slices, in the key layout of the reference's sweep driver
        (scripts/run_thesis_sweep.py:219-243): phi_3d, u_3d, solid_3d, xz_slice,
        yz_slice, xz_solid, step, nx, ny, nz."""
        if self.ndim == 2:
            raise NotImplementedError("snapshots in the sweep-driver layout are 3-D")
        phi, vel = self.fields("phi", "u")
        phi_np = phi.detach().cpu().numpy()
        u_np = vel.detach().cpu().numpy()
        solid_np = self.solid.cpu().numpy()
        nx, ny, nz = self.shape
        np.savez_compressed(path, phi_3d=phi_np, u_3d=u_np, solid_3d=solid_np,
                            xz_slice=phi_np[:, ny // 2, :], yz_slice=phi_np[nx // 2, :, :],
                            xz_solid=solid_np[:, ny // 2, :],
                            step=self.step_count if step is None else step, nx=nx, ny=ny, nz=nz)

    def status(self):
        v = ctypes.c_uint32()
        nat.check(self._lib.lbm_status(self._h, ctypes.byref(v)), "lbm_status")
        return int(v.value)
