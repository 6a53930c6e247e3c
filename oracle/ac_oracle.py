"""CPU oracle for the Allen-Cahn phase-field LBM time step -- TEST INFRASTRUCTURE.

This module is a numpy restatement of the reference solver's per-timestep
algorithm (pytorch-lbm, ``lbm/fe_ac_solver.py`` and ``lbm/fe_wetting.py``).
It is the checker for the CUDA path: only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it.  The product package
never imports it and never falls back to it.

Parity status: pinned.  ``tests/golden/make_golden.py`` runs the reference
itself (PyTorch, CPU) on small seeded cases and commits its outputs;
``tests/test_oracle_golden.py`` checks this restatement against them
(setup tables bit-exact, fields within a few float ulps -- torch's CPU
reductions use a size- and thread-dependent summation order that no
restatement can reproduce bit for bit).

Arithmetic follows the reference operation by operation, in the dtype the
reference computes in (float32 or float64):
  * python scalars enter an array operation cast to the array dtype
    (numpy NEP 50 "weak" scalars == torch wrapped-number semantics);
  * ``scalar / tensor`` in torch is ``reciprocal(tensor) * scalar``
    (torch/_tensor.py ``__rdiv__``) and is restated that way;
  * the lattice tables are float32 even in float64 runs
    (lbm/lattice.py:19-21, cast at lbm/fe_ac_solver.py:118-119);
  * wall geometry (normals, n.e, wall weight) is float32 in every mode
    (lbm/fe_wetting.py:147,237,281,299);
  * sums over the 19 populations / 3 components run sequentially in index
    order (the reference's order is torch-internal; see the parity note).
"""
from __future__ import annotations

import math

import numpy as np

# ---------------------------------------------------------------------------
# D3Q19 tables -- same velocity ordering, weights and opposites as
# lbm/lattice.py:60-96 (the ordering is part of the population layout).
# ---------------------------------------------------------------------------
E = np.array([
    [0, 0, 0],
    [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
    [1, 1, 0], [-1, 1, 0], [-1, -1, 0], [1, -1, 0],
    [1, 0, 1], [-1, 0, 1], [-1, 0, -1], [1, 0, -1],
    [0, 1, 1], [0, -1, 1], [0, -1, -1], [0, 1, -1],
], dtype=np.int64)
W32 = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, dtype=np.float32)
OPP = np.array([0, 2, 1, 4, 3, 6, 5, 9, 10, 7, 8, 13, 14, 11, 12, 17, 18, 15, 16],
               dtype=np.int64)
Q = 19
# D2Q9 tables of the 2-D (nz == 1) grids, lbm/lattice.py:36-57.
E2 = np.array([[0, 0], [1, 0], [-1, 0], [0, 1], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]], dtype=np.int64)
W2_32 = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4, dtype=np.float32)
OPP2 = np.array([0, 2, 1, 4, 3, 7, 8, 5, 6], dtype=np.int64)
CS2 = 1.0 / 3.0


def lattice_tables(ndim):
    """(e, float32 w, opp, q) of D2Q9 for ndim == 2, D3Q19 for ndim == 3."""
    return (E2, W2_32, OPP2, 9) if ndim == 2 else (E, W32, OPP, Q)
XI_NEAR_WALL = 5.0  # hard-coded interface width of the near-wall weight (lbm/fe_wetting.py:81)


def _seqsum(a):
    """Sum over axis 0 in index order (acc = a[0]; acc += a[1]; ...)."""
    acc = a[0].copy()
    for k in range(1, a.shape[0]):
        acc = acc + a[k]
    return acc


def _shift_from(a, e):
    """Return b with b[x] = a[x + e] (periodic) == torch.roll(a, -e)."""
    return np.roll(a, shift=tuple(-int(x) for x in e), axis=tuple(range(len(e))))


def _shift_to(a, e):
    """Return b with b[x] = a[x - e] (periodic) == torch.roll(a, +e)."""
    return np.roll(a, shift=tuple(int(x) for x in e), axis=tuple(range(len(e))))


def _exp_f32(x):
    """float32 exp, correctly rounded (matches torch.exp on float32 for the
    near-wall weight table; numpy's own float32 exp differs by 1 ulp on some
    of those inputs)."""
    x = np.asarray(x, dtype=np.float32)
    return np.exp(x.astype(np.float64)).astype(np.float32)


# ---------------------------------------------------------------------------
# Wetting precompute: ConningtonLeeWetting.__init__ / _precompute_*
# (lbm/fe_wetting.py:39-367)
# ---------------------------------------------------------------------------
class OracleWetting:
    def __init__(self, solid, phi_c, kappa, sigma, theta_deg, mode,
                 ghost_scale=None, geo_amplification=1.0, solid_fraction=None):
        self.solid = solid
        self.mode = mode
        self.theta_deg = theta_deg
        self.kappa = kappa
        self.sigma = sigma
        self.phi_c = phi_c
        # lbm/fe_wetting.py:85-115
        if mode == 'linear':
            cos_t = math.cos(math.radians(theta_deg))
            self.h = sigma * cos_t
            if ghost_scale is None:
                ghost_scale = 3.0 if abs(theta_deg - 90.0) > 60.0 else 2.0
            self.h_over_kappa = self.h / kappa * ghost_scale
            self.mu_wall = -self.h * 2.0
            self.ghost_scale = ghost_scale
        else:
            self.phi_c_over_kappa = phi_c / kappa
            self.h = 0.0
            self.h_over_kappa = 0.0
            self.mu_wall = 0.0
        self.geo_amplification = geo_amplification
        self._precompute(solid_fraction)

    def _precompute(self, frac):
        solid = self.solid
        shape = solid.shape
        D = solid.ndim
        E_, _, _, Q_ = lattice_tables(D)
        self.E, self.Q = E_, Q_
        # is_boundary: fluid node with a solid neighbour, periodic (fe_wetting.py:129-140)
        isb = np.zeros(shape, dtype=bool)
        for i in range(1, Q_):
            isb |= _shift_to(solid, E_[i]) & ~solid
        self.is_boundary = isb

        wn = np.zeros((D,) + shape, dtype=np.float32)
        if frac is not None:
            # smooth normals: -grad(frac)/|grad(frac)| in frac's dtype (fe_wetting.py:242-267)
            grad = np.gradient(frac)
            mag = np.sqrt(sum(gd ** 2 for gd in grad))
            mag[mag < 1e-10] = 1e-10
            for d in range(D):
                wn[d] = (-grad[d] / mag * isb).astype(np.float32)
        else:
            # discrete neighbour counting, non-periodic bounds (fe_wetting.py:152-203)
            for x in np.argwhere(isb):
                normal = np.zeros(D)
                count = 0
                for i in range(1, Q_):
                    j = x + E_[i]
                    if all(0 <= j[d] < shape[d] for d in range(D)) and solid[tuple(j)]:
                        normal -= E_[i]
                        count += 1
                if count > 0:
                    normal /= count
                    acc = normal[0] ** 2
                    for d in range(1, D):
                        acc = acc + normal[d] ** 2
                    norm = np.sqrt(acc)
                    if norm > 1e-10:
                        normal /= norm
                wn[(slice(None),) + tuple(x)] = normal
        self.wall_normal = wn

        # near-wall distance: 11 passes of periodic face-neighbour min-plus (fe_wetting.py:280-311)
        dist = np.full(shape, 100.0, dtype=np.float32)
        dist[isb] = 0.0
        for _ in range(int(2 * XI_NEAR_WALL) + 1):
            new = dist.copy()
            for d in range(D):
                for s in (-1, 1):
                    new = np.minimum(new, np.roll(dist, s, axis=d) + np.float32(1.0))
            dist = new
        dist[solid] = 100.0
        ww = _exp_f32(-dist / np.float32(XI_NEAR_WALL / 2.0))
        ww[solid] = 0.0
        self.dist = dist
        self.wall_weight = ww
        self.near_wall_mask = (dist < 2.0 * XI_NEAR_WALL) & ~solid

        # next-interior node of every boundary node, one step along the rounded
        # wall normal (round half to even, clamped to the grid, not periodic),
        # and whether it is fluid (fe_wetting.py:313-367)
        bnd = np.argwhere(isb)
        shift = np.rint(np.stack([wn[d][isb] for d in range(D)], axis=1)).astype(np.int64)
        nsw = np.clip(bnd + shift, 0, np.array(shape) - 1)
        self.bnd_flat = np.ravel_multi_index(bnd.T, shape)
        self.nsw_flat = np.ravel_multi_index(nsw.T, shape)
        self.nsw_is_fluid = ~solid.reshape(-1)[self.nsw_flat]
        self.cubic_a = 6.0 * self.sigma * math.cos(math.radians(self.theta_deg)) / self.kappa

        # per-direction ghost masks and n.e_i in float32 (fe_wetting.py:221-240)
        self.ghost_mask = [None] * Q_
        self.n_dot_e = [None] * Q_
        for i in range(1, Q_):
            m = _shift_from(solid, E_[i]) & isb
            if m.any():
                nde = np.zeros(shape, dtype=np.float32)
                for d in range(D):
                    nde = nde + wn[d] * np.float32(E_[i, d])
                self.ghost_mask[i] = m
                self.n_dot_e[i] = nde

    def cubic_boundary_phi(self, phi):
        """Boundary phi from the cubic wall energy (fe_wetting.py:369-416):
        the root of a phi_b^2 + (1 - a) phi_b - phi_nsw = 0 at boundary nodes
        whose next-interior node is fluid and 0.01 < phi < 0.99."""
        a = self.cubic_a
        if self.bnd_flat.size == 0 or abs(a) < 1e-10:
            return phi
        T = phi.dtype.type
        flat = phi.reshape(-1)
        phi_nsw = flat[self.nsw_flat]
        old = flat[self.bnd_flat].copy()
        oma = 1.0 - a
        disc = np.maximum(oma ** 2 + (4.0 * a) * phi_nsw, T(0))
        pb = np.clip((-oma + np.sqrt(disc)) / (2.0 * a), T(0), T(1))
        active = self.nsw_is_fluid & (old > 0.01) & (old < 0.99)
        out = phi.copy()
        of = out.reshape(-1)
        of[self.bnd_flat[active]] = pb[active]
        return out

    def correct_shifted(self, phi, phi_shifted, i):
        """fe_wetting.py:418-446."""
        m = self.ghost_mask[i]
        if m is None:
            return phi_shifted
        nde = self.n_dot_e[i]
        if self.mode == 'linear':
            val = phi - nde * self.h_over_kappa
        else:
            val = phi + nde * self.phi_c_over_kappa * phi * (1.0 - phi)
        return np.where(m, val, phi_shifted)

    def correct_gradient(self, grad):
        """Geometric contact-angle gradient correction with amplification
        (fe_wetting.py:448-539, near_wall_only=True)."""
        T = grad.dtype.type
        if not self.near_wall_mask.any():
            return grad
        n_w = self.wall_normal.astype(T)
        g_n = _seqsum(n_w * grad)
        g_t = grad - g_n[None] * n_w
        g_t_mag = np.maximum(np.sqrt(_seqsum(g_t * g_t)), T(1e-10))
        cos_t = math.cos(math.radians(self.theta_deg))
        sin_t = math.sin(math.radians(self.theta_deg))
        if abs(sin_t) < 1e-10:
            return grad
        g_n_des = -g_t_mag * cos_t / sin_t
        amp = self.geo_amplification
        if isinstance(amp, np.ndarray):
            a = amp.astype(T)
            delta = g_n_des - g_n
            g_n_des = np.where(a > 1.0, g_n + delta * a, g_n_des)
        elif amp is not None and amp > 1.0:
            delta = g_n_des - g_n
            g_n_des = g_n + delta * amp
        gc = g_t + g_n_des[None] * n_w
        grad_mag = np.sqrt(_seqsum(grad * grad))
        apply = self.near_wall_mask & (grad_mag > 1e-6)
        blend = self.wall_weight.astype(T)
        corrected = grad + blend[None] * (gc - grad)
        return np.where(apply[None], corrected, grad)


# ---------------------------------------------------------------------------
# The solver restatement (lbm/fe_ac_solver.py:54-639)
# ---------------------------------------------------------------------------
class OracleSolver:
    """numpy restatement of AllenCahnSolver: D3Q19 on 3-D grids, D2Q9 on
    2-D grids (nz == 1, shape (nx, ny)).

    ``cfg`` is any object with the FEConfig fields (nx, ny, nz, rho_l, rho_g,
    sigma, xi, beta, kappa, phi_c, tau_l, tau_g, tau_h, theta_eq, g_force).
    """

    def __init__(self, cfg, dtype=np.float64, stab_mode='auto', boundary_relax=0.3,
                 ghost_scale=None, sharpen_reduce=0.8, mu_wall_scale=1.0,
                 geometric_wetting=False, geo_amplification=1.0, ac_scale=1.0,
                 interface_mode='allen-cahn', mu_drive=0.0, direct_wetting=False):
        self.cfg = cfg
        self.T = np.dtype(dtype).type
        T = self.T
        self.shape = (cfg.nx, cfg.ny) if cfg.nz == 1 else (cfg.nx, cfg.ny, cfg.nz)
        self.D = len(self.shape)
        self.E, W32_, self.OPP, self.Q = lattice_tables(self.D)
        self.stab_mode = 'fakhari' if stab_mode == 'auto' else stab_mode
        self.boundary_relax = boundary_relax
        self.ghost_scale = ghost_scale
        self.sharpen_reduce = sharpen_reduce
        self.mu_wall_scale = mu_wall_scale
        self.geometric_wetting = geometric_wetting
        self.geo_amplification = geo_amplification
        self.ac_scale = ac_scale
        self.interface_mode = interface_mode
        self.mu_drive = mu_drive
        self.direct_wetting = direct_wetting
        self.rho_floor = 0.5 * cfg.rho_l
        self.w = W32_.astype(T)
        self.w_view = self.w.reshape((self.Q,) + (1,) * self.D)
        self.tau_f = cfg.tau_h if cfg.tau_h > 0 else cfg.tau_l
        self.tau_g = cfg.tau_g
        self.step_count = 0
        self.solid = np.zeros(self.shape, dtype=bool)
        self.solid_any = False
        self.partial = None
        self.has_partial = False
        self.wetting = None
        self.phi_mass_init = None
        self.phi_u_prev = None
        # lbm/fe_ac_solver.py:165-177
        self.phi_wall_target = None
        if cfg.theta_eq != 90.0:
            cos_t = math.cos(math.radians(cfg.theta_eq))
            disc = 1.0 - 4.0 * (-cos_t / 3.0)
            if disc >= 0:
                self.phi_wall_target = 0.5 * (1.0 - math.sqrt(disc))
            else:
                comp = math.pi - math.radians(cfg.theta_eq)
                self.phi_wall_target = 0.5 * (1.0 - math.cos(comp))

    # -- setup ------------------------------------------------------------
    def set_solid(self, solid, solid_fraction=None):
        """lbm/fe_ac_solver.py:193-237."""
        T = self.T
        self.solid = np.asarray(solid, dtype=bool)
        self.solid_any = bool(self.solid.any())
        if solid_fraction is not None:
            fr = np.asarray(solid_fraction)
            self.partial = (fr > 0.01) & (fr < 0.99) & ~self.solid
            self.eps = fr.astype(T)
            self.has_partial = bool(self.partial.any())
        else:
            self.has_partial = False
        cfg = self.cfg
        if cfg.theta_eq != 90.0 and cfg.kappa > 0:
            mode = 'linear' if cfg.theta_eq > 130.0 or cfg.theta_eq < 50.0 else 'quadratic'
            self.wetting = OracleWetting(self.solid, cfg.phi_c, cfg.kappa, cfg.sigma,
                                         cfg.theta_eq, mode, ghost_scale=self.ghost_scale,
                                         geo_amplification=self.geo_amplification,
                                         solid_fraction=solid_fraction)

    def init_fields(self, phi_init, u_init=None):
        """lbm/fe_ac_solver.py:239-261."""
        T = self.T
        phi = np.asarray(phi_init).astype(T)
        u = (np.asarray(u_init).astype(T) if u_init is not None
             else np.zeros((self.D,) + self.shape, dtype=T))
        self.phi = np.clip(phi, T(0), T(1))
        self.rho = self.phi * self.cfg.rho_l + (1.0 - self.phi) * self.cfg.rho_g
        self.u = u
        self.P = np.zeros_like(self.phi)
        self.p = self.rho * CS2
        self.phi_mass_init = float(T(self.phi.astype(np.float64).sum()))
        self.mu_phi = self._mu(self.phi, self._lap_only(self.phi))
        self.f = self._f_eq(self.phi, self.u)
        self.g = self._g_eq(self.P, self.u)
        self.phi_u_prev = None

    # -- operators ----------------------------------------------------------
    def _grad_lap(self, phi):
        """Fused isotropic gradient + laplacian with ghost correction
        (lbm/fe_ac_solver.py:296-320)."""
        T = self.T
        E = self.E
        grad = np.zeros((self.D,) + self.shape, dtype=T)
        lap = np.zeros(self.shape, dtype=T)
        w_over_cs2 = self.w / CS2
        for i in range(1, self.Q):
            ps = _shift_from(phi, E[i])
            if self.wetting is not None:
                ps = self.wetting.correct_shifted(phi, ps, i)
            diff = ps - phi
            wi = w_over_cs2[i]
            for d in range(self.D):
                if E[i, d] != 0:
                    grad[d] = grad[d] + (wi * T(E[i, d])) * ps
            lap = lap + (2.0 * wi) * diff
        return grad, lap

    def _lattice_gradient(self, v):
        """Unfused isotropic gradient with the ghost correction applied to v
        itself (lbm/fe_ac_solver.py:267-280): per direction i, per axis d with
        e_id != 0, grad_d += ((w_i e_id) v(x + e_i)) / cs2."""
        T = self.T
        E = self.E
        grad = np.zeros((self.D,) + self.shape, dtype=T)
        for i in range(1, self.Q):
            vs = _shift_from(v, E[i])
            if self.wetting is not None:
                vs = self.wetting.correct_shifted(v, vs, i)
            for d in range(self.D):
                if E[i, d] != 0:
                    grad[d] = grad[d] + ((self.w[i] * T(E[i, d])) * vs) / CS2
        return grad

    def _lap_only(self, phi):
        """Unfused laplacian used by init_fields (lbm/fe_ac_solver.py:282-294):
        ((2 w_i) (phi_i - phi)) / cs2 per direction."""
        T = self.T
        lap = np.zeros(self.shape, dtype=T)
        for i in range(1, self.Q):
            ps = _shift_from(phi, self.E[i])
            if self.wetting is not None:
                ps = self.wetting.correct_shifted(phi, ps, i)
            lap = lap + (2.0 * self.w[i]) * (ps - phi) / CS2
        return lap

    def _mu(self, phi, lap):
        """lbm/fe_ac_solver.py:326-340."""
        cfg = self.cfg
        mu = 4.0 * cfg.beta * phi * (phi - 1.0) * (phi - 0.5) - cfg.kappa * lap
        if self.wetting is not None:
            m = self.wetting.is_boundary
            if self.wetting.mode == 'linear':
                mu[m] = mu[m] + self.wetting.mu_wall * self.mu_wall_scale
            else:
                c = phi[m]
                mu[m] = mu[m] + cfg.phi_c * c * (1.0 - c)
        return mu

    def _eu(self, v):
        """einsum('qd,d...->q...', e, v): at most two non-zero terms per row."""
        T = self.T
        E = self.E
        out = np.empty((self.Q,) + v.shape[1:], dtype=T)
        for i in range(self.Q):
            acc = None
            for d in range(self.D):
                if E[i, d] != 0:
                    t = v[d] if E[i, d] > 0 else -v[d]
                    acc = t if acc is None else acc + t
            out[i] = T(0) if acc is None else acc
        return out

    def _f_eq(self, phi, u):
        """lbm/fe_ac_solver.py:346-356."""
        eu_cs2 = self._eu(u) / CS2
        u_sq = _seqsum(u * u)
        gamma = self.w_view * (1.0 + eu_cs2 + eu_cs2 * eu_cs2 / 2.0 - u_sq[None] / (2.0 * CS2))
        return phi[None] * gamma

    def _g_eq(self, P, u):
        """lbm/fe_ac_solver.py:358-367."""
        eu_cs2 = self._eu(u) / CS2
        u_sq = _seqsum(u * u)
        s = self.w_view * (eu_cs2 + eu_cs2 * eu_cs2 / 2.0 - u_sq[None] / (2.0 * CS2))
        return P[None] * self.w_view + s

    # -- mid-run droplet injection (lbm/fe_ac_solver.py:645-732) ----------
    def inject_droplet(self, center, radius, xi, u_impact=None):
        """Blend a new droplet into phi (max inside its core C > 0.1), blend
        u towards u_impact with weight C everywhere, reset f and g to their
        equilibria (with the current P) at the core nodes, re-base the phi
        mass and drop the previous phi u."""
        T = self.T
        if u_impact is None:
            u_impact = (0.0,) * self.D
        mesh = np.meshgrid(*[np.arange(n) for n in self.shape], indexing="ij")
        dist = np.sqrt(sum((M - center[d]) ** 2 for d, M in enumerate(mesh)))
        C = np.clip(0.5 + 0.5 * np.tanh(2.0 * (radius - dist) / xi), 0.0, 1.0).astype(np.float32).astype(T)
        core = C > T(0.1)
        phi = np.where(core, np.maximum(self.phi, C), self.phi)
        phi = np.clip(phi, T(0), T(1))
        if self.solid_any:
            phi = np.where(self.solid, T(0), phi)
        self.phi = phi.astype(T)
        self.rho = self.phi * self.cfg.rho_l + (1.0 - self.phi) * self.cfg.rho_g
        u_new = np.stack([np.full(self.shape, u_impact[d], dtype=T) for d in range(self.D)])
        u = (T(1) - C)[None] * self.u + C[None] * u_new
        if self.solid_any:
            u = np.where(self.solid[None], T(0), u)
        self.u = u.astype(T)
        f_eq = self._f_eq(self.phi, self.u)
        g_eq = self._g_eq(self.P, self.u)
        self.f = np.where(core[None], f_eq, self.f).astype(T)
        self.g = np.where(core[None], g_eq, self.g).astype(T)
        self.phi_mass_init = float(T(self.phi.astype(np.float64).sum()))
        self.phi_u_prev = None
        return int(core.sum())

    # -- the time step (lbm/fe_ac_solver.py:380-639) -----------------------
    def step(self):
        T = self.T
        cfg = self.cfg
        E, Q, OPP, D = self.E, self.Q, self.OPP, self.D
        # 1. phi recovery
        phi = np.clip(_seqsum(self.f), T(0), T(1))
        if self.solid_any:
            phi = np.where(self.solid, T(0), phi)
        self.phi = phi
        # 2. density, mu, gradients
        phi_safe = np.clip(phi, T(0), T(1))
        self.rho = phi_safe * cfg.rho_l + (1.0 - phi_safe) * cfg.rho_g
        rho_eff = np.maximum(self.rho, T(self.rho_floor))
        grad, lap = self._grad_lap(phi)
        self.mu_phi = self._mu(phi, lap)
        if self.wetting is not None and self.geometric_wetting:
            grad = self.wetting.correct_gradient(grad)
        # 3. pressure
        self.P = _seqsum(self.g)
        self.p = self.P * CS2
        # 4. non-equilibrium stress with new P, old u
        g_neq = self.g - self._g_eq(self.P, self.u)
        sig = {}
        for a in range(D):
            for b in range(D):
                acc = None
                for i in range(Q):
                    c = int(E[i, a] * E[i, b])
                    if c == 0:
                        continue
                    t = g_neq[i] if c > 0 else -g_neq[i]
                    acc = t if acc is None else acc + t
                sig[a, b] = acc
        # 5. forces (Fakhari 2017)
        drho = cfg.rho_l - cfg.rho_g
        F_s = self.mu_phi[None] * grad
        Fp = -self.P[None] * drho * CS2 * grad
        visc = (0.5 - self.tau_g) / self.tau_g
        if D == 3:
            m = np.stack([(sig[a, 0] * grad[0] + sig[a, 1] * grad[1]) + sig[a, 2] * grad[2]
                          for a in range(3)])
        else:
            m = np.stack([sig[a, 0] * grad[0] + sig[a, 1] * grad[1] for a in range(2)])
        Fm = visc * m * drho
        gf = tuple(cfg.g_force[:D])
        if any(x != 0 for x in gf):
            F_body = np.asarray(gf, dtype=T).reshape((D,) + (1,) * D) * self.rho[None]
        else:
            F_body = np.zeros_like(F_s)
        if self.stab_mode == 'fakhari':
            F = F_s + Fp + Fm + F_body
        elif self.stab_mode == 'liang':
            F = F_s + Fp + F_body
        else:
            F = F_s + F_body
        # 6. velocity
        u_from_g = np.stack([_seqsum(np.stack([self.g[i] if E[i, d] > 0 else -self.g[i]
                                               for i in range(Q) if E[i, d] != 0]))
                             for d in range(D)])
        u = u_from_g + 0.5 * F / rho_eff[None]
        if self.solid_any:
            u = np.where(self.solid[None], T(0), u)
        self.u = u
        # 7. Allen-Cahn source
        phi_u_now = phi_safe[None] * u
        if self.phi_u_prev is None:
            self.phi_u_prev = phi_u_now.copy()
        d_phi_u = phi_u_now - self.phi_u_prev
        self.phi_u_prev = phi_u_now.copy()
        gmag = np.sqrt(_seqsum(grad * grad))
        n = grad / np.maximum(gmag, T(1e-10))[None]
        lam = 4.0 * phi_safe * (1.0 - phi_safe) / cfg.xi
        sharp = CS2 * lam[None] * n * self.ac_scale
        if self.wetting is not None:
            sharp = sharp * (1.0 - self.sharpen_reduce * self.wetting.wall_weight.astype(T))[None]
        mobility = CS2 * (self.tau_f - 0.5)
        if self.interface_mode == 'cahn-hilliard' or self.mu_drive > 0.0:
            grad_mu = self._lattice_gradient(self.mu_phi)
        if self.interface_mode == 'cahn-hilliard':
            # lbm/fe_ac_solver.py:457-461
            guo = self.tau_f / (self.tau_f - 0.5)
            src = d_phi_u + mobility * (grad_mu - grad) * guo
        else:
            src = d_phi_u + sharp
            if self.mu_drive > 0.0:
                # lbm/fe_ac_solver.py:484-486
                src = src + (self.mu_drive * mobility) * grad_mu
        ac_coeff = 1.0 - 0.5 / self.tau_f
        F_src = ac_coeff * self.w_view * self._eu(src) / CS2
        # 8. collisions
        f_eq = self._f_eq(phi_safe, u)
        self.f = self.f - (1.0 / self.tau_f) * (self.f - f_eq) + F_src
        tau_l, tau_g = cfg.tau_l, self.tau_g
        if tau_g != tau_l:
            eta = phi_safe * cfg.rho_l * (tau_l - 0.5) + (1.0 - phi_safe) * cfg.rho_g * (tau_g - 0.5)
            rden = phi_safe * cfg.rho_l + (1.0 - phi_safe) * cfg.rho_g
            tau_eff = 0.5 + eta / rden
        else:
            tau_eff = np.full_like(phi_safe, T(tau_l))
        recip = T(1) / tau_eff
        ns = 1.0 - recip * 0.5
        G = ns[None] * self.w_view * self._eu(F) / (rho_eff[None] * CS2)
        g_eq = self._g_eq(self.P, u)
        self.g = self.g - recip[None] * (self.g - g_eq) + G
        # 9-10b. streaming, bounce-back, volume penalisation
        f_pre, g_pre = self.f, self.g
        fs = np.empty_like(f_pre)
        gs = np.empty_like(g_pre)
        for i in range(Q):
            fs[i] = _shift_to(f_pre[i], E[i])
            gs[i] = _shift_to(g_pre[i], E[i])
        if self.solid_any:
            s = self.solid
            for i in range(Q):
                fs[i][s] = f_pre[OPP[i]][s]
                gs[i][s] = g_pre[OPP[i]][s]
        if self.has_partial:
            pm = self.partial
            eps = self.eps[pm]
            for i in range(Q):
                j = OPP[i]
                fs[i][pm] = (1.0 - eps) * fs[i][pm] + eps * f_pre[j][pm]
                gs[i][pm] = (1.0 - eps) * gs[i][pm] + eps * g_pre[j][pm]
        self.f, self.g = fs, gs
        # 11. global phi-mass correction
        if self.phi_mass_init is not None:
            mass = T(self.phi.astype(np.float64).sum())
            safe = max(mass, T(1e-6))
            corr = (T(1) / safe) * T(self.phi_mass_init) if mass > 1e-6 else T(1)
            self.phi = np.clip(self.phi * corr, T(0), T(1))
            self.f = self.f * corr
        # 12. boundary-phi relaxation
        wt = self.wetting
        if wt is not None and self.boundary_relax > 0:
            m = wt.is_boundary
            phi_b = self.phi[m].copy()
            n_w = wt.wall_normal.astype(T)
            nz_abs = np.abs(n_w[D - 1])
            nmag = np.maximum(np.sqrt(_seqsum(n_w * n_w)), T(1e-10))
            top = (nz_abs[m] / nmag[m]) > 0.5
            inside = (phi_b > 0.15) & (phi_b < 0.85)
            tgt = self.phi_wall_target
            if self.direct_wetting:
                # lbm/fe_ac_solver.py:609-612
                target = wt.cubic_boundary_phi(self.phi)[m]
                active = inside & top
            elif tgt is not None and abs(tgt - 0.5) > 0.05:
                target = np.full_like(phi_b, T(tgt))
                active = inside & top
            else:
                active = np.zeros_like(phi_b, dtype=bool)
            if active.any():
                pnew = phi_b[active] + self.boundary_relax * (target[active] - phi_b[active])
                pnew = np.clip(pnew, T(0), T(1))
                phi_b[active] = pnew
                self.phi[m] = phi_b
                old = _seqsum(self.f)[m][active]
                scale = np.clip(pnew / np.maximum(old, T(1e-10)), T(0.5), T(2.0))
                idx = np.flatnonzero(m.reshape(-1))[active]
                for i in range(Q):
                    fl = self.f[i].reshape(-1)
                    fl[idx] = fl[idx] * scale
        self.step_count += 1


def measure_spread(phi, solid=None):
    """Spread extents / volume / C_max of lbm/fe_measure.py:11-82 plus the
    interface z centre of mass used by the sweep drivers
    (scripts/run_thesis_sweep.py:182-199)."""
    c = np.array(phi, copy=True)
    if solid is not None:
        c[np.asarray(solid, bool)] = 0.0
    iface = c > 0.5
    out = {'volume': float(c.sum(dtype=np.float64)), 'C_max': float(c.max())}
    if not iface.any():
        out.update(Dx=0.0, Dy=0.0, Dz=0.0, k=0.0, z_com=0.0, count=0)
        return out
    co = np.argwhere(iface)
    mn, mx = co.min(0), co.max(0)
    ext = [float(mx[a] - mn[a] + 1) for a in range(c.ndim)]
    Dx, Dy = ext[0], ext[1]
    Dz = ext[2] if c.ndim == 3 else 0.0
    # z_com: centre of the interface along the last axis (the wall-normal one)
    out.update(Dx=Dx, Dy=Dy, Dz=Dz, k=Dx / Dy if Dy > 0 else 0.0,
               z_com=float(co[:, -1].mean()), count=int(co.shape[0]))
    return out
