#!/usr/bin/env python3
"""Benchmark of the GB300 Allen-Cahn phase-field LBM step.

Workload (default): the drop-in GPU case -- 150x150x107 D3Q19 grid, ridge
substrate (R* = 1, R_d = 22.5, smooth solid fraction), droplet R = 22.5 at
(75, 75, 80) with impact velocity (0, 0, -0.05), theta_eq = 162 deg,
alpha_geo = 1.5, rho_l/rho_g = 828, sigma = 0.01424, tau = 0.53, float32.
Inputs are synthetic, built by the package's generators (same arrays as the
reference's generators).

One "step" is one lattice time step of the whole grid.  Reported:
  value      MLUPS (million lattice-node updates per second) over K timed
             steps (one lbm_step call) with the state resident on the device,
             CUDA events on the launching stream.  The K-step region is
             repeated until --min-seconds of device time have passed and the
             median repetition is reported.  The state (f, g: 732 MB) is
             larger than L2, so no flush is needed between steps.
  e2e        the same metric through the public API (AllenCahnSolver) from
             host numpy arrays: construction, set_solid, init_fields (H2D),
             K steps, the sweep drivers' read of phi to host every 50 steps
             (D2H), final spread measurement.
  roofline   the dominant kernel (k_update): algorithmic bytes per launch /
             its CUDA-event duration (from a separate pass with events between
             the kernels), against the measured HBM copy peak; step_roofline:
             the whole step's 336 B/node over the timed region.
  cpu_baseline  the numpy oracle (oracle/ac_oracle.py) on a bounded sample of
             the same workload, one host core; the reference's own PyTorch
             CPU figure, measured where the reference is installed, beside it.
  fp64_error the e2e run's phi, u, sum(phi) drift and spread factor after K
             steps against a float64 run of the same configuration.

--impl reference times the CPU implementation of the path (the oracle port;
the reference itself is Python/PyTorch and is not present on the GPU host)
on the same workload and prints the same JSON line with "impl": "reference".
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "pytorch-lbm_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

# Algorithmic bytes per node and step, float32 state: f and g (2 x 19
# populations), u (3) and the previous phi (1), each read once and written
# once: 2 x 4 x (38 + 3 + 1) = 336 B.  Half-precision population storage:
# 2 x 2 x 38 + 2 x 4 x 4 = 184 B.
B_ALG_STEP = {"fp32": 336, "fp16": 184}
# Per kernel (each adds the node-class byte it reads):
#   k_phi     f read (76 | 38), phi written (4), in the half form also the
#             previous phi (4, the deviation reference)
#   k_update  g (76 | 38), u (12) and previous phi (4) read; f, g (76 + 76 |
#             38 + 38) and u (12) written; the phi stencil comes from L2
#   k_step    the fused kernel: the whole step
B_ALG_KERNEL = {"fp32": {"k_phi": 81, "k_update": 257, "k_step": 337},
                "fp16": {"k_phi": 47, "k_update": 143, "k_step": 185}}
# 2-D (D2Q9) grids, float32: f and g (2 x 9), u (2), previous phi (1), read
# and written once: 2 x 4 x 21 = 168 B per node and step.  k2_phi reads f
# (36) and the class byte and writes phi (4); k2_update reads g (36), u (8),
# the previous phi (4) and the class byte and writes f, g (72) and u (8).
# (k2_update also reads f again for the collision: traffic beyond these
# algorithmic bytes.)
B_ALG_STEP_2D = 168
B_ALG_KERNEL_2D = {"k2_phi": 41, "k2_update": 129}

WORKLOADS = {
    "ridge150": dict(grid=(150, 150, 107), substrate=("ridge", 1.0, 22.5), center=(75, 75, 80),
                     radius=22.5, u=(0.0, 0.0, -0.05), theta=162.0,
                     label="ridge 150x150x107 D3Q19 droplet impact, theta=162, alpha_geo=1.5"),
    "flat64": dict(grid=(64, 64, 48), substrate=("flat_z2",), center=(32, 32, 14), radius=12.0,
                   u=(0.0, 0.0, 0.0), theta=120.0,
                   label="flat 64x64x48 D3Q19 static droplet, theta=120, alpha_geo=1.5"),
    # the large single solve of the precision form: convex hemisphere of radius 60 (R* = 60/45)
    # a 2-D (D2Q9) grid of about the default case's node count: ridge R* = 1, droplet R = 150
    "ridge2d": dict(grid=(2048, 1024, 1), substrate=("ridge", 1.0, 150.0), center=(1024, 310), radius=150.0,
                    u=(0.0, -0.05), theta=162.0,
                    label="ridge 2048x1024 D2Q9 (2-D) droplet impact, droplet R=150, theta=162, alpha_geo=1.5"),
    "convex384": dict(grid=(384, 384, 256), substrate=("convex", 60.0 / 45.0, 45.0), center=(192, 192, 180),
                      radius=45.0, u=(0.0, 0.0, -0.06), theta=150.0,
                      label="convex 384x384x256 D3Q19 droplet impact, hemisphere R=60, droplet R=45, "
                            "theta=150, alpha_geo=1.5"),
}


def make_case(name):
    from geometry.substrate import create_substrate_with_fraction
    from lbm.fe_config import FEConfig
    from lbm.fe_droplet import create_fe_droplet_with_impact
    w = WORKLOADS[name]
    nx, ny, nz = w["grid"]
    cfg = FEConfig(nx=nx, ny=ny, nz=nz, rho_l=1.0, rho_g=1.0 / 828.0, sigma=0.01424, xi=4.0,
                   tau_l=0.53, tau_g=0.53, theta_eq=w["theta"], device="cuda", max_steps=2000)
    if w["substrate"][0] == "flat_z2":
        solid = np.zeros(tuple(cfg.grid_shape), dtype=bool)
        solid[..., :2] = True
        frac = solid.astype(np.float32)
    else:
        t, rs, rd = w["substrate"]
        solid, frac = create_substrate_with_fraction(nx, ny, nz, t, R_star=rs, R_d=rd)
    C, _, u = create_fe_droplet_with_impact(nx, ny, nz, center=w["center"], radius=w["radius"], xi=4.0,
                                            u_impact=w["u"])
    return cfg, solid, frac, C, u


# Solver options of the drop-in case (geometric wetting, alpha_geo = 1.5) and
# of its variants (--mode): the reference's other interface sources and
# wetting options on the same inputs.
MODES = {
    "default": dict(),
    "cahn-hilliard": dict(interface_mode="cahn-hilliard"),
    "mu-drive": dict(mu_drive=0.5),
    "direct-wetting": dict(direct_wetting=True),
    "alpha-field": dict(alpha_field=(0.5, 2.5)),
}


def solver_kwargs(mode, shape):
    kw = dict(geo_amplification=1.5, geometric_wetting=True)
    m = dict(MODES[mode])
    if "alpha_field" in m:
        lo, hi = m.pop("alpha_field")
        nx = shape[0]
        ramp = np.linspace(lo, hi, nx, dtype=np.float32).reshape((nx,) + (1,) * (len(shape) - 1))
        kw["geo_amplification"] = np.ascontiguousarray(np.broadcast_to(ramp, shape))
    kw.update(m)
    return kw


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(kernel):
    """DRAM bytes per node of `kernel` from the committed ncu summary
    (a line 'dram_bytes_per_node <kernel> <value>' in profiles/*.md)."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for fn in sorted(os.listdir(pdir)):
        if not fn.endswith((".md", ".txt")):
            continue
        with open(os.path.join(pdir, fn)) as fh:
            for line in fh:
                parts = line.strip().strip("`").split()
                if len(parts) == 3 and parts[0] == "dram_bytes_per_node" and parts[1] == kernel:
                    try:
                        return float(parts[2])
                    except ValueError:
                        pass
    return None


class Clocks:
    """nvidia-smi sampling of SM clocks / throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", f"lbm_bench_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            with open(self.path) as fh:
                for line in fh:
                    p = [x.strip() for x in line.split(",")]
                    if len(p) < 9:
                        continue
                    try:
                        sm.append(float(p[1]))
                        mx.append(float(p[2]))
                    except ValueError:
                        continue
                    for nm, v in zip(names, p[5:9]):
                        if v.lower() == "active":
                            reasons.add(nm)
            os.remove(self.path)
        except Exception:
            return None
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_oracle_mlups(name, steps, warmup=1):
    """The numpy oracle on the same workload: `warmup` + `steps` steps."""
    from oracle.ac_oracle import OracleSolver
    cfg, solid, frac, C, u = make_case(name)
    s = OracleSolver(cfg, dtype=np.float32, geo_amplification=1.5, geometric_wetting=True)
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    for _ in range(warmup):
        s.step()
    t = time.perf_counter()
    for _ in range(steps):
        s.step()
    dt = time.perf_counter() - t
    n = cfg.nx * cfg.ny * cfg.nz
    return n * steps / dt / 1e6, dt


def run_reference_arm(args, rank, world):
    name = args.workload
    out = None
    if rank == 0:
        # bounded sample: K timed steps of the full grid, at most --ref-steps of
        # them (1.3-5 s each on one core at 2.4 M nodes), after up to 3 warm-up steps
        steps = max(1, min(args.steps, args.ref_steps))
        wu = min(args.warmup, 3)
        mlups, dt = cpu_oracle_mlups(name, steps, warmup=wu)
        w = WORKLOADS[name]
        n = int(np.prod(w["grid"]))
        sample = (f"{steps} timed steps (+{wu} warm-up) of the full {w['grid'][0]}x{w['grid'][1]}x{w['grid'][2]} "
                  "grid")
        out = {"impl": "reference", "metric": "MLUPS", "value": mlups, "unit": "MLUPS", "n_gpus": world,
               "steps": steps, "warmup": wu, "ms_per_step": dt / steps * 1e3,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic", "config": {"workload": w["label"], "nodes": n, "precision": "fp32"},
               "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": 1, "kind": "port",
                                "sample": sample + " with the numpy restatement of the reference step"},
               "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return out


def run_ours(args, rank, world, device):
    import torch
    from lbm import _native as nat
    from lbm.fe_ac_solver import AllenCahnSolver
    name = args.workload
    cfg, solid, frac, C, u = make_case(name)
    cfg.device = str(device)
    n = cfg.nx * cfg.ny * cfg.nz
    K, W = args.steps, args.warmup

    # --- device-resident timed region -------------------------------------
    pdt = torch.float16 if args.precision == "fp16" else torch.float32
    skw = solver_kwargs(args.mode, tuple(cfg.grid_shape))
    s = AllenCahnSolver(cfg, dtype=pdt, **skw)
    s.set_solid(solid, frac)
    if args.layout != "auto":
        s.set_layout(args.layout == "paired")
    s.init_fields(C, u)
    for _ in range(W):
        s.step()
    two_d = s.ndim == 2
    if two_d:
        tile, tune_ms = (0, 0, 0), 0.0  # 2-D grids: the per-node kernels only
    elif args.tile:
        s.set_tile(*[int(x) for x in args.tile.split(",")])
        tile, tune_ms = tuple(int(x) for x in args.tile.split(",")), 0.0
    elif not args.no_tune:
        tile, tune_ms = s.autotune(reps=5)
    else:
        tile, tune_ms = (0, 0, 0), 0.0
    for _ in range(2):
        s.step()
    lib, h = s._lib, s._h
    stream = torch.cuda.current_stream(device)
    # timed region: K steps in one lbm_step call, CUDA events on the launching
    # stream, bracketed by a barrier and a device synchronisation.  The K-step
    # region is repeated until at least --min-seconds of device time have
    # passed (so that the clock sampler sees the load) and the median
    # repetition is reported.
    reps_ms = []
    with Clocks(device.index) as clk:
        while True:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            barrier(world)
            torch.cuda.synchronize(device)
            e0.record(stream)
            nat.check(lib.lbm_step(h, K, nat.stream_ptr(stream)), "lbm_step")
            e1.record(stream)
            torch.cuda.synchronize(device)
            barrier(world)
            s.step_count += K
            reps_ms.append(e0.elapsed_time(e1))
            # every rank repeats as often as rank 0 decides
            more = sum(reps_ms) < args.min_seconds * 1e3 and len(reps_ms) < args.max_reps
            if not bcast_flag(more, world, device):
                break
    tot_ms = statistics.median(reps_ms)
    # per-kernel durations: a separate pass with events recorded between the
    # two kernels of every step (which serialises them: durations are upper bounds)
    Kp = min(K, 200)
    ms3 = (__import__("ctypes").c_float * 3)()
    nat.check(lib.lbm_step_profiled(h, Kp, nat.stream_ptr(stream), ms3), "lbm_step_profiled")
    s.step_count += Kp
    phi_ms, upd_ms = float(ms3[0]) * K / Kp, float(ms3[1]) * K / Kp
    two_kernel = tuple(s.get_tile()) == (0, 0, 0)
    tot_ms = max_over_ranks(tot_ms, world, device)
    status = s.status()
    meas = s.measure()
    if status & nat.STATUS_NAN or meas["has_nan"]:
        raise RuntimeError("NaN in the benchmark run")
    value = replica_mlups(n, K, tot_ms, world)
    layout = "paired" if s.paired else "linear"
    launch = dict(zip(("phi_nodes_per_thread", "update_block"), s.launch_shape()))
    nq = s.lattice.q
    # the timed solver is closed before the end-to-end run: its state arrays
    # go to the library's cache, from which the next solver's come, as in a
    # process that solves case after case
    s.close()

    # --- end to end through the public API from host arrays ----------------
    # the whole solve (construct, set-up from host arrays, K steps with phi to
    # the host every 50 steps, measure) is repeated like the timed region:
    # until ~0.5 s have passed (at most 5 times); the median is reported
    e2e_reps = []
    while True:
        torch.cuda.synchronize(device)
        barrier(world)
        t0 = time.perf_counter()
        s2 = AllenCahnSolver(cfg, dtype=pdt, **skw)
        s2.set_solid(solid, frac)
        s2.init_fields(C, u)
        reads = 0
        for k in range(1, K + 1):
            s2.step()
            if k % 50 == 0:
                _ = s2.phi.cpu().numpy()
                reads += 1
        m2 = s2.measure()
        torch.cuda.synchronize(device)
        e2e_reps.append(max_over_ranks(time.perf_counter() - t0, world, device))
        more = sum(e2e_reps) < 0.5 and len(e2e_reps) < 5
        if not bcast_flag(more, world, device):
            break
        s2.close()
    e2e_s = statistics.median(e2e_reps)
    s2_fields = [x.double().cpu().numpy() for x in s2.fields("phi", "u")]
    s2_meas = dict(m2, phi_mass_init=s2.phi_mass_init)
    s2.close()
    # the same run with the sweep drivers' every-50-steps check (extents, z
    # centre, NaN) reduced on the device instead of copying phi to the host
    torch.cuda.synchronize(device)
    barrier(world)
    t0 = time.perf_counter()
    s3 = AllenCahnSolver(cfg, dtype=pdt, **skw)
    s3.set_solid(solid, frac)
    s3.init_fields(C, u)
    for k in range(1, K + 1):
        s3.step()
        if k % 50 == 0:
            _ = s3.measure()
    torch.cuda.synchronize(device)
    e2e_m_s = max_over_ranks(time.perf_counter() - t0, world, device)
    s3.close()
    e2e = replica_mlups(n, K, e2e_s * 1e3, world)
    h2d = solid.nbytes + frac.nbytes + C.nbytes + u.nbytes
    d2h = reads * n * 4 + 9 * 8
    # the error of this run (K steps from the initial state, the e2e solve)
    # against a float64 run of the same configuration and inputs
    fp64 = None
    if rank == 0 and not args.no_fp64_check:
        fp64 = fp64_error(s2_fields, s2_meas, cfg, solid, frac, C, u, skw, K, WORKLOADS[name]["radius"])

    out = None
    if rank == 0:
        peak, peak_kind = peaks()
        f16 = args.precision == "fp16"
        b_step = B_ALG_STEP_2D if two_d else B_ALG_STEP[args.precision]
        # the dominant kernel of the step: k_update (two-kernel step) or k_step (fused)
        kname = ("k2_update" if two_d else "k_update") if two_kernel else "k_step"
        b_ker = B_ALG_KERNEL_2D[kname] if two_d else B_ALG_KERNEL[args.precision][kname]
        ker_s = upd_ms / K / 1e3
        achieved = b_ker * n / ker_s / 1e9
        traffic_pn = profiled_traffic(kname + ("_f16" if f16 else ""))
        step_bw = b_step * n / (tot_ms / K / 1e3) / 1e9
        kernels = {}
        if two_kernel:
            pname = "k2_phi" if two_d else "k_phi"
            b_phi = B_ALG_KERNEL_2D[pname] if two_d else B_ALG_KERNEL[args.precision][pname]
            kernels = {pname: {"ms_per_launch": phi_ms / K, "bytes_per_node": b_phi,
                               "achieved_gbs": b_phi * n / (phi_ms / K / 1e3) / 1e9},
                       kname: {"ms_per_launch": upd_ms / K, "bytes_per_node": b_ker,
                               "achieved_gbs": achieved}}
        w = WORKLOADS[name]
        cpu = None
        if not args.no_cpu_baseline:
            cm, cdt = cpu_oracle_mlups(name, args.cpu_steps, warmup=1)
            cpu = {"value": cm, "unit": "MLUPS", "cores": 1, "kind": "port",
                   "sample": f"{args.cpu_steps} steps (+1 warm-up) of the full grid, numpy oracle, "
                             f"{cdt:.1f} s",
                   "what": "one host core running the numpy restatement of the reference step (numpy "
                           "array operations are single-threaded); the reference itself is PyTorch and "
                           "does not exist on this host",
                   "reference_torch_cpu": REF_TORCH_CPU.get(name)}
        out = {
            "metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": tot_ms / K,
            "timed_reps": {"reps": len(reps_ms), "ms_per_rep_median": tot_ms, "ms_per_rep_min": min(reps_ms),
                           "ms_per_rep_max": max(reps_ms), "device_s_total": sum(reps_ms) / 1e3,
                           "what": f"the K-step region repeated until >= {args.min_seconds} s of device time; "
                                   "value and ms_per_step from the median repetition"}, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["label"], "nodes": n,
                       "precision": ("fp16 deviation-stored populations, fp32 math and fields, fp64 global sum"
                                     if f16 else "fp32 populations, fp32 math, fp64 global sum"),
                       "parallelism": "replicas" if world > 1 else "single",
                       "mode": args.mode,
                       "layout": layout,
                       "tile": list(tile), "tuned_ms": tune_ms,
                       "launch": launch,
                       "l2": f"state (f, g: {4 * nq * n * (2 if f16 else 4) / 1e6:.0f} MB) larger "
                             "than L2 (129 MB): no flush"},
            "e2e": {"value": e2e, "unit": "MLUPS", "h2d_bytes_per_step": h2d / K,
                    "d2h_bytes_per_step": d2h / K,
                    "what": f"AllenCahnSolver from host arrays: create + set_solid + init_fields + {K} steps "
                            f"+ phi to host every 50 steps + measure; median of {len(e2e_reps)} repetitions "
                            f"{e2e_s * 1e3:.2f} ms (first {e2e_reps[0] * 1e3:.2f} ms); the state arrays come "
                            "from the library's cache (the timed solver's, closed before)",
                    "reps_ms": [round(x * 1e3, 3) for x in e2e_reps],
                    "device_diagnostics": {
                        "value": replica_mlups(n, K, e2e_m_s * 1e3, world), "unit": "MLUPS",
                        "d2h_bytes_per_step": (K // 50) * 9 * 8 / K,
                        "what": "the same with measure() (device reduction, 9 doubles to the host) every 50 "
                                f"steps instead of phi; {e2e_m_s:.3f} s"}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": traffic_pn * n if traffic_pn is not None else None,
                         "kernel": kname, "bytes_per_node": b_ker,
                         "ms_per_launch": upd_ms / K,
                         "timing": f"{kname} launches timed with CUDA events over a separate pass of {Kp} "
                                   "steps with an event between the two kernels of every step"},
            "step_roofline": {"achieved_gbs": step_bw, "bytes_per_node": b_step, "peak": peak,
                              "frac": step_bw / peak, "mlups_roofline": peak * 1e3 / b_step},
            "kernels": kernels,
            # two kernels per step (four with the mu and grad-mu passes of the grad-mu modes)
            "gpu_launches": ((4 if args.mode in ("cahn-hilliard", "mu-drive") else 2) * K) if two_kernel else K,
            "cpu_baseline": cpu,
            "fp64_error": fp64,
            "clocks": clk.summary(),
            "spread_after": {k2: meas[k2] for k2 in ("Dx", "Dy", "k", "z_com", "volume")},
        }
    return out


def _events_time(fn, device):
    """Seconds of device time of fn() on the current stream (CUDA events)."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize(device)
    return e0.elapsed_time(e1) / 1e3


def run_sweep(args, device):
    """The batched sweep: `--sweep-cases` seeded impact cases (grids
    96^3 / 128x128x96 / 150x150x107 / 192x192x128, four substrates, R_d, theta,
    u_z drawn per case) advanced `--sweep-steps` steps each.  Timed: the
    batched half-precision form (one launch per kernel per step for all cases,
    CUDA graph, autotuned launch shape), the batched float32 form, both again
    as one cooperative launch per step, and the plain form (float32, one case
    at a time, each run to completion); device time only, with the state
    resident.  Check: spread factor D/(2 R_d), aspect k and
    volume of the first `--sweep-check` cases against float64 runs."""
    import torch
    from lbm.batch import AllenCahnBatch
    from lbm.impact import SWEEP_GRIDS, build_impact_case, sample_impact_case
    n_steps = args.sweep_steps
    cases = [sample_impact_case(args.seed + i, SWEEP_GRIDS, (n_steps, n_steps)) for i in range(args.sweep_cases)]
    updates = float(sum(c.nodes for c in cases)) * n_steps

    def batched(dtype, coop=False):
        t = time.perf_counter()
        solvers = [build_impact_case(c, dtype) for c in cases]
        setup = time.perf_counter() - t
        b = AllenCahnBatch(solvers)
        if coop:
            b.set_cooperative(True)
        b.run(1)
        b.autotune(reps=3)
        per = b.launch_shape()
        secs = _events_time(lambda: b.run(n_steps - 1), device)
        meas = [s.measure() for s in solvers[:args.sweep_check]]
        b.close()
        for s in solvers:
            s.close()
        return float(sum(c.nodes for c in cases)) * (n_steps - 1) / secs / 1e6, secs, setup, per, meas

    m16, t16, set16, per16, meas16 = batched(torch.float16)
    m32b, t32b, _, per32, meas32 = batched(torch.float32)
    # the same batches stepped by one cooperative launch per step (A/B)
    c16, ct16, _, cper16, _ = batched(torch.float16, coop=True)
    c32, ct32, _, cper32, _ = batched(torch.float32, coop=True)
    plain = 0.0
    for c in cases:
        s = build_impact_case(c, torch.float32)
        s.run(1)
        plain += _events_time(lambda: s.run(n_steps - 1), device)
        s.close()
    m32p = float(sum(c.nodes for c in cases)) * (n_steps - 1) / plain / 1e6
    check = []
    for c, a16, a32 in zip(cases[:args.sweep_check], meas16, meas32):
        s = build_impact_case(c, torch.float64)
        s.run(n_steps)
        m = s.measure()
        s.close()
        beta = lambda d: max(d["Dx"], d["Dy"]) / (2.0 * c.R_d)
        check.append({"case": c.seed, "grid": list(c.grid), "substrate": c.substrate,
                      "beta_f64": beta(m), "beta_f16": beta(a16), "beta_f32": beta(a32),
                      "k_f64": m["k"], "k_f16": a16["k"],
                      "volume_rel_err_f16": abs(a16["volume"] - m["volume"]) / m["volume"],
                      "beta_rel_err_f16": abs(beta(a16) - beta(m)) / beta(m)})
    return {"metric": "MLUPS", "value": m16, "unit": "MLUPS", "n_gpus": 1, "steps": n_steps,
            "higher_is_better": True, "dtype": "f16 storage / f32 math", "data": "synthetic",
            "config": {"workload": f"batched sweep: {len(cases)} impact cases x {n_steps} steps, grids "
                                   "96^3 / 128x128x96 / 150x150x107 / 192x192x128, flat/ridge/convex/concave, "
                                   "R_d~U[15,30], theta~U[90,162], u_z~U[-0.08,-0.02], seeds "
                                   f"{args.seed}..{args.seed + len(cases) - 1}",
                       "node_updates": updates},
            "batched_f16": {"mlups": m16, "seconds": t16, "setup_s": set16, "launch_shape": per16},
            "batched_f32": {"mlups": m32b, "seconds": t32b, "launch_shape": per32},
            "batched_f16_single_launch": {"mlups": c16, "seconds": ct16, "launch_shape": cper16},
            "batched_f32_single_launch": {"mlups": c32, "seconds": ct32, "launch_shape": cper32},
            "plain_f32": {"mlups": m32p, "seconds": plain, "what": "one case at a time, each to completion"},
            "speedup_f16_batched_vs_plain_f32": m16 / m32p,
            "fp64_check": check}


def run_precision(args, device):
    """The precision form's large single solve (384x384x256 convex hemisphere,
    droplet R = 45 at height 180, u_z = -0.06, theta = 150): the same case in
    half-precision population storage, float32 and float64 for
    `--precision-steps` steps each; device time per form; spread factor
    beta = max(Dx, Dy) / (2 R), aspect k, contact angles (the reference's
    layer scan, and the angle against the local wall normal that a curved
    substrate needs) and sum(phi) drift of each form every
    `--precision-every` steps, and the half and float32 forms' errors against
    the float64 run (the oracle at this size)."""
    import torch
    from lbm.fe_ac_solver import AllenCahnSolver
    from lbm.fe_measure import measure_contact_angle, measure_contact_angle_wall
    cfg, solid, frac, C, u = make_case("convex384")
    cfg.device = str(device)
    w = WORKLOADS["convex384"]
    n = cfg.nx * cfg.ny * cfg.nz
    K, every = args.precision_steps, args.precision_every
    forms = {}
    for name, dt in (("f16", torch.float16), ("f32", torch.float32), ("f64", torch.float64)):
        t = time.perf_counter()
        s = AllenCahnSolver(cfg, dtype=dt, geo_amplification=1.5, geometric_wetting=True)
        s.set_solid(solid, frac)
        s.init_fields(C, u)
        setup = time.perf_counter() - t
        m0 = s.phi_mass_init
        hist, secs, done = [], 0.0, 0
        while done < K:
            k = min(every, K - done)
            secs += _events_time(lambda: s.run(k), device)
            done += k
            m = s.measure()
            phi = s.phi
            ca = measure_contact_angle(phi, s.solid)
            caw = measure_contact_angle_wall(phi, s.solid, s.wetting.wall_normal, s.wetting.is_boundary)
            hist.append({"step": done, "beta": max(m["Dx"], m["Dy"]) / (2.0 * w["radius"]), "k": m["k"],
                         "contact_angle": ca, "contact_angle_wall": caw, "mass_drift": (m["volume"] - m0) / m0,
                         "nan": m["has_nan"]})
        forms[name] = {"ms_per_step": secs * 1e3 / K, "mlups": n * K / secs / 1e6, "setup_s": setup,
                       "history": hist}
        s.close()
        del s
        torch.cuda.empty_cache()
    ref = forms["f64"]["history"][-1]
    for name in ("f16", "f32"):
        last = forms[name]["history"][-1]
        forms[name]["vs_f64"] = {
            "beta_rel_err": abs(last["beta"] - ref["beta"]) / ref["beta"] if ref["beta"] else None,
            "k_abs_err": abs(last["k"] - ref["k"]),
            "contact_angle_abs_err_deg": abs(last["contact_angle"] - ref["contact_angle"]),
            "contact_angle_wall_abs_err_deg": abs(last["contact_angle_wall"] - ref["contact_angle_wall"]),
            "max_contact_angle_wall_err_over_run_deg": max(abs(a["contact_angle_wall"] - b["contact_angle_wall"])
                                                           for a, b in zip(forms[name]["history"],
                                                                           forms["f64"]["history"])),
            "mass_drift_diff": last["mass_drift"] - ref["mass_drift"],
            "max_beta_rel_err_over_run": max(abs(a["beta"] - b["beta"]) / b["beta"] if b["beta"] else 0.0
                                             for a, b in zip(forms[name]["history"], forms["f64"]["history"]))}
    return {"metric": "MLUPS", "value": forms["f16"]["mlups"], "unit": "MLUPS", "n_gpus": 1, "steps": K,
            "higher_is_better": True, "dtype": "f16 storage / f32 math", "data": "synthetic",
            "config": {"workload": w["label"] + f", {K} steps", "nodes": n},
            "forms": forms, "speedup_f16_vs_f32": forms["f16"]["mlups"] / forms["f32"]["mlups"]}


def run_serve(args, device):
    """The serving loop: `--serve-requests` impact requests (grids up to
    256x256x192, steps U[1000, 4000]) with Poisson arrivals (4 per second),
    admitted by HBM footprint within `--serve-budget-gb`; continuous batching
    in half precision against the plain one-at-a-time float32 path on the
    same request stream.  Wall-clock times include each case's set-up."""
    import torch
    from lbm.impact import SERVE_GRIDS, sample_impact_case
    from lbm.serve import GpuBackend, Request, poisson_arrivals, serve, serve_sequential
    arr = poisson_arrivals(args.serve_requests, 4.0, args.seed)
    reqs = [Request(i, sample_impact_case(args.seed + 1000 + i, SERVE_GRIDS, (1000, 4000)), a)
            for i, a in enumerate(arr)]
    budget = int(args.serve_budget_gb * 1e9)
    res_b, st_b = serve(reqs, GpuBackend(torch.float16), budget, tick=100, builders=4)
    # shortest remaining work first, at least args.serve_saturate nodes per tick
    res_r, st_r = serve(reqs, GpuBackend(torch.float16), budget, tick=100, builders=4,
                        saturate_nodes=int(args.serve_saturate))
    res_s, st_s = serve_sequential(reqs, GpuBackend(torch.float32))
    return {"metric": "MLUPS", "value": st_b["mlups"], "unit": "MLUPS", "n_gpus": 1, "higher_is_better": True,
            "dtype": "f16 storage / f32 math", "data": "synthetic",
            "config": {"workload": f"serving: {len(reqs)} impact requests, Poisson 4/s, grids up to 256x256x192, "
                                   f"steps U[1000,4000], HBM budget {args.serve_budget_gb} GB",
                       "node_updates": float(sum(r.case.nodes * r.case.steps for r in reqs))},
            "served_f16_batched": st_b, "served_f16_srpt": dict(st_r, saturate_nodes=int(args.serve_saturate)),
            "plain_f32_sequential": st_s,
            "mlups_ratio": st_b["mlups"] / st_s["mlups"], "p99_ratio": st_b["p99_s"] / st_s["p99_s"],
            "srpt_mlups_ratio": st_r["mlups"] / st_s["mlups"], "srpt_p50_ratio": st_r["p50_s"] / st_s["p50_s"],
            "srpt_p99_ratio": st_r["p99_s"] / st_s["p99_s"]}


# The reference's own PyTorch CPU path on the drop-in cases, measured where the
# reference is installed (8-core Xeon @ 2.7 GHz, torch 2.11 CPU build, 8
# intra-op threads): it does not exist on the GPU host, so it is reported
# beside the numpy port that is timed there.
REF_TORCH_CPU = {
    "ridge150": {"mlups": 1.98, "ms_per_step": 1213.7, "cores": 8, "dtype": "float32",
                 "where": "8-core Xeon @ 2.7 GHz, torch 2.11 CPU, 5 steps"},
    "flat64": {"mlups": 3.04, "ms_per_step": 64.7, "cores": 8, "dtype": "float32",
               "where": "8-core Xeon @ 2.7 GHz, torch 2.11 CPU, 20 steps"},
}


def fp64_error(fields, meas, cfg, solid, frac, C, u, skw, K, radius):
    """Error of a run's phi, u, sum(phi) drift and spread factor after K steps
    against a float64 run of the same configuration from the same inputs."""
    import torch
    from lbm.fe_ac_solver import AllenCahnSolver
    s = AllenCahnSolver(cfg, dtype=torch.float64, **skw)
    s.set_solid(solid, frac)
    s.init_fields(C, u)
    s.run(K)
    phi64, u64 = [x.cpu().numpy() for x in s.fields("phi", "u")]
    m64 = dict(s.measure(), phi_mass_init=s.phi_mass_init)
    s.close()
    phi, vel = fields
    drift = lambda m: (m["volume"] - m["phi_mass_init"]) / m["phi_mass_init"]
    beta = lambda m: max(m["Dx"], m["Dy"]) / (2.0 * radius)
    return {"steps": K,
            "max_abs_dphi": float(np.abs(phi - phi64).max()),
            "rel_l2_du": float(np.linalg.norm(vel - u64) / max(np.linalg.norm(u64), 1e-300)),
            "sum_phi_drift": drift(meas), "sum_phi_drift_f64": drift(m64),
            "sum_phi_drift_diff": drift(meas) - drift(m64),
            "spread_factor": beta(meas), "spread_factor_f64": beta(m64),
            "spread_factor_rel_err": abs(beta(meas) - beta(m64)) / beta(m64) if beta(m64) else None,
            "k": meas["k"], "k_f64": m64["k"],
            "what": "this run (the e2e solve: K steps from the initial state) against a float64 run of the "
                    "same configuration and inputs; the 150x150x107 impact amplifies rounding differences "
                    "(one float32 ulp of the initial state gives max|dphi| ~6e-3 by step 60), so the "
                    "pointwise figures grow with K while the spread factor and sum(phi) drift stay close"}


def bcast_flag(flag, world, device):
    """Rank 0's boolean on every rank."""
    if world == 1:
        return flag
    import torch
    import torch.distributed as dist
    t = torch.tensor([1 if flag else 0], dtype=torch.int32, device=device)
    dist.broadcast(t, 0)
    return bool(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def replica_mlups(nodes, steps, ms, world):
    """Whole-job MLUPS of `world` independent replicas that each advance a
    grid of `nodes` nodes by `steps` steps; `ms` is the slowest rank's time."""
    return world * nodes * steps / (ms / 1e3) / 1e6


def max_over_ranks(x, world, device):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)  # the drop-in case's own step count
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ridge150", choices=sorted(WORKLOADS) + ["serve", "sweep", "precision"])
    ap.add_argument("--seed", type=int, default=0, help="first seed of the sweep / serving cases")
    ap.add_argument("--sweep-cases", type=int, default=64)
    ap.add_argument("--sweep-steps", type=int, default=1500)
    ap.add_argument("--sweep-check", type=int, default=4, help="sweep cases also run in float64")
    ap.add_argument("--precision-steps", type=int, default=5000, help="steps of the precision-form solve")
    ap.add_argument("--precision-every", type=int, default=500, help="measurement interval of that solve")
    ap.add_argument("--serve-requests", type=int, default=24)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-saturate", type=float, default=4e6,
                    help="nodes per tick of the shortest-remaining-work-first serving policy")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--ref-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true", help="skip the float64 run of the same workload")
    ap.add_argument("--min-seconds", type=float, default=0.5,
                    help="repeat the timed K-step region until this much device time has passed")
    ap.add_argument("--max-reps", type=int, default=1000)
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp16"])
    ap.add_argument("--mode", default="default", choices=sorted(MODES),
                    help="solver option variant of the drop-in case (the bench line's config names it)")
    ap.add_argument("--tile", default=None, help="fixed tile 'tx,ty,tz' of the step kernel (no autotune)")
    ap.add_argument("--layout", default="auto", choices=["auto", "paired", "linear"],
                    help="state storage layout of the timed solver (auto: the library's default, linear)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference_arm(args, rank, world)), flush=True)
        return
    import torch
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    if args.workload in ("sweep", "serve", "precision"):
        if world > 1:
            raise SystemExit("the sweep, serving and precision workloads run on one GPU")
        run = {"sweep": run_sweep, "serve": run_serve, "precision": run_precision}[args.workload]
        out = run(args, device)
        print(json.dumps(out), flush=True)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=device)
    out = run_ours(args, rank, world, device)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
