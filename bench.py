#!/usr/bin/env python3
"""Benchmark of the plain explicit heat sweep (the ScaFES update phase).

Workload (the large heat configuration): 3D heat equation u_t = Laplace(u)
on the unit cube, 512^3 nodes, FP64, 7-point stencil, homogeneous Dirichlet
border, u0 = sin(pi x) sin(pi y) sin(pi z) plus seeded (seed 2) uniform
noise in [-1e-3, 1e-3] at inner nodes, tau = 0.9 h^2/6.  One bench step is
one solve: 1000 explicit Euler time steps (1000 sweep launches).  Synthetic
data; every field (1 GiB) is larger than L2, so no L2 flush is needed.

  value  : GLUP/s (nodes x time steps / s, all nodes counted) with the field
           resident in HBM, CUDA events on the launching stream
  e2e    : same metric through the C ABI with host buffers: per step an
           upload (pinned host -> device), 1000 steps and a download
           (device -> pinned host), two handles on two streams so that one
           step's copies overlap the other's sweeps; e2e.serial is the same
           on one handle, one call after the other
  roofline / cpu_baseline / clocks / variants: see the keys' comments.

``--impl reference`` times the reference's CPU path (the C restatement of
the reference's update in oracle/, all host threads) on a bounded sample of
the same workload and prints the same JSON line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import re
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GLUP/s and % HBM roofline, plain vs batched vs adjoint on 1 GB300, at stated error"
UNIT = "GLUP/s"
B_PER_LUP = {"f64": 16, "f32x2": 16, "f32": 8}   # algorithmic bytes per node update
FP64_OPS_PER_LUP = 7                               # DMUL + 3 DADD + 3 DFMA
INT_SUMS_PER_LUP = 3   # of which the three neighbour sums run on the integer pipe (exact)


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--kernel-case", choices=sorted(KERNEL_CASES), default=None,
                    help="run one small case of one kernel (for an ncu capture) and exit")
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--time-steps", type=int, default=1000)
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-instances", type=int, default=256)
    ap.add_argument("--batch-time-steps", type=int, default=500)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--adj-n", type=int, default=256)
    ap.add_argument("--adj-time-steps", type=int, default=2000)
    ap.add_argument("--adj-fd-directions", type=int, default=16)
    ap.add_argument("--no-multifield", action="store_true")
    ap.add_argument("--lame-n", type=int, default=384)
    ap.add_argument("--yee-n", type=int, default=512)
    ap.add_argument("--mf-time-steps", type=int, default=100)
    ap.add_argument("--no-oracle-error", action="store_true",
                    help="skip the errors against the CPU oracle (each section states one by default)")
    ap.add_argument("--temporal-depth", choices=["auto", "1", "2"], default="auto",
                    help="temporal blocking depth of the plain sweep (auto: the autotuner's choice)")
    ap.add_argument("--no-tissue", action="store_true")
    ap.add_argument("--tissue-n", type=int, default=512)
    ap.add_argument("--ref-sweeps", type=int, default=10,
                    help="sweeps of the 512^3 field per step of the reference arm (even)")
    return ap.parse_args()


def workload_config(args, world: int) -> dict:
    """The workload both arms measure (the same dict in both JSON lines)."""
    n, T = args.n, args.time_steps
    return {"workload": f"heat3d {n}^3 FP64 plain sweep, sine+noise(seed 2), Dirichlet 0, "
                        f"tau=0.9h^2/6, {T} explicit Euler steps per bench step",
            "nodes": [n, n, n], "time_steps_per_step": T, "parallelism": f"replicas x{world}",
            "l2": (f"inputs larger than L2 ({n ** 3 * 8 / 2 ** 30:.3g} GiB per field), no flush"
                   if n ** 3 * 8 > 129e6 else "field smaller than L2 (a test size, not the workload)")}


def rel_err(a, ref) -> float:
    """Relative max-norm error max|a - ref| / max|ref|."""
    return float(np.max(np.abs(a - ref))) / float(np.max(np.abs(ref)))


# ---- process group (replicas only: no data-path collective) ---------------

class Dist:
    def __init__(self, backend: str):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---- inputs -----------------------------------------------------------------

def workload(n: int):
    h = 1.0 / (n - 1)
    tau = 0.9 * h * h / 6.0
    return h, tau


def make_u0(n: int, out: np.ndarray, seed: int = 2) -> np.ndarray:
    """Sine mode + seeded noise at inner nodes, border 0, written into out
    (shape (n, n, n), x fastest)."""
    h, _ = workload(n)
    s = np.sin(np.pi * h * np.arange(n))
    rng = np.random.default_rng(seed)
    inner = np.zeros(n, dtype=bool)
    inner[1:-1] = True
    for k in range(n):
        plane = s[k] * (s[:, None] * s[None, :])
        plane = plane + rng.uniform(-1e-3, 1e-3, (n, n))
        if inner[k]:
            plane[0, :] = plane[-1, :] = 0.0
            plane[:, 0] = plane[:, -1] = 0.0
        else:
            plane[:] = 0.0
        out[k] = plane
    return out


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def pipe_peaks():
    """FP64 and FP32 FMA issue rates of this GPU (G op/s), measured live by
    scafes_probe_pipe_rates (CUDA events)."""
    import ctypes as C

    import masterthesis_gb300 as M
    f64, f32 = C.c_double(), C.c_double()
    if M.lib().scafes_probe_pipe_rates(C.byref(f64), C.byref(f32)) != 0:
        return None, None
    return f64.value, f32.value


def ncu_figure(name: str, kernel_key: str):
    """One figure of an ncu capture (e.g. traffic_bytes_per_launch, the DRAM
    bytes read + written per launch), from the committed profile summary of
    that kernel."""
    for p in sorted((ROOT / "profiles").glob("*.md")):
        txt = p.read_text()
        m = re.search(rf"{re.escape(name)}\[{re.escape(kernel_key)}\]:\s*([0-9.eE+]+)", txt)
        if m:
            return float(m.group(1))
    return None


def ncu_traffic(kernel_key: str):
    return ncu_figure("traffic_bytes_per_launch", kernel_key)


# ---- GPU clock sampling during the timed region -----------------------------

class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        rows = [r for r in csv.reader(io.StringIO(out)) if len(r) >= 9]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        load = [v for v in sm if v > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


# ---- CPU baseline (the oracle port of the reference's update) ---------------

def cpu_sample_glups(n: int, target_s: float, max_sweeps: int = 60):
    """Times the reference's update (C restatement, all host threads) on the
    512^3 workload for a bounded, even number of sweeps (~target_s seconds),
    on fields allocated and first-touched before the timed region."""
    import oracle as O
    _, tau = workload(n)
    g = O.make_grid((n, n, n), tau=tau)
    threads = os.cpu_count() or 1
    u = O.first_touched((n, n, n), threads)
    w = O.first_touched((n, n, n), threads)
    make_u0(n, u)
    t0 = time.perf_counter()
    O.heat_dirichlet_ws(g, u, w, 2, nthreads=threads)
    one = (time.perf_counter() - t0) / 2
    sweeps = 2 * int(max(1, min(max_sweeps, target_s / max(one, 1e-3)) // 2))
    t0 = time.perf_counter()
    O.heat_dirichlet_ws(g, u, w, sweeps, nthreads=threads)
    dt = time.perf_counter() - t0
    return n ** 3 * sweeps / dt / 1e9, threads, sweeps, dt


def cpu_section_baselines(args) -> dict:
    """CPU baselines of the other workloads (the oracle's restatements, all
    host threads), each timed on a bounded sample of its workload:
    batched -- the first 16 ensemble instances x 50 steps; adjoint -- the
    forward solve and the adjoint at 64^3 x 200 steps (every state stored);
    Lame 192^3 x 40 steps; Yee 256^3 x 80 steps; tissue 256^3 x 40 steps."""
    import oracle as O
    from masterthesis_gb300 import workloads as W
    threads = os.cpu_count() or 1
    out = {}
    # Batched ensemble: instance by instance, as the reference runs them.
    specs = W.pennes_ensemble(n_inst=args.batch_instances, seed=8)[:16]
    T = 50
    lup, t0 = 0, time.perf_counter()
    for sp in specs:
        n = sp["n"]
        shape = (n[2], n[1], n[0])
        g = O.make_grid(n, tau=sp["tau"])
        u0 = np.full(shape, W.T_ARTERIAL)
        O.pennes_mri(g, u0, T, 1.0, 1.0, sp["k"], 1.0, 1.0, sp["w_b"], W.T_ARTERIAL, sp["q"], u0, nthreads=threads)
        lup += int(np.prod(n)) * T
    dt = time.perf_counter() - t0
    out["batched"] = {"value": lup / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                      "sample": f"first {len(specs)} instances x {T} steps, one after the other ({dt:.1f} s)"}
    # Adjoint: forward solve and gradient (every state stored) at 64^3.
    n, T = (64, 64, 64), 200
    rng = np.random.default_rng(5)
    shape = (64, 64, 64)
    k = np.exp(0.3 * rng.standard_normal(shape))
    tau = 0.9 / (2.0 * k.max() * sum((m - 1) ** 2 for m in n))
    g = O.make_grid(n, tau=tau)
    u0 = rng.uniform(-1.0, 1.0, shape)
    t0 = time.perf_counter()
    _, traj = O.kheat_forward(g, k, u0, T, keep_traj=True, nthreads=threads)
    t1 = time.perf_counter()
    O.kheat_adjoint(g, k, traj, np.zeros(shape), nthreads=threads)
    t2 = time.perf_counter()
    out["adjoint"] = {"value": 64 ** 3 * T / (t1 - t0) / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                      "gradient_over_forward": (t2 - t0) / (t1 - t0),
                      "sample": f"64^3 x {T} steps, forward {1e3 * (t1 - t0):.0f} ms, adjoint {1e3 * (t2 - t1):.0f} ms"}
    # Lame and Yee.
    n, T = (192, 192, 192), 40
    u0 = W.gaussian_bump_displacement(n, seed=3)
    g = O.make_grid(n, tau=W.lame_tau(n))
    t0 = time.perf_counter()
    O.lame(g, u0, u0.copy(), T, 1.0, 0.5, 1.0, nthreads=threads)
    dt = time.perf_counter() - t0
    out["lame_f64"] = {"value": 192 ** 3 * T / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                       "sample": f"192^3 x {T} steps ({dt:.1f} s)"}
    n, T = (256, 256, 256), 80
    tau, src, par = W.yee_setup(n)
    g = O.make_grid(n, tau=tau)
    t0 = time.perf_counter()
    O.yee(g, np.zeros((6, 256, 256, 256)), T, src, *par, nthreads=threads)
    dt = time.perf_counter() - t0
    out["yee_f64"] = {"value": 256 ** 3 * T / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                      "sample": f"256^3 x {T} steps ({dt:.1f} s)"}
    # Tissue (the MRI-data example's update with per-node coefficients).
    m, T = 256, 40
    nn = (m, m, m)
    f = W.tissue_fields_slab(nn, 0, m, 31)
    g = O.make_grid(nn, last=TISSUE_LAST, tau=W.tissue_tau(nn, TISSUE_LAST))
    u0 = np.full((m, m, m), 37.0)
    t0 = time.perf_counter()
    O.pennes_tissue(g, u0, T, f, zmax_kind=0, q_bc=TISSUE_FLUX["q_bc"], q_skull=TISSUE_FLUX["q_skull"],
                    nthreads=threads)
    dt = time.perf_counter() - t0
    out["tissue"] = {"value": m ** 3 * T / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                     "sample": f"{m}^3 x {T} steps ({dt:.1f} s)"}
    return out


# ---- batched ensemble ---------------------------------------------------------

def run_batched(M, args, dist: Dist, hbm_peak: float):
    """Pennes ensemble (256 instances, sizes {32..160}^3 drawn by seed 8,
    500 steps, FP64): all instances in one persistent launch per step with
    the loop replayed from a CUDA graph, against one plain launch per
    instance per step.  24 algorithmic bytes per node update (T read and
    write, source read)."""
    from masterthesis_gb300 import workloads as W
    specs = W.pennes_ensemble(n_inst=args.batch_instances, seed=8)
    T = args.batch_time_steps
    out = {"workload": f"Pennes ensemble: {len(specs)} instances, sizes {{32,48,...,160}}^3 (seed 8), "
                       f"FP64, {T} steps, Dirichlet 37, Gaussian source"}
    f64_final = []
    sample = list(range(0, len(specs), 8))       # instances checked against the oracle
    kept = {}
    for prec in ("f64", "f32x2"):
        b = M.Batch([W.pennes_batch_instance(s) for s in specs], precision=prec)
        err = None
        try:
            for i, s in enumerate(specs):
                b.upload(i, M.FIELD_F_A, W.pennes_source(s))
                b.upload(i, M.FIELD_U, np.full((s["n"][2], s["n"][1], s["n"][0]), W.T_ARTERIAL))
            tile, ctas = b.autotune(5)
            depth = b.temporal_depth()
            nodes = b.info()["nodes"]
            b.step(T)                  # warm-up: captures the graph
            dist.barrier()
            b.step(T)
            ms_b = dist.max(b.last_ms())
            launches_b = b.info()["launches"]
            b.step_looped(T)
            ms_l = dist.max(b.last_ms())
            launches_l = b.info()["launches"]
            # The pair result's distance to the FP64 one after the
            # workload's T steps (a fresh start from the initial iterate).
            for i, s in enumerate(specs):
                b.upload(i, M.FIELD_U, np.full((s["n"][2], s["n"][1], s["n"][0]), W.T_ARTERIAL))
            b.step(T)
            kept[prec] = {i: b.download(i) for i in sample}
            if prec == "f64":
                f64_final = [b.download(i) for i in range(len(specs))]
            else:
                err = 0.0
                for i in range(len(specs)):
                    ref = f64_final[i]
                    err = max(err, float(np.max(np.abs(b.download(i) - ref))) / float(np.max(np.abs(ref))))
                f64_final = []
        finally:
            b.close()
        lup = nodes * T
        g_b = dist.world * lup / (ms_b * 1e-3) / 1e9
        g_l = dist.world * lup / (ms_l * 1e-3) / 1e9
        out[prec] = {"value": g_b, "unit": UNIT, "looped_value": g_l, "speedup_vs_looped": ms_l / ms_b,
                     "hbm_frac": 24 * lup / (ms_b * 1e-3) / 1e9 / hbm_peak, "ms": ms_b, "looped_ms": ms_l,
                     "nodes": nodes, "tile": tile, "ctas_per_sm": ctas, "temporal_depth": depth["depth"],
                     "autotune_ms_by_depth": {"1": depth["ms_depth1"], "2": depth["ms_depth2"], "trial_steps": 6},
                     "launches": launches_b, "looped_launches": launches_l}
        if err is not None:
            out[prec]["max_rel_err_vs_f64"] = err
            out[prec]["steps_compared"] = T
    if not args.no_oracle_error and dist.rank == 0:
        # Every 8th instance after the workload's T steps against the CPU
        # oracle of the MRI-form Pennes update (after the timed runs).
        import oracle as O
        errs = {p: 0.0 for p in kept}
        t0 = time.perf_counter()
        for i in sample:
            sp = specs[i]
            n = sp["n"]
            g = O.make_grid(n, tau=sp["tau"])
            u0 = np.full((n[2], n[1], n[0]), W.T_ARTERIAL)
            ref = O.pennes_mri(g, u0, T, 1.0, 1.0, sp["k"], 1.0, 1.0, sp["w_b"], W.T_ARTERIAL, sp["q"], u0,
                               nthreads=os.cpu_count() or 1)
            for p in kept:
                errs[p] = max(errs[p], rel_err(kept[p][i], ref))
        for p, e in errs.items():
            out[p]["error_vs_oracle"] = {"max_rel": e, "instances": len(sample), "steps": T,
                                         "sample": f"instances 0, 8, ..., {sample[-1]} of {len(specs)}, "
                                                   f"full {T} steps each (oracle {time.perf_counter() - t0:.0f} s)"}
    return out


# ---- adjoint --------------------------------------------------------------------

def smooth_gauss(n, seed):
    """Seeded standard-normal field smoothed by 3 Jacobi passes (x fastest)."""
    g = np.random.default_rng(seed).standard_normal((n[2], n[1], n[0]))
    for _ in range(3):
        g[1:-1, 1:-1, 1:-1] = (g[2:, 1:-1, 1:-1] + g[:-2, 1:-1, 1:-1] + g[1:-1, 2:, 1:-1] + g[1:-1, :-2, 1:-1]
                               + g[1:-1, 1:-1, 2:] + g[1:-1, 1:-1, :-2]) / 6.0
    return g


def run_adjoint(M, args, dist: Dist):
    """Adjoint workload: flux-form heat with k = exp(0.3 g), g a seeded
    (seed 5) smoothed Gaussian field, 256^3, 2000 steps, u0 = sine mode,
    target = the forward solve with a second conductivity (seed 6).  For
    each arithmetic (FP64; compensated FP32 pairs): the forward solve's
    time, and for 45, 128, 256 and 512 snapshots and (where it fits in
    device memory) every state stored, the gradient's time, its ratio to
    the forward solve in the same arithmetic, the forward steps of the
    binomial schedule and the snapshot memory.  Both gradients are checked
    against central differences of J (FP64 forward solves) on seeded
    directions."""
    import torch
    from masterthesis_gb300 import workloads as W
    n = (args.adj_n,) * 3
    T = args.adj_time_steps
    k = np.exp(0.3 * smooth_gauss(n, 5))
    k2 = np.exp(0.3 * smooth_gauss(n, 6))
    tau = 0.9 / (2.0 * max(k.max(), k2.max()) * sum((m - 1) ** 2 for m in n))
    u0 = W.heat_sine_noise(n, amp=0.0)
    out = {"workload": f"adjoint heat, k=exp(0.3 g) (seed 5), {n[0]}^3, {T} steps, "
                       f"J=0.5||u_T-u_target||^2, u_target from k seed 6"}
    field = int(np.prod(n)) * 8
    lups = float(np.prod(n)) * T

    def forward_ms(prec):
        with M.Adjoint(n, tau, 2, precision=prec) as a:
            a.set_conductivity(k)
            a.forward(u0, 2)  # warm-up
            a.forward(u0, T)
            return a.stats()["forward_ms"]

    def gradient(prec, snaps):
        with M.Adjoint(n, tau, snaps, precision=prec) as a:
            a.set_conductivity(k)
            J, gk, gu = a.gradient(u0, target, T)
            return J, gk, gu, a.stats()

    with M.Adjoint(n, tau, 2) as a:
        a.set_conductivity(k2)
        target = a.forward(u0, T)
    grads = {}
    for prec in ("f64", "f32x2"):
        f_ms = forward_ms(prec)
        sec = {"forward_ms": f_ms, "forward_glups": lups / (f_ms * 1e-3) / 1e9, "gradient": {}}
        torch.cuda.empty_cache()
        free, _ = torch.cuda.mem_get_info()
        for snaps in (45, 128, 256, 512, T + 1):
            if (snaps + 16) * field > free:
                continue
            J, gk, gu, st = gradient(prec, snaps)
            name = "store_all" if snaps == T + 1 else f"snapshots_{snaps}"
            sec["gradient"][name] = {"gradient_ms": st["gradient_ms"], "cost_ratio": st["gradient_ms"] / f_ms,
                                     "forward_steps": st["forward_steps"], "adjoint_steps": st["adjoint_steps"],
                                     "snapshot_bytes": snaps * field, "J": J}
            if snaps == 45:
                grads[prec] = (J, gk, gu)
        out[prec] = sec
    if "f64" in grads and "f32x2" in grads:
        (J64, gk64, gu64), (J, gk, gu) = grads["f64"], grads["f32x2"]
        out["f32x2"]["rel_diff_vs_f64"] = {"J": abs(J - J64) / abs(J64),
                                           "grad_k": float(np.abs(gk - gk64).max() / np.abs(gk64).max()),
                                           "grad_u0": float(np.abs(gu - gu64).max() / np.abs(gu64).max())}
    # Central differences of J on seeded directions (k relative), FP64.
    errs = {p: [] for p in grads}
    with M.Adjoint(n, tau, 2) as a:
        def J_of(kk, uu):
            a.set_conductivity(kk)
            uT = a.forward(uu, T)
            return 0.5 * float(np.sum((uT - target) ** 2))
        for seed in range(args.adj_fd_directions):
            rng = np.random.default_rng(7000 + seed)
            dk = rng.standard_normal(k.shape) * k
            # eps 1e-4: the difference's truncation error (~eps^2) and its
            # rounding noise (~1e-16 J / eps) both stay near 1e-8 here.
            eps = 1e-4
            fd = (J_of(k + eps * dk, u0) - J_of(k - eps * dk, u0)) / (2 * eps)
            for p, (_, g, _) in grads.items():
                errs[p].append(abs(fd - float(np.sum(g * dk))) / abs(fd))
    out["fd_directions"] = args.adj_fd_directions
    for p, e in errs.items():
        out[p]["fd_max_rel_err"] = max(e) if e else None
    if not args.no_oracle_error and dist.rank == 0:
        out["error_vs_oracle"] = adjoint_oracle_error(M)
    return out


def adjoint_oracle_error(M, m: int = 64, T: int = 200, snaps: int = 12):
    """J, dJ/dk and dJ/du0 of the GPU gradient (checkpointed) against the
    CPU oracle's adjoint on the workload's problem at m^3 x T steps (the
    oracle keeps every forward state in host memory, so the full 256^3 x
    2000 run, 268 GB of states, is out of its reach)."""
    import oracle as O
    from masterthesis_gb300 import workloads as W
    n = (m,) * 3
    k = np.exp(0.3 * smooth_gauss(n, 5))
    k2 = np.exp(0.3 * smooth_gauss(n, 6))
    tau = 0.9 / (2.0 * max(k.max(), k2.max()) * sum((v - 1) ** 2 for v in n))
    u0 = W.heat_sine_noise(n, amp=0.0)
    g = O.make_grid(n, tau=tau)
    threads = os.cpu_count() or 1
    target = O.kheat_forward(g, k2, u0, T, nthreads=threads)
    _, traj = O.kheat_forward(g, k, u0, T, keep_traj=True, nthreads=threads)
    J_ref, gk_ref, gu_ref = O.kheat_adjoint(g, k, traj, target, nthreads=threads)
    out = {"sample": f"{m}^3 x {T} steps, {snaps} snapshots, same k (seed 5) and target (seed 6) construction"}
    for prec in ("f64", "f32x2"):
        with M.Adjoint(n, tau, snaps, precision=prec) as a:
            a.set_conductivity(k)
            J, gk, gu = a.gradient(u0, target, T)
        out[prec] = {"J_rel": abs(J - J_ref) / abs(J_ref), "grad_k_rel": rel_err(gk, gk_ref),
                     "grad_u0_rel": rel_err(gu, gu_ref)}
    return out


# ---- multi-field leapfrog workloads ------------------------------------------

def run_multifield(M, args, dist: Dist, hbm_peak: float):
    """Lame-Navier 384^3 in FP64 and FP32 pairs (lambda=1, mu=0.5, rho=1,
    seeded Gaussian bump, seed 3) and Yee 512^3 in FP32, FP32 pairs and FP64
    (eps=mu=1, Courant 0.5, seeded point dipole, seed 4): GLUP/s over a timed
    run of leapfrog steps.  Algorithmic bytes per node update: Lame 72 (u^n
    and u^{n-1} read, u^{n+1} written, 3 components), Yee 6 fields read +
    written (96 B FP64 and pairs, 48 B FP32)."""
    from masterthesis_gb300 import workloads as W
    T = args.mf_time_steps
    out = {}
    n = (args.lame_n,) * 3
    check = not args.no_oracle_error and dist.rank == 0
    E = 10  # steps of the full-size comparison with the oracle
    for prec in ("f64", "f32x2"):
        u0 = W.gaussian_bump_displacement(n, seed=3)
        with M.MultiField(M.MF_LAME, n, W.lame_tau(n), (1.0, 0.5, 1.0), precision=prec) as mf:
            for c in range(3):
                mf.upload(c, u0[c])
                mf.upload(3 + c, u0[c])
            del u0
            mf.step(5)
            dist.barrier()
            mf.step(T)
            ms = dist.max(mf.last_ms())
        lup = float(np.prod(n)) * T
        g = dist.world * lup / (ms * 1e-3) / 1e9
        out[f"lame_{prec}"] = {"workload": f"Lame-Navier {n[0]}^3 {prec.upper()}, leapfrog, {T} steps", "value": g,
                               "unit": UNIT, "hbm_frac": 72 * g / hbm_peak, "bytes_per_lup": 72, "ms": ms}
    if check:
        import oracle as O
        threads = os.cpu_count() or 1
        u0 = W.gaussian_bump_displacement(n, seed=3)
        ref, _ = O.lame(O.make_grid(n, tau=W.lame_tau(n)), u0, u0, E, 1.0, 0.5, 1.0, nthreads=threads)
        for prec in ("f64", "f32x2"):
            with M.MultiField(M.MF_LAME, n, W.lame_tau(n), (1.0, 0.5, 1.0), precision=prec) as mf:
                for c in range(3):
                    mf.upload(c, u0[c])
                    mf.upload(3 + c, u0[c])
                mf.step(E)
                u = np.stack([mf.download(c) for c in range(3)])
            out[f"lame_{prec}"]["error_vs_oracle"] = {"max_rel": rel_err(u, ref),
                                                      "sample": f"{n[0]}^3, first {E} steps (full grid)"}
            del u
        del u0, ref
    n = (args.yee_n,) * 3
    tau, src, par = W.yee_setup(n)
    for prec, bpl in (("f32", 48), ("f32x2", 96), ("f64", 96)):
        with M.MultiField(M.MF_YEE, n, tau, par, precision=prec, src=src) as mf:
            mf.step(5)
            dist.barrier()
            mf.step(T)
            ms = dist.max(mf.last_ms())
        lup = float(np.prod(n)) * T
        g = dist.world * lup / (ms * 1e-3) / 1e9
        out[f"yee_{prec}"] = {"workload": f"Yee FDTD {n[0]}^3 {prec.upper()}, PEC, point dipole, {T} steps",
                              "value": g, "unit": UNIT, "hbm_frac": bpl * g / hbm_peak, "bytes_per_lup": bpl,
                              "ms": ms}
    # The same cavity (no source) as recorded linear rules on the generic
    # multi-field kernel (scafes_lin_*: what the drop-in runs for a Yee
    # class written against the callbacks): FP64, plain loads.
    with M.Linear(n, 6, 2) as lin:
        for (ph, f, c), terms in W.yee_linear_rules(tau * (n[0] - 1)).items():
            lin.set_rule(ph, f, c, terms)
        rng = np.random.default_rng(4)
        for f in range(6):
            lin.upload(f, rng.uniform(-1.0, 1.0, (n[2], n[1], n[0])))
        lin.step(2)
        dist.barrier()
        lin.step(T)
        ms = dist.max(lin.last_ms())
    lup = float(np.prod(n)) * T
    g = dist.world * lup / (ms * 1e-3) / 1e9
    out["yee_linear_f64"] = {"workload": f"Yee cavity {n[0]}^3 as recorded linear rules (scafes_lin), FP64, "
                                         f"seeded fields (seed 4), no source, {T} steps",
                             "value": g, "unit": UNIT, "hbm_frac": 96 * g / hbm_peak, "bytes_per_lup": 96, "ms": ms,
                             "launches_per_step": 2}
    if check:
        # Both precisions against the oracle after 2E steps from the
        # workload's initial state (zero fields, the dipole switched on).
        ref = O.yee(O.make_grid(n, tau=tau), np.zeros((6, n[2], n[1], n[0])), 2 * E, src, *par, nthreads=threads)
        for prec in ("f32", "f32x2", "f64"):
            with M.MultiField(M.MF_YEE, n, tau, par, precision=prec, src=src) as mf:
                mf.step(2 * E)
                f = np.stack([mf.download(i) for i in range(6)])
            out[f"yee_{prec}"]["error_vs_oracle"] = {"max_rel": rel_err(f, ref),
                                                     "sample": f"{n[0]}^3, first {2 * E} steps (full grid)"}
            del f
        # The linear-rule path against the oracle's Yee without a source.
        m = (128, 128, 128)
        tau_m, _, _ = W.yee_setup(m)
        f0 = np.random.default_rng(4).uniform(-1.0, 1.0, (6, m[2], m[1], m[0]))
        with M.Linear(m, 6, 2) as lin:
            for (ph, f, c), terms in W.yee_linear_rules(tau_m * (m[0] - 1)).items():
                lin.set_rule(ph, f, c, terms)
            for f in range(6):
                lin.upload(f, f0[f])
            lin.step(2 * E)
            got = np.stack([lin.download(f) for f in range(6)])
        ref = O.yee(O.make_grid(m, tau=tau_m), f0, 2 * E, (0, 0, 0), 0.0, 1.0, 1.0, 1.0, nthreads=threads)
        out["yee_linear_f64"]["error_vs_oracle"] = {"max_rel": rel_err(got, ref),
                                                    "sample": f"{m[0]}^3, {2 * E} steps, same construction"}
    return out


# ---- variable coefficients (the tissue examples' update) ----------------------

TISSUE_LAST = (0.05, 0.04, 0.03)          # domain of the MRI-data example's golden case (m)
TISSUE_FLUX = {"zmax_kind": 0, "q_bc": 5.0, "q_skull": -3.0}
TISSUE_FP64_OPS = 8                       # 3 DADD, 1 DMUL, 4 DFMA per inner node


def tissue_arrays(n: int, seed: int = 31):
    """The MRI-data Pennes update on n^3 nodes of the 5 x 4 x 3 cm domain:
    seeded coefficient fields over the nodes (workloads.tissue_fields_slab)
    folded slab by slab into C0, CA and the source F, Neumann borders as
    per-node rules.  Returns (C0, CA, F, rules, cp, tau)."""
    from masterthesis_gb300 import workloads as W
    nn = (n, n, n)
    tau = W.tissue_tau(nn, TISSUE_LAST)
    h = [TISSUE_LAST[p] / (n - 1) for p in range(3)]
    C0, CA, F = (np.empty((n, n, n)) for _ in range(3))
    rules = []
    for z0 in range(0, n, 32):
        z1 = min(n, z0 + 32)
        d = W.tissue_device_form(nn, h, tau, W.tissue_fields_slab(nn, z0, z1, seed), z0, TISSUE_FLUX)
        C0[z0:z1], CA[z0:z1], F[z0:z1] = d["C0"], d["CA"], d["F"]
        rules.append(d["rules"])
    return C0, CA, F, np.concatenate(rules), d["cp"], tau


def tissue_problem(M, arrays, prec: str):
    """An open Plain handle of the tissue problem (initial temperature 37)."""
    C0, CA, F, rules, cp, tau = arrays
    n = C0.shape[0]
    cfg = M.make_cfg((n, n, n), last=TISSUE_LAST, tau=tau, precision=prec, border=M.BORDER_NODES, c0=0.0, cp=cp,
                     cf=1.0)
    p = M.Plain(cfg)
    p.upload(M.FIELD_C0, C0)
    p.upload(M.FIELD_CA, CA)
    p.upload(M.FIELD_F_A, F)
    p.set_border_node_rules(rules)
    p.upload(M.FIELD_U, np.full((n, n, n), 37.0))
    return p


def run_tissue(M, args, dist: Dist, hbm_peak: float, fp64_peak):
    """Variable-coefficient Pennes (the MRI-data example's update): 512^3,
    eight seeded coefficient fields folded into C0, CA and the source F,
    per-node Neumann border rules, 200 steps, FP64 and FP32.  Algorithmic
    bytes per node update: the iterate read and written plus C0, CA, F read
    (40 B FP64, 20 B FP32).  Error: the same construction at 96^3 x 100
    steps against the oracle's restatement of the example."""
    n, T = args.tissue_n, 200
    out = {"workload": f"tissue Pennes (MRI-data example's update), {n}^3, coefficients per node (seed 31), "
                       f"Neumann borders per node, {T} steps"}
    arrays = tissue_arrays(n)
    for prec, bpl in (("f64", 40), ("f32", 20)):
        p = tissue_problem(M, arrays, prec)
        try:
            tile, _ = p.autotune(5)
            p.step(T)  # warm-up
            dist.barrier()
            p.step(T)
            ms = dist.max(p.last_step_ms())
        finally:
            p.close()
        lup = float(n) ** 3 * T
        g = dist.world * lup / (ms * 1e-3) / 1e9
        out[prec] = {"value": g, "unit": UNIT, "hbm_frac": bpl * g / hbm_peak, "bytes_per_lup": bpl, "ms": ms,
                     "tile": tile}
        if prec == "f64" and fp64_peak:
            out[prec]["fp64_pipe_frac"] = TISSUE_FP64_OPS * g / fp64_peak
    if not args.no_oracle_error and dist.rank == 0:
        import oracle as O
        from masterthesis_gb300 import workloads as W
        m, Te = 96, 100
        nn = (m, m, m)
        f = W.tissue_fields_slab(nn, 0, m, 31)
        tau = W.tissue_tau(nn, TISSUE_LAST)
        g = O.make_grid(nn, last=TISSUE_LAST, tau=tau)
        ref = O.pennes_tissue(g, np.full((m, m, m), 37.0), Te, f, zmax_kind=0, q_bc=TISSUE_FLUX["q_bc"],
                              q_skull=TISSUE_FLUX["q_skull"], nthreads=os.cpu_count() or 1)
        small = tissue_arrays(m)
        for prec in ("f64", "f32"):
            p = tissue_problem(M, small, prec)
            try:
                p.step(Te)
                out[prec]["error_vs_oracle"] = {"max_rel": rel_err(p.download(), ref),
                                                "sample": f"{m}^3 x {Te} steps, same construction"}
            finally:
                p.close()
    del arrays
    return out


# ---- GPU arm ----------------------------------------------------------------

def run_ours(args, dist: Dist):
    import torch

    import masterthesis_gb300 as M
    from masterthesis_gb300 import build as B

    B.build_library()
    torch.cuda.set_device(dist.local_rank)
    n, T = args.n, args.time_steps
    _, tau = workload(n)
    nn = n ** 3
    # Host arrays of the end-to-end copies: pinned and backed by huge pages,
    # so that the copies after a long solve keep the link rate.
    host_u0 = M.HostArray((n, n, n))
    host_out = M.HostArray((n, n, n))
    u0 = host_u0.a
    make_u0(n, u0)
    out = host_out.a
    stream = torch.cuda.Stream()
    tuned = {}

    def device_timed(prec: str, steps: int, warmup: int, clocks: Clocks | None):
        cfg = M.make_cfg((n, n, n), tau=tau, precision=prec, heat=(1.0, 1.0, 0.0),
                         stream=stream.cuda_stream)
        with M.Plain(cfg) as p:
            p.upload(M.FIELD_U, u0)
            # picks the sweep's CTA tile variant and the temporal blocking depth
            tile_ms = p.autotune(10)
            if args.temporal_depth != "auto":
                p.set_temporal_depth(int(args.temporal_depth))
            tuned[prec] = tile_ms + (p.temporal_depth,)
            for _ in range(warmup):
                p.step(T)
            stream.synchronize()
            dist.barrier()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            if clocks:
                clocks.start()
            e0.record(stream)
            launches = 0
            for _ in range(steps):
                p.step(T)
                launches += p.last_step_launches()
            e1.record(stream)
            e1.synchronize()
            clk = clocks.stop() if clocks else None
            torch.cuda.synchronize()
            dist.barrier()
            dt = dist.max(e0.elapsed_time(e1) / 1e3)
        return dt, launches, clk

    # Headline: FP64 storage and arithmetic.
    dt, launches, clk = device_timed("f64", args.steps, args.warmup, Clocks(dist.local_rank))
    value = dist.world * nn * T * args.steps / dt / 1e9
    launch_s = dt / (args.steps * T)
    hbm_peak, peak_src = measured_peaks()
    achieved_gbs = B_PER_LUP["f64"] * nn / launch_s / 1e9
    # DRAM bytes per launch from the committed ncu summary of this kernel at
    # this grid size (null when no capture of this size exists).
    key = f"star7_tma<PolF64>@{args.n}"
    traffic = ncu_traffic(key)
    roofline = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved_gbs / hbm_peak, "traffic": traffic,
                "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                "kernel": "star7_tma<PolF64>", "bytes_per_launch_alg": B_PER_LUP["f64"] * nn,
                "launch_ms": launch_s * 1e3}
    fp64_peak, fp32_peak = pipe_peaks()
    if fp64_peak:
        # The update is 7 FP64 operations; the three neighbour sums run on the
        # integer pipe (bit-identical), the rest (plus the sums of warps that
        # fall back to FP64) on the FP64 pipe.
        ncu_fp64 = ncu_figure("fp64_ops_per_lup", key)
        on_pipe = ncu_fp64 if ncu_fp64 else FP64_OPS_PER_LUP - INT_SUMS_PER_LUP
        ach = FP64_OPS_PER_LUP * nn / launch_s / 1e9
        pipe_ach = on_pipe * nn / launch_s / 1e9
        roofline["fp64_pipe"] = {"achieved_gops": pipe_ach, "peak_gops": fp64_peak, "frac": pipe_ach / fp64_peak,
                                 "ops_on_fp64_pipe_per_lup": on_pipe,
                                 "ops_per_lup": FP64_OPS_PER_LUP, "int_pipe_sums_per_lup": INT_SUMS_PER_LUP,
                                 "fp64_equivalent_gops": ach, "fp64_equivalent_frac": ach / fp64_peak,
                                 "fp32_fma_gops": fp32_peak,
                                 "peak_source": "measured live (scafes_probe_pipe_rates)",
                                 "ncu": {"fp64_ops_per_lup": ncu_fp64,
                                         "fp64_pipe_active": ncu_figure("fp64_pipe_active", key),
                                         "alu_pipe_active": ncu_figure("alu_pipe_active", key),
                                         "issue_active": ncu_figure("issue_active", key),
                                         "source": "profiles/star7_f64_heat512.md"},
                                 "note": "the FP64 pipe and the integer ALU, not HBM, bind this kernel on GB300: "
                                         "7 FP64 operations per node, 3 of them as exact integer additions"}

    # e2e through the C ABI with host buffers, pipelined: two handles on two
    # streams, step k on handle k % 2 (upload_async, step, download_async).
    # The sweeps of one handle wait for the other's (an event), so the GPU
    # runs one solve at a time while one step's copies overlap the other
    # handle's sweeps.  Every step copies its 1 GiB input in and its 1 GiB
    # result out inside the timed region; the wall clock spans the first
    # upload to the last download's completion.
    host_in2 = M.HostArray((n, n, n))
    host_out2 = M.HostArray((n, n, n))
    host_in2.a[...] = u0
    ins, outs = [u0, host_in2.a], [out, host_out2.a]
    streams = [stream, torch.cuda.Stream()]
    handles = [M.Plain(M.make_cfg((n, n, n), tau=tau, precision="f64", heat=(1.0, 1.0, 0.0),
                                  stream=s_.cuda_stream, tile=tuned["f64"][0])) for s_ in streams]
    try:
        for h_ in handles:
            h_.set_temporal_depth(tuned["f64"][2])
            h_.upload(M.FIELD_U, u0)     # warm-up
            h_.step(T)
            h_.download(M.FIELD_U, out)
        dist.barrier()
        torch.cuda.synchronize()
        swept = [torch.cuda.Event(), torch.cuda.Event()]
        t0 = time.perf_counter()
        for k in range(args.steps):
            i = k % 2
            h_ = handles[i]
            if k >= 2:
                h_.synchronize()         # its previous step's result has landed
            h_.upload_async(ins[i])      # overlaps the other handle's sweeps
            if k >= 1:
                streams[i].wait_event(swept[1 - i])
            h_.step(T)
            swept[i].record(streams[i])
            h_.download_async(outs[i])   # overlaps the other handle's next sweeps
        for h_ in handles:
            h_.synchronize()
        t1 = time.perf_counter()
    finally:
        for h_ in handles:
            h_.close()
        host_in2.close()
        host_out2.close()
    e2e_pipe_dt = dist.max(t1 - t0)
    # The same calls one after the other on one handle (upload, step,
    # download, each step waiting for the previous one).
    cfg = M.make_cfg((n, n, n), tau=tau, precision="f64", heat=(1.0, 1.0, 0.0), stream=stream.cuda_stream,
                     tile=tuned["f64"][0])
    e2e_times = []
    parts = np.zeros(3)  # upload, upload-to-download (steps), download (s)
    with M.Plain(cfg) as p:
        p.set_temporal_depth(tuned["f64"][2])
        for it in range(1 + args.steps):
            dist.barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            p.upload(M.FIELD_U, u0)
            ta = time.perf_counter()
            p.step(T)
            tb = time.perf_counter()
            p.download(M.FIELD_U, out)
            t1 = time.perf_counter()
            if it > 0:
                e2e_times.append(t1 - t0)
                parts += (ta - t0, tb - ta, t1 - tb)
    e2e_dt = dist.max(sum(e2e_times))
    e2e = {"value": dist.world * nn * T * args.steps / e2e_pipe_dt / 1e9, "unit": UNIT,
           "h2d_bytes_per_step": nn * 8, "d2h_bytes_per_step": nn * 8,
           "ms_per_step": e2e_pipe_dt / args.steps * 1e3,
           "path": f"two handles on two streams, per step scafes_gpu_upload_async + scafes_gpu_step({T}) + "
                   f"scafes_gpu_download_async, scafes_gpu_synchronize before a handle's next step; the sweeps "
                   f"of one handle wait for the other's (a stream event), so one solve runs at a time and each "
                   f"step's copies overlap the other handle's sweeps; huge-page pinned host buffers "
                   f"(scafes_host_alloc)",
           "serial": {"value": dist.world * nn * T * len(e2e_times) / e2e_dt / 1e9,
                      "ms_per_step": e2e_dt / len(e2e_times) * 1e3,
                      "ms_upload_enqueue_download": [float(v) for v in parts / len(e2e_times) * 1e3],
                      "path": f"one handle: scafes_gpu_upload + scafes_gpu_step({T}) + scafes_gpu_download"}}

    variants = {}
    # One solve of the workload per precision from the same initial iterate:
    # the results whose errors the line states.
    finals = {}
    for prec in (("f64",) if args.no_variants else ("f64", "f32x2", "f32")):
        cfg = M.make_cfg((n, n, n), tau=tau, precision=prec, heat=(1.0, 1.0, 0.0), stream=stream.cuda_stream)
        with M.Plain(cfg) as p:
            p.upload(M.FIELD_U, u0)
            p.step(T)
            finals[prec] = p.download()
    if not args.no_variants:
        for prec in ("f32x2", "f32"):
            vdt, vl, _ = device_timed(prec, max(1, args.steps // 2), 1, None)
            lps = vdt / (max(1, args.steps // 2) * T)
            variants[prec] = {"value": dist.world * nn * T * max(1, args.steps // 2) / vdt / 1e9,
                              "unit": UNIT, "hbm_frac": B_PER_LUP[prec] * nn / lps / 1e9 / hbm_peak,
                              "bytes_per_lup": B_PER_LUP[prec], "launch_ms": lps * 1e3}
        # Stated error: each variant against FP64 on the same inputs, one solve.
        for prec in ("f32x2", "f32"):
            variants[prec]["rel_err_vs_f64"] = rel_err(finals[prec], finals["f64"])

    tissue = None if args.no_tissue else run_tissue(M, args, dist, hbm_peak, fp64_peak)
    batched = None if args.no_batched else run_batched(M, args, dist, hbm_peak)
    adjoint = None if args.no_adjoint else run_adjoint(M, args, dist)
    multifield = None if args.no_multifield else run_multifield(M, args, dist, hbm_peak)

    error = {"note": "relative max-norm max|u - u_oracle| / max|u_oracle| after the workload's full solve; "
                     "f64 is the reference's arithmetic with FMA contraction"}
    if not args.no_oracle_error and dist.rank == 0:
        # The CPU oracle (C restatement of the reference's update, pinned
        # bit-exact to the reference's own driver) runs the same solve after
        # every timed region of this process.
        import oracle as O
        threads = os.cpu_count() or 1
        g = O.make_grid((n, n, n), tau=tau)
        ou = O.first_touched((n, n, n), threads)
        ow = O.first_touched((n, n, n), threads)
        ou[...] = u0
        t0 = time.perf_counter()
        ref = O.heat_dirichlet_ws(g, ou, ow, T, nthreads=threads)
        error["oracle_s"] = time.perf_counter() - t0
        error["steps"] = T
        for prec, v in finals.items():
            error[f"{prec}_vs_oracle"] = rel_err(v, ref)
        del ou, ow, ref
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, dist.world),
        "e2e": e2e, "roofline": roofline, "gpu_launches": launches,
        "autotune": {k: {"tile": v[0], "ms_per_sweep_by_tile": v[1], "temporal_depth": v[2]}
                     for k, v in tuned.items()},
        "error": error,
    }
    for prec in variants:
        if f"{prec}_vs_oracle" in error:
            variants[prec]["rel_err_vs_oracle"] = error[f"{prec}_vs_oracle"]
    if variants:
        res["variants"] = variants
    if tissue:
        res["tissue"] = tissue
    if batched:
        res["batched"] = batched
    if adjoint:
        res["adjoint"] = adjoint
    if multifield:
        res["multifield"] = multifield
    if clk:
        res["clocks"] = clk
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        v, cores, sweeps, cdt = cpu_sample_glups(n, target_s=10.0)
        res["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": f"{sweeps} sweeps of the {n}^3 workload ({cdt:.1f} s), "
                                         f"C restatement of the reference update (oracle/), OpenMP"}
        # The other workloads' CPU baselines sit beside their GPU numbers.
        sec = cpu_section_baselines(args)
        if batched:
            batched["cpu_baseline"] = sec["batched"]
        if adjoint:
            adjoint["cpu_baseline"] = sec["adjoint"]
        if multifield:
            multifield["cpu_baseline"] = {"lame_f64": sec["lame_f64"], "yee_f64": sec["yee_f64"]}
        if tissue:
            tissue["cpu_baseline"] = sec["tissue"]
    return res


def run_reference(args, dist: Dist):
    """The reference's CPU update on the workload: the C restatement of the
    reference's update in oracle/ (bit-exact to the reference's own
    Problem::iterateOverTime on the golden cases; the reference's driver
    itself is not built on the GPU machine), all host threads.  Both fields are
    allocated and their pages mapped before the timed region, and each step
    times only sweeps: --ref-sweeps sweeps of the 512^3 field (a bounded
    sample of the 1000-sweep solve)."""
    if dist.rank != 0:
        return None
    import oracle as O
    O.build()
    n = args.n
    _, tau = workload(n)
    g = O.make_grid((n, n, n), tau=tau)
    threads = os.cpu_count() or 1
    u = O.first_touched((n, n, n), threads)
    w = O.first_touched((n, n, n), threads)
    make_u0(n, u)
    sweeps = max(2, args.ref_sweeps + args.ref_sweeps % 2)  # even: the iterate ends in u
    for _ in range(args.warmup):
        O.heat_dirichlet_ws(g, u, w, sweeps, nthreads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.heat_dirichlet_ws(g, u, w, sweeps, nthreads=threads)
        times.append(time.perf_counter() - t0)
    dt = sum(times)
    value = n ** 3 * sweeps * args.steps / dt / 1e9
    sample = (f"{sweeps} sweeps of the {n}^3 workload per step (the solve has {args.time_steps}), "
              f"fields allocated and first-touched outside the timed region; C restatement of the "
              f"reference update (oracle/), OpenMP {threads} threads")
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(args, dist.world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ---- single-kernel cases for profiler captures ----------------------------------

def case_adjoint(prec: str, m: int = 160, T: int = 6):
    """The adjoint workload's problem at m^3: a forward solve and a gradient
    of T steps (16 snapshots: every state kept)."""
    import masterthesis_gb300 as M
    from masterthesis_gb300 import workloads as W
    n = (m,) * 3
    k = np.exp(0.3 * smooth_gauss(n, 5))
    tau = 0.9 / (2.0 * k.max() * sum((v - 1) ** 2 for v in n))
    u0 = W.heat_sine_noise(n, amp=0.0)
    with M.Adjoint(n, tau, 16, precision=prec) as a:
        a.set_conductivity(k)
        uT = a.forward(u0, T)
        J, gk, _ = a.gradient(u0, 0.5 * uT, T)
    return f"J {J:.6e}, max|dJ/dk| {float(np.abs(gk).max()):.6e}"


def case_lame(prec: str, m: int = 192, T: int = 4):
    import masterthesis_gb300 as M
    from masterthesis_gb300 import workloads as W
    n = (m,) * 3
    u0 = W.gaussian_bump_displacement(n, seed=3)
    with M.MultiField(M.MF_LAME, n, W.lame_tau(n), (1.0, 0.5, 1.0), precision=prec) as mf:
        for c in range(3):
            mf.upload(c, u0[c])
            mf.upload(3 + c, u0[c])
        mf.step(T)
        return f"max|u_x| {float(np.abs(mf.download(0)).max()):.6e}"


def case_yee(prec: str, m: int = 256, T: int = 4):
    import masterthesis_gb300 as M
    from masterthesis_gb300 import workloads as W
    n = (m,) * 3
    tau, src, par = W.yee_setup(n)
    with M.MultiField(M.MF_YEE, n, tau, par, precision=prec, src=src) as mf:
        mf.step(T)
        return f"max|Ez| {float(np.abs(mf.download(2)).max()):.6e}"


def case_tissue(prec: str, m: int = 256, T: int = 4):
    import masterthesis_gb300 as M
    p = tissue_problem(M, tissue_arrays(m), prec)
    try:
        p.step(T)
        return f"max T {float(p.download().max()):.6e}"
    finally:
        p.close()


def case_heat(prec: str, n: int = 512, T: int = 4, tile: int = 4):
    """The large heat workload's field at n^3 in one arithmetic, T sweeps
    with a fixed tile (the autotuner's choice at 512^3: {BY 16, R 4,
    4 stages} for the FP32 pair, {BY 8, R 1, 8 stages} for FP64) and
    depth 1: every launch is the same kernel."""
    import masterthesis_gb300 as M
    _, tau = workload(n)
    u0 = np.empty((n, n, n))
    make_u0(n, u0)
    with M.Plain(M.make_cfg((n, n, n), tau=tau, precision=prec, heat=(1.0, 1.0, 0.0), tile=tile)) as p:
        p.upload(M.FIELD_U, u0)
        p.set_temporal_depth(1)
        p.step(T)
        return f"max|u| {float(np.abs(p.download()).max()):.6e}"


KERNEL_CASES = {
    "heat_f32x2_512": lambda: case_heat("f32x2"),
    "heat_f64_512": lambda: case_heat("f64", tile=1),
    "adjoint_f64_160": lambda: case_adjoint("f64"),
    "adjoint_x2_160": lambda: case_adjoint("f32x2"),
    "lame_x2_192": lambda: case_lame("f32x2"),
    "lame_f64_192": lambda: case_lame("f64"),
    "yee_x2_256": lambda: case_yee("f32x2"),
    "yee_f32_256": lambda: case_yee("f32"),
    "tissue_f32_256": lambda: case_tissue("f32"),
    "tissue_f64_256": lambda: case_tissue("f64"),
}


def main():
    args = parse_args()
    if args.kernel_case:
        from masterthesis_gb300 import build as B
        B.build_library()
        print(f"{args.kernel_case}: {KERNEL_CASES[args.kernel_case]()}", flush=True)
        return
    if args.impl == "reference":
        dist = Dist("gloo")
        res = run_reference(args, dist)
    else:
        dist = Dist("nccl")
        res = run_ours(args, dist)
    if res is not None and dist.rank == 0:
        print(json.dumps(res), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
