#!/usr/bin/env python3
"""Benchmark of the forward/adjoint LBM hot path on GB300.

Workload: the D3Q19 MRT + partial-bounce-back (Brinkman) duct, 256x128x128
cells, tau = 0.6, other MRT rates 1.2, Hecht velocity inlet u_max = 0.04 and
pressure outlet, seeded synthetic design, FP32 shifted population storage
(the production precision).  One bench step = one forward time step plus one
adjoint time step over the whole lattice.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Rank 0 prints one JSON line.  Under torchrun each rank runs an independent
replica on its own GPU (weak scaling, no collective on the data path); the
timed region is bracketed by a barrier and the device time is the maximum
over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "lbm-topopt_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, os.path.join(ROOT, "tests"))

NX, NY, NZ = 256, 128, 128
NSTEPS_GRAD = 5000     # time steps of the full design gradient (the workload's horizon)
# Checkpoint slots in device memory, chosen from the HBM budget of one GB300
# (284 GB): 512 FP32 states of 319 MB = 163 GB.  Wang's schedule recomputes
# 8906 of the 5000 steps with 64 slots, 4873 with 128 and 4489 with 512; each
# further 128 slots save 128 recomputed steps (13 ms of a 1.8 s gradient).
NSNAP = 512
# the FP64 comparison gradient (638 MB states): 128 slots = 82 GB
NSNAP_FP64 = 128
METRIC = "MLUPS fwd+adjoint D3Q19"
CONFIG_NAME = ("D3Q19 MRT (d'Humieres, s_nu from tau=0.6, other rates 1.2) + Brinkman "
               "partial bounce-back duct 256x128x128, Hecht velocity inlet u_max=0.04, "
               "pressure outlet, FP32 shifted populations")


def bytes_per_lu(storage, kind):
    """Algorithmic bytes per lattice update: forward 2*Q*s + s_gamma,
    adjoint 3*Q*s (two adjoint passes + one forward read) + s_gamma + 16 (FP64
    sensitivity read-modify-write); FP16 storage keeps FP32 adjoints."""
    Q = 19
    s = {0: 8, 1: 4, 2: 2}[storage]
    sg = 8 if storage == 0 else 4
    sa = 8 if storage == 0 else 4
    if kind == "fwd":
        return 2 * Q * s + sg
    return 2 * Q * sa + Q * s + sg + 16


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup(init=True):
    """One process per GPU (torchrun env).  NCCL with GPUs, gloo without."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1 and init:
        import torch
        import torch.distributed as td
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            td.init_process_group("nccl")
        else:
            td.init_process_group("gloo")
        dist = td
    return world, rank, local, dist


def _on_gpu(dist):
    return dist is not None and dist.get_backend() == "nccl"


def barrier(dist):
    if dist is not None:
        dist.barrier()
        if _on_gpu(dist):
            import torch
            torch.cuda.synchronize()


def _reduce(dist, v, op):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device="cuda" if _on_gpu(dist) else "cpu")
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(dist, v):
    return _reduce(dist, v, dist.ReduceOp.MAX) if dist is not None else v


def sum_over_ranks(dist, v):
    return _reduce(dist, v, dist.ReduceOp.SUM) if dist is not None else v


def aggregate_mlups(dist, cells, steps, ms):
    """Whole-job throughput of independent replicas: all ranks' lattice updates
    over the slowest rank's device time."""
    total = sum_over_ranks(dist, cells * steps)
    slowest = max_over_ranks(dist, ms)
    return total / (slowest * 1e-3) / 1e6, slowest


# ----------------------------------------------------------------------------------------
# CPU legs (the oracle restatement of the reference's CPU path)

def cpu_time(cfg, gamma, nsteps, nthreads):
    import ctypes as C
    from oracle_lib import oracle
    o = oracle()
    o.lib.orc_time_steps.restype = C.c_int
    o.lib.orc_time_steps.argtypes = [C.POINTER(type(cfg.to_c())), C.POINTER(C.c_double), C.c_int,
                                     C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    c = cfg.to_c()
    g = np.ascontiguousarray(gamma, dtype=np.float64)
    tf, ta = C.c_double(), C.c_double()
    rc = o.lib.orc_time_steps(C.byref(c), g.ctypes.data_as(C.POINTER(C.c_double)), int(nsteps),
                              int(nthreads), C.byref(tf), C.byref(ta))
    if rc:
        raise RuntimeError("oracle timing failed: %d" % rc)
    return tf.value, ta.value


def host_threads():
    import ctypes as C
    from oracle_lib import oracle
    o = oracle()
    o.lib.orc_max_threads.restype = C.c_int
    return int(o.lib.orc_max_threads())


def cpu_model():
    """The host CPU as /proc/cpuinfo or lscpu names it (x86 'model name', Arm
    'CPU part' / lscpu 'Model name'), with the online core count."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.split(":")[0].strip() in ("Model name", "Vendor ID") and ":" in ln:
                v = ln.split(":", 1)[1].strip()
                name = v if name is None else name + " " + v
    except Exception:
        pass
    if not name:
        try:
            for ln in open("/proc/cpuinfo"):
                if ln.lower().startswith(("model name", "cpu part")):
                    name = ln.split(":", 1)[1].strip()
                    break
        except OSError:
            name = "unknown"
    return "%s, %d online cores" % (name, os.cpu_count() or 0)


def duct_case():
    """The bench workload itself (the full 256x128x128 duct) in FP64, the
    reference's precision."""
    import workloads as W
    cfg, g, _ = W.workload_duct_256x128x128(W.STORE_FP64, nx=NX, ny=NY, nz=NZ, nsteps=NSTEPS_GRAD)
    return cfg, g


def cpu_baseline_leg():
    """Single-thread oracle on a bounded sample of the bench workload: the
    full duct, as many forward + adjoint step pairs as fit in about 15 s of
    CPU work (at least one)."""
    cfg, g = duct_case()
    tf, ta = cpu_time(cfg, g, 1, 1)
    per = tf + ta
    n = max(1, min(60, int(15.0 / max(per, 1e-3))))
    if n > 1:
        tf, ta = cpu_time(cfg, g, n, 1)
    else:
        n = 1
    mlups = cfg.ncells * n / (tf + ta) / 1e6
    return {"value": round(mlups, 4), "unit": "MLUPS", "cores": 1, "kind": "port",
            "cpu": cpu_model(),
            "sample": "oracle (C restatement of the reference operators, FP64, 1 thread) on the "
                      "full 256x128x128 duct, %d forward + %d adjoint steps (%.1f s); "
                      "fwd %.3f / adj %.3f MLUPS" % (n, n, tf + ta, cfg.ncells * n / tf / 1e6,
                                                    cfg.ncells * n / ta / 1e6)}


def reference_arm(args, world, rank):
    if rank != 0:
        return
    nthr = host_threads()
    cfg, g = duct_case()
    cpu_time(cfg, g, 1, nthr)   # first touch / thread start-up
    for _ in range(args.warmup):
        cpu_time(cfg, g, 1, nthr)
    tot = 0.0
    for _ in range(args.steps):
        tf, ta = cpu_time(cfg, g, 1, nthr)
        tot += tf + ta
    v = cfg.ncells * args.steps / tot / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "MLUPS",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(tot / args.steps * 1e3, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": CONFIG_NAME.replace("FP32 shifted populations",
                                                       "FP64 (reference CPU path)"),
                       "cells": cfg.ncells,
                       "step": "one forward + one adjoint time step over the lattice"},
            "cpu_baseline": {"value": round(v, 4), "unit": "MLUPS", "cores": nthr, "kind": "port",
                             "cpu": cpu_model(),
                             "sample": "oracle (C restatement of the reference operators, FP64, "
                                       "OpenMP %d threads): 1 forward + 1 adjoint step of the "
                                       "full 256x128x128 duct per bench step" % nthr},
            "e2e": {"value": round(v, 4), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------------------

def precision_errors(G, W):
    """Population error of FP32 / FP16 storage against the FP64 path on a
    64x32x32 duct after 300 steps (the FP64 GPU path equals the oracle to 1e-12)."""
    cfg, g, _ = W.workload_duct_256x128x128(G.STORE_FP64, nx=64, ny=32, nz=32, nsteps=300)
    out = {}
    ref = None
    for name, st in (("fp64", G.STORE_FP64), ("fp32", G.STORE_FP32), ("fp16", G.STORE_FP16)):
        with G.Handle(cfg.replace(storage=st)) as h:
            h.set_design(g)
            h.init_equilibrium()
            h.forward(300)
            m = h.macros().reshape(-1, 4)
        u = m[:, 1:4]
        if ref is None:
            ref = u
        else:
            out[name] = float(np.linalg.norm(u - ref) / np.linalg.norm(ref))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        world, rank, _, _ = dist_setup(init=False)
        reference_arm(args, world, rank)   # rank 0 only; the others exit without work
        return
    world, rank, local, dist = dist_setup()

    import lbmgpu as G
    import workloads as W
    G.select_device(local)
    cfg, gamma, _ = W.workload_duct_256x128x128(G.STORE_FP32, nx=NX, ny=NY, nz=NZ, nsteps=NSTEPS_GRAD)
    cells = cfg.ncells
    h = G.Handle(cfg)
    h.set_design(gamma)
    h.init_equilibrium()
    shapes = h.autotune()   # thread-block shapes of the two step kernels
    h.forward(20)   # develop the inflow before timing
    # clocks over both timed regions (the step pairs and the end-to-end
    # gradients); nvidia-smi takes a moment to start reporting
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.5)
    # warm-up pairs
    h.time_steps(2, args.warmup)
    launches0 = h.launch_count()
    barrier(dist)
    ms_pairs = h.time_steps(2, args.steps)
    barrier(dist)
    launches = h.launch_count() - launches0
    # per-kernel device time of the same two kernels, same stream
    ms_fwd = h.time_steps(0, args.steps)
    ms_adj = h.time_steps(1, args.steps)
    value, ms_pairs = aggregate_mlups(dist, cells, args.steps, ms_pairs)
    ms_fwd = max_over_ranks(dist, ms_fwd)
    ms_adj = max_over_ranks(dist, ms_adj)
    total_cells = sum_over_ranks(dist, cells)

    # roofline of the dominant kernel (the adjoint step)
    peak, peak_kind = load_peaks()
    t_adj = ms_adj / args.steps * 1e-3
    t_fwd = ms_fwd / args.steps * 1e-3
    b_adj = bytes_per_lu(G.STORE_FP32, "adj") * cells
    b_fwd = bytes_per_lu(G.STORE_FP32, "fwd") * cells
    ach_adj = b_adj / t_adj / 1e9
    ach_fwd = b_fwd / t_fwd / 1e9
    traffic = traffic_fwd = None
    tr_path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if os.path.exists(tr_path):
        with open(tr_path) as f:
            for ln in f:
                parts = ln.split()
                if len(parts) == 2 and parts[0] == "k_adjoint_fp32_256x128x128":
                    traffic = int(parts[1])
                if len(parts) == 2 and parts[0] == "k_forward_fp32_256x128x128":
                    traffic_fwd = int(parts[1])

    # end to end through the C ABI with host buffers: design upload, full checkpointed
    # gradient (5000 steps, 64 device snapshots), sensitivity download
    e2e = None
    grad_fp64_s = None
    grad_fp32_s = None
    try:
        import torch
        pin_g = torch.from_numpy(gamma.copy()).pin_memory()
        pin_s = torch.empty(cells, dtype=torch.float64).pin_memory()
        g_np = pin_g.numpy()
        s_np = pin_s.numpy()
    except Exception:
        g_np = gamma.copy()
        s_np = np.empty(cells)
    import ctypes as C
    lib = G.load_library()
    Jbuf = np.zeros(1)
    st = G.CGradStats()

    def one_gradient(handle, nsnap=NSNAP):
        handle.set_design(g_np)
        rc = lib.lbm_gradient(handle.h, NSTEPS_GRAD, nsnap, Jbuf.ctypes.data_as(C.POINTER(C.c_double)),
                              s_np.ctypes.data_as(C.POINTER(C.c_double)), C.byref(st))
        if rc:
            raise G.LBMError(rc, lib.lbm_last_error(handle.h).decode())

    # warm-up (allocates the snapshot slots); a GPU with less free memory than
    # the slots need falls back to the FP64 comparison's count
    nsnap_fp32 = NSNAP
    try:
        one_gradient(h, nsnap_fp32)
    except G.LBMError as e:
        if e.code != G.ERR_MEM:
            raise
        nsnap_fp32 = NSNAP_FP64
        one_gradient(h, nsnap_fp32)
    e2e_runs = 2
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(e2e_runs):
        one_gradient(h, nsnap_fp32)
    t1 = time.perf_counter()
    barrier(dist)
    clocks = sampler.stop()
    grad_fp32_s = (t1 - t0) / e2e_runs
    J32, s32 = float(Jbuf[0]), s_np.copy()
    grad_fp32_s = max_over_ranks(dist, grad_fp32_s)
    recomputed = int(st.recomputed_steps)
    e2e_value = total_cells * NSTEPS_GRAD / grad_fp32_s / 1e6
    # the design goes up and dJ/dgamma (plus J) comes down once per gradient
    # of NSTEPS_GRAD time steps: per time step, a share of those copies
    h2d_grad, d2h_grad = cells * 8, cells * 8 + 8
    e2e = {"value": round(e2e_value, 2), "unit": "MLUPS",
           "h2d_bytes_per_step": round(h2d_grad / NSTEPS_GRAD, 1),
           "d2h_bytes_per_step": round(d2h_grad / NSTEPS_GRAD, 1),
           "h2d_bytes_per_gradient": h2d_grad, "d2h_bytes_per_gradient": d2h_grad,
           "what": "lbm_set_design (host FP64 design) + lbm_gradient (5000 forward steps, "
                   "%d recomputed by Wang checkpointing in %d device slots (%.0f GB), 5000 adjoint "
                   "steps) + dJ/dgamma to host; one design upload and one sensitivity download "
                   "per gradient, i.e. per 5000 time steps" % (recomputed, nsnap_fp32,
                                                              nsnap_fp32 * cells * 19 * 4 / 1e9),
           "gradient_s": round(grad_fp32_s, 4),
           "forward_sweep_ms": round(float(st.forward_ms), 2),
           "reverse_sweep_ms": round(float(st.reverse_ms), 2)}
    # the FP32 gradient with the FP64 comparison's slot count: the speed-up
    # of FP32 storage at equal recomputation (the first call re-sizes the slots)
    one_gradient(h, NSNAP_FP64)
    t0 = time.perf_counter()
    one_gradient(h, NSNAP_FP64)
    grad_fp32_same_slots_s = time.perf_counter() - t0
    h.close()

    # FP64 storage: same gradient, for the FP32-vs-FP64 comparison
    h64 = G.Handle(cfg.replace(storage=G.STORE_FP64))
    h64.set_design(gamma)
    h64.init_equilibrium()
    h64.autotune(2)
    one_gradient(h64, NSNAP_FP64)
    t0 = time.perf_counter()
    one_gradient(h64, NSNAP_FP64)
    grad_fp64_s = time.perf_counter() - t0
    J64, s64 = float(Jbuf[0]), s_np.copy()
    grad_err = {"J_rel": abs(J32 - J64) / abs(J64),
                "dJdgamma_rel_l2": float(np.linalg.norm(s32 - s64) / np.linalg.norm(s64)),
                "dJdgamma_max_rel": float(np.abs(s32 - s64).max() / np.abs(s64).max())}
    h64.set_design(gamma)
    h64.init_equilibrium()
    ms64 = h64.time_steps(2, max(10, args.steps // 4))
    mlups64 = cells * max(10, args.steps // 4) / (ms64 * 1e-3) / 1e6
    h64.close()
    errs = precision_errors(G, W)

    cpu = cpu_baseline_leg() if rank == 0 else None
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_pairs / args.steps, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded SplitMix64 design, 3x3x3-smoothed, thresholded at 0.5, "
                "2-cell blend",
        "config": {"workload": CONFIG_NAME, "cells": cells,
                   "step": "one forward + one adjoint time step over the lattice",
                   "l2": "inputs larger than L2 (FP32 state 319 MB > 129 MB L2); no flush",
                   "parallelism": "replicas (one independent duct per GPU)",
                   "block_shapes": {"forward": list(shapes[0]), "adjoint": list(shapes[1])}},
        "mlups_fwd": round(cells * args.steps / (ms_fwd * 1e-3) / 1e6, 2),
        "mlups_adj": round(cells * args.steps / (ms_adj * 1e-3) / 1e6, 2),
        "roofline": {"bound": "hbm", "kernel": "k_adjoint<D3Q19,MRT,float>",
                     "achieved": round(ach_adj, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(ach_adj / peak, 4), "peak_kind": peak_kind,
                     "bytes_per_lu": bytes_per_lu(G.STORE_FP32, "adj"),
                     "traffic": traffic,
                     "forward": {"kernel": "k_forward<D3Q19,MRT,float>",
                                 "achieved": round(ach_fwd, 1), "frac": round(ach_fwd / peak, 4),
                                 "bytes_per_lu": bytes_per_lu(G.STORE_FP32, "fwd"),
                                 "traffic": traffic_fwd}},
        "precision": {"fp32_vs_fp64_velocity_rel_l2_300_steps": errs.get("fp32"),
                      "fp16_vs_fp64_velocity_rel_l2_300_steps": errs.get("fp16"),
                      "fp64_mlups_fwd_adj": round(mlups64, 2),
                      "gradient_s_fp32": round(grad_fp32_s, 4),
                      "gradient_slots_fp32": nsnap_fp32,
                      "gradient_s_fp32_%d_slots" % NSNAP_FP64: round(grad_fp32_same_slots_s, 4),
                      "gradient_s_fp64": round(grad_fp64_s, 4),
                      "gradient_slots_fp64": NSNAP_FP64,
                      "gradient_speedup_fp32_vs_fp64": round(grad_fp64_s / grad_fp32_same_slots_s, 3),
                      "gradient_fp32_vs_fp64_full_size": grad_err},
        "e2e": e2e,
        "cpu_baseline": cpu,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
