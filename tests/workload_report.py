"""Measurements of the six workloads on the GPU, one JSON line each, with the
oracle as the checker (test infrastructure: it lives beside the tests because
it imports the oracle; the product package does not).

    python tests/workload_report.py [--workloads channel duct ...] [--quick]

channel           128x64 D2Q9 BGK + Brinkman, FP64, 2000 steps: forward and
                  gradient time, agreement with the FP64 oracle.
unsteady_channel  1024x512 D2Q9, unsteady inlet, dissipated energy, 20000
                  steps with 64 device snapshots: gradient wall time FP64 vs
                  FP32 shifted storage, FP32 error against FP64, dJ/dgamma
                  against central differences (h = 1e-6, FP64) at 16 seeded
                  cells on a 2000-step horizon (one inlet period), and against
                  the reference adjoint (the oracle, bit-identical to the
                  reference's own operators) on a 128x64 cut-down.
duct              256x128x128 D3Q19 MRT duct: FP64 / FP32 / FP16 storage MLUPS
                  and errors (bench.py measures its FP32 headline).
thermal           512x256 D2Q9 + D2Q5 thermal, 10000 steps, FP32 with FP64
                  objective accumulation: gradient time, error against FP64.
batch             8 D2Q9 lattices (3 projected designs of 1024x512 + 5 uneven
                  ones), 4000 steps: batched gradient (one launch per step,
                  CUDA graph) against the same lattices one at a time.
robust            robust design iteration on the device: 3 realisations of the
                  1024x512 channel, double projection filter, batched
                  gradient, chain rule and one min-max MMA step, with the CPU
                  oracle's filter and MMA beside it.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "lbm-topopt_gb300"))
sys.path.insert(0, HERE)

import lbmgpu as G  # noqa: E402
import workloads as W  # noqa: E402


def _oracle():
    from oracle_lib import oracle
    return oracle()


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def timed_gradient(cfg, gamma, n, k, reps=1):
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        h.autotune(3)
        h.gradient(min(n, 20), k)   # warm-up, allocates the slots
        t0 = time.perf_counter()
        for _ in range(reps):
            J, s, st = h.gradient(n, k)
        dt = (time.perf_counter() - t0) / reps
    return J, s, st, dt


def step_rates(cfg, gamma, nsteps=50):
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        h.autotune(3)
        h.forward(10)
        mf = h.time_steps(0, nsteps)
        ma = h.time_steps(1, nsteps)
    return cfg.ncells * nsteps / mf / 1e3, cfg.ncells * nsteps / ma / 1e3


def report_channel(quick):
    cfg, g, n = W.workload_channel_128x64()
    orc = _oracle()
    with G.Handle(cfg) as h:
        h.set_design(g)
        h.init_equilibrium()
        t0 = time.perf_counter()
        J = h.forward(n)
        tf = time.perf_counter() - t0
        f = h.populations()
    fo, _, Jo = orc.forward(cfg, g, n)
    Jg, s, st, tg = timed_gradient(cfg, g, n, 64)
    return {"workload_name": "channel", "workload": "128x64 D2Q9 BGK + Brinkman, FP64, 2000 steps",
            "forward_s": tf, "gradient_s_64_snapshots": tg, "recomputed": st.recomputed_steps,
            "J": J, "J_rel_err_vs_oracle": abs(J - Jo) / abs(Jo),
            "populations_max_rel_err_vs_oracle": float(np.abs(f - fo).max() / np.abs(fo).max())}


def report_unsteady_channel(quick):
    n = 2000 if quick else 20000
    cfg64, g, _ = W.workload_unsteady_channel_1024x512(G.STORE_FP64, nsteps=n)
    cfg32 = cfg64.replace(storage=G.STORE_FP32)
    J64, s64, st, t64 = timed_gradient(cfg64, g, n, 64)
    J32, s32, _, t32 = timed_gradient(cfg32, g, n, 64)
    out = {"workload_name": "unsteady_channel", "workload": "1024x512 D2Q9 BGK + Brinkman, unsteady inlet, dissipated "
                                    "energy, %d steps, 64 device snapshots" % n,
           "recomputed": st.recomputed_steps, "gradient_s_fp64": t64, "gradient_s_fp32": t32,
           "speedup_fp32": t64 / t32, "J_fp64": J64, "J_fp32_rel_err": abs(J32 - J64) / abs(J64),
           "dJdgamma_fp32_rel_l2_err": rel(s32, s64)}
    mf, ma = step_rates(cfg32, g)
    out.update(mlups_fwd_fp32=mf, mlups_adj_fp32=ma)
    # central differences, FP64, one inlet period
    nfd = 2000
    cfd = cfg64.replace(obj_weight=1.0 / nfd)
    _, sfd, _, _ = timed_gradient(cfd, g, nfd, 64)
    rng = np.random.default_rng(W.SEED_BASE + 22)
    cells = rng.choice(cfg64.ncells, size=4 if quick else 16, replace=False)
    h_fd = 1e-6
    worst = 0.0
    with G.Handle(cfd) as h:
        for c in cells:
            vals = []
            for sgn in (1.0, -1.0):
                gg = g.copy()
                gg[c] = min(max(gg[c] + sgn * h_fd, 0.0), 1.0)
                h.set_design(gg)
                h.init_equilibrium()
                vals.append((h.forward(nfd), gg[c]))
            fd = (vals[0][0] - vals[1][0]) / (vals[0][1] - vals[1][1])
            worst = max(worst, abs(fd - sfd[c]) / np.abs(sfd).max())
    out.update(fd_cells=int(len(cells)), fd_steps=nfd, fd_h=h_fd, fd_max_err_rel_to_max_sens=worst)
    # reference adjoint on the 128x64 cut-down
    orc = _oracle()
    ccut, gcut, _ = W.workload_unsteady_channel_1024x512(G.STORE_FP64, nx=128, ny=64, nsteps=2000)
    Jc, sc, _, _ = timed_gradient(ccut, gcut, 2000, 64)
    Jo, so = orc.gradient(ccut, gcut, 2000)
    out.update(cutdown_J_rel_err=abs(Jc - Jo) / abs(Jo),
               cutdown_dJdgamma_max_rel_err=float(np.abs(sc - so).max() / np.abs(so).max()))
    return out


def report_duct(quick):
    out = {"workload_name": "duct", "workload": "256x128x128 D3Q19 MRT + Brinkman duct"}
    for name, st in (("fp64", G.STORE_FP64), ("fp32", G.STORE_FP32), ("fp16", G.STORE_FP16)):
        cfg, g, _ = W.workload_duct_256x128x128(st)
        mf, ma = step_rates(cfg, g, 10 if st == G.STORE_FP64 else 50)
        out["mlups_fwd_" + name] = mf
        out["mlups_adj_" + name] = ma
    cfg, g, _ = W.workload_duct_256x128x128(G.STORE_FP64, nx=64, ny=32, nz=32, nsteps=300)
    J64, s64, _, _ = timed_gradient(cfg, g, 300, 32)
    for name, st in (("fp32", G.STORE_FP32), ("fp16", G.STORE_FP16)):
        J, s, _, _ = timed_gradient(cfg.replace(storage=st), g, 300, 32)
        out["dJdgamma_rel_l2_err_%s_64x32x32_300_steps" % name] = rel(s, s64)
        out["J_rel_err_%s" % name] = abs(J - J64) / abs(J64)
    return out


def report_thermal(quick):
    n = 2000 if quick else 10000
    cfg64, g, _ = W.workload_thermal_512x256(G.STORE_FP64, nsteps=n)
    cfg32 = cfg64.replace(storage=G.STORE_FP32)
    J64, s64, st, t64 = timed_gradient(cfg64, g, n, 64)
    J32, s32, _, t32 = timed_gradient(cfg32, g, n, 64)
    mf, ma = step_rates(cfg32, g)
    return {"workload_name": "thermal", "workload": "512x256 D2Q9 + D2Q5 thermal, heat flux, %d steps" % n,
            "gradient_s_fp64": t64, "gradient_s_fp32": t32, "recomputed": st.recomputed_steps,
            "J_fp64": J64, "J_fp32_rel_err": abs(J32 - J64) / abs(J64),
            "dJdgamma_fp32_rel_l2_err": rel(s32, s64), "mlups_fwd_fp32": mf, "mlups_adj_fp32": ma}


def report_batch(quick):
    n = 400 if quick else 4000
    insts, _ = W.workload_batch_8_channels(G.STORE_FP32, nsteps=n)
    cells = sum(c.ncells for c, _ in insts)
    # one at a time
    t_single = 0.0
    Js = []
    for cfg, g in insts:
        J, s, st, dt = timed_gradient(cfg, g, n, 64)
        t_single += dt
        Js.append(J)
    with G.Batch([c for c, _ in insts]) as b:
        for i, (_, g) in enumerate(insts):
            b[i].set_design(g)
        shape = b.autotune(3)
        b.gradient(n, 64, use_graph=True)          # capture + first replay
        t0 = time.perf_counter()
        J, sens, st = b.gradient(n, 64, use_graph=True)
        t_batch = time.perf_counter() - t0
        t0 = time.perf_counter()
        b.gradient(n, 64, use_graph=False)
        t_eager = time.perf_counter() - t0
    return {"workload_name": "batch", "workload": "8 D2Q9 lattices (3 projected 1024x512 + 256x128 .. 768x384), "
                                     "FP32, %d steps, 64 snapshots each" % n,
            "cells": cells, "batch_block_shape": list(shape),
            "gradient_s_batched_graph": t_batch, "gradient_s_batched_no_graph": t_eager,
            "gradient_s_one_at_a_time": t_single,
            "aggregate_mlups_batched": cells * n / t_batch / 1e6,
            "aggregate_mlups_one_at_a_time": cells * n / t_single / 1e6,
            "max_J_rel_diff_batched_vs_single": float(max(abs(a - b) / abs(b) for a, b in zip(J, Js)))}


def report_robust(quick):
    """Robust design iteration at the batch scale: three realisations (the
    second projection's eta 0.3 / 0.5 / 0.7) of the 1024x512 channel, the
    double projection filter of RobustPump2d (radii 8 and 4), one batched
    FP32 gradient, the chain rule of each realisation and one min-max MMA step
    with a fluid-volume constraint, all on the device; the CPU oracle's filter
    chain and MMA on the same inputs for comparison."""
    import design_lib as D
    n = 400 if quick else 4000
    nx, ny = 1024, 512
    cfg = W.channel_2d(nx, ny, storage=G.STORE_FP32, nsteps=n)
    box = (32, nx - 33, 1, ny - 2, 0, 0)
    stages = [(8, True, 2.0, 0.5), (4, True, 1.0, 0.5)]
    etas = [0.3, 0.5, 0.7]
    mask = np.zeros((ny, nx), bool)
    mask[box[2]:box[3] + 1, box[0]:box[1] + 1] = True
    x0 = W.design_2d(nx, ny, W.SEED_BASE + 6).reshape(ny, nx)[mask]
    x0 = np.clip(x0, 0.0, 1.0)
    out = {"workload_name": "robust", "workload": "robust design iteration: 3 realisations of a 1024x512 D2Q9 "
                                    "channel, double projection (R 8 + 4), FP32 gradient of %d "
                                    "steps, min-max MMA with a fluid-volume constraint" % n,
           "design_variables": int(mask.sum())}
    with G.TopOpt(nx, ny, 1, box, stages, nreal=3, real_eta=etas, volume_type=G.VOLUME_FLUID,
                  volume=0.8, move_limit=0.1, x0=x0) as t, G.Batch([cfg] * 3) as b:
        times = {}

        def iteration(record):
            t0 = time.perf_counter()
            for r in range(3):
                t.apply(r, b[r])
            t1 = time.perf_counter()
            J, _, _ = b.gradient(n, 64, use_graph=True)
            t2 = time.perf_counter()
            for r in range(3):
                t.set_sensitivity(r, b[r], J[r])
            t3 = time.perf_counter()
            sens = [t.design_sensitivity(r) for r in range(3)]
            xb = t.variables()
            t4 = time.perf_counter()
            ch, cons = t.update()
            t5 = time.perf_counter()
            if record:
                times.update(apply_s=t1 - t0, gradient_s=t2 - t1, chain_rule_s=t3 - t2,
                             mma_update_s=t5 - t4, iteration_s=(t3 - t0) + (t5 - t4))
            return J, sens, xb, cons, ch

        J, sens, xb, cons, ch = iteration(False)          # graph capture on the first pass
        xa = t.variables()
        # the same first update on the CPU oracle
        a_const = np.array([1., 1., 1., 0.])
        # realisation 0's chain (the volume is measured on it): last eta = etas[0]
        st0 = [(r_, box, p_, b_, e_) for r_, p_, b_, e_ in stages]
        st0[-1] = st0[-1][:4] + (etas[0],)
        ch_o = D.make_chain(nx, ny, 1, st0)
        tc0 = time.perf_counter()
        xfull = np.ones(nx * ny)
        xfull[mask.reshape(-1)] = xb
        D.filter_forward(ch_o, xfull)
        tc1 = time.perf_counter()
        dvol = np.full(nx * ny, 1.0 / mask.sum())
        dvol_x = D.filter_transpose(ch_o, xfull, dvol)[mask.reshape(-1)]
        tc2 = time.perf_counter()
        orc = D.OracleMMA(len(xb), 4, xb, a_const)
        dg = np.vstack(sens + [dvol_x])
        x_o, _, _ = orc.update(xb, np.zeros(len(xb)), cons, dg, 0.1)
        tc3 = time.perf_counter()
        out.update(J=[float(v) for v in J], constraints=[float(v) for v in cons],
                   first_change=ch, mma_gpu_vs_oracle_max_abs=float(np.abs(xa - x_o).max()),
                   cpu_filter_forward_s=tc1 - tc0, cpu_filter_transpose_s=tc2 - tc1,
                   cpu_mma_update_s=tc3 - tc2)
        iteration(True)
        out.update(times)
    return out


REPORTS = {"channel": report_channel, "unsteady_channel": report_unsteady_channel,
           "duct": report_duct, "thermal": report_thermal, "batch": report_batch,
           "robust": report_robust}


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--workloads", nargs="*", choices=list(REPORTS), default=list(REPORTS))
    ap.add_argument("--quick", action="store_true", help="shorter horizons")
    a = ap.parse_args()
    for c in a.workloads:
        t0 = time.perf_counter()
        r = REPORTS[c](a.quick)
        r["wall_s"] = time.perf_counter() - t0
        print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()
