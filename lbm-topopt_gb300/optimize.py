"""Topology optimisation of a channel on one GPU: the loop of the reference's
robust pump application (applications/RobustPump2d/robustPump2d.cc:215-315)
with every vector on the device.

    python lbm-topopt_gb300/optimize.py [--robust] [--nx 256 --ny 128 --steps 2000 --iters 100]

Per iteration: the design variables on the design box pass the filter chain
(double projection for --robust, whose realisations differ in the second
eta, 0.3 / 0.5 / 0.7; one projection otherwise) into each realisation's
lattice, one batched checkpointed gradient (static schedule, CUDA graph)
gives J_r and dJ_r/dgamma, the chain rule takes them to the design
variables, and MMA takes one step: minimise J (plain) or max_r J_r (robust,
the reference's min-max form) under a fluid-volume constraint.  The
projection sharpness rises by 1.5x every 50 iterations up to iteration 500
(increaseBeta), and the loop stops when the design changes by less than
1e-4.  Designs are written as PETSc binary Vec files and the fields of
realisation 0 as .vts every --every iterations.

Under torchrun (several ranks, one GPU each) the realisations are split over
the ranks as MPISplit splits them over communicators (robustPump2d.cc:140-146):
rank k computes the gradients of realisations r = k, k + N, ...; one sum over
the ranks assembles every (J_r, dJ_r/dgamma) on every rank, and every rank
takes the same (deterministic) MMA step, so the designs stay identical.

    torchrun --nproc-per-node 3 --master-addr 127.0.0.1 lbm-topopt_gb300/optimize.py --robust
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import lbmgpu as G  # noqa: E402
import workloads as W  # noqa: E402


def make_problem(nx, ny, nsteps, robust, storage):
    cfg = W.channel_2d(nx, ny, nsteps=nsteps, storage=storage)
    cl = max(2, nx // 16)          # inlet and outlet channel lengths
    box = (cl, nx - 1 - cl, 1, ny - 2, 0, 0)
    if robust:
        stages = [(max(2, nx // 64), True, 2.0, 0.5), (max(1, nx // 128), True, 1.0, 0.5)]
        etas = [0.3, 0.5, 0.7]
    else:
        stages = [(max(2, nx // 64), True, 1.0, 0.5)]
        etas = [0.5]
    return cfg, box, stages, etas


def owned_realisations(nreal, rank, world):
    """The realisations rank `rank` of `world` computes: r = rank, rank + world, ..."""
    return [r for r in range(nreal) if r % world == rank]


def exchange_realisations(nreal, ncells, local, group=None):
    """(J_r, dJ_r/dgamma) of every realisation on every rank.  `local` maps this
    rank's realisations to theirs; each rank fills its own rows of a zero
    (nreal, 1 + ncells) FP64 block and one sum over the ranks assembles the
    block (every row has a single nonzero contributor, so the sum is exact)."""
    import torch
    import torch.distributed as td
    buf = torch.zeros(nreal, ncells + 1, dtype=torch.float64)
    for r, (J, s) in local.items():
        buf[r, 0] = float(J)
        buf[r, 1:] = torch.from_numpy(np.ascontiguousarray(s, dtype=np.float64))
    td.all_reduce(buf, op=td.ReduceOp.SUM, group=group)
    return [(float(buf[r, 0]), buf[r, 1:].numpy().copy()) for r in range(nreal)]


def optimise(nx=256, ny=128, nsteps=2000, iters=100, robust=False, volume=0.6, nsnap=10,
             storage=G.STORE_FP32, out_dir=None, every=50, tol=1e-4, log=print,
             rank=0, world=1, group=None):
    cfg, box, stages, etas = make_problem(nx, ny, nsteps, robust, storage)
    nreal = len(etas)
    nb = (box[1] - box[0] + 1) * (box[3] - box[2] + 1)
    mine = owned_realisations(nreal, rank, world)
    if not mine:
        raise ValueError("rank %d of %d has no realisation (%d realisations)" % (rank, world, nreal))
    history = []
    with G.TopOpt(nx, ny, 1, box, stages, nreal=nreal, real_eta=etas if robust else None,
                  volume_type=G.VOLUME_FLUID, volume=volume, move_limit=0.1,
                  x0=np.full(nb, volume)) as t, G.Batch([cfg] * len(mine)) as b:
        beta = stages[-1][2]
        for it in range(iters):
            t0 = time.perf_counter()
            for i, r in enumerate(mine):
                t.apply(r, b[i])
            J, sens, _ = b.gradient(nsteps, nsnap, use_graph=True, schedule=G.SCHEDULE_STATIC)
            if world == 1:
                for r in range(nreal):
                    t.set_sensitivity(r, b[r], J[r])
            else:
                every_r = exchange_realisations(nreal, cfg.ncells,
                                                {r: (J[i], sens[i]) for i, r in enumerate(mine)},
                                                group)
                J = [Jr for Jr, _ in every_r]
                for r, (Jr, sr) in enumerate(every_r):
                    t.set_sensitivity_host(r, sr, Jr)
            ch, cons = t.update()
            dt = time.perf_counter() - t0
            rec = {"iteration": it, "J": [float(v) for v in J], "volume": float(cons[-1]),
                   "change": ch, "seconds": dt}
            history.append(rec)
            if rank == 0:
                log(json.dumps(rec))
            if rank == 0 and out_dir and (it % every == 0 or ch < tol or it == iters - 1):
                os.makedirs(out_dir, exist_ok=True)
                G.write_petsc_vec(os.path.join(out_dir, "design_iter_%d.bin" % it), t.variables())
                b[0].write_vts(os.path.join(out_dir, "fields_iter_%d.vts" % it), t.physical(mine[0]))
            if (it + 1) % 50 == 0 and it + 1 <= 500:
                beta *= 1.5
                t.set_beta(len(stages) - 1, beta)
            if ch < tol:
                break
        x = t.variables()
    return x, history


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--ny", type=int, default=128)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--iters", type=int, default=100)
    ap.add_argument("--volume", type=float, default=0.6)
    ap.add_argument("--robust", action="store_true")
    ap.add_argument("--fp64", action="store_true", help="FP64 populations (default FP32)")
    ap.add_argument("--out", default=None, help="folder for designs and .vts fields")
    ap.add_argument("--every", type=int, default=50)
    a = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    group = None
    if world > 1:
        import torch.distributed as td
        td.init_process_group("gloo")   # host-side exchange of the realisations' results
        import torch
        ndev = max(1, torch.cuda.device_count())
        # one GPU per rank; ranks beyond the GPU count share them (their
        # kernels never wait on one another)
        G.select_device(int(os.environ.get("LOCAL_RANK", "0")) % ndev)
        group = td.group.WORLD
    optimise(a.nx, a.ny, a.steps, a.iters, a.robust, a.volume,
             storage=G.STORE_FP64 if a.fp64 else G.STORE_FP32, out_dir=a.out, every=a.every,
             rank=rank, world=world, group=group)
    if world > 1:
        td.destroy_process_group()


if __name__ == "__main__":
    main()
