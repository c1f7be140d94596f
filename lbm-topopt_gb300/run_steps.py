"""Run forward and reverse time steps of one of the five workloads on the GPU.

    python lbm-topopt_gb300/run_steps.py --workload 3 --storage fp32 --fwd 20 --adj 20

Prints the device time per step (CUDA events on the library's stream) and the
MLUPS.  Small enough to run under a profiler: it launches only the forward
and reverse step kernels (plus one initialisation and one design upload).
"""
import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import lbmgpu as G  # noqa: E402
import workloads as W  # noqa: E402

STORAGE = {"fp64": G.STORE_FP64, "fp32": G.STORE_FP32, "fp16": G.STORE_FP16}


def build_workload(which: int, storage: int, size=None):
    kw = {}
    if size:
        kw = dict(nx=size[0], ny=size[1])
        if which == 3:
            if len(size) != 3:
                raise ValueError("workload 3 takes --size nx ny nz")
            kw["nz"] = size[2]
        elif len(size) != 2:
            raise ValueError("2D workloads take --size nx ny")
    if which == 1:
        if size:
            raise ValueError("workload 1 has a fixed size")
        cfg, g, n = W.workload_config1(storage)
    elif which == 2:
        cfg, g, n = W.workload_config2(storage, **kw)
    elif which == 3:
        cfg, g, n = W.workload_config3(storage, **kw)
    elif which == 4:
        cfg, g, n = W.workload_config4(storage, **kw)
    else:
        raise ValueError("workload must be 1-4")
    return cfg, g, n


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--workload", type=int, default=3)
    ap.add_argument("--storage", choices=sorted(STORAGE), default="fp32")
    ap.add_argument("--size", type=int, nargs="+", default=None,
                    help="nx ny nz (workload 3) or nx ny (workloads 2 and 4)")
    ap.add_argument("--fwd", type=int, default=10)
    ap.add_argument("--adj", type=int, default=10)
    ap.add_argument("--autotune", action="store_true", help="pick block shapes first")
    ap.add_argument("--shape", type=int, nargs=4, default=None, metavar=("FBX", "FBY", "ABX", "ABY"),
                    help="fixed block shapes of the forward and reverse steps (reproducible "
                         "profiles: the autotuner's choice can change under a profiler)")
    a = ap.parse_args()
    cfg, gamma, _ = build_workload(a.workload, STORAGE[a.storage], a.size)
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        if a.shape:
            h.set_launch_shape(0, a.shape[0], a.shape[1])
            h.set_launch_shape(1, a.shape[2], a.shape[3])
        elif a.autotune:
            print("block shapes (forward, reverse):", h.autotune())
        ms_f = h.time_steps(0, a.fwd) if a.fwd > 0 else 0.0
        ms_a = h.time_steps(1, a.adj) if a.adj > 0 else 0.0
        n = cfg.ncells
        if a.fwd:
            print("forward: %.4f ms/step, %.1f MLUPS" % (ms_f / a.fwd, n * a.fwd / ms_f / 1e3))
        if a.adj:
            print("adjoint: %.4f ms/step, %.1f MLUPS" % (ms_a / a.adj, n * a.adj / ms_a / 1e3))
        print("kernel launches: %d" % h.launch_count())


if __name__ == "__main__":
    main()
