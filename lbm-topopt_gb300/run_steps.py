"""Run forward and reverse time steps of one of the workloads on the GPU.

    python lbm-topopt_gb300/run_steps.py --workload duct --storage fp32 --fwd 20 --adj 20

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

WORKLOADS = ("channel", "unsteady_channel", "duct", "thermal", "batch")
STORAGE = {"fp64": G.STORE_FP64, "fp32": G.STORE_FP32, "fp16": G.STORE_FP16}


def build_workload(which: str, storage: int, size=None):
    kw = {}
    if size:
        if which == "channel":
            raise ValueError("the 128x64 channel has a fixed size")
        kw = dict(nx=size[0], ny=size[1])
        if which == "duct":
            if len(size) != 3:
                raise ValueError("the duct takes --size nx ny nz")
            kw["nz"] = size[2]
        elif len(size) != 2:
            raise ValueError("2D workloads take --size nx ny")
    if which == "channel":
        return W.workload_channel_128x64(storage)
    if which == "unsteady_channel":
        return W.workload_unsteady_channel_1024x512(storage, **kw)
    if which == "duct":
        return W.workload_duct_256x128x128(storage, **kw)
    if which == "thermal":
        return W.workload_thermal_512x256(storage, **kw)
    raise ValueError("unknown workload %r" % (which,))


def run_batch(a):
    """The 8-channel batch: one launch per step for all eight lattices."""
    if a.size:
        raise ValueError("the 8-channel batch has fixed sizes")
    insts, _ = W.workload_batch_8_channels(STORAGE[a.storage])
    n = sum(c.ncells for c, _ in insts)
    with G.Batch([c for c, _ in insts]) as b:
        for i, (_, g) in enumerate(insts):
            b[i].set_design(g)
            b[i].init_equilibrium()
        if a.shape:
            b.set_launch_shape(0, a.shape[0], a.shape[1])
            b.set_launch_shape(1, a.shape[2], a.shape[3])
        elif a.autotune:
            print("block shapes (forward, reverse):", b.autotune(), b.reverse_shape())
            for i, (_, g) in enumerate(insts):
                b[i].init_equilibrium()
        ms_f = b.time_steps(0, a.fwd) if a.fwd > 0 else 0.0
        ms_a = b.time_steps(1, a.adj) if a.adj > 0 else 0.0
        if a.fwd:
            print("forward: %.4f ms/step, %.1f MLUPS" % (ms_f / a.fwd, n * a.fwd / ms_f / 1e3))
        if a.adj:
            print("adjoint: %.4f ms/step, %.1f MLUPS" % (ms_a / a.adj, n * a.adj / ms_a / 1e3))
        print("kernel launches: %d" % b.launch_count())


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--workload", choices=WORKLOADS, default="duct",
                    help="channel: 128x64 D2Q9 BGK; unsteady_channel: 1024x512 D2Q9 BGK with "
                         "pulsed inlet; duct: 256x128x128 D3Q19 MRT; thermal: 512x256 D2Q9 + D2Q5; "
                         "batch: 8 D2Q9 channels (3 of 1024x512, 256x128 .. 768x384)")
    ap.add_argument("--storage", choices=sorted(STORAGE), default="fp32")
    ap.add_argument("--size", type=int, nargs="+", default=None,
                    help="nx ny nz (duct) or nx ny (unsteady_channel, thermal)")
    ap.add_argument("--fwd", type=int, default=10)
    ap.add_argument("--adj", type=int, default=10)
    ap.add_argument("--autotune", action="store_true", help="pick block shapes first")
    ap.add_argument("--shape", type=int, nargs=4, default=None, metavar=("FBX", "FBY", "ABX", "ABY"),
                    help="fixed block shapes of the forward and reverse steps (reproducible "
                         "profiles: the autotuner's choice can change under a profiler)")
    a = ap.parse_args()
    if a.workload == "batch":
        return run_batch(a)
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
