"""The D3Q19 MRT duct at its full 256x128x128 size (4,194,304 cells), where
the CPU oracle would take hours: size-independent properties over a 200-step
horizon.

* The dynamic and the static checkpoint schedule give bit-identical FP32
  gradients (the states every reverse step sees are the same ones).
* FP32 storage against FP64 storage on the GPU (the FP64 path equals the
  oracle within 1e-12 at the sizes the oracle runs): J within 1e-6 and
  dJ/dgamma within 1e-5 (relative L2).
* A repeated gradient is bit-identical (rounding streams are keyed by cell
  and step, not by launch order).
* The FP64 gradient agrees with central differences (h = 1e-6) of the FP64
  objective at the four cells of largest sensitivity."""
import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from helpers import rel_l2

pytestmark = pytest.mark.gpu

N = 200


@pytest.fixture(scope="module")
def duct():
    cfg, gamma, _ = W.workload_duct_256x128x128(G.STORE_FP32, nsteps=N)
    return cfg, gamma


def gradient(cfg, gamma, k, schedule=G.SCHEDULE_DYNAMIC):
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        return h.gradient(N, k, schedule)


def test_full_size_schedules_and_repeat_agree_bitwise(duct):
    cfg, gamma = duct
    Jd, sd, std = gradient(cfg, gamma, 16)
    Js, ss, sts = gradient(cfg, gamma, 16, G.SCHEDULE_STATIC)
    assert std.recomputed_steps == G.wang_recompute_count(N, 16)
    assert Jd == Js
    assert np.array_equal(sd, ss)
    Jr, sr, _ = gradient(cfg, gamma, 16)
    assert Jr == Jd
    assert np.array_equal(sr, sd)


def test_full_size_fp32_against_fp64(duct):
    cfg, gamma = duct
    J32, s32, _ = gradient(cfg, gamma, 16)
    J64, s64, _ = gradient(cfg.replace(storage=G.STORE_FP64), gamma, 16)
    assert abs(J32 - J64) <= 1e-6 * abs(J64)
    e = rel_l2(s32, s64)
    print("full-size 200-step FP32 vs FP64: J %.3e, dJ/dgamma %.3e" % (abs(J32 - J64) / abs(J64), e))
    assert e < 1e-5


def test_full_size_fp64_gradient_matches_central_differences(duct):
    cfg, gamma = duct
    cfg = cfg.replace(storage=G.STORE_FP64)
    J, sens, _ = gradient(cfg, gamma, 16)
    cells = np.argsort(-np.abs(sens))[:4]
    h = 1e-6
    with G.Handle(cfg) as hd:
        for c in cells:
            vals = []
            for sg in (1, -1):
                g = gamma.copy()
                g[c] = min(1.0, max(0.0, g[c] + sg * h))
                hd.set_design(g)
                hd.init_equilibrium()
                vals.append((hd.forward(N), g[c]))
            fd = (vals[0][0] - vals[1][0]) / (vals[0][1] - vals[1][1])
            print("cell %d: adjoint %.6e, central difference %.6e" % (c, sens[c], fd))
            assert abs(fd - sens[c]) <= 1e-4 * abs(sens[c])
