"""The unsteady channel, the thermal channel and the 8-lattice batch at their
stated sizes on the GPU.

* 1024x512 D2Q9 channel, unsteady inlet u(t) = 0.05 (1 + 0.2 sin(2 pi t/2000)),
  dissipated-energy objective averaged over 20,000 steps:
  - FP64 against the oracle over the first 100 steps (populations, per-step
    objective and dJ/dgamma within 1e-12);
  - FP32 storage against FP64 over the full 20,000-step gradient with 64
    device snapshots (J and dJ/dgamma within 1e-4);
  - the FP64 gradient against central differences (h = 1e-6) of the FP64
    objective at 16 seeded cells, on the full 20,000-step horizon (the
    reference's own check, topOpt/finiteDifferenceCheck2d.cc:58-113, with
    central instead of one-sided differences).
* 512x256 D2Q9 + D2Q5 thermal channel, 10,000 steps, heat flux:
  - FP64 against the oracle over 100 steps (1e-12) from a flowing start
    with the obstacle hot, the heat flux measured on a column just downstream
    of it (from rest, neither flow nor heat reaches any column within 100
    steps);
  - FP32 against FP64 over the full 10,000-step gradient (1e-4).
* The batch of 3 projected 1024x512 designs and 5 uneven channels:
  - every lattice of the FP64 batch against the oracle over 50 steps (1e-12);
  - the FP32 batch (one launch per step, CUDA graph) against the same lattices
    one at a time over the full 4,000-step gradient.
Each test runs in a few minutes at most."""
import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from helpers import rel_inf, rel_l2

pytestmark = pytest.mark.gpu

SHORT = 100


def gpu_forward_and_gradient(cfg, gamma, n, k, macros=None):
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium(macros)
        J, js = h.forward(n, per_step=True)
        f = h.populations()
        Jg, sens, _ = h.gradient(n, k)
    return f, js, J, Jg, sens


def check_against_oracle(orc, cfg, gamma, n, k, macros=None):
    f, js, J, Jg, sens = gpu_forward_and_gradient(cfg, gamma, n, k, macros)
    fo, jso, Jo = orc.forward(cfg, gamma, n, macros)
    Jgo, so = orc.gradient(cfg, gamma, n, macros)
    assert Jgo != 0.0 and np.abs(so).max() > 0.0   # the comparison sees a nonzero objective
    print("%dx%d, %d steps: populations %.2e, J_steps %.2e, J %.2e, dJ/dgamma %.2e" % (
        cfg.nx, cfg.ny, n, rel_inf(f, fo), rel_inf(js, jso), abs(Jg - Jgo) / abs(Jgo),
        rel_inf(sens, so)))
    assert rel_inf(f, fo) < 1e-12
    assert rel_inf(js, jso) < 1e-12
    assert abs(J - Jo) <= 1e-12 * abs(Jo)
    assert abs(Jg - Jgo) <= 1e-12 * abs(Jgo)
    assert rel_inf(sens, so) < 1e-12


# -- unsteady channel 1024x512 -------------------------------------------------------

@pytest.fixture(scope="module")
def unsteady():
    cfg, gamma, n = W.workload_unsteady_channel_1024x512()
    assert (cfg.nx, cfg.ny, n) == (1024, 512, 20000)
    return cfg, gamma, n


def test_unsteady_channel_fp64_matches_oracle_at_full_size(orc, unsteady):
    cfg, gamma, _ = unsteady
    check_against_oracle(orc, cfg, gamma, SHORT, 8)


@pytest.fixture(scope="module")
def unsteady_fp64_gradient(unsteady):
    cfg, gamma, n = unsteady
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        J, sens, st = h.gradient(n, 64)
    assert st.recomputed_steps == G.wang_recompute_count(n, 64) == 38813
    return J, sens


def test_unsteady_channel_fp32_against_fp64_full_gradient(unsteady, unsteady_fp64_gradient):
    cfg, gamma, n = unsteady
    J64, s64 = unsteady_fp64_gradient
    with G.Handle(cfg.replace(storage=G.STORE_FP32)) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        J32, s32, _ = h.gradient(n, 64)
    eJ, es = abs(J32 - J64) / abs(J64), rel_l2(s32, s64)
    print("1024x512, 20000 steps, 64 snapshots: FP32 vs FP64 J %.2e, dJ/dgamma %.2e" % (eJ, es))
    assert eJ < 1e-4
    assert es < 1e-4


def test_unsteady_channel_gradient_matches_central_differences(unsteady,
                                                               unsteady_fp64_gradient):
    cfg, gamma, n = unsteady
    _, sens = unsteady_fp64_gradient
    rng = np.random.default_rng(20261203 + 2)
    cells = rng.choice(np.flatnonzero((gamma > 1e-5) & (gamma < 1 - 1e-5)), 16, replace=False)
    h = 1e-6
    scale = np.abs(sens).max()
    worst = 0.0
    with G.Handle(cfg) as hd:
        for c in cells:
            vals = []
            for sg in (1.0, -1.0):
                g = gamma.copy()
                g[c] += sg * h
                hd.set_design(g)
                hd.init_equilibrium()
                vals.append(hd.forward(n))
            fd = (vals[0] - vals[1]) / (2 * h)
            worst = max(worst, abs(fd - sens[c]) / scale)
            print("cell %d: adjoint %.8e, central difference %.8e" % (c, sens[c], fd))
    print("worst |fd - adjoint| / max|dJ/dgamma| = %.2e" % worst)
    assert worst < 1e-5


# -- thermal channel 512x256 ---------------------------------------------------------

@pytest.fixture(scope="module")
def thermal():
    cfg, gamma, n = W.workload_thermal_512x256()
    assert (cfg.nx, cfg.ny, n) == (512, 256, 10000)
    return cfg, gamma, n


def test_thermal_fp64_matches_oracle_at_full_size(orc, thermal):
    cfg, gamma, _ = thermal
    # From rest with a cold inlet no heat leaves the obstacle's neighbourhood
    # and no flow reaches it within 100 steps: start instead from the inlet
    # velocity everywhere and the solid already hot (T = 1 - gamma), and
    # measure the heat flux on a column just downstream of the heated disc
    # (x = 144..220 for this seed).
    solid_x = np.flatnonzero((gamma.reshape(cfg.ny, cfg.nx) < 1.0).any(axis=0))
    col = int(solid_x.max()) + 3
    macros = np.zeros((cfg.ncells, 4))
    macros[:, 0] = 1.0
    macros[:, 1] = 0.03 * gamma
    macros[:, 3] = 1.0 - gamma
    check_against_oracle(orc, cfg.replace(obj_out=(col, col, 1, cfg.ny - 2, 0, 0)), gamma, SHORT, 8,
                         macros.ravel())


def test_thermal_fp32_against_fp64_full_gradient(thermal):
    cfg, gamma, n = thermal
    out = {}
    for st in (G.STORE_FP64, G.STORE_FP32):
        with G.Handle(cfg.replace(storage=st)) as h:
            h.set_design(gamma)
            h.init_equilibrium()
            out[st] = h.gradient(n, 64)[:2]
    (J64, s64), (J32, s32) = out[G.STORE_FP64], out[G.STORE_FP32]
    eJ, es = abs(J32 - J64) / abs(J64), rel_l2(s32, s64)
    print("thermal 512x256, 10000 steps: FP32 vs FP64 J %.2e, dJ/dgamma %.2e" % (eJ, es))
    assert eJ < 1e-4
    assert es < 1e-4


# -- the 8-lattice batch -------------------------------------------------------------

def test_batch_fp64_every_lattice_matches_oracle(orc):
    insts, _ = W.workload_batch_8_channels(G.STORE_FP64)
    n = 50
    with G.Batch([c for c, _ in insts]) as b:
        for i, (_, g) in enumerate(insts):
            b[i].set_design(g)
        J, sens, _ = b.gradient(n, 8, use_graph=True)
    for i, (cfg, g) in enumerate(insts):
        Jo, so = orc.gradient(cfg, g, n)
        print("lattice %d (%dx%d): J %.2e, dJ/dgamma %.2e" % (
            i, cfg.nx, cfg.ny, abs(J[i] - Jo) / abs(Jo), rel_inf(sens[i], so)))
        assert abs(J[i] - Jo) <= 1e-12 * abs(Jo)
        assert rel_inf(sens[i], so) < 1e-12


def test_batch_fp32_full_gradient_equals_one_at_a_time():
    insts, n = W.workload_batch_8_channels(G.STORE_FP32)
    assert n == 4000 and sum(c.ncells for c, _ in insts) == 2310144
    with G.Batch([c for c, _ in insts]) as b:
        for i, (_, g) in enumerate(insts):
            b[i].set_design(g)
        J, sens, st = b.gradient(n, 64, use_graph=True)
    assert st.recomputed_steps == G.wang_recompute_count(n, 64)
    for i, (cfg, g) in enumerate(insts):
        with G.Handle(cfg) as h:
            h.set_design(g)
            h.init_equilibrium()
            Js, ss, _ = h.gradient(n, 64)
        eJ, es = abs(J[i] - Js) / abs(Js), rel_l2(sens[i], ss)
        print("lattice %d (%dx%d): batched vs alone J %.2e, dJ/dgamma %.2e" % (
            i, cfg.nx, cfg.ny, eJ, es))
        assert eJ < 1e-9
        assert es < 1e-6
