"""The oracle (C restatement of the reference hot path) against the golden
vectors produced by the reference's own compiled operators, the reference's
checkpoint-schedule known answers, the operators' conservation identities and
central finite differences.  CPU only."""
import os

import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from helpers import rel_inf
from oracle_lib import reference

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


_MG = golden_module()
CASES = _MG.cases()
TABLES = _MG.TABLES              # boundary tables of a case ({slot: table})
FORWARD_ONLY = _MG.FORWARD_ONLY  # cases without a reference adjoint


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_reference_golden(orc, name):
    cfg, gamma, n = CASES[name]
    g = np.load(os.path.join(GOLD, name + ".npz"))
    assert np.array_equal(g["gamma"], gamma)           # seeded inputs are reproducible
    orc.set_tables(TABLES.get(name))
    try:
        f, js, J = orc.forward(cfg, gamma, n)
        assert rel_inf(f, g["f"]) < 1e-13
        assert rel_inf(js, g["J_steps"]) < 1e-13
        if name not in FORWARD_ONLY:
            Jg, sens = orc.gradient(cfg, gamma, n)
            assert abs(Jg - g["J_grad"]) <= 1e-13 * abs(g["J_grad"])
            assert rel_inf(sens, g["sens"]) < 1e-13
    finally:
        orc.set_tables(None)
    for k in range(len(g["cell_gamma"])):
        fo, mac = orc.collide_cell(cfg, g["cell_fin"][k], g["cell_gamma"][k])
        assert rel_inf(fo, g["cell_fout"][k]) < 1e-15
        assert rel_inf(mac, g["cell_mac"][k]) < 1e-15
        li, dg = orc.reverse_cell(cfg, g["cell_fin"][k], g["cell_gamma"][k], g["cell_lam_out"][k])
        assert rel_inf(li, g["cell_lam_in"][k]) < 1e-14
        assert abs(dg - g["cell_dgamma"][k]) <= 1e-14 * max(abs(g["cell_dgamma"][k]), 1e-3)


def test_wang_schedule_known_answers(orc):
    table = np.loadtxt(os.path.join(GOLD, "wang_schedule.txt"), dtype=np.int64)
    for N, K, rec, ok in table:
        r, good = orc.wang_count(int(N), int(K))
        assert (r, int(good)) == (rec, ok), (N, K)
    # the headline schedule: 20000 steps in 64 slots
    assert orc.wang_count(20000, 64) == (38813, True)


def test_wang_schedule_of_the_library_host_code(lib):
    """The library's C++ schedule (no GPU involved) gives the same counts."""
    table = np.loadtxt(os.path.join(GOLD, "wang_schedule.txt"), dtype=np.int64)
    for N, K, rec, ok in table:
        assert G.wang_recompute_count(int(N), int(K)) == rec, (N, K)


def test_static_schedule_known_answers(orc, lib):
    """StaticCheckpointing(K, N + 1): the oracle's restatement and the library's
    host schedule against the table made by the reference's own
    staticCheckpointing.cc (recomputed steps, exact reversal, states kept)."""
    table = np.loadtxt(os.path.join(GOLD, "static_schedule.txt"), dtype=np.int64)
    assert len(table) >= 70
    for N, K, rec, ok, saved in table:
        assert ok == 1
        assert orc.static_count(int(N), int(K)) == (rec, True, saved), (N, K)
        assert G.schedule_count(int(N), int(K), G.SCHEDULE_STATIC) == (rec, saved), (N, K)
    ref = reference()
    if ref is not None:   # where the reference tree exists: a wider sweep
        for N in (5, 33, 257, 3000):
            for K in (2, 5, 9, 40):
                assert orc.static_count(N, K) == ref.static_count(N, K), (N, K)


def test_oracle_matches_reference_build_on_fresh_inputs(orc):
    ref = reference()
    if ref is None:
        pytest.skip("reference operators not built here (no reference tree)")
    cfg = W.channel_2d(20, 10, amp=0.3, period=17.0, nsteps=40)
    g = W.design_2d(20, 10, 4242)
    fo, jo, Jo = orc.forward(cfg, g, 40)
    fr, jr, Jr = ref.forward(cfg, g, 40)
    assert np.array_equal(fo, fr)
    cfg3 = W.duct_3d(10, 6, 6, nsteps=20)
    g3 = W.design_3d(10, 6, 6, 4243)
    Jo, so = orc.gradient(cfg3, g3, 20)
    Jr, sr = ref.gradient(cfg3, g3, 20)
    assert rel_inf(so, sr) < 1e-13


EX = {G.D2Q9: [0, 1, 0, -1, -1, -1, 0, 1, 1],
      G.D3Q19: [0, 0, 0, -1, 0, 0, -1, 1, -1, 1, 0, 0, 1, 0, 0, 1, -1, 1, -1]}


@pytest.mark.parametrize("cfg", [W.channel_2d(8, 6), W.channel_2d(8, 6, collision=G.MRT),
                                 W.duct_3d(6, 5, 5), W.duct_3d(6, 5, 5).replace(collision=G.BGK)],
                         ids=["d2q9_bgk", "d2q9_mrt", "d3q19_mrt", "d3q19_bgk"])
def test_collision_conserves_mass(orc, cfg):
    """Sum f is kept by BGK, MRT and partial bounce-back; momentum only without PBB."""
    rng = np.random.default_rng(3)
    for _ in range(10):
        fin = (1.0 / cfg.npop) * (1 + 0.1 * rng.standard_normal(cfg.npop))
        fo, _ = orc.collide_cell(cfg, fin, rng.uniform(0.05, 0.95))
        assert abs(fo.sum() - fin.sum()) < 1e-14
        fo1, _ = orc.collide_cell(cfg.replace(interp_scale=0.0), fin, 0.5)
        e = np.array(EX[cfg.lattice])
        assert abs(fo1.sum() - fin.sum()) < 1e-14
        assert abs(e @ fo1 - e @ fin) < 1e-14          # momentum kept without bounce-back
        if abs(e @ fin) > 1e-3:
            assert abs(e @ fo - e @ fin) > 1e-6       # and removed by partial bounce-back


def test_gradient_matches_central_differences(orc):
    """The oracle's adjoint against central differences (h = 1e-6), the
    reference's own verification (topOpt/finiteDifferenceCheck2d.cc:58-113)."""
    cfg = W.channel_2d(20, 10, amp=0.2, period=15.0, objective=G.OBJ_DISSIPATION, nsteps=40)
    gamma = np.clip(W.design_2d(20, 10, 55), 0.05, 0.95)
    _, s = orc.gradient(cfg, gamma, 40)
    rng = np.random.default_rng(1)
    for c in rng.choice(cfg.ncells, 5, replace=False):
        gp, gm = gamma.copy(), gamma.copy()
        gp[c] += 1e-6
        gm[c] -= 1e-6
        fd = (orc.forward(cfg, gp, 40)[2] - orc.forward(cfg, gm, 40)[2]) / 2e-6
        assert abs(fd - s[c]) <= 1e-6 * np.abs(s).max()


def test_thermal_gradient_matches_central_differences(orc):
    cfg, gamma, _ = W.workload_thermal_512x256(nx=20, ny=10, nsteps=40)
    gamma = np.clip(gamma + 0.05 * np.sin(np.arange(gamma.size)), 0.02, 0.98)
    _, s = orc.gradient(cfg, gamma, 40)
    rng = np.random.default_rng(2)
    for c in rng.choice(cfg.ncells, 5, replace=False):
        gp, gm = gamma.copy(), gamma.copy()
        gp[c] += 1e-6
        gm[c] -= 1e-6
        fd = (orc.forward(cfg, gp, 40)[2] - orc.forward(cfg, gm, 40)[2]) / 2e-6
        assert abs(fd - s[c]) <= 1e-6 * np.abs(s).max()
