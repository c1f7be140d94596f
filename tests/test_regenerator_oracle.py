"""The regenerator driver on the oracle (CPU): the steady-then-unsteady gradient
against central differences for the regenerator efficiency (with a time
average, where the reference's own adjoint sources would be off) and the
domain temperature, and the StageTemp ramp against an independent
tabulation of its law."""
import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from helpers import rel_inf


def regen_case(objective=G.OBJ_REGENERATOR_EFFICIENCY, nx=40, ny=14, n_unsteady=120):
    cfg = W.regenerator_2d(nx, ny, n_unsteady=n_unsteady, ramp=40.0, objective=objective)
    return cfg, W.regenerator_design(nx, ny, 11)


@pytest.mark.parametrize("objective", [G.OBJ_REGENERATOR_EFFICIENCY, G.OBJ_DOMAIN_TEMPERATURE],
                         ids=["regenerator_efficiency", "domain_temperature"])
def test_steady_unsteady_gradient_matches_central_differences(orc, objective):
    cfg, gamma = regen_case(objective)
    gamma = np.clip(gamma + 0.02 * np.sin(np.arange(gamma.size)), 0.0, 1.0)
    # tol = 0: the steady phase runs its maximum, so its length cannot change
    # between the perturbed designs
    args = (300, 100, 0.0, 120)
    J, s, S = orc.gradient_steady(cfg, gamma, *args)
    assert S == 300 and J != 0.0
    rng = np.random.default_rng(5)
    box = cfg.obj_out
    inside = [c for c in range(cfg.ncells)
              if box[0] <= c % cfg.nx <= box[1] and 0.05 < gamma[c] < 0.95]
    cells = list(rng.choice(inside, 3, replace=False)) + [int(np.argmax(np.abs(s)))]
    for c in cells:
        gp, gm = gamma.copy(), gamma.copy()
        gp[c] += 1e-6
        gm[c] -= 1e-6
        fd = (orc.gradient_steady(cfg, gp, *args)[0] - orc.gradient_steady(cfg, gm, *args)[0]) / 2e-6
        assert abs(fd - s[c]) <= 1e-6 * np.abs(s).max(), (c, fd, s[c])


def test_steady_phase_length_follows_the_tolerance(orc):
    cfg, gamma = regen_case()
    _, _, S1 = orc.gradient_steady(cfg, gamma, 5000, 100, 1e-4, 20)
    _, _, S2 = orc.gradient_steady(cfg, gamma, 5000, 100, 1e-5, 20)
    assert S1 % 100 == 0 and S2 % 100 == 0 and 0 < S1 < S2 < 5000


def test_stage_temperature_ramp_matches_its_law(orc):
    """T_in(t) = T0 through the steady phase (t <= S), then T0 + dT sin(pi (t-S) /
    (2 ramp)) for t - S < ramp, then T0 + dT (regenerator2d.cc:53-69), against
    the same law tabulated per step."""
    cfg, gamma = regen_case(n_unsteady=60)
    S, ramp, dT, T0 = 30, 40.0, 2.0, 0.5
    b = cfg.bcs[2]
    ramped = cfg.replace(bcs=[cfg.bcs[0], cfg.bcs[1],
                              G.Boundary(G.BC_TEMPERATURE, G.FACE_WEST, b.box, dT, amp=T0 / dT,
                                         period=ramp, time_law=G.TIME_RAMP)])
    n = S + 60
    law = np.array([T0 if t <= S else T0 + dT * (np.sin(np.pi * (t - S) / (2 * ramp))
                                                 if t - S < ramp else 1.0) for t in range(n + 1)])
    tab = cfg.replace(bcs=[cfg.bcs[0], cfg.bcs[1],
                           G.Boundary(G.BC_TEMPERATURE, G.FACE_WEST, b.box, 1.0,
                                      G.PROFILE_TABLE)])
    npos = b.box[3] - b.box[2] + 1
    orc.set_phase(S, 1)
    try:
        f1, _, _ = orc.forward(ramped, gamma, n)
    finally:
        orc.set_phase()
    orc.set_tables({2: np.repeat(law[:, None], npos, axis=1)})
    try:
        f2, _, _ = orc.forward(tab, gamma, n)
    finally:
        orc.set_tables(None)
    assert rel_inf(f1, f2) < 1e-14
    # before any steady phase the ramp never starts
    f3, _, _ = orc.forward(ramped, gamma, n)
    orc.set_tables({2: np.full((1, npos), T0)})
    try:
        f4, _, _ = orc.forward(tab, gamma, n)
    finally:
        orc.set_tables(None)
    assert rel_inf(f3, f4) < 1e-14
