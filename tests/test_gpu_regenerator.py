"""The regenerator driver on the GPU: lbm_gradient_steady (steady phase,
unsteady objective steps, reverse sweep through both) against the oracle for
the regenerator efficiency and the domain temperature, FP32 against FP64, the
steady forward with the StageTemp ramp, and reverse steps one at a time with
the regenerator efficiency's per-step design term."""
import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from helpers import rel_inf, rel_l2

pytestmark = pytest.mark.gpu


def regen_case(objective=G.OBJ_REGENERATOR_EFFICIENCY, nx=64, ny=20, n_unsteady=300,
               storage=G.STORE_FP64):
    cfg = W.regenerator_2d(nx, ny, n_unsteady=n_unsteady, ramp=60.0, objective=objective,
                           storage=storage)
    return cfg, W.regenerator_design(nx, ny, 12)


@pytest.mark.parametrize("objective", [G.OBJ_REGENERATOR_EFFICIENCY, G.OBJ_DOMAIN_TEMPERATURE],
                         ids=["regenerator_efficiency", "domain_temperature"])
def test_gradient_steady_matches_the_oracle(orc, objective):
    cfg, gamma = regen_case(objective)
    args = (6000, 100, 1e-4, 300)
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        J, s, st, S = h.gradient_steady(*args, 16)
    Jo, so, So = orc.gradient_steady(cfg, gamma, *args)
    assert S == So and 0 < S < 6000
    assert st.forward_steps == S + 300
    assert abs(J - Jo) <= 1e-12 * abs(Jo)
    assert rel_inf(s, so) < 1e-12


def test_gradient_steady_fp32_against_fp64():
    cfg, gamma = regen_case(n_unsteady=1000)
    out = {}
    for st in (G.STORE_FP64, G.STORE_FP32):
        with G.Handle(cfg.replace(storage=st)) as h:
            h.set_design(gamma)
            h.init_equilibrium()
            # tol = 0: both run the full steady phase, so the sweeps are the same length
            J, s, _, S = h.gradient_steady(1500, 100, 0.0, 1000, 32)
            assert S == 1500
            out[st] = (J, s)
    (J64, s64), (J32, s32) = out[G.STORE_FP64], out[G.STORE_FP32]
    assert abs(J32 - J64) <= 1e-4 * abs(J64)
    assert rel_l2(s32, s64) < 1e-4


def test_steady_forward_starts_the_ramp(orc):
    """lbm_forward_steady and lbm_forward after it: the inlet temperature ramps
    from the step the steady phase ended, as the oracle's forward with that phase."""
    cfg, gamma = regen_case()
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        S, _ = h.forward_steady(6000, 100, 1e-4)
        J, js = h.forward(150, per_step=True)
        f = h.populations()
    fo, _, _ = orc.forward(cfg, gamma, S)
    orc.set_phase(S, 1)
    try:
        import ctypes
        c = cfg.to_c()
        jso = np.zeros(150)
        rc = orc.lib.orc_forward_from(ctypes.byref(c), gamma.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                      fo.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), S, 150,
                                      jso.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
        assert rc == 0
    finally:
        orc.set_phase()
    assert rel_inf(f, fo) < 1e-12
    assert rel_inf(js, jso) < 1e-12


def test_reverse_steps_carry_the_design_term(orc):
    """Reverse steps one at a time (lbm_adjoint_step) with the regenerator
    efficiency: each adds its step's share J_t (Tb - Ti)/D of the 1/D design
    term, as the oracle's adjoint step does."""
    cfg, gamma = regen_case(nx=40, ny=14, n_unsteady=40)
    n = 40
    macros = np.zeros((cfg.ncells, 4))
    macros[:, 0] = 1.0
    macros[:, 1] = 0.03 * gamma
    macros[:, 3] = 1.5 * (1.0 - gamma)     # warm solid plates: a nonzero efficiency
    f0, _, _ = orc.forward(cfg, gamma, 0, macros.ravel())
    import ctypes
    states = [f0.copy()]
    ft = f0.copy()
    c = cfg.to_c()
    for t in range(1, n + 1):
        rc = orc.lib.orc_forward_from(ctypes.byref(c),
                                      gamma.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                      ft.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), t - 1, 1,
                                      None, None)
        assert rc == 0
        states.append(ft.copy())
    lam_o = np.zeros(cfg.ncells * cfg.npop)
    sens_o = np.zeros(cfg.ncells)
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.adjoint_reset()
        for t in range(n, n - 8, -1):
            h.set_populations(states[t], t)
            h.adjoint_step()
            lam_o, sens_o = orc.adjoint_step(cfg, gamma, states[t], t, lam_o, sens_o)
            assert rel_inf(h.adjoint(), lam_o) < 1e-12
            assert rel_inf(h.sensitivity(), sens_o) < 1e-12
    assert np.abs(sens_o).max() > 0


def test_batches_refuse_the_regenerator_efficiency():
    cfg, _ = regen_case()
    with pytest.raises(G.LBMError) as e:
        G.Batch([cfg, cfg])
    assert e.value.code == G.ERR_SUP
