"""Boundaries on every face on the GPU: each face and kind against the oracle
(FP64 within 1e-12), reduced-precision storage on the y faces, tabulated
inputs, and the robust pump's set-up (north inlet with a zero-mean sine,
pressure segments west and east, through-flow objective) in a batch."""
import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from boundary_cases import pressure_driven_reverse, rotate_config, west_to_east_channel
from helpers import rel_inf, rel_l2

pytestmark = pytest.mark.gpu


def mirrored_inlets(nx=18, ny=12, n=50, storage=G.STORE_FP64):
    north = (4, 13, ny - 1, ny - 1, 0, 0)
    south = (4, 13, 0, 0, 0, 0)
    west = (0, 0, 1, ny - 2, 0, 0)
    base = W.channel_2d(nx, ny, nsteps=n, storage=storage)
    return [base.replace(bcs=[G.Boundary(G.BC_VELOCITY, face, box, 0.04, G.PROFILE_PARABOLIC,
                                         0.3, 20.0, G.TIME_OFFSET_SINE, (0.01, sgn, 0.0)),
                              G.Boundary(G.BC_PRESSURE, G.FACE_WEST, west, 1.0)],
                         objective=G.OBJ_PRESSURE_DROP, obj_in=box, obj_out=west)
            for face, box, sgn in ((G.FACE_NORTH, north, -1.0), (G.FACE_SOUTH, south, 1.0))]


def standard_channel(kind_v, kind_p, nx=24, ny=12, n=60, storage=G.STORE_FP64):
    cfg = W.channel_2d(nx, ny, amp=0.2, period=30.0, nsteps=n, storage=storage)
    a, b = cfg.bcs
    return cfg.replace(bcs=[G.Boundary(kind_v, a.face, a.box, a.value, a.profile, a.amp, a.period),
                            G.Boundary(kind_p, b.face, b.box, 1.0)])


CASES = {
    "west_velocity_east_pressure": west_to_east_channel(),
    "south_velocity_north_pressure": rotate_config(west_to_east_channel()),
    "west_pressure_east_velocity": pressure_driven_reverse(),
    "south_pressure_north_velocity": rotate_config(pressure_driven_reverse()),
    "north_inlet_west_outlet": mirrored_inlets()[0],
    "south_inlet_west_outlet": mirrored_inlets()[1],
    "standard_velocity_west": standard_channel(G.BC_VELOCITY_STANDARD, G.BC_PRESSURE),
    "standard_pressure_east": standard_channel(G.BC_VELOCITY, G.BC_PRESSURE_STANDARD),
    "mrt_south_velocity_north_pressure": rotate_config(
        west_to_east_channel().replace(collision=G.MRT)),
}


def run(cfg, gamma, n, k=5, tables=None):
    with G.Handle(cfg) as h:
        for i, t in (tables or {}).items():
            h.set_bc_profile(i, t)
        h.set_design(gamma)
        h.init_equilibrium()
        J, js = h.forward(n, per_step=True)
        f = h.populations()
        Jg, sens, _ = h.gradient(n, k)
    return f, js, Jg, sens


@pytest.mark.parametrize("name", sorted(CASES))
def test_every_face_matches_the_oracle(orc, name):
    cfg = CASES[name]
    gamma = W.design_2d(cfg.nx, cfg.ny, 601)
    n = 50
    f, js, Jg, sens = run(cfg, gamma, n)
    fo, jso, _ = orc.forward(cfg, gamma, n)
    Jgo, so = orc.gradient(cfg, gamma, n)
    assert rel_inf(f, fo) < 1e-12
    assert rel_inf(js, jso) < 1e-12
    assert abs(Jg - Jgo) <= 1e-12 * abs(Jgo)
    assert rel_inf(sens, so) < 1e-12


@pytest.mark.parametrize("storage,tol_f", [(G.STORE_FP32, 2e-6), (G.STORE_FP16, 2e-3)])
@pytest.mark.parametrize("name", ["south_velocity_north_pressure", "south_pressure_north_velocity",
                                  "standard_velocity_west"])
def test_reduced_precision_on_every_face(orc, name, storage, tol_f):
    cfg = CASES[name].replace(storage=storage)
    gamma = W.design_2d(cfg.nx, cfg.ny, 602)
    n = 50
    f, _, Jg, sens = run(cfg, gamma, n)
    fo, _, _ = orc.forward(cfg.replace(storage=G.STORE_FP64), gamma, n)
    Jgo, so = orc.gradient(cfg.replace(storage=G.STORE_FP64), gamma, n)
    assert rel_inf(f, fo) < tol_f
    assert abs(Jg - Jgo) <= 1e-4 * abs(Jgo)
    assert rel_l2(sens, so) < 1e-4


def test_tables_match_the_analytic_boundary_and_are_checked():
    cfg = W.channel_2d(24, 12, amp=0.25, period=12.0, nsteps=40)
    gamma = W.design_2d(24, 12, 603)
    n = 40
    f0, js0, J0, s0 = run(cfg, gamma, n)
    y = np.arange(1, 11, dtype=np.float64)
    m = (12 - 1) / 2.0
    par = ((m * m - (y - m) * (y - m)) / (m * m))[None, :]
    tab = cfg.replace(bcs=[G.Boundary(G.BC_VELOCITY, G.FACE_WEST, cfg.bcs[0].box, 0.05,
                                      G.PROFILE_TABLE, 0.25, 12.0), cfg.bcs[1]])
    f1, js1, J1, s1 = run(tab, gamma, n, tables={0: par})
    assert np.array_equal(f1, f0) and np.array_equal(js1, js0)
    assert J1 == J0 and np.array_equal(s1, s0)
    vec = np.zeros((12, 10, 2))
    for t in range(12):
        vec[t, :, 0] = (0.05 * (1 + 0.25 * np.sin(2 * np.pi * t / 12.0))) * par[0]
    f2, _, J2, s2 = run(tab, gamma, n, tables={0: vec})
    assert rel_inf(f2, f0) < 1e-15 and abs(J2 - J0) <= 1e-14 * abs(J0)
    assert rel_inf(s2, s0) < 1e-13
    with G.Handle(tab) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        with pytest.raises(G.LBMError) as e:
            h.forward(3)                     # the table was never set
        assert e.value.code == G.ERR_STATE
        with pytest.raises(G.LBMError) as e:
            h.set_bc_profile(0, np.zeros((1, 10, 3)))   # a 2D velocity has 2 components
        assert e.value.code == G.ERR_ARG
        with pytest.raises(G.LBMError) as e:
            h.set_bc_profile(1, par)          # boundary 1 is not a table boundary
        assert e.value.code == G.ERR_STATE
        h.set_bc_profile(0, par)
        h.forward(3)


def test_pump_setup_fp32_against_fp64():
    cfg = W.pump_2d(36, nsteps=600, period=200.0)
    gamma = W.design_2d(36, 36, 604)
    prof = {2: W.pump_inflow_profile(cfg)}
    _, _, J64, s64 = run(cfg, gamma, 600, 16, prof)
    _, _, J32, s32 = run(cfg.replace(storage=G.STORE_FP32), gamma, 600, 16, prof)
    assert abs(J32 - J64) <= 1e-4 * abs(J64)
    assert rel_l2(s32, s64) < 1e-4


def test_pump_realisations_in_a_batch_with_tables(orc):
    """Three realisations of the pump (the robust design's eta = 0.3/0.5/0.7
    projections of one field) in one batch, each lattice with its own inflow
    table; a changed table is seen by the captured graph's next replay."""
    n = 120
    cfg = W.pump_2d(36, nsteps=n, period=60.0)
    base = W.design_2d(36, 36, 605)
    designs = [W.tanh_projection(base, 8.0, eta) for eta in (0.3, 0.5, 0.7)]
    prof = W.pump_inflow_profile(cfg)
    with G.Batch([cfg] * 3) as b:
        for i, g in enumerate(designs):
            b[i].set_bc_profile(2, prof)
            b[i].set_design(g)
        J, sens, _ = b.gradient(n, 8, use_graph=True)
        for i, g in enumerate(designs):
            orc.set_tables({2: prof})
            try:
                Jo, so = orc.gradient(cfg, g, n)
            finally:
                orc.set_tables(None)
            assert abs(J[i] - Jo) <= 1e-12 * abs(Jo)
            assert rel_inf(sens[i], so) < 1e-12
        # a stronger inlet on lattice 1, same table size: the replayed graph reads it
        b[1].set_bc_profile(2, 2.0 * prof)
        J2, sens2, _ = b.gradient(n, 8, use_graph=True)
        # a two-row table (new layout): the batch captures a new graph
        b[2].set_bc_profile(2, np.vstack([prof, prof]))
        J3, sens3, _ = b.gradient(n, 8, use_graph=True)
    orc.set_tables({2: 2.0 * prof})
    try:
        Jo1, so1 = orc.gradient(cfg, designs[1], n)
    finally:
        orc.set_tables(None)
    assert abs(J2[1] - Jo1) <= 1e-12 * abs(Jo1) and rel_inf(sens2[1], so1) < 1e-12
    assert J2[0] == J[0] and J2[2] == J[2]
    assert J3[2] == J[2] and np.array_equal(sens3[2], sens[2])   # same values, two rows
