"""The boundaries without a reference counterpart (south velocity, north and
south pressure) pinned by rotation against the reference-pinned west/east
operators, on the oracle; the tabulated boundary input against the analytic
one; and the argument checks of the widened boundary interface (no GPU)."""
import ctypes as C

import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from boundary_cases import (pressure_driven_reverse, rotate_cells, rotate_config,
                            rotate_populations, west_to_east_channel)
from helpers import rel_inf


@pytest.mark.parametrize("make", [west_to_east_channel, pressure_driven_reverse],
                         ids=["velocity_south_pressure_north", "pressure_south_velocity_north"])
def test_rotated_problem_gives_rotated_fields(orc, make):
    cfg = make()
    gamma = W.design_2d(cfg.nx, cfg.ny, 501)
    n = 60
    rcfg = rotate_config(cfg)
    faces = sorted(b.face for b in rcfg.bcs)
    assert faces == sorted([G.FACE_SOUTH, G.FACE_NORTH])
    rgamma = rotate_cells(gamma, cfg)
    f, js, J = orc.forward(cfg, gamma, n)
    fr, jsr, Jr = orc.forward(rcfg, rgamma, n)
    assert rel_inf(fr, rotate_populations(f, cfg)) < 1e-13
    assert rel_inf(jsr, js) < 1e-12
    Jg, s = orc.gradient(cfg, gamma, n)
    Jgr, sr = orc.gradient(rcfg, rgamma, n)
    assert abs(Jgr - Jg) <= 1e-12 * abs(Jg)
    assert rel_inf(sr, rotate_cells(s, cfg)) < 1e-11


def test_south_velocity_is_the_mirrored_north_one(orc):
    """A north inlet (the reference's IncompressibleZouHeVelocityNorth2d) and a
    south inlet on the channel mirrored in y give mirrored fields."""
    nx, ny, n = 18, 12, 50
    MIR = np.array([0, 7, 6, 5, 4, 3, 2, 1, 8])   # e_i -> (ex, -ey)
    north = (4, 13, ny - 1, ny - 1, 0, 0)
    south = (4, 13, 0, 0, 0, 0)
    west = (0, 0, 1, ny - 2, 0, 0)
    base = W.channel_2d(nx, ny, nsteps=n)
    cn = base.replace(bcs=[G.Boundary(G.BC_VELOCITY, G.FACE_NORTH, north, 0.04, G.PROFILE_PARABOLIC,
                                      0.3, 20.0, G.TIME_OFFSET_SINE, (0.01, -1.0, 0.0)),
                           G.Boundary(G.BC_PRESSURE, G.FACE_WEST, west, 1.0)],
                      objective=G.OBJ_PRESSURE_DROP, obj_in=north, obj_out=west)
    cs = base.replace(bcs=[G.Boundary(G.BC_VELOCITY, G.FACE_SOUTH, south, 0.04, G.PROFILE_PARABOLIC,
                                      0.3, 20.0, G.TIME_OFFSET_SINE, (0.01, 1.0, 0.0)),
                           G.Boundary(G.BC_PRESSURE, G.FACE_WEST, west, 1.0)],
                      objective=G.OBJ_PRESSURE_DROP, obj_in=south, obj_out=west)
    g = W.design_2d(nx, ny, 502)
    gm = g.reshape(ny, nx)[::-1].ravel()
    fn, _, Jn = orc.forward(cn, g, n)
    fs, _, Js = orc.forward(cs, gm, n)
    fn_m = fn.reshape(ny, nx, 9)[::-1][:, :, MIR].reshape(-1)
    assert rel_inf(fs, fn_m) < 1e-13
    assert abs(Js - Jn) <= 1e-12 * abs(Jn)
    _, sn = orc.gradient(cn, g, n)
    _, ss = orc.gradient(cs, gm, n)
    assert rel_inf(ss, sn.reshape(ny, nx)[::-1].ravel()) < 1e-11


def test_tabulated_input_equals_the_analytic_one(orc):
    """A one-row factor table holding the parabola, and a per-step vector table
    holding value * T(t) * parabola * dir, reproduce the analytic boundary."""
    cfg = W.channel_2d(16, 10, amp=0.25, period=12.0, nsteps=40)
    g = W.design_2d(16, 10, 503)
    n = 40
    f0, _, J0 = orc.forward(cfg, g, n)
    _, s0 = orc.gradient(cfg, g, n)
    y = np.arange(1, 9, dtype=np.float64)
    m = (10 - 1) / 2.0
    par = (m * m - (y - m) * (y - m)) / (m * m)
    tab = cfg.replace(bcs=[G.Boundary(G.BC_VELOCITY, G.FACE_WEST, cfg.bcs[0].box, 0.05,
                                      G.PROFILE_TABLE, 0.25, 12.0), cfg.bcs[1]])
    orc.set_tables({0: par[None, :]})
    try:
        f1, _, J1 = orc.forward(tab, g, n)
        _, s1 = orc.gradient(tab, g, n)
    finally:
        orc.set_tables(None)
    assert np.array_equal(f1, f0) and J1 == J0 and np.array_equal(s1, s0)
    # the velocity vectors themselves over one period of 12 steps
    vec = np.zeros((12, 8, 2))
    for t in range(12):
        vec[t, :, 0] = (0.05 * (1 + 0.25 * np.sin(2 * np.pi * t / 12.0))) * par
    orc.set_tables({0: vec})
    try:
        f2, _, J2 = orc.forward(tab, g, n)
    finally:
        orc.set_tables(None)
    assert rel_inf(f2, f0) < 1e-15 and abs(J2 - J0) <= 1e-14 * abs(J0)


@pytest.mark.parametrize("kind,face,code", [
    (G.BC_VELOCITY_STANDARD, G.FACE_EAST, -2),     # the reference has the west face only
    (G.BC_VELOCITY_STANDARD, G.FACE_NORTH, -2),
    (G.BC_PRESSURE_STANDARD, G.FACE_SOUTH, -2),
    (G.BC_TEMPERATURE, G.FACE_WEST, -2),           # needs the thermal lattice
    (9, G.FACE_WEST, -2),
])
def test_boundary_kind_face_combinations_checked(lib, kind, face, code):
    nx, ny = 16, 8
    box = {G.FACE_WEST: (0, 0, 1, 6, 0, 0), G.FACE_EAST: (15, 15, 1, 6, 0, 0),
           G.FACE_SOUTH: (1, 14, 0, 0, 0, 0), G.FACE_NORTH: (1, 14, 7, 7, 0, 0)}[face]
    cfg = W.channel_2d(nx, ny).replace(
        bcs=[G.Boundary(kind, face, box, 0.02)], objective=G.OBJ_NONE)
    h = C.c_void_p()
    assert lib.lbm_create(C.byref(cfg.to_c()), C.byref(h)) == code
    assert lib.lbm_last_error(None)


def test_boundary_box_must_lie_on_its_face(lib):
    h = C.c_void_p()
    cfg = W.channel_2d(16, 8).replace(
        bcs=[G.Boundary(G.BC_VELOCITY, G.FACE_NORTH, (1, 14, 6, 6, 0, 0), 0.02)],
        objective=G.OBJ_NONE)
    assert lib.lbm_create(C.byref(cfg.to_c()), C.byref(h)) == -1
    cfg = W.channel_2d(16, 8).replace(
        bcs=[G.Boundary(G.BC_PRESSURE, G.FACE_SOUTH, (0, 15, 0, 0, 0, 0), 1.0,
                        time_law=7)], objective=G.OBJ_NONE)
    assert lib.lbm_create(C.byref(cfg.to_c()), C.byref(h)) == -1   # unknown time law


def test_through_flow_objective_needs_both_boxes(lib):
    h = C.c_void_p()
    cfg = W.pump_2d(12).replace(obj_in=(0, 0, 5, 20, 0, 0))   # past the lattice
    assert lib.lbm_create(C.byref(cfg.to_c()), C.byref(h)) == -1


def test_pump_setup_is_expressible(lib):
    """The robust pump's boundaries (north inlet segment with a zero-mean sine,
    west/east pressure segments) pass the configuration checks."""
    cfg = W.pump_2d(36)
    assert [b.face for b in cfg.bcs] == [G.FACE_WEST, G.FACE_EAST, G.FACE_NORTH]
    assert cfg.bcs[2].time_law == G.TIME_SINE and cfg.bcs[2].profile == G.PROFILE_TABLE
    prof = W.pump_inflow_profile(cfg)
    # the reference's InflowVelocity centres its parabola on (ny-1)/2 = 17.5 with
    # radius th/2 = 6 over the inlet x = 13..24, so it is lopsided and turns
    # negative at x = 24 (robustPump2d.cc:17-19, 100-102)
    assert prof.shape == (1, 12)
    assert abs(prof[0, 0] - (36 - 4.5 ** 2) / 36) < 1e-15
    assert abs(prof[0, -1] - (36 - 6.5 ** 2) / 36) < 1e-15
