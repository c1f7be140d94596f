"""GPU parity: the CUDA path through the C ABI against the oracle on the same
seeded inputs.

Tolerances (norm-wise, max|gpu - oracle| / max|oracle|):
* FP64 storage: populations, per-step objective, adjoint and dJ/dgamma within 1e-12.
* FP32 shifted storage: populations within 2e-6, dJ/dgamma within 1e-4 (the
  target for the FP32 gradient against the FP64 oracle).
* FP16 storage with FP32 compute: populations within 2e-3.
"""
import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from helpers import rel_inf, rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def run_forward(cfg, gamma, n, macros=None):
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium(macros)
        J, js = h.forward(n, per_step=True)
        return h.populations(), js, J, h.macros()


def run_gradient(cfg, gamma, n, k):
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        return h.gradient(n, k)


# -- 128x64 channel: D2Q9 BGK + Brinkman, FP64, 2000 steps ---------------------------

def test_channel_128x64_forward_matches_oracle(orc):
    cfg, gamma, n = W.workload_channel_128x64()
    f, js, J, mac = run_forward(cfg, gamma, n)
    fo, jo, Jo = orc.forward(cfg, gamma, n)
    assert rel_inf(f, fo) < FP64_TOL
    assert rel_inf(js, jo) < FP64_TOL
    assert abs(J - Jo) <= FP64_TOL * abs(Jo)
    # macros are the reference's: rho = sum f, u = j (incompressible)
    m = mac.reshape(-1, 3)
    fr = fo.reshape(-1, 9)
    assert rel_inf(m[:, 0], fr.sum(axis=1)) < FP64_TOL


def test_channel_128x64_gradient_matches_oracle(orc):
    cfg, gamma, _ = W.workload_channel_128x64()
    n = 400
    cfg = cfg.replace(obj_weight=1.0 / n)
    J, s, st = run_gradient(cfg, gamma, n, 16)
    Jo, so = orc.gradient(cfg, gamma, n)
    assert abs(J - Jo) <= FP64_TOL * abs(Jo)
    assert rel_inf(s, so) < FP64_TOL
    assert st.recomputed_steps == G.wang_recompute_count(n, 16)


def test_unsteady_inlet_and_dissipation_gradient(orc):
    cfg = W.channel_2d(64, 32, amp=0.2, period=50.0, objective=G.OBJ_DISSIPATION, nsteps=150)
    gamma = W.design_2d(64, 32, 99)
    J, s, _ = run_gradient(cfg, gamma, 150, 7)
    Jo, so = orc.gradient(cfg, gamma, 150)
    assert abs(J - Jo) <= FP64_TOL * abs(Jo)
    assert rel_inf(s, so) < FP64_TOL


def test_mrt2d_forward_and_gradient(orc):
    cfg = W.channel_2d(40, 20, collision=G.MRT, nsteps=120)
    gamma = W.design_2d(40, 20, 5)
    f, js, J, _ = run_forward(cfg, gamma, 120)
    fo, jo, Jo = orc.forward(cfg, gamma, 120)
    assert rel_inf(f, fo) < FP64_TOL
    Jg, s, _ = run_gradient(cfg, gamma, 120, 4)
    Jgo, so = orc.gradient(cfg, gamma, 120)
    assert abs(Jg - Jgo) <= FP64_TOL * abs(Jgo)
    assert rel_inf(s, so) < FP64_TOL


# -- duct family: D3Q19 MRT + Brinkman ------------------------------------------------

def test_d3q19_mrt_forward_matches_oracle(orc):
    cfg, gamma, _ = W.workload_duct_256x128x128(nx=32, ny=16, nz=12, nsteps=150)
    f, js, J, mac = run_forward(cfg, gamma, 150)
    fo, jo, Jo = orc.forward(cfg, gamma, 150)
    assert rel_inf(f, fo) < FP64_TOL
    assert rel_inf(js, jo) < FP64_TOL


def test_d3q19_mrt_gradient_matches_oracle(orc):
    cfg, gamma, _ = W.workload_duct_256x128x128(nx=20, ny=12, nz=10, nsteps=80)
    J, s, st = run_gradient(cfg, gamma, 80, 6)
    Jo, so = orc.gradient(cfg, gamma, 80)
    assert abs(J - Jo) <= FP64_TOL * abs(Jo)
    assert rel_inf(s, so) < FP64_TOL


def test_d3q19_bgk_forward_and_gradient(orc):
    cfg, gamma, _ = W.workload_duct_256x128x128(nx=18, ny=10, nz=9, nsteps=60)
    cfg = cfg.replace(collision=G.BGK)
    f, _, _, _ = run_forward(cfg, gamma, 60)
    fo, _, _ = orc.forward(cfg, gamma, 60)
    assert rel_inf(f, fo) < FP64_TOL
    J, s, _ = run_gradient(cfg, gamma, 60, 5)
    Jo, so = orc.gradient(cfg, gamma, 60)
    assert rel_inf(s, so) < FP64_TOL


# -- thermal double distribution --------------------------------------------------------

def test_thermal_forward_and_gradient(orc):
    cfg, gamma, _ = W.workload_thermal_512x256(nx=48, ny=24, nsteps=100)
    f, js, J, _ = run_forward(cfg, gamma, 100)
    fo, jo, Jo = orc.forward(cfg, gamma, 100)
    assert rel_inf(f, fo) < FP64_TOL
    assert abs(J - Jo) <= FP64_TOL * abs(Jo)
    Jg, s, _ = run_gradient(cfg, gamma, 100, 5)
    Jgo, so = orc.gradient(cfg, gamma, 100)
    assert rel_inf(s, so) < FP64_TOL


# -- single reverse steps through the step API ----------------------------------------

def test_adjoint_steps_match_oracle(orc):
    cfg = W.channel_2d(30, 14, nsteps=40)
    gamma = W.design_2d(30, 14, 3)
    # forward trajectory from the oracle
    f = np.zeros(cfg.ncells * 9)
    import ctypes
    states = []
    ft, _, _ = orc.forward(cfg, gamma, 0)
    states.append(ft.copy())
    for t in range(1, 41):
        ft2 = ft.copy()
        c = cfg.to_c()
        orc.lib.orc_forward_from(ctypes.byref(c), gamma.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                 ft2.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), t - 1, 1, None, None)
        ft = ft2
        states.append(ft.copy())
    lam_o = np.zeros(cfg.ncells * 9)
    sens_o = np.zeros(cfg.ncells)
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.adjoint_reset()
        for t in range(40, 30, -1):
            h.set_populations(states[t], t)
            h.adjoint_step()
            lam_o, sens_o = orc.adjoint_step(cfg, gamma, states[t], t, lam_o, sens_o)
            assert rel_inf(h.adjoint(), lam_o) < FP64_TOL
            assert rel_inf(h.sensitivity(), sens_o) < FP64_TOL
        del f


# -- reduced precision against the FP64 oracle -------------------------------------------

def test_fp32_fp16_storage_error_vs_fp64_oracle(orc):
    cfg, gamma, _ = W.workload_duct_256x128x128(nx=32, ny=16, nz=16, nsteps=200)
    fo, jo, Jo = orc.forward(cfg, gamma, 200)
    f32, _, J32, _ = run_forward(cfg.replace(storage=G.STORE_FP32), gamma, 200)
    f16, _, J16, _ = run_forward(cfg.replace(storage=G.STORE_FP16), gamma, 200)
    e32, e16 = rel_inf(f32, fo), rel_inf(f16, fo)
    print("D3Q19 populations after 200 steps: FP32 rel %.3e, FP16 rel %.3e" % (e32, e16))
    assert e32 < 2e-6
    assert e16 < 2e-3


def test_fp32_gradient_vs_fp64_oracle(orc):
    cfg, gamma, _ = W.workload_duct_256x128x128(nx=24, ny=12, nz=12, nsteps=120)
    Jo, so = orc.gradient(cfg, gamma, 120)
    J, s, _ = run_gradient(cfg.replace(storage=G.STORE_FP32), gamma, 120, 8)
    e = rel_l2(s, so)
    print("D3Q19 FP32 gradient rel L2 error %.3e, J rel %.3e" % (e, abs(J - Jo) / abs(Jo)))
    assert e < 1e-4
    assert abs(J - Jo) < 1e-4 * abs(Jo)


def _model(name):
    if name == "d2q9_bgk":
        cfg = W.channel_2d(48, 24, amp=0.2, period=100.0, nsteps=150)
        return cfg, W.design_2d(48, 24, 11)
    if name == "d2q9_mrt":
        cfg = W.channel_2d(48, 24, collision=G.MRT, nsteps=150)
        return cfg, W.design_2d(48, 24, 12)
    if name == "d3q19_bgk":
        cfg = W.duct_3d(20, 12, 10, nsteps=150).replace(collision=G.BGK)
        return cfg, W.design_3d(20, 12, 10, 13)
    cfg = W.thermal_2d(48, 24, nsteps=150)
    return cfg, W.thermal_design(48, 24, 14)


@pytest.mark.parametrize("name", ["d2q9_bgk", "d2q9_mrt", "d3q19_bgk", "thermal"])
def test_reduced_precision_every_model_vs_fp64_oracle(orc, name):
    """FP32 and FP16 storage of every other collision model against the FP64
    oracle: populations after 150 steps (FP32 within 2e-6, FP16 within 2e-3
    of the largest value) and the FP32 gradient (within 1e-4, rel. L2)."""
    cfg, gamma = _model(name)
    fo, _, _ = orc.forward(cfg, gamma, 150)
    f32, _, _, _ = run_forward(cfg.replace(storage=G.STORE_FP32), gamma, 150)
    f16, _, _, _ = run_forward(cfg.replace(storage=G.STORE_FP16), gamma, 150)
    e32, e16 = rel_inf(f32, fo), rel_inf(f16, fo)
    Jo, so = orc.gradient(cfg, gamma, 150)
    J, s, _ = run_gradient(cfg.replace(storage=G.STORE_FP32), gamma, 150, 8)
    eg = rel_l2(s, so)
    print("%s: populations FP32 %.3e, FP16 %.3e; FP32 gradient %.3e, J %.3e"
          % (name, e32, e16, eg, abs(J - Jo) / abs(Jo)))
    assert e32 < 2e-6
    assert e16 < 2e-3
    assert eg < 1e-4
    assert abs(J - Jo) < 1e-4 * abs(Jo)


@pytest.mark.parametrize("lattice", ["d2q9", "d3q19", "thermal"])
def test_fp32_fluid_cells_feel_no_porosity(lattice):
    """Where gamma = 1 the Brinkman term must vanish exactly in FP32 too: an
    all-fluid lattice steps bit for bit like the same lattice with the
    porosity scale set to 0 (a fluid cell whose interpolation is off by one
    unit in the last place gets a small spurious drag every step, which
    accumulates over long runs)."""
    if lattice == "d2q9":
        cfg = W.channel_2d(96, 40, storage=G.STORE_FP32)
    elif lattice == "d3q19":
        cfg = W.duct_3d(40, 20, 16, storage=G.STORE_FP32)
    else:
        cfg = W.thermal_2d(96, 40, storage=G.STORE_FP32)
    ones = np.ones(cfg.ncells)
    f1, _, J1, _ = run_forward(cfg, ones, 150)
    f0, _, J0, _ = run_forward(cfg.replace(interp_scale=0.0), ones, 150)
    assert np.array_equal(f1, f0)
    assert J1 == J0


@pytest.mark.parametrize("which", ["d2q9_bgk", "d3q19_mrt", "thermal"])
def test_reverse_variant_does_not_change_results(which):
    """The register-lean reverse kernel does the same arithmetic up to the
    compiler's multiply-add fusion under a tighter register budget: the FP32
    gradients of the two variants agree to FP32 rounding (bit-identical on
    D3Q19 MRT and the thermal model as built; a few cells of the D2Q9 BGK
    channel differ by about 1e-9 relative).  FP64 has one variant only."""
    if which == "d2q9_bgk":
        cfg, g = W.channel_2d(96, 40, storage=G.STORE_FP32, nsteps=80), W.design_2d(96, 40, 31)
    elif which == "d3q19_mrt":
        cfg, g = W.duct_3d(40, 20, 16, storage=G.STORE_FP32, nsteps=80), W.design_3d(40, 20, 16, 32)
    else:
        cfg, g = W.thermal_2d(96, 40, storage=G.STORE_FP32, nsteps=80), W.thermal_design(96, 40, 33)
    out = []
    for lean in (0, 1):
        with G.Handle(cfg) as h:
            h.set_reverse_variant(lean)
            assert h.reverse_variant == lean
            h.set_design(g)
            h.init_equilibrium()
            out.append(h.gradient(80, 8))
    assert abs(out[0][0] - out[1][0]) <= 1e-12 * abs(out[0][0])
    scale = np.abs(out[0][1]).max()
    assert np.abs(out[0][1] - out[1][1]).max() <= 1e-7 * scale
    with G.Handle(cfg.replace(storage=G.STORE_FP64)) as h:
        with pytest.raises(G.LBMError) as e:
            h.set_reverse_variant(1)
        assert e.value.code == G.ERR_SUP


# -- finite differences --------------------------------------------------------------------

def test_gradient_matches_central_differences():
    """dJ/dgamma against central FD (h = 1e-6, FP64) at seeded cells, the
    reference's verification (topOpt/finiteDifferenceCheck2d.cc:58-113) with
    central instead of one-sided differences."""
    cfg = W.channel_2d(32, 16, amp=0.2, period=30.0, objective=G.OBJ_DISSIPATION, nsteps=80)
    gamma = W.design_2d(32, 16, 21)
    _, s, _ = run_gradient(cfg, gamma, 80, 5)
    rng = np.random.default_rng(12)
    cells = rng.choice(cfg.ncells, size=8, replace=False)
    hstep = 1e-6
    with G.Handle(cfg) as h:
        for c in cells:
            vals = []
            for sgn in (1.0, -1.0):
                g = gamma.copy()
                g[c] = min(max(g[c] + sgn * hstep, 0.0), 1.0)
                h.set_design(g)
                h.init_equilibrium()
                vals.append((h.forward(80), g[c]))
            fd = (vals[0][0] - vals[1][0]) / (vals[0][1] - vals[1][1])
            assert abs(fd - s[c]) <= 1e-5 * max(abs(s).max(), 1e-30), (c, fd, s[c])


# -- edge cases ------------------------------------------------------------------------------

@pytest.mark.parametrize("nx,ny", [(37, 19), (5, 3), (300, 7)])
def test_ragged_sizes(orc, nx, ny):
    cfg = W.channel_2d(nx, ny, nsteps=30)
    gamma = W.design_2d(nx, ny, nx * 100 + ny)
    f, js, J, _ = run_forward(cfg, gamma, 30)
    fo, jo, Jo = orc.forward(cfg, gamma, 30)
    assert rel_inf(f, fo) < FP64_TOL
    Jg, s, _ = run_gradient(cfg, gamma, 30, 2)
    Jgo, so = orc.gradient(cfg, gamma, 30)
    assert rel_inf(s, so) < FP64_TOL


def test_lattice_larger_than_l2_matches_oracle(orc):
    """A 2D reverse step whose working set is larger than L2 adds to dJ/dgamma
    with a read-modify-write (smaller ones use an atomic add): a 1536x768
    channel, 283 MB per FP64 reverse step, against the oracle."""
    nx, ny, n = 1536, 768, 8
    assert nx * ny * (3 * 9 * 8 + 8 + 16) > 256 * 2**20
    cfg = W.channel_2d(nx, ny, nsteps=n)
    gamma = W.design_2d(nx, ny, 17)
    J, s, _ = run_gradient(cfg, gamma, n, 3)
    Jo, so = orc.gradient(cfg, gamma, n)
    assert abs(J - Jo) <= FP64_TOL * abs(Jo)
    assert rel_inf(s, so) < FP64_TOL


def test_gradient_snapshot_counts_agree():
    cfg = W.channel_2d(24, 12, nsteps=50)
    gamma = W.design_2d(24, 12, 8)
    ref = None
    for k in (2, 3, 7, 51, 60):
        J, s, st = run_gradient(cfg, gamma, 50, k)
        assert st.recomputed_steps == G.wang_recompute_count(50, k)
        if ref is None:
            ref = (J, s)
        else:
            assert J == ref[0]
            assert np.array_equal(s, ref[1])   # recomputation is bitwise reproducible


def test_single_step_and_roundtrip(orc):
    cfg = W.channel_2d(20, 10, nsteps=1)
    gamma = W.design_2d(20, 10, 4)
    f, js, J, _ = run_forward(cfg, gamma, 1)
    fo, jo, Jo = orc.forward(cfg, gamma, 1)
    assert rel_inf(f, fo) < FP64_TOL
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.set_populations(fo, 1)
        assert h.time() == 1
        assert np.array_equal(h.populations(), fo)


def test_errors_are_reported():
    cfg = W.channel_2d(20, 10)
    with G.Handle(cfg) as h:
        with pytest.raises(G.LBMError) as e:
            h.forward(3)
        assert e.value.code == -5
        g = W.design_2d(20, 10, 1)
        g[5] = np.nan
        with pytest.raises(G.LBMError) as e:
            h.set_design(g)
        assert e.value.code == -6
    bad = cfg.replace(omega=2.5)
    with pytest.raises(G.LBMError) as e:
        G.Handle(bad)
    assert e.value.code == -1
    # the largest lattice: Q * P must stay below 2^31 (32-bit population offsets);
    # 19 x 1024 x 1024 x 128 = 2.55e9 is refused before anything is allocated
    with pytest.raises(G.LBMError) as e:
        G.Handle(W.duct_3d(1024, 1024, 128, storage=G.STORE_FP32))
    assert e.value.code == G.ERR_SUP
    # an empty horizon and a single snapshot are refused
    with G.Handle(cfg) as h:
        h.set_design(W.design_2d(20, 10, 1))
        h.init_equilibrium()
        for n, k in ((0, 8), (10, 1)):
            with pytest.raises(G.LBMError) as e:
                h.gradient(n, k)
            assert e.value.code == G.ERR_ARG


@pytest.mark.parametrize("storage", [G.STORE_FP64, G.STORE_FP32])
def test_launch_shape_does_not_change_results(storage):
    """Every block shape gives the same populations bit for bit (the FP32
    rounding noise is keyed on the cell, not the block); an invalid shape is
    refused."""
    cfg = W.duct_3d(40, 12, 10, nsteps=30).replace(storage=storage)
    gamma = W.design_3d(40, 12, 10, 5)
    out = []
    for shape in ((128, 2), (32, 4), (64, 2), (64, 1), (32, 2)):
        with G.Handle(cfg) as h:
            h.set_launch_shape(0, *shape)
            h.set_launch_shape(1, *shape)
            assert h.launch_shape(0) == shape and h.launch_shape(1) == shape
            h.set_design(gamma)
            h.init_equilibrium()
            J = h.forward(30)
            out.append((h.populations(), J))
    for f, J in out[1:]:
        assert np.array_equal(f, out[0][0])
        assert abs(J - out[0][1]) <= 1e-13 * abs(out[0][1])
    with G.Handle(cfg) as h:
        for bad in ((48, 4), (32, 3), (16, 8)):
            with pytest.raises(G.LBMError) as e:
                h.set_launch_shape(0, *bad)
            assert e.value.code == -1


def test_static_schedule_gives_the_same_gradient(orc):
    """LBStaticCheckpointing and LBDynamicCheckpointing: the same dJ/dgamma bit
    for bit (recomputation is exact) and the reference's recompute counts."""
    n, k = 90, 6
    cfg = W.channel_2d(30, 14, nsteps=n, amp=0.1, period=40.0)
    gamma = W.design_2d(30, 14, 17)
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        Jd, sd, std = h.gradient(n, k, G.SCHEDULE_DYNAMIC)
        Js, ss, sts = h.gradient(n, k, G.SCHEDULE_STATIC)
    assert Js == Jd and np.array_equal(ss, sd)
    assert sts.recomputed_steps == orc.static_count(n, k)[0]
    assert std.recomputed_steps == orc.wang_count(n, k)[0]
    insts = [(cfg, gamma), (W.channel_2d(20, 10, nsteps=n), W.design_2d(20, 10, 18))]
    with G.Batch([c for c, _ in insts]) as b:
        for i, (_, g) in enumerate(insts):
            b[i].set_design(g)
        Jb, sb, _ = b.gradient(n, k, use_graph=True, schedule=G.SCHEDULE_STATIC)
    assert abs(Jb[0] - Jd) <= 1e-12 * abs(Jd)
    assert rel_inf(sb[0], sd) < 1e-12


@pytest.mark.parametrize("storage,tol", [(G.STORE_FP64, 1e-9), (G.STORE_FP32, 1e-6)])
def test_forward_until_steady(orc, storage, tol):
    """The steady-state run of the regenerator application: it stops at a
    check step once max |f_t - f_{t-1}| < tol, and has then taken exactly that
    many steps (the state equals the oracle's after the same number of steps);
    max_steps bounds it."""
    cfg = W.channel_2d(48, 20, nsteps=100).replace(storage=storage)
    gamma = W.design_2d(48, 20, 33)
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        n, ch = h.forward_steady(40000, 100, tol)
        assert n < 40000 and n % 100 == 0 and 0 <= ch < tol
        assert h.time() == n
        f = h.populations()
        h.init_equilibrium()
        n2, ch2 = h.forward_steady(250, 100, 0.0)   # never below 0: runs to max_steps
        assert n2 == 250 and ch2 > 0
    fo, _, _ = orc.forward(cfg.replace(storage=G.STORE_FP64), gamma, n)
    lim = 1e-12 if storage == G.STORE_FP64 else 1e-5
    assert rel_inf(f, fo) < lim
    fp, _, _ = orc.forward(cfg.replace(storage=G.STORE_FP64), gamma, n - 1)
    assert np.abs(fo - fp).max() < 10 * tol
