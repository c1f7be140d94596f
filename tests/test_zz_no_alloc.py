"""lbm_objective_noalloc: the objective of a caller-owned device state computed
without any device allocation, for applications that reserve all of their
device memory themselves or may not call cudaMalloc at that point (fixed
memory budgets, real-time loops).

The caller's buffers here are made with torch (the test may allocate; the
entry point may not).  The states come from the oracle: its FP64 populations
after a forward run, laid out in the handle's SoA form (shifted by the lattice
weights and rounded for FP32/FP16 storage).  Two calls in a row of the entry
point must reproduce the oracle's objective of the same populations
(orc_objective, evaluated on the populations exactly as stored): within 1e-12
relative for FP64 storage, 1e-5 for FP32 and FP16 (FP32 arithmetic).  The
cases cover every objective, every storage, D2Q9 / D3Q19 / the thermal
lattice, boundaries on x and y faces, and t = 0 (no boundary applied) against
t > 0 (boundaries of step t applied on load).  The second call must leave the
device's free memory unchanged.  The rejections of oversized requests happen
before any device call and run without a GPU.  This file is collected last
so a failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from boundary_cases import rotate_config

W2 = np.array([4 / 9, 1 / 36, 1 / 9, 1 / 36, 1 / 9, 1 / 36, 1 / 9, 1 / 36, 1 / 9])
W3 = np.array([1 / 3] + [1 / 18] * 3 + [1 / 36] * 6 + [1 / 18] * 3 + [1 / 36] * 6)
STORE_NP = {G.STORE_FP64: np.float64, G.STORE_FP32: np.float32, G.STORE_FP16: np.float16}

# populations each boundary kind/face overwrites (perturbing them tests whether
# the boundary of step t is applied on load)
UNKNOWN = {G.FACE_WEST: [1, 7, 8], G.FACE_EAST: [3, 4, 5], G.FACE_NORTH: [1, 2, 3],
           G.FACE_SOUTH: [5, 6, 7]}


def _stored(cfg, f_aos):
    """Host AoS FP64 populations -> (device planes in the storage type, the FP64
    populations those planes hold)."""
    n, q = cfg.ncells, cfg.npop
    P = (n + 127) // 128 * 128
    f = f_aos.reshape(n, q).copy()
    w = W3 if cfg.lattice == G.D3Q19 else W2
    if cfg.storage != G.STORE_FP64:
        f[:, :len(w)] -= w          # shifted storage holds f_i - w_i (flow populations)
    dev = f.astype(STORE_NP[cfg.storage])
    held = dev.astype(np.float64)
    if cfg.storage != G.STORE_FP64:
        held[:, :len(w)] += w
    planes = np.zeros((q, P), dtype=dev.dtype)
    planes[:, :n] = dev.T
    return planes, held.ravel()


def _noalloc(lib, cfg, t, planes, gamma, check_memory=False):
    import torch
    gdt = torch.float64 if cfg.storage == G.STORE_FP64 else torch.float32
    fd = torch.from_numpy(planes).to(device="cuda").contiguous()
    gd = torch.from_numpy(np.asarray(gamma, dtype=np.float64)).to(dtype=gdt, device="cuda")
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    c = cfg.to_c()
    torch.cuda.synchronize()
    free = []
    for k in range(2):   # two calls in a row share the same scratch
        rc = lib.lbm_objective_noalloc(C.byref(c), int(t), C.c_void_p(fd.data_ptr()),
                                       C.c_void_p(gd.data_ptr()),
                                       C.cast(C.c_void_p(out.data_ptr() + 8 * k),
                                              C.POINTER(C.c_double)), None)
        assert rc == 0, lib.lbm_last_error(None).decode()
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
    if check_memory:
        assert free[1] == free[0]     # the second call allocated nothing
    return out.cpu().numpy()


@pytest.fixture(scope="module")
def nlib():
    lib = G.load_library()
    lib.lbm_objective_noalloc.restype = C.c_int
    lib.lbm_objective_noalloc.argtypes = [C.POINTER(G.CConfig), C.c_int, C.c_void_p, C.c_void_p,
                                          C.POINTER(C.c_double), C.c_void_p]
    return lib


def case(name, storage):
    if name == "d2q9_pressure_drop":
        cfg = W.channel_2d(64, 32, amp=0.2, period=40.0, nsteps=60, storage=storage)
        return cfg, W.design_2d(64, 32, 77)
    if name == "d2q9_outflow":
        cfg = W.channel_2d(48, 24, nsteps=60, storage=storage).replace(objective=G.OBJ_OUTFLOW)
        return cfg, W.design_2d(48, 24, 78)
    if name == "d2q9_dissipation":
        cfg = W.channel_2d(48, 24, nsteps=60, storage=storage, objective=G.OBJ_DISSIPATION)
        return cfg, W.design_2d(48, 24, 79)
    if name == "d2q9_through_flow_y_faces":
        # the pump's north inlet (parabolic here: tabulated inputs are refused)
        # with the west/east pressure segments and the through-flow objective
        cfg = W.pump_2d(36, nsteps=60, period=150.0, collision=G.BGK, storage=storage)
        b = cfg.bcs[2]
        cfg.bcs[2] = G.Boundary(b.kind, b.face, b.box, b.value, G.PROFILE_PARABOLIC, b.amp,
                                b.period, b.time_law, b.dir)
        # a higher pressure west drives a net flow west to east (the two means
        # of the objective then add up instead of cancelling)
        cfg.bcs[0] = G.Boundary(G.BC_PRESSURE, G.FACE_WEST, cfg.bcs[0].box, 1.01)
        return cfg, W.design_2d(36, 36, 80)
    if name == "d2q9_rotated_channel":
        # south velocity inlet and north pressure outlet
        cfg = rotate_config(W.channel_2d(40, 24, nsteps=60, storage=storage))
        return cfg, W.design_2d(24, 40, 82)
    if name == "d3q19_pressure_drop":
        cfg, gamma, _ = W.workload_duct_256x128x128(storage, nx=24, ny=12, nz=12, nsteps=60)
        return cfg, gamma
    if name == "thermal_heat_flux":
        # the heat flux through a column just behind the heated disc
        gamma = W.thermal_design(48, 24, 81)
        solid_x = np.flatnonzero((gamma.reshape(24, 48) < 1.0).any(axis=0))
        col = int(solid_x.max()) + 2
        cfg = W.thermal_2d(48, 24, nsteps=60, storage=storage).replace(
            obj_out=(col, col, 1, 22, 0, 0))
        return cfg, gamma
    raise KeyError(name)


def initial_macros(cfg, gamma):
    """A flowing start with the heated solid hot for the thermal case (from rest,
    no heat reaches any column within the run); rest for the others."""
    if cfg.lattice != G.D2Q9_D2Q5:
        return None
    m = np.zeros((cfg.ncells, 4))
    m[:, 0] = 1.0
    m[:, 1] = 0.03 * gamma
    m[:, 3] = 1.0 - gamma
    return m.ravel()


NAMES = ["d2q9_pressure_drop", "d2q9_outflow", "d2q9_dissipation", "d2q9_through_flow_y_faces",
         "d2q9_rotated_channel", "d3q19_pressure_drop", "thermal_heat_flux"]


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [G.STORE_FP64, G.STORE_FP32, G.STORE_FP16],
                         ids=["fp64", "fp32", "fp16"])
@pytest.mark.parametrize("name", NAMES)
def test_noalloc_objective_matches_the_oracle(nlib, orc, name, storage):
    pytest.importorskip("torch")
    cfg, gamma = case(name, storage)
    n = 200
    f, _, _ = orc.forward(cfg.replace(storage=G.STORE_FP64), gamma, n,
                          initial_macros(cfg, gamma))
    tol = 1e-12 if storage == G.STORE_FP64 else 1e-5
    gam = gamma if storage == G.STORE_FP64 else gamma.astype(np.float32).astype(np.float64)
    # t = n: the boundaries of step n are applied on load.  The boundary cells'
    # unknown populations are perturbed first: the boundary overwrites them.
    q = cfg.npop
    fp = f.reshape(cfg.ncells, q).copy()
    for b in cfg.bcs:
        if b.kind in (G.BC_VELOCITY, G.BC_PRESSURE) and cfg.lattice != G.D3Q19:
            x0, x1, y0, y1 = b.box[:4]
            for y in range(y0, y1 + 1):
                for x in range(x0, x1 + 1):
                    fp[y * cfg.nx + x, UNKNOWN[b.face]] += 1e-3
    planes, held = _stored(cfg, fp.ravel())
    vals = _noalloc(nlib, cfg, n, planes, gamma, check_memory=True)
    c64 = cfg.replace(storage=G.STORE_FP64)
    ref = orc.objective(c64, orc.apply_bcs(c64, held, n), gam)
    for v in vals:
        assert abs(v - ref) <= tol * max(abs(ref), 1e-30), (v, ref)
    # t = 0: no boundary applied, the objective of the populations as given
    vals0 = _noalloc(nlib, cfg, 0, planes, gamma)
    ref0 = orc.objective(cfg.replace(storage=G.STORE_FP64), held, gam)
    for v in vals0:
        assert abs(v - ref0) <= tol * max(abs(ref0), 1e-30), (v, ref0)


@pytest.mark.gpu
def test_noalloc_at_the_block_limit(nlib, orc):
    """The largest request the scratch holds: 32,768 thread blocks (a 3 x 8 x
    32768 D3Q19 lattice: blocks of 32 x 8 threads, one per z layer)."""
    pytest.importorskip("torch")
    cfg, gamma, _ = W.workload_duct_256x128x128(G.STORE_FP32, nx=3, ny=8, nz=32768, nsteps=1)
    # uniform inflow: a parabolic one would need 6 x 32766 profile values
    cfg.bcs[0] = G.Boundary(G.BC_VELOCITY, G.FACE_WEST, cfg.bcs[0].box, 0.04)
    # a density falling along x (the pressure drop between the x = 0 and x = 2
    # faces is then well conditioned), with some noise on top
    x = np.arange(cfg.ncells) % cfg.nx
    f0 = W3[None, :] * (1.0 + 0.01 * (2 - x)[:, None])
    f0 = (f0 * (1 + 0.001 * np.sin(np.arange(f0.size)).reshape(f0.shape))).ravel()
    planes, held = _stored(cfg, f0)
    vals = _noalloc(nlib, cfg, 0, planes, gamma)
    ref = orc.objective(cfg.replace(storage=G.STORE_FP64), held,
                        gamma.astype(np.float32).astype(np.float64))
    for v in vals:
        assert abs(v - ref) <= 1e-5 * abs(ref), (v, ref)


def _reject(lib, cfg):
    out = C.c_double(0.0)
    # the pointers are never touched: the request is refused before any device call
    return lib.lbm_objective_noalloc(C.byref(cfg.to_c()), 1, C.c_void_p(256), C.c_void_p(256),
                                     C.pointer(out), None)


def test_noalloc_rejects_one_block_too_many(nlib):
    cfg, _, _ = W.workload_duct_256x128x128(G.STORE_FP32, nx=3, ny=8, nz=32769, nsteps=10)
    assert _reject(nlib, cfg) == G.ERR_ARG
    assert b"thread blocks" in nlib.lbm_last_error(None)
    # fewer cells than 8,388,608 but more blocks than the scratch holds: the
    # limit is on blocks (257 columns take two 256-wide blocks per row)
    cfg2 = W.channel_2d(257, 32640, nsteps=10)
    assert cfg2.ncells < 8388608
    assert _reject(nlib, cfg2) == G.ERR_ARG


def test_noalloc_rejects_too_many_profile_entries(nlib):
    """More tabulated inflow-profile values than the scratch holds (32,768):
    five parabolic velocity boundaries of 6,600 cells each."""
    ny = 6602
    cfg = W.channel_2d(8, ny, nsteps=10)
    box = (0, 0, 1, ny - 2, 0, 0)
    cfg = cfg.replace(bcs=[G.Boundary(G.BC_VELOCITY, G.FACE_WEST, box, 0.01, G.PROFILE_PARABOLIC)
                           for _ in range(5)])
    assert _reject(nlib, cfg) == G.ERR_ARG
    assert b"profile" in nlib.lbm_last_error(None)


def test_noalloc_refuses_tabulated_profiles(nlib):
    cfg = W.pump_2d(36)
    assert _reject(nlib, cfg) == G.ERR_SUP
