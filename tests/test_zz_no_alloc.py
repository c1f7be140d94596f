"""lbm_objective_noalloc: the objective of a caller-owned device state computed
without any device allocation, for applications that reserve all of their
device memory themselves or may not call cudaMalloc at that point (fixed
memory budgets, real-time loops).

The caller's buffers here are made with torch (the test may allocate; the
entry point may not).  The state comes from the existing entry points: a
handle runs the forward sweep with lbm_forward (per-step objective) and hands
its populations out with lbm_get_populations; they are laid out in the
handle's SoA form in a torch buffer, and two calls in a row of the new entry
point must reproduce lbm_forward's objective of that step: within 1e-12
relative for FP64 storage, 1e-5 for FP32.  This file is collected last so a
failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

import lbmgpu as G
import workloads as W

pytestmark = pytest.mark.gpu

W2 = np.array([4 / 9, 1 / 36, 1 / 9, 1 / 36, 1 / 9, 1 / 36, 1 / 9, 1 / 36, 1 / 9])
W3 = np.array([1 / 3] + [1 / 18] * 3 + [1 / 36] * 6 + [1 / 18] * 3 + [1 / 36] * 6)


def _soa(cfg, f_aos):
    """Host AoS FP64 populations -> the handle's device layout (planes of P)."""
    n, q = cfg.ncells, cfg.npop
    P = (n + 127) // 128 * 128
    f = f_aos.reshape(n, q)
    if cfg.storage != G.STORE_FP64:
        w = W3 if cfg.lattice == G.D3Q19 else W2
        f = f.copy()
        f[:, :len(w)] -= w          # shifted storage holds f_i - w_i
    planes = np.zeros((q, P))
    planes[:, :n] = f.T
    return planes


def _noalloc(lib, cfg, t, f_aos, gamma):
    import torch
    dt = {G.STORE_FP64: torch.float64, G.STORE_FP32: torch.float32,
          G.STORE_FP16: torch.float16}[cfg.storage]
    gdt = torch.float64 if cfg.storage == G.STORE_FP64 else torch.float32
    fd = torch.from_numpy(_soa(cfg, f_aos)).to(dtype=dt, device="cuda").contiguous()
    gd = torch.from_numpy(np.asarray(gamma, dtype=np.float64)).to(dtype=gdt, device="cuda")
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    c = cfg.to_c()
    vals = []
    for k in range(2):   # two calls in a row share the same scratch
        rc = lib.lbm_objective_noalloc(C.byref(c), int(t), C.c_void_p(fd.data_ptr()),
                                       C.c_void_p(gd.data_ptr()),
                                       C.cast(C.c_void_p(out.data_ptr() + 8 * k),
                                              C.POINTER(C.c_double)), None)
        assert rc == 0, lib.lbm_last_error(None).decode()
    torch.cuda.synchronize()
    vals = out.cpu().numpy()
    return vals


@pytest.fixture(scope="module")
def nlib():
    lib = G.load_library()
    lib.lbm_objective_noalloc.restype = C.c_int
    lib.lbm_objective_noalloc.argtypes = [C.POINTER(G.CConfig), C.c_int, C.c_void_p, C.c_void_p,
                                          C.POINTER(C.c_double), C.c_void_p]
    return lib


@pytest.mark.parametrize("case,storage,tol", [
    ("d2q9", G.STORE_FP64, 1e-12),
    ("d2q9", G.STORE_FP32, 1e-5),
    ("d3q19", G.STORE_FP64, 1e-12),
    ("d3q19", G.STORE_FP32, 1e-5),
])
def test_noalloc_objective_matches_forward(nlib, case, storage, tol):
    pytest.importorskip("torch")
    if case == "d2q9":
        cfg = W.channel_2d(64, 32, amp=0.2, period=40.0, nsteps=60, storage=storage)
        gamma = W.design_2d(64, 32, 77)
    else:
        cfg, gamma, _ = W.workload_duct_256x128x128(storage, nx=24, ny=12, nz=12, nsteps=60)
    n = 60
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        _, js = h.forward(n, per_step=True)
        f = h.populations()
    vals = _noalloc(nlib, cfg, n, f, gamma)
    ref = js[-1]
    for v in vals:
        assert abs(v - ref) <= tol * max(abs(ref), 1e-30), (v, ref)


def test_noalloc_rejects_oversized_lattice(nlib):
    pytest.importorskip("torch")
    import torch
    cfg, _, _ = W.workload_duct_256x128x128(G.STORE_FP32, nx=512, ny=256, nz=128, nsteps=10)
    dummy = torch.zeros(1, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    c = cfg.to_c()
    rc = nlib.lbm_objective_noalloc(C.byref(c), 1, C.c_void_p(dummy.data_ptr()),
                                    C.c_void_p(dummy.data_ptr()),
                                    C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_double)), None)
    assert rc == -1
    assert "thread blocks" in nlib.lbm_last_error(None).decode()
