"""The C ABI without a GPU: the library loads, exports every entry point that
include/lbmgpu.h declares, fills reference defaults, rejects bad
configurations before touching a device, and fails loudly (no CPU fallback)
when there is no CUDA device."""
import ctypes as C
import os
import re
import subprocess

import pytest

import lbmgpu as G
import workloads as W
from conftest import HAS_GPU

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lbmgpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(lbm_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_the_api():
    names = declared_functions()
    for n in ("lbm_create", "lbm_destroy", "lbm_forward", "lbm_adjoint_step", "lbm_gradient",
              "lbm_objective_noalloc", "lbm_autotune"):
        assert n in names


def test_library_exports_every_declared_function(lib):
    for n in declared_functions():
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", G.LIB_PATH], capture_output=True, text=True)
    if out.returncode == 0:
        exported = set(re.findall(r"\sT\s(lbm_\w+)", out.stdout))
        assert set(declared_functions()) <= exported


def test_config_defaults(lib):
    c = G.CConfig()
    lib.lbm_config_default(C.byref(c))
    assert (c.lattice, c.collision, c.storage) == (G.D2Q9, G.BGK, G.STORE_FP64)
    assert c.omega == 1.0 and c.interp_scale == 1.0 and c.interp_q == 1.0
    assert list(c.mrt) == list(G.MRT3D_DEFAULT)       # MRT3d_Compile_constants


@pytest.mark.parametrize("bad,code", [
    (dict(omega=2.5), -1),
    (dict(nx=2), -1),
    (dict(interp_q=0.0), -1),
    (dict(storage=7), -1),
    (dict(lattice=9), -1),
])
def test_bad_configs_rejected_before_any_device_call(lib, bad, code):
    cfg = W.channel_2d(16, 8).replace(**bad)
    h = C.c_void_p()
    rc = lib.lbm_create(C.byref(cfg.to_c()), C.byref(h))
    assert rc == code
    assert lib.lbm_last_error(None)


def test_bad_boundary_boxes_rejected(lib):
    cfg = W.channel_2d(16, 8)
    cfg.bcs[0].box = (1, 1, 1, 6, 0, 0)        # a west velocity box off the west face
    h = C.c_void_p()
    assert lib.lbm_create(C.byref(cfg.to_c()), C.byref(h)) == -1
    cfg = W.channel_2d(16, 8)
    cfg.bcs[1].box = (15, 15, 1, 8, 0, 0)       # past the lattice
    assert lib.lbm_create(C.byref(cfg.to_c()), C.byref(h)) == -1
    cfg3 = W.duct_3d(8, 6, 6)
    cfg3.bcs[0].face = G.FACE_EAST               # unsupported Hecht face
    cfg3.bcs[0].box = (7, 7, 1, 4, 1, 4)
    assert lib.lbm_create(C.byref(cfg3.to_c()), C.byref(h)) == -2


def test_unsupported_combinations(lib):
    h = C.c_void_p()
    cfg = W.thermal_2d(16, 8).replace(collision=G.MRT)
    assert lib.lbm_create(C.byref(cfg.to_c()), C.byref(h)) == -2
    cfg = W.channel_2d(16, 8).replace(objective=G.OBJ_HEAT_FLUX)
    assert lib.lbm_create(C.byref(cfg.to_c()), C.byref(h)) == -2


def test_no_device_fails_loudly(lib):
    if HAS_GPU:
        pytest.skip("a CUDA device is present")
    h = C.c_void_p()
    rc = lib.lbm_create(C.byref(W.channel_2d(16, 8).to_c()), C.byref(h))
    assert rc == -3
    assert b"CUDA" in lib.lbm_last_error(None)
    with pytest.raises(G.LBMError):
        G.Handle(W.channel_2d(16, 8))


def test_wang_schedule_argument_checks(lib):
    r = C.c_int64()
    assert lib.lbm_wang_recompute_count(10, 1, C.byref(r)) == -1
    assert lib.lbm_wang_recompute_count(0, 4, C.byref(r)) == -1
    assert lib.lbm_wang_recompute_count(10, 11, C.byref(r)) == 0 and r.value == 0


def test_seeded_workloads_are_reproducible():
    a = W.design_3d(16, 8, 8, 7)
    b = W.design_3d(16, 8, 8, 7)
    assert (a == b).all() and a.min() >= 0.0 and a.max() <= 1.0
    g = W.design_2d(128, 64, W.SEED_BASE + 1)
    assert g.shape == (128 * 64,) and 0.0 <= g.min() and g.max() <= 1.0
    cfg, gamma, n = W.workload_channel_128x64()
    assert (cfg.nx, cfg.ny, n) == (128, 64, 2000)
    assert abs(cfg.omega - 1.25) < 1e-15 and abs(cfg.interp_scale - 0.1) < 1e-15
    insts, n5 = W.workload_batch_8_channels(scale=8)
    assert len(insts) == 8 and n5 == 4000
    p = W.tanh_projection(np.linspace(0, 1, 11), 8.0, 0.5)
    assert abs(p[0]) < 1e-15 and abs(p[-1] - 1.0) < 1e-15


import numpy as np  # noqa: E402


def handle_functions():
    """Entry points whose first argument is a handle, batch or design-update
    object."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(
        r"^\s*(?:int|const char\*)\s+(lbm_\w+)\s*\(\s*(?:const\s+)?lbm_(?:handle|batch|topopt)\s*\*",
        src, flags=re.M)))


def test_null_handles_are_argument_errors(lib):
    """Like a PETSc call on a null object: every entry point given a null
    handle returns LBM_ERR_ARG (-1) with a message and touches nothing;
    destroying a null handle is a no-op."""
    names = handle_functions()
    assert len(names) >= 50
    for n in names:
        f = getattr(lib, n)
        assert f.argtypes is not None, n
        args = [0.0 if t in (C.c_double, C.c_float) else
                0 if t in (C.c_int, C.c_int64, C.c_uint, C.c_size_t) else None
                for t in f.argtypes]
        r = f(*args)
        if n.endswith("_last_error"):
            assert isinstance(r, bytes) and r, n
        elif n.endswith("_destroy"):
            assert r == 0, n
        else:
            assert r == -1, (n, r)
