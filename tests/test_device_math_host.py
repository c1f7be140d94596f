"""The GPU kernels' per-cell collision operators and their transposes, built
for the host from the same source (tests/device_math_host.cpp stubs the CUDA
qualifiers), against the oracle: FP64 within 1e-14, FP32 within 5e-6 on
shifted-scale inputs.  Runs without a GPU."""
import ctypes as C
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from helpers import rel_inf

HERE = os.path.dirname(os.path.abspath(__file__))


def _cuda_include():
    for cand in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        inc = os.path.join(cand, "include") if cand else ""
        if inc and os.path.exists(os.path.join(inc, "cuda_fp16.h")):
            return inc
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
        if os.path.exists(os.path.join(inc, "cuda_fp16.h")):
            return inc
    return None


@pytest.fixture(scope="module")
def devmath():
    inc = _cuda_include()
    if inc is None or shutil.which("g++") is None:
        pytest.skip("needs g++ and the CUDA headers")
    d = tempfile.mkdtemp()
    so = os.path.join(d, "libdevmath.so")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-ffp-contract=off",
                           "-I" + inc, os.path.join(HERE, "device_math_host.cpp"), "-o", so])
    lib = C.CDLL(so)
    dp = C.POINTER(C.c_double)
    lib.dev_collide.argtypes = [C.POINTER(G.CConfig), C.c_int, dp, C.c_double, dp]
    lib.dev_reverse.argtypes = [C.POINTER(G.CConfig), C.c_int, dp, C.c_double, dp, dp, dp]
    return lib


CASES = {
    "d2q9_bgk": W.channel_2d(16, 8),
    "d2q9_mrt": W.channel_2d(16, 8, collision=G.MRT),
    "d3q19_mrt": W.duct_3d(8, 6, 6),
    "d3q19_mrt_default_rates": W.duct_3d(8, 6, 6).replace(mrt=G.MRT3D_DEFAULT),
    "d3q19_bgk": W.duct_3d(8, 6, 6).replace(collision=G.BGK),
    "thermal": W.thermal_2d(16, 8),
}


def _inputs(cfg, rng):
    L = {G.D2Q9: [4 / 9] + [1 / 36, 1 / 9] * 4,
         G.D3Q19: [1 / 3] + [1 / 18] * 3 + [1 / 36] * 6 + [1 / 18] * 3 + [1 / 36] * 6,
         G.D2Q9_D2Q5: [4 / 9] + [1 / 36, 1 / 9] * 4 + [1 / 3 * 0.4] + [1 / 6 * 0.4] * 4}[cfg.lattice]
    fin = np.array(L) * (1 + 0.05 * rng.standard_normal(len(L)))
    return fin, float(rng.uniform(0.02, 0.98)), rng.standard_normal(len(L))


@pytest.mark.parametrize("name", sorted(CASES))
def test_device_operators_match_oracle(devmath, orc, name):
    cfg = CASES[name]
    c = cfg.to_c()
    dp = C.POINTER(C.c_double)
    rng = np.random.default_rng(hash(name) % 2**32)
    for _ in range(20):
        fin, g, lo = _inputs(cfg, rng)
        fo, _ = orc.collide_cell(cfg, fin, g)
        li_o, dg_o = orc.reverse_cell(cfg, fin, g, lo)
        for fp32, tol in ((0, 1e-14), (1, 5e-6)):
            out = np.zeros(cfg.npop)
            devmath.dev_collide(C.byref(c), fp32, fin.ctypes.data_as(dp), g, out.ctypes.data_as(dp))
            assert rel_inf(out, fo) < tol, (name, fp32, rel_inf(out, fo))
            li = np.zeros(cfg.npop)
            dg = np.zeros(1)
            devmath.dev_reverse(C.byref(c), fp32, fin.ctypes.data_as(dp), g, lo.ctypes.data_as(dp),
                                li.ctypes.data_as(dp), dg.ctypes.data_as(dp))
            assert rel_inf(li, li_o) < tol * 10, (name, fp32, rel_inf(li, li_o))
            assert abs(dg[0] - dg_o) <= tol * 10 * max(abs(dg_o), np.abs(lo).max() * 1e-3), (name, fp32)
