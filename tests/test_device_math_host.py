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
    lib.dev_collide_inc.argtypes = [C.POINTER(G.CConfig), C.c_int, dp, C.c_double, dp, dp]
    lib.dev_reverse_inc.argtypes = [C.POINTER(G.CConfig), C.c_int, dp, C.c_double, dp, dp, dp]
    lib.dev_round.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, C.c_uint, dp]
    lib.dev_round.restype = None
    lib.dev_batch_div.argtypes = [C.c_uint, C.c_uint, C.c_ulonglong]
    lib.dev_batch_div.restype = C.c_uint
    lib.dev_batch_div_magic.argtypes = [C.c_ulonglong, C.c_ulonglong]
    lib.dev_batch_div_magic.restype = C.c_uint
    lib.dev_bp.argtypes = [C.c_int, C.c_double, C.c_double, dp]
    lib.dev_bp.restype = None
    lib.dev_round_pair.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, C.c_uint, dp]
    lib.dev_round_pair.restype = None
    ip = C.POINTER(C.c_int)
    lib.dev_mrt3d_table.argtypes = [ip, ip]
    lib.dev_mrt3d_table.restype = None
    lib.dev_mrt3d_moments.argtypes = [dp, dp]
    lib.dev_mrt3d_moments.restype = None
    lib.dev_mrt3d_back.argtypes = [dp, dp]
    lib.dev_mrt3d_back.restype = None
    lib.dev_mrt3d_rows_t.argtypes = [dp, dp]
    lib.dev_mrt3d_rows_t.restype = None
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


@pytest.mark.parametrize("name", sorted(CASES))
def test_increment_form_matches_oracle(devmath, orc, name):
    """The FP32/FP16 storage path computes the collision (and, for BGK and the
    thermal model, its transpose) as increments: f + d must be the same
    operator (FP64 instantiation within 1e-14, FP32 within 5e-6)."""
    cfg = CASES[name]
    c = cfg.to_c()
    dp = C.POINTER(C.c_double)
    rng = np.random.default_rng(hash(name) % 2**32 + 1)
    for _ in range(20):
        fin, g, lo = _inputs(cfg, rng)
        fo, _ = orc.collide_cell(cfg, fin, g)
        li_o, dg_o = orc.reverse_cell(cfg, fin, g, lo)
        for fp32, tol in ((0, 1e-14), (1, 5e-6)):
            out = np.zeros(cfg.npop)
            sums = np.zeros(5)
            devmath.dev_collide_inc(C.byref(c), fp32, fin.ctypes.data_as(dp), g,
                                    out.ctypes.data_as(dp), sums.ctypes.data_as(dp))
            assert rel_inf(out, fo) < tol, (name, fp32, rel_inf(out, fo))
            if cfg.collision != G.BGK:
                continue
            li = np.zeros(cfg.npop)
            dg = np.zeros(1)
            rc = devmath.dev_reverse_inc(C.byref(c), fp32, fin.ctypes.data_as(dp), g,
                                         lo.ctypes.data_as(dp), li.ctypes.data_as(dp),
                                         dg.ctypes.data_as(dp))
            assert rc == 0
            assert rel_inf(li, li_o) < tol * 10, (name, fp32, rel_inf(li, li_o))
            assert abs(dg[0] - dg_o) <= tol * 10 * max(abs(dg_o), np.abs(lo).max() * 1e-3)


@pytest.mark.parametrize("name", ["d2q9_bgk", "d2q9_mrt", "d3q19_bgk", "d3q19_mrt"])
def test_increments_conserve_mass_and_momentum(devmath, orc, name):
    """In a fluid cell (gamma = 1, no partial bounce-back) the FP32 increments
    carry no mass and no momentum up to their own rounding: near equilibrium
    |sum d| stays below 1e-6 of the largest increment, far below the rounding
    of f itself that the plain form leaves in them."""
    cfg = CASES[name]
    c = cfg.to_c()
    dp = C.POINTER(C.c_double)
    rng = np.random.default_rng(7)
    for _ in range(20):
        fin, _, _ = _inputs(cfg, rng)
        feq, _ = orc.collide_cell(cfg.replace(omega=1.0), fin, 1.0)   # the equilibrium of fin
        fin = feq + 1e-4 * feq * rng.standard_normal(len(feq))        # small non-equilibrium part
        out = np.zeros(cfg.npop)
        sums = np.zeros(5)
        devmath.dev_collide_inc(C.byref(c), 1, fin.ctypes.data_as(dp), 1.0,
                                out.ctypes.data_as(dp), sums.ctypes.data_as(dp))
        assert sums[4] > 0
        assert np.abs(sums[:4]).max() < 1e-6 * sums[4], (name, sums)


@pytest.mark.parametrize("half", [0, 1])
def test_stochastic_rounding_is_unbiased(devmath, half):
    """Round<S>::apply(f, d) takes one of the two representable neighbours of
    f + d, and over many cells its mean is f + d: round to nearest would be
    off by the same fraction of a unit every time."""
    n = 200000
    out = np.zeros(n)
    dp = C.POINTER(C.c_double)
    dt = np.float16 if half else np.float32
    for f, d in ((0.0123456, 3.1e-7), (-0.0071, 2.2e-6), (0.3, -1.3e-8)):
        devmath.dev_round(half, f, d, n, 12345, out.ctypes.data_as(dp))
        x = float(np.float32(f)) + float(np.float32(d))   # f and d as the kernel holds them
        lo = float(dt(x))
        if lo > x:
            lo = float(np.nextafter(dt(x), dt(-np.inf)))
        hi = float(np.nextafter(dt(lo), dt(np.inf)))
        assert set(np.unique(out)) <= {lo, hi}, (f, d, np.unique(out)[:5])
        ulp = hi - lo
        assert abs(out.mean() - x) < 0.01 * ulp, (f, d, (out.mean() - x) / ulp)
        rn_err = abs(float(dt(x)) - x) / ulp
        assert rn_err > 0.05   # the cases are not trivially exact under round to nearest
    # Within one unit of a power of two the noise, scaled to one binade, spans
    # two or three neighbours; the mean stays within 0.25 units of the lower
    # binade (such values are 1 in 2^23 of FP32 and 1 in 2^10 of FP16 ones).
    for f, d in ((0.25, -1.3e-8), (0.5, -4e-9), (0.25, 1.3e-8)) if not half else \
            ((0.25, -1e-4), (0.25, 3e-5), (0.5, -2e-4)):
        devmath.dev_round(half, f, d, n, 999, out.ctypes.data_as(dp))
        x = float(np.float32(f)) + float(np.float32(d))
        ulp_lo = float(np.spacing(dt(min(abs(x), f) * 0.999)))
        assert abs(out.mean() - x) < 0.25 * ulp_lo, (f, d, (out.mean() - x) / ulp_lo)


def test_batch_block_division(devmath):
    """The batched kernels split a virtual block index with a multiply-high
    by ceil(2^32 / d), exact while n * d < 2^32; outside that bound (and for
    d = 1) the magic number is 0 and the kernel divides."""
    rng = np.random.default_rng(9)
    for d in list(range(1, 300)) + [int(v) for v in rng.integers(2, 1 << 16, 300)]:
        nmax = (1 << 32) // d
        m = devmath.dev_batch_div_magic(d, nmax)
        assert (m == 0) == (d == 1 or nmax * d >= (1 << 32))
        if d > 1:
            assert devmath.dev_batch_div_magic(d, nmax - 1) != 0
        lim = min(nmax - 1, (1 << 32) - 1)
        for n in [0, 1, d - 1, d, d + 1, lim, lim - d, lim // 2] + [int(v) for v in rng.integers(0, lim + 1, 40)]:
            if 0 <= n <= lim:
                assert devmath.dev_batch_div(n, d, lim + 1) == n // d, (n, d)


def test_porosity_interpolation(devmath):
    """BP_q(s) = 1 - s(1+q)/(q+s) (interpolationFunctions.hh:18-25): the FP32
    form q(1-s)/(q+s) is exactly 0 in fluid cells (s = 1) and 1 in solid
    ones, matches the FP64 value to FP32 rounding, and both derivatives match
    central differences of FP64."""
    dp = C.POINTER(C.c_double)
    out = np.zeros(2)
    for q in (0.1, 0.01, 1.0):
        devmath.dev_bp(1, 1.0, q, out.ctypes.data_as(dp))
        assert out[0] == 0.0
        devmath.dev_bp(1, 0.0, q, out.ctypes.data_as(dp))
        assert abs(out[0] - 1.0) < 1e-6
        for s in np.linspace(0, 1, 11):
            ref = np.zeros(2)
            devmath.dev_bp(0, s, q, ref.ctypes.data_as(dp))
            assert abs(ref[0] - (1 - s * (1 + q) / (q + s))) < 1e-15
            devmath.dev_bp(1, s, q, out.ctypes.data_as(dp))
            assert abs(out[0] - ref[0]) < 1e-6
            assert abs(out[1] - ref[1]) < 1e-6 * abs(ref[1])
            hi, lo = np.zeros(2), np.zeros(2)
            devmath.dev_bp(0, s + 1e-6, q, hi.ctypes.data_as(dp))
            devmath.dev_bp(0, s - 1e-6, q, lo.ctypes.data_as(dp))
            assert abs((hi[0] - lo[0]) / 2e-6 - ref[1]) < 1e-6 * abs(ref[1])


@pytest.mark.parametrize("half", [0, 1])
def test_pair_rounding_is_unbiased_and_uncorrelated(devmath, half):
    """Round<S>::apply_pair draws the noise of two populations from one step
    of the sequence: each output takes one of the two neighbours of f + d
    with mean f + d, and the two rounding errors of a cell are nearly
    uncorrelated over the cells (FP32 and FP16 storage)."""
    n = 200000
    out = np.zeros(2 * n)
    dp = C.POINTER(C.c_double)
    dt = np.float16 if half else np.float32
    cases = ((0.0123456, 3.1e-7), (-0.0071, 2.2e-6), (0.3, -1.3e-8)) if not half else \
        ((0.0123456, 3.1e-6), (-0.0071, 2.2e-6), (0.3, -1.3e-5))
    for f, d in cases:
        devmath.dev_round_pair(half, f, d, n, 4321, out.ctypes.data_as(dp))
        x = float(np.float32(f)) + float(np.float32(d))
        lo = float(dt(x))
        if lo > x:
            lo = float(np.nextafter(dt(x), dt(-np.inf)))
        hi = float(np.nextafter(dt(lo), dt(np.inf)))
        ulp = hi - lo
        a, b = out[0::2], out[1::2]
        for v in (a, b):
            assert set(np.unique(v)) <= {lo, hi}
            assert abs(v.mean() - x) < 0.01 * ulp, (f, d, (v.mean() - x) / ulp)
        assert abs(np.corrcoef(a, b)[0, 1]) < 0.02, np.corrcoef(a, b)[0, 1]


def test_factored_d3q19_moments_match_the_table(devmath):
    """The pair-form D3Q19 moments and back-map are written with shared
    sub-sums; row by row they must equal the moment table (MRT3d.hh:50-90):
    m = M f, the back-map -M^T diag(1/N) r split into the rest population,
    the pair sums (twice the even part) and differences, and the transposed
    even rows M_even^T m of the adjoint."""
    ip = C.POINTER(C.c_int)
    dp = C.POINTER(C.c_double)
    M = np.zeros((15, 19), dtype=np.int32)
    N = np.zeros(15, dtype=np.int32)
    devmath.dev_mrt3d_table(M.ctypes.data_as(ip), N.ctypes.data_as(ip))
    ex = np.array([0, 0, 0, -1, 0, 0, -1, 1, -1, 1, 0, 0, 1, 0, 0, 1, -1, 1, -1])
    ey = np.array([0, 0, -1, 0, -1, 1, 0, 0, -1, -1, 0, 1, 0, 1, -1, 0, 0, 1, 1])
    ez = np.array([0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 1, 0, 0, 1, 1, 1, 1, 0, 0])
    full = np.vstack([np.ones(19), ex, ey, ez, M]).astype(float)
    assert np.linalg.matrix_rank(full) == 19
    rng = np.random.default_rng(5)
    out = np.zeros(19)
    for _ in range(10):
        f = rng.standard_normal(19)
        devmath.dev_mrt3d_moments(f.ctypes.data_as(dp), out.ctypes.data_as(dp))
        assert np.abs(out - full @ f).max() < 1e-13
        r = rng.standard_normal(15)
        devmath.dev_mrt3d_back(r.ctypes.data_as(dp), out.ctypes.data_as(dp))
        back = -(M.T.astype(float) / N) @ r
        assert abs(out[0] - back[0]) < 1e-14
        assert np.abs(out[1:10] - (back[1:10] + back[10:19])).max() < 1e-14
        assert np.abs(out[10:19] - (back[1:10] - back[10:19])).max() < 1e-14
        m = rng.standard_normal(15)
        even = np.array([np.all(M[k, 1:10] == M[k, 10:19]) for k in range(15)])
        devmath.dev_mrt3d_rows_t(m.ctypes.data_as(dp), out.ctypes.data_as(dp))
        gt = M[even].T.astype(float) @ m[even]
        assert abs(out[0] - gt[0]) < 1e-13
        assert np.abs(out[1:10] - gt[1:10]).max() < 1e-13
