"""The C++ facade (include/lbmgpu.hpp) used by a reference-style C++ driver
(tests/cpp_driver.cpp): it compiles against the C ABI here, and on a GPU its
objective, populations and dJ/dgamma equal the oracle's within 1e-12."""
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
ROOT = os.path.dirname(HERE)


def _build(name):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    d = tempfile.mkdtemp()
    exe = os.path.join(d, name)
    subprocess.check_call(["g++", "-std=c++14", "-O2", "-Wall", "-Werror",
                           os.path.join(HERE, name + ".cpp"), "-o", exe,
                           "-L" + os.path.dirname(G.LIB_PATH), "-llbmgpu",
                           "-Wl,-rpath," + os.path.dirname(G.LIB_PATH)])
    return exe, d


@pytest.fixture(scope="module")
def driver():
    return _build("cpp_driver")


@pytest.fixture(scope="module")
def pump_driver():
    return _build("cpp_pump_driver")


def test_cpp_driver_builds(driver):
    assert os.path.exists(driver[0])


def test_cpp_pump_driver_builds(pump_driver):
    assert os.path.exists(pump_driver[0])


@pytest.mark.gpu
def test_cpp_pump_driver_with_a_reference_style_input_functor(pump_driver, orc):
    """The pump set-up with the reference's InflowVelocity law as a C++ functor
    (tabulated by the facade) against the oracle given the same velocities."""
    exe, d = pump_driver
    n, nsteps, freq = 36, 150, 50
    gamma = W.design_2d(n, n, 32)
    path = os.path.join(d, "gamma.bin")
    gamma.tofile(path)
    out = subprocess.run([exe, str(n), str(nsteps), str(freq), path], capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = {ln.split()[0]: ln.split()[1:] for ln in out.stdout.splitlines()}
    J = float(lines["J"][0])
    sens = np.array([float(v) for v in lines["sens"]])
    cfg = W.pump_2d(n, nsteps=nsteps, period=float(freq))
    cfg.bcs[2] = G.Boundary(G.BC_VELOCITY, G.FACE_NORTH, cfg.bcs[2].box, 1.0, G.PROFILE_TABLE)
    th = n // 3
    x = np.arange(th + 1, 2 * th + 1, dtype=np.float64)
    mid, r = (n - 1) / 2.0, th / 2.0
    vec = np.zeros((freq, th, 2))
    for t in range(freq):
        vec[t, :, 1] = -np.sin(2.0 * np.pi * t / freq) * (0.05 * (r * r - (x - mid) ** 2)) / (r * r)
    orc.set_tables({2: vec})
    try:
        Jo, so = orc.gradient(cfg, gamma, nsteps)
    finally:
        orc.set_tables(None)
    assert abs(J - Jo) <= 1e-12 * abs(Jo)
    assert rel_inf(sens, so) < 1e-11


@pytest.mark.gpu
def test_cpp_driver_matches_oracle(driver, orc):
    exe, d = driver
    nx, ny, n = 40, 20, 150
    gamma = W.design_2d(nx, ny, 31)
    path = os.path.join(d, "gamma.bin")
    gamma.tofile(path)
    out = subprocess.run([exe, str(nx), str(ny), str(n), path], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    lines = {ln.split()[0]: ln.split()[1:] for ln in out.stdout.splitlines()}
    J, Jg = float(lines["J"][0]), float(lines["Jgrad"][0])
    sens = np.array([float(v) for v in lines["sens"]])
    f = np.array([float(v) for v in lines["f"]])
    cfg = W.channel_2d(nx, ny, nsteps=n)
    fo, _, Jo = orc.forward(cfg, gamma, n)
    Jgo, so = orc.gradient(cfg, gamma, n)
    assert abs(J - Jo) <= 1e-12 * abs(Jo)
    assert abs(Jg - Jgo) <= 1e-12 * abs(Jgo)
    assert rel_inf(f, fo) < 1e-12
    assert rel_inf(sens, so) < 1e-12
    assert int(lines["recomputed"][0]) == G.wang_recompute_count(n, 8)
    # LBStaticCheckpointing: same gradient bit for bit, the reference's recompute count
    assert lines["static_same"][0] == "1"
    assert int(lines["static_recomputed"][0]) == orc.static_count(n, 8)[0]
