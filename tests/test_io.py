"""File formats (core/binaryIO.cc, LBSolver::outputMacros): PETSc binary Vec
files byte for byte, and .vts files read back by an independent parser.  The
CPU tests need no GPU; the last test writes a handle's macros on the GPU."""
import os
import struct

import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from vts_reader import read_vts


def test_petsc_vec_layout_and_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    v = np.concatenate([rng.standard_normal(37), [0.0, -0.0, 1e-300, np.inf, -np.inf]])
    p = str(tmp_path / "design.bin")
    G.write_petsc_vec(p, v)
    raw = open(p, "rb").read()
    assert len(raw) == 8 + 8 * v.size
    assert struct.unpack(">ii", raw[:8]) == (1211214, v.size)
    assert np.array_equal(np.frombuffer(raw[8:], dtype=">f8"), v)
    back = G.read_petsc_vec(p)
    assert back.tobytes() == v.tobytes()


def test_petsc_vec_rejects_other_files(tmp_path):
    p = str(tmp_path / "bad.bin")
    with open(p, "wb") as f:
        f.write(struct.pack(">ii", 1211216, 3) + b"\0" * 24)   # a Mat class id
    with pytest.raises(G.LBMError):
        G.read_petsc_vec(p)
    with open(p, "wb") as f:
        f.write(struct.pack(">ii", 1211214, 10) + b"\0" * 16)  # truncated
    with pytest.raises(G.LBMError):
        G.read_petsc_vec(p)


@pytest.mark.parametrize("dims", [(7, 5, 1), (4, 3, 6)])
def test_vts_round_trip(tmp_path, dims):
    n = int(np.prod(dims))
    rng = np.random.default_rng(2)
    fields = {"rho": rng.standard_normal(n), "velocity": rng.standard_normal(3 * n)}
    p = str(tmp_path / "f.vts")
    G.write_vts(p, dims, fields)
    d, out = read_vts(p)
    assert d == dims
    assert np.array_equal(out["rho"], fields["rho"])
    assert np.array_equal(out["velocity"].reshape(-1), fields["velocity"])
    pts = out["Points"]
    c = np.arange(n)
    assert np.array_equal(pts[:, 0], c % dims[0])
    assert np.array_equal(pts[:, 1], (c // dims[0]) % dims[1])
    assert np.array_equal(pts[:, 2], c // (dims[0] * dims[1]))


@pytest.mark.gpu
def test_handle_vts_holds_its_macros(tmp_path):
    cfg = W.channel_2d(30, 12, nsteps=50)
    gamma = W.design_2d(30, 12, 5)
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        h.forward(50)
        assert h.dims() == (30, 12, 1)
        mac = h.macros().reshape(-1, 3)
        p = str(tmp_path / "m.vts")
        h.write_vts(p, gamma)
    d, out = read_vts(p)
    assert d == (30, 12, 1)
    assert np.array_equal(out["rho"], mac[:, 0])
    assert np.array_equal(out["velocity"][:, :2], mac[:, 1:])
    assert np.all(out["velocity"][:, 2] == 0)
    assert np.array_equal(out["gamma"], gamma)
