"""Batched lattices (one launch per time step for all, optional CUDA graph):
each lattice's objective and dJ/dgamma equal the single-lattice path's and the
oracle's (FP64 within 1e-12), graph replays reproduce the captured run
bit for bit, and uneven sizes and objectives mix in one batch."""
import numpy as np
import pytest

import lbmgpu as G
import workloads as W
from helpers import rel_inf

pytestmark = pytest.mark.gpu


def uneven_2d(storage=G.STORE_FP64, n=60):
    out = []
    for k, (nx, ny) in enumerate([(48, 24), (37, 19), (64, 32)]):
        cfg = W.channel_2d(nx, ny, storage=storage, nsteps=n, amp=0.1 * k, period=30.0)
        if k == 1:
            cfg = cfg.replace(objective=G.OBJ_OUTFLOW)
        out.append((cfg, W.design_2d(nx, ny, 900 + k)))
    return out


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_gradient_matches_single_and_oracle(orc, use_graph):
    n = 60
    insts = uneven_2d(n=n)
    with G.Batch([c for c, _ in insts]) as b:
        for i, (_, g) in enumerate(insts):
            b[i].set_design(g)
        J, sens, st = b.gradient(n, 7, use_graph=use_graph)
        if use_graph:   # replay of the captured graph
            J2, sens2, _ = b.gradient(n, 7, use_graph=True)
            assert np.array_equal(J, J2)
            for a, c in zip(sens, sens2):
                assert np.array_equal(a, c)
    assert st.recomputed_steps == G.wang_recompute_count(n, 7)
    for i, (cfg, g) in enumerate(insts):
        with G.Handle(cfg) as h:
            h.set_design(g)
            Js, ss, _ = h.gradient(n, 7)
        Jo, so = orc.gradient(cfg, g, n)
        assert abs(J[i] - Js) <= 1e-12 * abs(Js)
        assert rel_inf(sens[i], ss) < 1e-12
        assert rel_inf(sens[i], so) < 1e-12


def test_batch_forward_matches_single(orc):
    insts = uneven_2d(n=40)
    with G.Batch([c for c, _ in insts]) as b:
        for i, (_, g) in enumerate(insts):
            b[i].set_design(g)
            b[i].init_equilibrium()
        J = b.forward(40)
        fs = [b[i].populations() for i in range(len(insts))]
    for i, (cfg, g) in enumerate(insts):
        fo, _, Jo = orc.forward(cfg, g, 40)
        assert rel_inf(fs[i], fo) < 1e-12
        # the outflow objective of a 40-step start-up is a near-cancelling sum
        # (|J| ~ 2e-9): the block-partial order differs between grids, so the
        # bound gets an absolute floor of 1e-15
        assert abs(J[i] - Jo) <= 1e-12 * abs(Jo) + 1e-15


def test_batch_d3q19_fp32_autotuned():
    cfgs, gs = [], []
    for k, (nx, ny, nz) in enumerate([(32, 16, 16), (24, 12, 12)]):
        cfg, g, _ = W.workload_duct_256x128x128(G.STORE_FP32, nx=nx, ny=ny, nz=nz, nsteps=40)
        cfgs.append(cfg)
        gs.append(g)
    with G.Batch(cfgs) as b:
        for i, g in enumerate(gs):
            b[i].set_design(g)
        shape = b.autotune(2)
        assert shape[0] * shape[1] in (64, 128, 256)
        rshape = b.reverse_shape()
        assert rshape[0] * rshape[1] in (64, 128, 256) and rshape[0] % 32 == 0
        J, sens, _ = b.gradient(40, 5)
    for cfg, g, Jb, sb in zip(cfgs, gs, J, sens):
        with G.Handle(cfg) as h:
            h.set_design(g)
            Js, ss, _ = h.gradient(40, 5)
        assert abs(Jb - Js) <= 1e-5 * abs(Js)
        assert rel_inf(sb, ss) < 1e-4


def test_batch_reverse_variant_does_not_change_results():
    """As for a single lattice: the batched reverse step's two register
    variants agree to FP32 rounding."""
    insts = uneven_2d(storage=G.STORE_FP32, n=50)
    out = []
    for lean in (0, 1):
        with G.Batch([c for c, _ in insts]) as b:
            b.set_reverse_variant(lean)
            assert b.reverse_variant == lean
            for i, (_, g) in enumerate(insts):
                b[i].set_design(g)
            out.append(b.gradient(50, 6, use_graph=True))
    assert np.allclose(out[0][0], out[1][0], rtol=1e-12, atol=0)
    for a, c in zip(out[0][1], out[1][1]):
        assert np.abs(a - c).max() <= 1e-7 * np.abs(a).max()


def test_batch_launch_shape_does_not_change_results():
    """Every shape the batch tuner may pick gives the same FP32 gradient bit
    for bit (rounding streams are keyed by cell and step); shapes outside the
    tuner's set are refused."""
    n = 40
    insts = uneven_2d(storage=G.STORE_FP32, n=n)
    out = []
    for fwd, rev in (((128, 2), (128, 2)), ((256, 1), (32, 4)), ((32, 8), (64, 2))):
        with G.Batch([c for c, _ in insts]) as b:
            for i, (_, g) in enumerate(insts):
                b[i].set_design(g)
            b.set_reverse_variant(0)
            b.set_launch_shape(0, *fwd)
            b.set_launch_shape(1, *rev)
            assert b.reverse_shape() == rev
            J, sens, _ = b.gradient(n, 7, use_graph=True)
            out.append((J, sens))
            with pytest.raises(G.LBMError, match="not one of the tuner's shapes"):
                b.set_launch_shape(0, 96, 2)
    for J, sens in out[1:]:
        assert np.array_equal(J, out[0][0])
        for a, c in zip(sens, out[0][1]):
            assert np.array_equal(a, c)
