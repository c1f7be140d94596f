"""The design-update oracle (oracle/design_oracle.c) on the CPU: its MMA
against the reference's own MMA.cc (golden trajectories made by the reference
build, and the reference build itself where present), and its density filter
and projection against their defining properties (row normalisation, box and
boundary handling, exact transposes, central differences).  Runs without a GPU."""
import os

import numpy as np
import pytest

import design_lib as D

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("kind", ["plain", "minmax"])
def test_mma_matches_reference_trajectory(kind):
    """30 MMA iterations (asymptotes adapting, move limit 0.1) of a plain
    volume-constrained problem and of the reference's min-max form: the
    oracle's iterates equal the reference MMA's within 1e-10."""
    gold = np.load(os.path.join(GOLD, "mma_%s.npz" % kind))
    xs, chs = D.mma_trajectory(D.OracleMMA, kind)
    assert np.abs(xs - gold["x"]).max() < 1e-10
    assert np.allclose(chs, gold["change"], rtol=1e-6, atol=1e-11)
    if D.reference_mma_available():   # the reference build itself, another seed and size
        for seed in (5, 9):
            a, _ = D.mma_trajectory(D.OracleMMA, kind, n=137, seed=seed, iters=12, movlim=0.2)
            b, _ = D.mma_trajectory(D.ReferenceMMA, kind, n=137, seed=seed, iters=12, movlim=0.2)
            assert np.abs(a - b).max() < 1e-10


def test_mma_solves_the_problem():
    """The plain problem's KKT point: the volume constraint is active and the
    trajectory has settled."""
    xs, chs = D.mma_trajectory(D.OracleMMA, "plain", iters=60)
    assert abs(xs[-1].mean() - 0.4) < 1e-6
    assert chs[-1] < 1e-6


CHAINS = {
    "2d_one_stage": (20, 14, 1, [(3, (4, 15, 2, 11, 0, 0), 1, 2.0, 0.5)]),
    "2d_two_stages": (22, 13, 1, [(4, (3, 18, 1, 11, 0, 0), 1, 2.0, 0.5),
                                  (2, (3, 18, 1, 11, 0, 0), 1, 1.0, 0.3)]),
    "2d_filter_only": (15, 9, 1, [(2, (0, 14, 0, 8, 0, 0), 0, 1.0, 0.5)]),
    "3d_one_stage": (10, 8, 7, [(2, (2, 7, 1, 6, 1, 5), 1, 3.0, 0.5)]),
}


@pytest.mark.parametrize("name", sorted(CHAINS))
def test_filter_chain_properties(name):
    nx, ny, nz, stages = CHAINS[name]
    ch = D.make_chain(nx, ny, nz, stages)
    rng = np.random.default_rng(11)
    n = nx * ny * nz
    x = rng.uniform(0, 1, n)
    g = D.filter_forward(ch, x)
    # a constant field stays constant through the filter, projections map [0,1] into [0,1]
    if not any(s[2] for s in stages):
        assert np.allclose(D.filter_forward(ch, np.full(n, 0.37)), 0.37, atol=1e-15)
    assert g.min() >= -1e-15 and g.max() <= 1 + 1e-15
    # cells outside every stage's box are untouched
    box = stages[0][1]
    xx, yy, zz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    inside = np.zeros((nx, ny, nz), bool)
    for s in stages:
        b = s[1]
        inside |= (xx >= b[0]) & (xx <= b[1]) & (yy >= b[2]) & (yy <= b[3]) & (zz >= b[4]) & (zz <= b[5])
    out = ~inside.transpose(2, 1, 0).reshape(-1)
    assert np.array_equal(g[out], x[out])
    # the transpose is the exact adjoint of the linearised chain: central differences
    s = rng.standard_normal(n)
    grad = D.filter_transpose(ch, x, s)
    for c in rng.choice(n, 12, replace=False):
        h = 1e-6
        xp, xm = x.copy(), x.copy()
        xp[c] += h
        xm[c] -= h
        fd = (s @ D.filter_forward(ch, xp) - s @ D.filter_forward(ch, xm)) / (2 * h)
        assert abs(fd - grad[c]) <= 1e-7 * max(1.0, abs(grad[c])), (c, fd, grad[c])


def test_filter_weights_by_hand():
    """A single interior unit impulse through a radius-2 filter: the cone
    weights R - |d| (zero at |d| = R) divided by the row sums."""
    nx, ny = 9, 9
    ch = D.make_chain(nx, ny, 1, [(2, (0, 8, 0, 8, 0, 0), 0, 1.0, 0.5)])
    x = np.zeros(nx * ny)
    x[4 * nx + 4] = 1.0
    g = D.filter_forward(ch, x).reshape(ny, nx)
    offs = [(dx, dy) for dx in range(-2, 3) for dy in range(-2, 3)]
    wsum = sum(max(0.0, 2 - np.hypot(dx, dy)) for dx, dy in offs)
    assert abs(g[4, 4] - 2.0 / wsum) < 1e-15
    assert abs(g[4, 5] - (2 - 1.0) / wsum) < 1e-15
    assert abs(g[5, 5] - (2 - np.sqrt(2.0)) / wsum) < 1e-15
    assert g[4, 6] == 0.0 and g[6, 6] == 0.0
