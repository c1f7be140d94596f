"""The design update on the GPU (lbm_topopt_*) against the CPU oracle:

* filter + projection chains (one and two stages, 2D and 3D, a filter box
  inside the grid) and their transposes within 1e-13 of the oracle;
* MMA trajectories (plain and the reference's min-max form) within 1e-10 of
  the oracle, whose MMA equals the reference's MMA.cc (tests/golden);
* the whole chain design -> filters -> solver -> adjoint -> filters^T ->
  dJ/dx against central differences on a channel, FP64;
* a short optimisation loop lowers the objective and meets the volume
  constraint."""
import os

import numpy as np
import pytest

import design_lib as D
import lbmgpu as G
import workloads as W

pytestmark = pytest.mark.gpu


def box_mask(nx, ny, nz, b):
    x, y, z = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    m = (x >= b[0]) & (x <= b[1]) & (y >= b[2]) & (y <= b[3]) & (z >= b[4]) & (z <= b[5])
    return m.transpose(2, 1, 0).reshape(-1)


CHAINS = {
    "2d_one_stage": (26, 17, 1, (3, 22, 2, 14, 0, 0), [(3, True, 2.0, 0.5)]),
    "2d_two_stages": (30, 19, 1, (4, 25, 1, 17, 0, 0), [(4, True, 2.0, 0.5), (2, True, 1.0, 0.3)]),
    "2d_filter_only": (21, 12, 1, (0, 20, 0, 11, 0, 0), [(2, False, 1.0, 0.5)]),
    "3d_one_stage": (14, 10, 9, (2, 11, 1, 8, 1, 7), [(2, True, 3.0, 0.5)]),
}


@pytest.mark.parametrize("name", sorted(CHAINS))
def test_filter_chain_matches_oracle(name):
    nx, ny, nz, box, stages = CHAINS[name]
    rng = np.random.default_rng(21)
    N = nx * ny * nz
    bg = rng.uniform(0, 1, N)
    mask = box_mask(nx, ny, nz, box)
    n = int(mask.sum())
    x = rng.uniform(0, 1, n)
    with G.TopOpt(nx, ny, nz, box, stages, background=bg, x0=x) as t:
        assert t.n == n
        gam = t.physical(0)
        s = rng.standard_normal(N)
        t.set_sensitivity_host(0, s, 1.0)
        dx = t.design_sensitivity(0)
    ch = D.make_chain(nx, ny, nz, [(r, box, p, b, e) for r, p, b, e in stages])
    xfull = bg.copy()
    xfull[mask] = x
    gam_o = D.filter_forward(ch, xfull)
    assert np.abs(gam - gam_o).max() <= 1e-13
    dx_o = D.filter_transpose(ch, xfull, s)[mask]
    assert np.abs(dx - dx_o).max() <= 1e-13 * max(1.0, np.abs(dx_o).max())


@pytest.mark.parametrize("kind", ["plain", "minmax"])
def test_mma_matches_oracle(kind):
    """No filter stage, the design box is the whole grid: the update is MMA on
    the problem of design_lib, step for step against the oracle."""
    n = 300
    m, a, ev = D.mma_problem(kind, n, 3)
    nreal = 1 if kind == "plain" else 3
    vol = 0.4 if kind == "plain" else 0.5
    x = np.full(n, 0.5)
    orc = D.OracleMMA(n, m, x, a)
    xo = x.copy()
    with G.TopOpt(n, 1, 1, (0, n - 1, 0, 0, 0, 0), stages=(), nreal=nreal, volume=vol,
                  move_limit=0.1, magic=5.0, x0=x) as t:
        for it in range(20):
            df0, g, dg = ev(x)
            if kind == "plain":
                t.set_sensitivity_host(0, df0, 0.0)
            else:
                for r in range(3):
                    t.set_sensitivity_host(r, dg[r], g[r] - 5.0)
            ch, cons = t.update()
            x = t.variables()
            df0o, go, dgo = ev(xo)
            xo, cho, _ = orc.update(xo, df0o, go, dgo, 0.1)
            assert np.allclose(cons, go, rtol=0, atol=1e-13)
            assert np.abs(x - xo).max() < 1e-10, (it, np.abs(x - xo).max())
            assert abs(ch - cho) < 1e-10


def channel_problem(nx=36, ny=18, n=120):
    cfg = W.channel_2d(nx, ny, nsteps=n)
    box = (6, nx - 7, 2, ny - 3, 0, 0)
    return cfg, box


def solve(t, h, n, k=16):
    t.apply(0, h)
    J, _, _ = h.gradient(n, k)
    t.set_sensitivity(0, h, J)
    return J


def test_design_gradient_matches_central_differences():
    cfg, box = channel_problem()
    n = 120
    rng = np.random.default_rng(4)
    nb = (box[1] - box[0] + 1) * (box[3] - box[2] + 1)
    x = np.clip(0.6 + 0.3 * rng.standard_normal(nb), 0.05, 0.95)
    with G.Handle(cfg) as h, G.TopOpt(cfg.nx, cfg.ny, 1, box, [(2, True, 2.0, 0.5)], x0=x) as t:
        solve(t, h, n)
        dx = t.design_sensitivity(0)
        scale = np.abs(dx).max()
        assert scale > 0
        for i in rng.choice(nb, 6, replace=False):
            vals = []
            for sg in (1, -1):
                xp = x.copy()
                xp[i] += sg * 1e-6
                t.set_variables(xp)
                t.apply(0, h)
                h.init_equilibrium()
                vals.append(h.forward(n))
            fd = (vals[0] - vals[1]) / 2e-6
            assert abs(fd - dx[i]) <= 2e-5 * scale, (i, fd, dx[i])
        t.set_variables(x)


def test_short_optimisation_lowers_the_pressure_drop():
    """Minimise the pressure drop of a channel with at most 60% of the box
    fluid (ConstrainFluid): fluid everywhere would be best, so the volume
    constraint must end up active and the objective must fall."""
    cfg, box = channel_problem(40, 20, 150)
    n = 150
    nb = (box[1] - box[0] + 1) * (box[3] - box[2] + 1)
    with G.Handle(cfg) as h, G.TopOpt(cfg.nx, cfg.ny, 1, box, [(2, True, 1.0, 0.5)],
                                     volume_type=G.VOLUME_FLUID, volume=0.6, move_limit=0.2,
                                     x0=np.full(nb, 0.6)) as t:
        Js, vols = [], []
        for it in range(12):
            Js.append(solve(t, h, n))
            ch, cons = t.update()
            vols.append(cons[0])
        assert Js[-1] < Js[0]
        assert abs(vols[-1]) < 0.02
        x = t.variables()
        assert x.min() >= 0 and x.max() <= 1


def test_robust_minmax_loop(tmp_path):
    """The robust loop of optimize.py (3 realisations in one batch, double
    projection, static checkpoints, min-max MMA): the worst case falls, the
    realisations keep the order of their eta (a larger eta projects less
    fluid, so a larger pressure drop), the volume constraint ends near
    active, and the designs and fields are written."""
    import optimize as O
    x, hist = O.optimise(64, 32, 120, iters=15, robust=True, volume=0.6, nsnap=8,
                         storage=G.STORE_FP64, out_dir=str(tmp_path), every=10, log=lambda s: None)
    worst = [max(h["J"]) for h in hist]
    assert worst[-1] < worst[0]
    J = hist[-1]["J"]
    assert J[0] <= J[1] <= J[2]
    assert abs(hist[-1]["volume"]) < 0.05
    files = sorted(os.listdir(tmp_path))
    assert "design_iter_0.bin" in files and "fields_iter_0.vts" in files
    v = G.read_petsc_vec(str(tmp_path / "design_iter_0.bin"))
    assert v.size == x.size


def test_robust_loop_split_over_two_ranks_matches_one(tmp_path):
    """optimize.py under torchrun with two ranks (both on this GPU: their
    kernels are independent): rank 0 computes realisations 0 and 2, rank 1
    realisation 1, one sum over the ranks assembles all three, and every
    rank takes the same MMA step.  The design after three iterations equals
    the one-rank run's."""
    import socket
    import subprocess
    import sys
    import optimize as O
    x1, _ = O.optimise(64, 32, 60, iters=3, robust=True, volume=0.6, nsnap=10,
                       out_dir=str(tmp_path / "one"), every=100, log=lambda s: None)
    sock = socket.socket()
    sock.bind(("127.0.0.1", 0))
    port = sock.getsockname()[1]
    sock.close()
    here = os.path.dirname(os.path.abspath(__file__))
    script = os.path.join(os.path.dirname(here), "lbm-topopt_gb300", "optimize.py")
    out = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                          "--nproc-per-node=2", "--master-addr=127.0.0.1", "--master-port=%d" % port,
                          script, "--robust", "--nx", "64", "--ny", "32", "--steps", "60",
                          "--iters", "3", "--every", "100", "--out", str(tmp_path / "two")],
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    x2 = G.read_petsc_vec(str(tmp_path / "two" / "design_iter_2.bin"))
    assert x2.size == x1.size
    assert np.abs(x2 - x1).max() <= 1e-12
