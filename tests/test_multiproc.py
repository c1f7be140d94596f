"""The multi-rank paths on CPU with two gloo ranks: the replica reduction of
bench.py (barrier, max over ranks of the device time, sum of the lattice
updates), the reference arm printing from rank 0 only, and the split of the
robust realisations over ranks in optimize.py (each rank computes its own
realisations; one sum assembles every (J_r, dJ_r/dgamma) on every rank)."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    _, r, _, dist = bench.dist_setup()
    bench.barrier(dist)
    # rank r pretends to have timed 10 + r ms for 1000 + r cells x 5 steps
    v, slowest = bench.aggregate_mlups(dist, 1000 + r, 5, 10.0 + r)
    q.put((r, v, slowest))
    dist.destroy_process_group()


def test_replica_reduction_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    expect = (1000 + 1001) * 5 / (11.0e-3) / 1e6
    for _, v, slowest in res:
        assert slowest == 11.0
        assert abs(v - expect) < 1e-12 * expect


def test_reference_arm_prints_on_rank0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "1"], env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0
    assert out.stdout.strip() == ""


def _robust_worker(rank, world, port, nreal, ncells, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, os.path.join(ROOT, "lbm-topopt_gb300"))
    import numpy as np
    import torch.distributed as td
    import optimize as O
    td.init_process_group("gloo")
    mine = O.owned_realisations(nreal, rank, world)
    # realisation r's stand-in results: J_r = r + 0.25, dJ_r/dgamma = (r + 1) * [1, 2, ...] / 7
    local = {r: (r + 0.25, (r + 1) * np.arange(1, ncells + 1) / 7.0) for r in mine}
    full = O.exchange_realisations(nreal, ncells, local)
    q.put((rank, mine, [J for J, _ in full], [s.tolist() for _, s in full]))
    td.destroy_process_group()


def test_robust_realisations_split_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import numpy as np
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    nreal, ncells = 3, 37
    procs = [mp.Process(target=_robust_worker, args=(r, 2, port, nreal, ncells, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every realisation is computed by exactly one rank
    owned = [r for _, mine, _, _ in res for r in mine]
    assert sorted(owned) == list(range(nreal))
    assert res[0][1] == [0, 2] and res[1][1] == [1]
    # and every rank ends with the same, exact results of all of them
    for _, _, Js, ss in res:
        assert Js == [r + 0.25 for r in range(nreal)]
        for r in range(nreal):
            assert np.array_equal(np.array(ss[r]), (r + 1) * np.arange(1, ncells + 1) / 7.0)
