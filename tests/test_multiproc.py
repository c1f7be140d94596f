"""The N-GPU bench path on CPU: two gloo ranks run the replica reduction of
bench.py (barrier, max over ranks of the device time, sum of the lattice
updates), and the reference arm prints from rank 0 only."""
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
