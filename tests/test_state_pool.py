"""Zero-copy checkpoint storage, simulated on the host: the Wang schedule
drives the StatePool exactly as the gradient does, with each buffer holding
the step whose state it contains.  Every reverse step must see its own
forward state, no step may write its input or a live checkpoint, the pool
must ask for no copy, and the recompute count must match the oracle's Wang
restatement (pinned to the reference's own schedule).  Runs without a GPU."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "lbm-topopt_gb300", "csrc")


@pytest.fixture(scope="module")
def sim():
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    d = tempfile.mkdtemp()
    exe = os.path.join(d, "state_pool_sim")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", CSRC,
                           os.path.join(HERE, "state_pool_sim.cpp"), "-o", exe])
    yield exe
    shutil.rmtree(d, ignore_errors=True)


CASES = [(1, 2), (2, 2), (7, 2), (10, 3), (25, 4), (60, 7), (100, 5), (257, 16),
         (400, 64), (1000, 8), (2000, 64), (5000, 64)]


@pytest.mark.parametrize("planned", [False, True], ids=["dynamic", "static"])
@pytest.mark.parametrize("nsteps,nsnap", CASES)
def test_zero_copy_schedule(sim, orc, nsteps, nsnap, planned):
    out = subprocess.run([sim, str(nsteps), str(nsnap)] + (["static"] if planned else []),
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    tag, copies, recomputed = out.stdout.split()
    assert tag == "ok"
    assert int(copies) == 0
    expect = orc.static_count(nsteps, nsnap)[0] if planned else orc.wang_count(nsteps, nsnap)[0]
    assert int(recomputed) == expect
