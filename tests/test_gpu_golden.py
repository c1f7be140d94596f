"""The CUDA path against the golden vectors of the reference's own operators
(tests/golden, FP64 storage): populations, per-step objective and dJ/dgamma
within 1e-12 relative."""
import os

import numpy as np
import pytest

import lbmgpu as G
from helpers import rel_inf
from test_oracle import CASES, GOLD

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_reproduces_reference_golden(name):
    cfg, gamma, n = CASES[name]
    g = np.load(os.path.join(GOLD, name + ".npz"))
    with G.Handle(cfg) as h:
        h.set_design(gamma)
        h.init_equilibrium()
        J, js = h.forward(n, per_step=True)
        f = h.populations()
        Jg, sens, _ = h.gradient(n, 6)
    assert rel_inf(f, g["f"]) < 1e-12
    assert rel_inf(js, g["J_steps"]) < 1e-12
    assert abs(Jg - g["J_grad"]) <= 1e-12 * abs(g["J_grad"])
    assert rel_inf(sens, g["sens"]) < 1e-12
