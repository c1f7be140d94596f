"""The CUDA path against the golden vectors of the reference's own operators
(tests/golden, FP64 storage): populations, per-step objective and dJ/dgamma
within 1e-12 relative."""
import os

import numpy as np
import pytest

import lbmgpu as G
from helpers import rel_inf
from test_oracle import CASES, FORWARD_ONLY, GOLD, TABLES

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_reproduces_reference_golden(orc, name):
    """Forward populations, per-step objective and dJ/dgamma of the reference
    build; for the cases whose boundaries have no adjoint in the reference
    (standard Zou-He pressure), dJ/dgamma against the oracle's transposes."""
    cfg, gamma, n = CASES[name]
    g = np.load(os.path.join(GOLD, name + ".npz"))
    with G.Handle(cfg) as h:
        for k, t in TABLES.get(name, {}).items():
            h.set_bc_profile(k, t)
        h.set_design(gamma)
        h.init_equilibrium()
        J, js = h.forward(n, per_step=True)
        f = h.populations()
        Jg, sens, _ = h.gradient(n, 6)
    assert rel_inf(f, g["f"]) < 1e-12
    assert rel_inf(js, g["J_steps"]) < 1e-12
    if name in FORWARD_ONLY:
        orc.set_tables(TABLES.get(name))
        try:
            Jo, so = orc.gradient(cfg, gamma, n)
        finally:
            orc.set_tables(None)
        assert abs(Jg - Jo) <= 1e-12 * abs(Jo)
        assert rel_inf(sens, so) < 1e-12
        return
    assert abs(Jg - g["J_grad"]) <= 1e-12 * abs(g["J_grad"])
    assert rel_inf(sens, g["sens"]) < 1e-12
