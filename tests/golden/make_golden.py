"""Generate the golden vectors in this directory from the reference's own
operators, loops and checkpoint schedule (oracle/_ref/libref.so, built from the
reference sources by `make -C oracle ref REF_SRC=<reference>/src`).  The reference has no tests or
stored results of its own; these fixtures are its outputs on seeded inputs.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "lbm-topopt_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import lbmgpu as G  # noqa: E402
import workloads as W  # noqa: E402
from oracle_lib import reference  # noqa: E402


def thermal_case(nx, ny, nsteps):
    """The thermal double distribution without the solid heating term (the
    reference has none): a T = 1 Zou-He inlet heats the channel instead."""
    cfg = W.thermal_2d(nx, ny, heat_rate=0.0, nsteps=nsteps, period=30.0)
    bcs = [G.Boundary(b.kind, b.face, b.box, 1.0 if b.kind == G.BC_TEMPERATURE else b.value,
                      b.profile, b.amp, b.period) for b in cfg.bcs]
    return cfg.replace(bcs=bcs)


def standard_case(nx, ny, nsteps, velocity_kind, pressure_kind, pressure_face):
    """A channel whose inlet or outlet uses the standard-equilibrium Zou-He
    operators (StandardZouHeVelocityWest2d / StandardZouHePressureEast/West2d)."""
    cfg = W.channel_2d(nx, ny, nsteps=nsteps, amp=0.2, period=30.0)
    inlet, outlet = cfg.bcs[0], cfg.bcs[1]
    if pressure_face == G.FACE_WEST:
        # pressure-driven: rho = 1.02 in the west, 1 in the east
        box_w, box_e = inlet.box, outlet.box
        bcs = [G.Boundary(pressure_kind, G.FACE_WEST, box_w, 1.02),
               G.Boundary(G.BC_PRESSURE, G.FACE_EAST, box_e, 1.0)]
        # the densities of the two boxes are prescribed: measure the outflow instead
        return cfg.replace(bcs=bcs, objective=G.OBJ_OUTFLOW)
    else:
        bcs = [G.Boundary(velocity_kind, G.FACE_WEST, inlet.box, inlet.value, inlet.profile,
                          inlet.amp, inlet.period),
               G.Boundary(pressure_kind, G.FACE_EAST, outlet.box, 1.0)]
    return cfg.replace(bcs=bcs)


# cases whose tables the library takes through lbm_set_bc_profile: {name: {slot: table}}
TABLES = {}
# cases with a boundary the reference has no adjoint for (the standard Zou-He
# pressure loops, boundaryConditions/ZouHe2d.hh:325-391): forward only
FORWARD_ONLY = {"d2q9_standard_pressure_east", "d2q9_standard_pressure_west"}


def cases():
    pump = W.pump_2d(36, nsteps=100, period=60.0)
    TABLES["d2q9_mrt_pump"] = {2: W.pump_inflow_profile(pump)}
    return {
        "d2q9_bgk": (W.channel_2d(32, 16, amp=0.2, period=25.0, nsteps=120),
                     W.design_2d(32, 16, 101), 120),
        "d2q9_mrt": (W.channel_2d(24, 12, collision=G.MRT, nsteps=80), W.design_2d(24, 12, 102), 80),
        "d2q9_bgk_outflow": (W.channel_2d(28, 14, nsteps=90).replace(objective=G.OBJ_OUTFLOW),
                             W.design_2d(28, 14, 105), 90),
        "d3q19_mrt": (W.duct_3d(16, 8, 8, nsteps=50), W.design_3d(16, 8, 8, 103), 50),
        "d3q19_mrt_default_rates": (W.duct_3d(12, 8, 8, nsteps=30).replace(mrt=G.MRT3D_DEFAULT),
                                    W.design_3d(12, 8, 8, 104), 30),
        "d2q9_d2q5_thermal": (thermal_case(24, 12, 80), W.design_2d(24, 12, 106), 80),
        "d2q9_mrt_pump": (pump, W.design_2d(36, 36, 107), 100),
        "d2q9_standard_velocity": (standard_case(26, 13, 90, G.BC_VELOCITY_STANDARD,
                                                 G.BC_PRESSURE, G.FACE_EAST),
                                   W.design_2d(26, 13, 108), 90),
        "d2q9_standard_pressure_east": (standard_case(26, 13, 90, G.BC_VELOCITY,
                                                      G.BC_PRESSURE_STANDARD, G.FACE_EAST),
                                        W.design_2d(26, 13, 109), 90),
        "d2q9_standard_pressure_west": (standard_case(26, 13, 90, None,
                                                      G.BC_PRESSURE_STANDARD, G.FACE_WEST),
                                        W.design_2d(26, 13, 110), 90),
    }


def cell_inputs(cfg, rng, n=16):
    d2q9 = [4 / 9] + [1 / 36, 1 / 9] * 4
    base = {G.D2Q9: d2q9,
            G.D3Q19: [1 / 3] + [1 / 18] * 3 + [1 / 36] * 6 + [1 / 18] * 3 + [1 / 36] * 6,
            G.D2Q9_D2Q5: d2q9 + [0.6 / 3] + [0.6 / 6] * 4}[cfg.lattice]
    fin = np.array(base)[None, :] * (1 + 0.05 * rng.standard_normal((n, len(base))))
    g = rng.uniform(0.02, 0.98, n)
    lo = rng.standard_normal((n, len(base)))
    return fin, g, lo


def main():
    ref = reference()
    if ref is None:
        raise SystemExit("build the reference operators first: make -C oracle ref REF_SRC=<reference>/src")
    rng = np.random.default_rng(20261203)
    for name, (cfg, gamma, n) in cases().items():
        ref.set_tables(TABLES.get(name))
        f, js, J = ref.forward(cfg, gamma, n)
        if name in FORWARD_ONLY:
            Jg, sens = np.nan, np.full(cfg.ncells, np.nan)
        else:
            Jg, sens = ref.gradient(cfg, gamma, n)
        ref.set_tables(None)
        fin, g, lo = cell_inputs(cfg, rng)
        fout = np.zeros_like(fin)
        mac = np.zeros((len(g), cfg.nmac))
        lin = np.zeros_like(fin)
        dg = np.zeros(len(g))
        for k in range(len(g)):
            fout[k], mac[k] = ref.collide_cell(cfg, fin[k], g[k])
            lin[k], dg[k] = ref.reverse_cell(cfg, fin[k], g[k], lo[k])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), gamma=gamma, nsteps=n, f=f,
                            J_steps=js, J=J, J_grad=Jg, sens=sens, cell_fin=fin, cell_gamma=g,
                            cell_fout=fout, cell_mac=mac, cell_lam_out=lo, cell_lam_in=lin,
                            cell_dgamma=dg)
        print(name, "J", J, "max|sens|", np.nanmax(np.abs(sens)) if name not in FORWARD_ONLY else "-")
    table = []
    for N in (1, 2, 3, 10, 50, 100, 777, 1000, 2000, 4000, 5000, 10000, 20000):
        for K in (2, 3, 7, 16, 20, 64):
            r, ok = ref.wang_count(N, K)
            table.append((N, K, r, int(ok)))
    np.savetxt(os.path.join(HERE, "wang_schedule.txt"), np.array(table, dtype=np.int64), fmt="%d",
               header="nsteps nsnapshots recomputed_steps reversal_exact (reference WangCheckpointing + DynamicCheckpointing)")
    print("wang table", len(table))
    table = []
    for N in (1, 2, 3, 10, 50, 100, 777, 1000, 2000, 4000, 5000, 10000, 20000):
        for K in (2, 3, 7, 16, 20, 64):
            r, ok, saved = ref.static_count(N, K)
            table.append((N, K, r, int(ok), saved))
    np.savetxt(os.path.join(HERE, "static_schedule.txt"), np.array(table, dtype=np.int64), fmt="%d",
               header="nsteps nsnapshots recomputed_steps reversal_exact saved_states "
                      "(reference StaticCheckpointing(K, nsteps + 1) + WangCheckpointing)")
    print("static table", len(table))
    # the reference's MMA (topOpt/MMA.cc) on the seeded problems of design_lib
    import design_lib as D
    for kind in ("plain", "minmax"):
        xs, chs = D.mma_trajectory(D.ReferenceMMA, kind)
        np.savez_compressed(os.path.join(HERE, "mma_%s.npz" % kind), x=xs, change=chs)
        print("mma", kind, "final change", chs[-1])


if __name__ == "__main__":
    main()
