"""Seeded synthetic workloads: the five problem set-ups the library is measured on.

The reference hard-codes its problems in application ``main()``s
(applications/*/*.cc) and draws random designs with PETSc ``VecSetRandom``
(topOpt/finiteDifferenceCheck2d.cc:24-32), which is not reproducible outside
PETSc.  Designs here come from a counter-based SplitMix64 generator with a
fixed seed per workload, so every run, the oracle and the GPU see the same
inputs.

Channel set-ups follow the reference's 2D applications: parabolic Zou-He
velocity inlet on the west column y = 1..ny-2 and Zou-He pressure outlet on
the east column (applications/Regenerator2d/regenerator2d.cc:392,398), walls
by the pull stream's mid-way bounce-back (dynamics/isothermalLBLoops2d.hh:79-82).
"""
from __future__ import annotations

import math

import numpy as np

from lbmgpu import (BC_PRESSURE, BC_TEMPERATURE, BC_VELOCITY, BGK, D2Q9, D2Q9_D2Q5, D3Q19,
                    FACE_EAST, FACE_NORTH, FACE_WEST, MRT, OBJ_DISSIPATION, OBJ_HEAT_FLUX,
                    OBJ_PRESSURE_DROP, OBJ_REGENERATOR_EFFICIENCY, OBJ_THROUGH_FLOW,
                    PROFILE_PARABOLIC, PROFILE_TABLE, STORE_FP64, TIME_RAMP, TIME_SINE, Boundary,
                    Config)

SEED_BASE = 20261203
MASK64 = (1 << 64) - 1


def splitmix64_uniform(seed: int, n: int) -> np.ndarray:
    """n doubles in [0,1) from SplitMix64 at counters 0..n-1 (Steele et al. 2014)."""
    with np.errstate(over="ignore"):
        x = (np.uint64(seed) + np.uint64(0x9E3779B97F4A7C15) *
             (np.arange(n, dtype=np.uint64) + np.uint64(1)))
        z = x
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def box_filter(a: np.ndarray) -> np.ndarray:
    """3^d box filter with edge replication (the mean over each cell's neighbourhood)."""
    p = np.pad(a, 1, mode="edge")
    out = np.zeros_like(a)
    if a.ndim == 2:
        for dy in range(3):
            for dx in range(3):
                out += p[dy:dy + a.shape[0], dx:dx + a.shape[1]]
        return out / 9.0
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                out += p[dz:dz + a.shape[0], dy:dy + a.shape[1], dx:dx + a.shape[2]]
    return out / 27.0


def design_2d(nx: int, ny: int, seed: int) -> np.ndarray:
    """Uniform noise, 3x3 box-filtered, clamped to [0,1]; shape (ny, nx), flattened x fastest."""
    g = splitmix64_uniform(seed, nx * ny).reshape(ny, nx)
    return np.clip(box_filter(g), 0.0, 1.0).ravel()


def design_3d(nx: int, ny: int, nz: int, seed: int) -> np.ndarray:
    """Smoothed noise (3x3x3 box, 2 passes) thresholded at 0.5 to {0,1}, then one
    more box pass, which blends each solid/fluid interface linearly over 2 cells."""
    g = splitmix64_uniform(seed, nx * ny * nz).reshape(nz, ny, nx)
    g = box_filter(box_filter(g))
    g = (g >= 0.5).astype(np.float64)
    g = box_filter(g)
    return np.clip(g, 0.0, 1.0).ravel()


def tanh_projection(x: np.ndarray, beta: float, eta: float) -> np.ndarray:
    """(tanh(b*eta)+tanh(b(x-eta)))/(tanh(b*eta)+tanh(b(1-eta))) (topOpt/projectionFilter2d.cc:39-40)."""
    return ((np.tanh(beta * eta) + np.tanh(beta * (x - eta))) /
            (np.tanh(beta * eta) + np.tanh(beta * (1.0 - eta))))


def channel_2d(nx: int, ny: int, *, tau: float = 0.8, u_max: float = 0.05, amp: float = 0.0,
               period: float = 2000.0, alpha_max: float = 0.05, q: float = 0.1,
               storage: int = STORE_FP64, objective: int = OBJ_PRESSURE_DROP,
               nsteps: int = 2000, collision: int = BGK) -> Config:
    inlet = (0, 0, 1, ny - 2, 0, 0)
    outlet = (nx - 1, nx - 1, 1, ny - 2, 0, 0)
    return Config(
        lattice=D2Q9, collision=collision, storage=storage, nx=nx, ny=ny, nz=1,
        omega=1.0 / tau, mrt=(1.4, 1.4, 1.2, 0, 0, 0, 0, 0),
        interp_scale=2.0 * alpha_max, interp_q=q,
        bcs=[Boundary(BC_VELOCITY, FACE_WEST, inlet, u_max, PROFILE_PARABOLIC, amp, period),
             Boundary(BC_PRESSURE, FACE_EAST, outlet, 1.0)],
        objective=objective, obj_in=inlet, obj_out=outlet, obj_weight=1.0 / nsteps)


def duct_3d(nx: int, ny: int, nz: int, *, tau: float = 0.6, rate: float = 1.2,
            u_max: float = 0.04, alpha_max: float = 0.05, q: float = 0.1,
            storage: int = STORE_FP64, nsteps: int = 5000) -> Config:
    inlet = (0, 0, 1, ny - 2, 1, nz - 2)
    outlet = (nx - 1, nx - 1, 1, ny - 2, 1, nz - 2)
    return Config(
        lattice=D3Q19, collision=MRT, storage=storage, nx=nx, ny=ny, nz=nz,
        omega=1.0 / tau, mrt=(rate, rate, rate, rate, rate, 3.0, -5.5, -0.5),
        interp_scale=2.0 * alpha_max, interp_q=q,
        bcs=[Boundary(BC_VELOCITY, FACE_WEST, inlet, u_max, PROFILE_PARABOLIC),
             Boundary(BC_PRESSURE, FACE_EAST, outlet, 1.0)],
        objective=OBJ_PRESSURE_DROP, obj_in=inlet, obj_out=outlet, obj_weight=1.0 / nsteps)


def thermal_2d(nx: int, ny: int, *, tau: float = 0.8, u0: float = 0.03, du: float = 0.01,
               period: float = 2000.0, prandtl: float = 0.7, ck: float = 0.1, q: float = 0.1,
               alpha_max: float = 0.05, heat_rate: float = 0.05, storage: int = STORE_FP64,
               nsteps: int = 10000) -> Config:
    nu = (tau - 0.5) / 3.0
    inlet = (0, 0, 1, ny - 2, 0, 0)
    outlet = (nx - 1, nx - 1, 1, ny - 2, 0, 0)
    return Config(
        lattice=D2Q9_D2Q5, collision=BGK, storage=storage, nx=nx, ny=ny, nz=1,
        omega=1.0 / tau, interp_scale=2.0 * alpha_max, interp_q=q,
        diffusivity=nu / prandtl, ramp_q=q, ramp_ck=ck, heat_rate=heat_rate, heat_T=1.0,
        bcs=[Boundary(BC_VELOCITY, FACE_WEST, inlet, u0, PROFILE_PARABOLIC, du / u0, period),
             Boundary(BC_PRESSURE, FACE_EAST, outlet, 1.0),
             Boundary(BC_TEMPERATURE, FACE_WEST, inlet, 0.0)],
        objective=OBJ_HEAT_FLUX, obj_in=inlet, obj_out=outlet, obj_weight=1.0 / nsteps)


def pump_2d(n: int, *, tau: float = 0.8, u_max: float = 0.05, period: float = 200.0,
            alpha_max: float = 0.05, q: float = 0.1, collision: int = MRT,
            storage: int = STORE_FP64, nsteps: int = 600) -> Config:
    """The robust pump's set-up (applications/RobustPump2d/robustPump2d.cc:52-104) on an
    n x n lattice, n divisible by 3, th = n/3: Zou-He pressure rho = 1 on the west
    and east segments y = th+1..2th, a north Zou-He velocity inlet on x =
    th+1..2th with the zero-mean oscillation u_y(t) = -u_max sin(2 pi t/period) p(x)
    (p from ``pump_inflow_profile``, the reference's InflowVelocity), and the
    through-flow objective over the two pressure segments (ThroughFlow2d,
    robustPump2d.cc:165-166).  The reference closes the rest of the box with
    on-grid bounce-back; here the pull stream's mid-way bounce-back walls do."""
    th = n // 3
    west = (0, 0, th + 1, 2 * th, 0, 0)
    east = (n - 1, n - 1, th + 1, 2 * th, 0, 0)
    north = (th + 1, 2 * th, n - 1, n - 1, 0, 0)
    return Config(
        lattice=D2Q9, collision=collision, storage=storage, nx=n, ny=n, nz=1,
        omega=1.0 / tau, mrt=(1.4, 1.4, 1.2, 0, 0, 0, 0, 0),
        interp_scale=2.0 * alpha_max, interp_q=q,
        bcs=[Boundary(BC_PRESSURE, FACE_WEST, west, 1.0),
             Boundary(BC_PRESSURE, FACE_EAST, east, 1.0),
             Boundary(BC_VELOCITY, FACE_NORTH, north, u_max, PROFILE_TABLE, 1.0, period,
                      TIME_SINE, (0.0, -1.0, 0.0))],
        objective=OBJ_THROUGH_FLOW, obj_in=west, obj_out=east, obj_weight=1.0 / nsteps)


def pump_inflow_profile(cfg: Config) -> np.ndarray:
    """Factors (r^2 - (x - mid)^2) / r^2 of the north inlet cells x = th+1..2th, mid
    = (n-1)/2, r = th/2 (the InflowVelocity of robustPump2d.cc:13-25), as the one-row
    table of ``lbm_set_bc_profile`` (shape (1, th))."""
    n = cfg.nx
    th = n // 3
    mid, r = (n - 1) / 2.0, th / 2.0
    x = np.arange(th + 1, 2 * th + 1, dtype=np.float64)
    return ((r * r - (x - mid) * (x - mid)) / (r * r))[None, :]


def regenerator_2d(nx: int, ny: int, *, velocity: float = 0.05, reynolds: float = 30.0,
                   prandtl: float = 0.71, ck: float = 0.0025, delta_T: float = 2.0,
                   ramp: float = 200.0, storage: int = STORE_FP64, n_unsteady: int = 2000,
                   objective: int = OBJ_REGENERATOR_EFFICIENCY) -> Config:
    """The regenerator's set-up (applications/Regenerator2d/regenerator2d.cc:346-436)
    on the D2Q9 + D2Q5 lattice: parabolic Zou-He velocity inlet (u_max = velocity,
    nu from Re on the channel height), Zou-He pressure outlet rho = 1, and a
    Dirichlet inlet temperature that holds T0 = 0 through the steady phase and then
    ramps to delta_T over `ramp` steps (StageTemp, regenerator2d.cc:53-69); the
    solid conducts Ck times the fluid (RAMP q = 1, regenerator2d.cc:376-381) and
    partial bounce-back uses the plain BP interpolation with q = 1
    (regenerator2d.cc:364).  The objective measures the middle of the channel
    (obj_out, x = nx/4 .. 3nx/4): by default the regenerator efficiency with
    Ti = 0, Tb = delta_T (functionals/regeneratorEfficiency2d.hh), averaged over
    the unsteady steps.  Differences from the reference: the D2Q5 temperature
    lattice instead of D2Q4, BGK flow instead of MRT, and the pull stream's mid-way
    bounce-back for the walls and the thermal outlet instead of on-grid bounce-back
    and a Neumann outlet."""
    nu = velocity * ny / reynolds
    omega = 1.0 / (3.0 * nu + 0.5)
    inlet = (0, 0, 1, ny - 2, 0, 0)
    outlet = (nx - 1, nx - 1, 1, ny - 2, 0, 0)
    region = (nx // 4, 3 * nx // 4, 0, ny - 1, 0, 0)
    return Config(
        lattice=D2Q9_D2Q5, collision=BGK, storage=storage, nx=nx, ny=ny, nz=1,
        omega=omega, interp_scale=1.0, interp_q=1.0,
        diffusivity=nu / prandtl, ramp_q=1.0, ramp_ck=ck, heat_rate=0.0, heat_T=0.0,
        bcs=[Boundary(BC_VELOCITY, FACE_WEST, inlet, velocity, PROFILE_PARABOLIC),
             Boundary(BC_PRESSURE, FACE_EAST, outlet, 1.0),
             Boundary(BC_TEMPERATURE, FACE_WEST, inlet, delta_T, amp=0.0, period=ramp,
                      time_law=TIME_RAMP)],
        objective=objective, obj_in=inlet, obj_out=region, obj_weight=1.0 / n_unsteady,
        obj_param=(0.0, delta_T, 0.0, 0.0))


def regenerator_design(nx: int, ny: int, seed: int) -> np.ndarray:
    """Fluid except seeded solid plates across the middle of the channel (the
    reference's initial plates, regenerator2d.cc:462-470, with seeded widths),
    box-filtered once."""
    r = splitmix64_uniform(seed, 8)
    g = np.ones((ny, nx))
    for k in range(3):
        x0 = int(nx * (0.3 + 0.15 * k + 0.05 * r[k]))
        w = max(3, int(nx * (0.04 + 0.02 * r[3 + k])))
        y0, y1 = (1, int(ny * 0.45)) if k % 2 == 0 else (int(ny * 0.55), ny - 2)
        g[y0:y1, x0:x0 + w] = 0.0
    return np.clip(box_filter(g), 0.0, 1.0).ravel()


def thermal_design(nx: int, ny: int, seed: int) -> np.ndarray:
    """Fluid (gamma=1) everywhere except a seeded disc of heated solid (gamma=0)."""
    r = splitmix64_uniform(seed, 3)
    cx = nx * (0.3 + 0.2 * r[0])
    cy = ny * (0.35 + 0.3 * r[1])
    rad = ny * (0.12 + 0.06 * r[2])
    y, x = np.mgrid[0:ny, 0:nx]
    d = np.sqrt((x - cx) ** 2 + (y - cy) ** 2)
    g = np.clip(d - rad, 0.0, 1.0)   # one-cell linear edge
    return g.ravel().astype(np.float64)


# -- the five workloads -------------------------------------------------------------

def workload_channel_128x64(storage: int = STORE_FP64):
    """128x64 D2Q9 BGK + Brinkman, FP64, 2000 steps from rest, pressure drop."""
    cfg = channel_2d(128, 64, storage=storage, nsteps=2000)
    return cfg, design_2d(128, 64, SEED_BASE + 1), 2000


def workload_unsteady_channel_1024x512(storage: int = STORE_FP64, nx: int = 1024, ny: int = 512,
                     nsteps: int = 20000):
    """1024x512 D2Q9 BGK + Brinkman, unsteady inlet, dissipated energy."""
    cfg = channel_2d(nx, ny, amp=0.2, period=2000.0, storage=storage,
                     objective=OBJ_DISSIPATION, nsteps=nsteps)
    return cfg, design_2d(nx, ny, SEED_BASE + 2), nsteps


def workload_duct_256x128x128(storage: int = STORE_FP64, nx: int = 256, ny: int = 128, nz: int = 128,
                     nsteps: int = 5000):
    """256x128x128 D3Q19 MRT + Brinkman duct, pressure drop."""
    cfg = duct_3d(nx, ny, nz, storage=storage, nsteps=nsteps)
    return cfg, design_3d(nx, ny, nz, SEED_BASE + 3), nsteps


def workload_thermal_512x256(storage: int = STORE_FP64, nx: int = 512, ny: int = 256,
                     nsteps: int = 10000):
    """512x256 D2Q9 + D2Q5 thermal, oscillating inlet, heat flux out of the outlet."""
    cfg = thermal_2d(nx, ny, storage=storage, nsteps=nsteps)
    return cfg, thermal_design(nx, ny, SEED_BASE + 4), nsteps


BATCH_GRIDS = [(1024, 512)] * 3 + [(256, 128), (384, 192), (512, 256), (640, 320), (768, 384)]


def workload_batch_8_channels(storage: int = STORE_FP64, nsteps: int = 4000, scale: int = 1):
    """3 projected designs (beta=8, eta 0.3/0.5/0.7) of a 1024x512 channel plus 5 extra
    channels from independent seeds.  `scale` divides every grid edge (for tests)."""
    out = []
    base = design_2d(1024 // scale, 512 // scale, SEED_BASE + 5)
    for k, (nx, ny) in enumerate(BATCH_GRIDS):
        nx, ny = nx // scale, ny // scale
        cfg = channel_2d(nx, ny, storage=storage, nsteps=nsteps)
        if k < 3:
            g = tanh_projection(base, 8.0, (0.3, 0.5, 0.7)[k])
        else:
            g = design_2d(nx, ny, SEED_BASE + 50 + k)
        out.append((cfg, g))
    return out, nsteps
