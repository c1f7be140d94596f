"""Boundary set-ups on every face, shared by the oracle and GPU boundary tests.

The reference has Zou-He operators on the west, east and north faces
(boundaryConditions/ZouHe2d.hh); the library adds the south velocity and the
north/south pressure operators.  Those are pinned by rotation: a channel
turned by +90 degrees (x' = ny-1-y, y' = x) moves its west inlet to the south
face and its east outlet to the north face, so the rotated problem must give
the rotated populations, objective and dJ/dgamma of the original one, whose
operators the reference build pins."""
import numpy as np

import lbmgpu as G
import workloads as W

# D2Q9 direction i turned by +90 degrees: e_i = (ex, ey) -> (-ey, ex)
ROT = np.array([0, 7, 8, 1, 2, 3, 4, 5, 6])
FACE_ROT = {G.FACE_WEST: G.FACE_SOUTH, G.FACE_EAST: G.FACE_NORTH,
            G.FACE_SOUTH: G.FACE_EAST, G.FACE_NORTH: G.FACE_WEST}


def rot_box(box, ny):
    x0, x1, y0, y1, z0, z1 = box
    return (ny - 1 - y1, ny - 1 - y0, x0, x1, z0, z1)


def rotate_config(cfg):
    """The configuration turned by +90 degrees (2D)."""
    bcs = []
    for b in cfg.bcs:
        d = b.dir if any(b.dir) else (1.0, 0.0, 0.0)
        bcs.append(G.Boundary(b.kind, FACE_ROT[b.face], rot_box(b.box, cfg.ny), b.value,
                              b.profile, b.amp, b.period, b.time_law, (-d[1], d[0], 0.0)))
    return cfg.replace(nx=cfg.ny, ny=cfg.nx, bcs=bcs, obj_in=rot_box(cfg.obj_in, cfg.ny),
                       obj_out=rot_box(cfg.obj_out, cfg.ny))


def rotate_cells(a, cfg):
    """Per-cell field (ncells, ...) of the original lattice onto the rotated one."""
    nx, ny = cfg.nx, cfg.ny
    a = np.asarray(a).reshape((ny, nx) + np.asarray(a).shape[1:])
    out = np.empty((nx, ny) + a.shape[2:], dtype=a.dtype)   # rotated lattice: ny' = nx, nx' = ny
    for y in range(ny):
        for x in range(nx):
            out[x, ny - 1 - y] = a[y, x]
    return out.reshape((nx * ny,) + a.shape[2:])


def rotate_populations(f, cfg):
    q = cfg.npop
    fr = rotate_cells(np.asarray(f).reshape(-1, q), cfg)
    out = np.empty_like(fr)
    out[:, ROT[:9]] = fr[:, :9]
    if q > 9:
        out[:, 9:] = fr[:, 9:]
    return out.ravel()


def west_to_east_channel(nx=20, ny=12, n=60, storage=G.STORE_FP64):
    """Velocity inlet west (parabolic, oscillating), pressure outlet east."""
    return W.channel_2d(nx, ny, amp=0.2, period=25.0, nsteps=n, storage=storage)


def pressure_driven_reverse(nx=20, ny=12, n=60, storage=G.STORE_FP64):
    """Pressure inlet west (rho = 1.02), velocity boundary east (outflow
    u_x = 0.03 with a parabolic profile), outflow objective on the east box."""
    cfg = W.channel_2d(nx, ny, nsteps=n, storage=storage)
    west = (0, 0, 1, ny - 2, 0, 0)
    east = (nx - 1, nx - 1, 1, ny - 2, 0, 0)
    return cfg.replace(
        bcs=[G.Boundary(G.BC_PRESSURE, G.FACE_WEST, west, 1.02),
             G.Boundary(G.BC_VELOCITY, G.FACE_EAST, east, 0.03, G.PROFILE_PARABOLIC)],
        objective=G.OBJ_PRESSURE_DROP, obj_in=west, obj_out=east)
