"""Python host mirror of the GB300 LBM library's C ABI (include/lbmgpu.h).

The classes below keep the reference's C++ surface so that driver code reads
like the reference applications:

* ``IsothermalLBSolver`` -- ``IsothermalLBSolver2d/3d<Op>`` plus the parts of
  ``LBSolver`` a driver calls (latticeBoltzmann/LBSolver.hh:14-73,
  isothermalLBSolver2d.hh:20-110): ``setFieldFromDesignVec``,
  ``initializeAtEquilibrium``, ``collideAndStream``, ``computeMacroFunctional``,
  ``getDistributions`` / ``setDistributions``.
* ``AdjointLBSolver`` -- adjointLatticeBoltzmann/adjointLBSolver.hh:11-46:
  ``resetAdjoints``, ``adjointStep`` (adjointCollide + computeCollideSource +
  adjointStream), ``getSensitivities``.
* ``LBDynamicCheckpointing`` -- the Wang et al. checkpointed gradient
  (topOpt/LBCheckpointing.hh:20-29) run inside the library with device slots.

All work happens in the compiled CUDA library ``liblbmgpu.so``; this module only
marshals arguments.  There is no CPU fallback: if the library is missing the
import of the solver classes raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbmgpu.so")

# lattices, operators, storage, boundaries, objectives (include/lbmgpu.h)
D2Q9, D3Q19, D2Q9_D2Q5 = 0, 1, 2
BGK, MRT = 0, 1
STORE_FP64, STORE_FP32, STORE_FP16 = 0, 1, 2
BC_VELOCITY, BC_PRESSURE, BC_TEMPERATURE = 1, 2, 3
BC_VELOCITY_STANDARD, BC_PRESSURE_STANDARD = 4, 5
FACE_WEST, FACE_EAST, FACE_SOUTH, FACE_NORTH = 0, 1, 2, 3
PROFILE_UNIFORM, PROFILE_PARABOLIC, PROFILE_TABLE = 0, 1, 2
TIME_OFFSET_SINE, TIME_SINE, TIME_RAMP = 0, 1, 2
OBJ_NONE, OBJ_PRESSURE_DROP, OBJ_DISSIPATION, OBJ_HEAT_FLUX, OBJ_OUTFLOW = 0, 1, 2, 3, 4
OBJ_THROUGH_FLOW, OBJ_DOMAIN_TEMPERATURE, OBJ_REGENERATOR_EFFICIENCY = 5, 6, 7
SCHEDULE_DYNAMIC, SCHEDULE_STATIC = 0, 1
MAX_BC = 8

ERR_ARG, ERR_SUP, ERR_CUDA, ERR_MEM, ERR_STATE, ERR_NONFINITE = -1, -2, -3, -4, -5, -6
STATUS_TEXT = {0: "ok", ERR_ARG: "bad argument", ERR_SUP: "unsupported", ERR_CUDA: "CUDA error",
               ERR_MEM: "out of memory", ERR_STATE: "call out of order",
               ERR_NONFINITE: "non-finite value"}

# MRT rates: d'Humieres defaults (dynamics/MRT3d.hh:9-22) and the 2D ones
# (dynamics/incompressibleMRT2d.hh:88-90)
MRT3D_DEFAULT = (1.19, 1.4, 1.2, 1.4, 1.4, 3.0, -5.5, -0.5)
MRT2D_DEFAULT = (1.4, 1.4, 1.2, 0.0, 0.0, 0.0, 0.0, 0.0)


class CBC(C.Structure):
    _fields_ = [("kind", C.c_int), ("face", C.c_int), ("profile", C.c_int),
                ("box", C.c_int * 6), ("value", C.c_double), ("amp", C.c_double),
                ("period", C.c_double), ("time_law", C.c_int), ("dir", C.c_double * 3)]


class CConfig(C.Structure):
    _fields_ = [("lattice", C.c_int), ("collision", C.c_int), ("storage", C.c_int),
                ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("omega", C.c_double), ("mrt", C.c_double * 8),
                ("interp_scale", C.c_double), ("interp_q", C.c_double),
                ("diffusivity", C.c_double), ("ramp_q", C.c_double), ("ramp_ck", C.c_double),
                ("heat_rate", C.c_double), ("heat_T", C.c_double),
                ("nbc", C.c_int), ("bc", CBC * MAX_BC),
                ("objective", C.c_int), ("obj_in", C.c_int * 6), ("obj_out", C.c_int * 6),
                ("obj_weight", C.c_double), ("obj_param", C.c_double * 4)]


class CGradStats(C.Structure):
    _fields_ = [("forward_steps", C.c_int64), ("recomputed_steps", C.c_int64),
                ("adjoint_steps", C.c_int64), ("forward_ms", C.c_double),
                ("reverse_ms", C.c_double)]


@dataclass
class Boundary:
    """One ``lbm_bc``: value(t) = value * T(t) * profile, T(t) = 1 + amp sin(2 pi t /
    period) (TIME_OFFSET_SINE) or amp sin(2 pi t / period) (TIME_SINE); a velocity
    boundary imposes that times ``dir`` ((0,0,0) = +x)."""
    kind: int
    face: int
    box: Sequence[int]
    value: float
    profile: int = PROFILE_UNIFORM
    amp: float = 0.0
    period: float = 1.0
    time_law: int = TIME_OFFSET_SINE
    dir: Sequence[float] = (0.0, 0.0, 0.0)


@dataclass
class Config:
    """Python view of ``lbm_config``; ``to_c()`` gives the C struct."""
    lattice: int = D2Q9
    collision: int = BGK
    storage: int = STORE_FP64
    nx: int = 1
    ny: int = 1
    nz: int = 1
    omega: float = 1.0
    mrt: Sequence[float] = MRT3D_DEFAULT
    interp_scale: float = 1.0
    interp_q: float = 1.0
    diffusivity: float = 0.0
    ramp_q: float = 1.0
    ramp_ck: float = 1.0
    heat_rate: float = 0.0
    heat_T: float = 1.0
    bcs: List[Boundary] = field(default_factory=list)
    objective: int = OBJ_NONE
    obj_in: Sequence[int] = (0, 0, 0, 0, 0, 0)
    obj_out: Sequence[int] = (0, 0, 0, 0, 0, 0)
    obj_weight: float = 1.0
    obj_param: Sequence[float] = (0.0, 0.0, 0.0, 0.0)

    @property
    def ncells(self) -> int:
        return self.nx * self.ny * (self.nz if self.lattice == D3Q19 else 1)

    @property
    def npop(self) -> int:
        return {D2Q9: 9, D3Q19: 19, D2Q9_D2Q5: 14}[self.lattice]

    @property
    def nmac(self) -> int:
        return {D2Q9: 3, D3Q19: 4, D2Q9_D2Q5: 4}[self.lattice]

    def replace(self, **kw) -> "Config":
        d = dict(self.__dict__)
        d["bcs"] = list(self.bcs)
        d.update(kw)
        return Config(**d)

    def to_c(self) -> CConfig:
        if len(self.bcs) > MAX_BC:
            raise ValueError("at most %d boundary conditions" % MAX_BC)
        c = CConfig()
        c.lattice, c.collision, c.storage = self.lattice, self.collision, self.storage
        c.nx, c.ny, c.nz = self.nx, self.ny, (self.nz if self.lattice == D3Q19 else 1)
        c.omega = self.omega
        for i, v in enumerate(list(self.mrt)[:8]):
            c.mrt[i] = v
        c.interp_scale, c.interp_q = self.interp_scale, self.interp_q
        c.diffusivity, c.ramp_q, c.ramp_ck = self.diffusivity, self.ramp_q, self.ramp_ck
        c.heat_rate, c.heat_T = self.heat_rate, self.heat_T
        c.nbc = len(self.bcs)
        for k, b in enumerate(self.bcs):
            cb = c.bc[k]
            cb.kind, cb.face, cb.profile = b.kind, b.face, b.profile
            for i in range(6):
                cb.box[i] = int(b.box[i])
            cb.value, cb.amp, cb.period = b.value, b.amp, b.period
            cb.time_law = b.time_law
            for i in range(3):
                cb.dir[i] = float(b.dir[i])
        c.objective = self.objective
        for i in range(6):
            c.obj_in[i] = int(self.obj_in[i])
            c.obj_out[i] = int(self.obj_out[i])
        c.obj_weight = self.obj_weight
        for i, v in enumerate(list(self.obj_param)[:4]):
            c.obj_param[i] = float(v)
        return c


class LBMError(RuntimeError):
    def __init__(self, code: int, text: str):
        super().__init__("%s (%d): %s" % (STATUS_TEXT.get(code, "error"), code, text))
        self.code = code


_lib = None


def load_library(path: Optional[str] = None) -> C.CDLL:
    """Load liblbmgpu.so (built in-tree by __graft_entry__.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or os.environ.get("LBMGPU_LIBRARY") or LIB_PATH
    if not os.path.exists(p):
        raise OSError("liblbmgpu.so not built at %s (run __graft_entry__.build())" % p)
    lib = C.CDLL(p)
    dp = C.POINTER(C.c_double)
    H = C.c_void_p
    sig = {
        "lbm_config_default": (None, [C.POINTER(CConfig)]),
        "lbm_create": (C.c_int, [C.POINTER(CConfig), C.POINTER(H)]),
        "lbm_destroy": (C.c_int, [H]),
        "lbm_last_error": (C.c_char_p, [H]),
        "lbm_get_sizes": (C.c_int, [H, C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
        "lbm_set_design": (C.c_int, [H, dp]),
        "lbm_set_bc_profile": (C.c_int, [H, C.c_int, C.c_int, C.c_int, dp]),
        "lbm_init_equilibrium": (C.c_int, [H, dp]),
        "lbm_forward": (C.c_int, [H, C.c_int, dp, dp]),
        "lbm_get_time": (C.c_int, [H, C.POINTER(C.c_int)]),
        "lbm_get_populations": (C.c_int, [H, dp]),
        "lbm_set_populations": (C.c_int, [H, dp, C.c_int]),
        "lbm_get_macros": (C.c_int, [H, dp]),
        "lbm_adjoint_reset": (C.c_int, [H]),
        "lbm_adjoint_step": (C.c_int, [H]),
        "lbm_get_adjoint": (C.c_int, [H, dp]),
        "lbm_get_sensitivity": (C.c_int, [H, dp]),
        "lbm_gradient": (C.c_int, [H, C.c_int, C.c_int, dp, dp, C.POINTER(CGradStats)]),
        "lbm_time_steps": (C.c_int, [H, C.c_int, C.c_int, C.POINTER(C.c_float)]),
        "lbm_get_launch_count": (C.c_int, [H, C.POINTER(C.c_int64)]),
        "lbm_select_device": (C.c_int, [C.c_int]),
        "lbm_batch_create": (C.c_int, [C.POINTER(CConfig), C.c_int, C.POINTER(H)]),
        "lbm_batch_destroy": (C.c_int, [H]),
        "lbm_batch_last_error": (C.c_char_p, [H]),
        "lbm_batch_handle": (C.c_int, [H, C.c_int, C.POINTER(H)]),
        "lbm_batch_autotune": (C.c_int, [H, C.c_int]),
        "lbm_batch_get_launch_shape": (C.c_int, [H, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "lbm_batch_get_reverse_shape": (C.c_int, [H, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "lbm_batch_set_launch_shape": (C.c_int, [H, C.c_int, C.c_int, C.c_int]),
        "lbm_batch_forward": (C.c_int, [H, C.c_int, dp]),
        "lbm_batch_gradient": (C.c_int, [H, C.c_int, C.c_int, C.c_int, dp, C.POINTER(dp),
                                         C.POINTER(CGradStats)]),
        "lbm_batch_time_steps": (C.c_int, [H, C.c_int, C.c_int, C.POINTER(C.c_float)]),
        "lbm_batch_get_launch_count": (C.c_int, [H, C.POINTER(C.c_int64)]),
        "lbm_autotune": (C.c_int, [H, C.c_int]),
        "lbm_get_launch_shape": (C.c_int, [H, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "lbm_set_launch_shape": (C.c_int, [H, C.c_int, C.c_int, C.c_int]),
        "lbm_set_reverse_variant": (C.c_int, [H, C.c_int]),
        "lbm_get_reverse_variant": (C.c_int, [H]),
        "lbm_batch_set_reverse_variant": (C.c_int, [H, C.c_int]),
        "lbm_batch_get_reverse_variant": (C.c_int, [H]),
        "lbm_forward_steady": (C.c_int, [H, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_int),
                                         C.POINTER(C.c_double)]),
        "lbm_gradient_steady": (C.c_int, [H, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                          C.POINTER(C.c_int), dp, dp, C.POINTER(CGradStats)]),
        "lbm_get_dims": (C.c_int, [H, C.POINTER(C.c_int)]),
        "lbm_write_petsc_vec": (C.c_int, [C.c_char_p, dp, C.c_int64]),
        "lbm_read_petsc_vec": (C.c_int, [C.c_char_p, dp, C.c_int64, C.POINTER(C.c_int64)]),
        "lbm_write_vts_fields": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.POINTER(C.c_char_p), C.POINTER(C.c_int),
                                           C.POINTER(dp)]),
        "lbm_write_vts": (C.c_int, [H, C.c_char_p, dp]),
        "lbm_set_design_device": (C.c_int, [H, C.c_void_p]),
        "lbm_get_sensitivity_device": (C.c_int, [H, C.POINTER(C.c_void_p)]),
        "lbm_topopt_config_default": (None, [C.c_void_p]),
        "lbm_topopt_create": (C.c_int, [C.c_void_p, dp, dp, C.POINTER(C.c_void_p)]),
        "lbm_topopt_destroy": (C.c_int, [C.c_void_p]),
        "lbm_topopt_last_error": (C.c_char_p, [C.c_void_p]),
        "lbm_topopt_num_variables": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
        "lbm_topopt_set_variables": (C.c_int, [C.c_void_p, dp]),
        "lbm_topopt_get_variables": (C.c_int, [C.c_void_p, dp]),
        "lbm_topopt_set_beta": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
        "lbm_topopt_physical": (C.c_int, [C.c_void_p, C.c_int, dp]),
        "lbm_topopt_apply": (C.c_int, [C.c_void_p, C.c_int, H]),
        "lbm_topopt_set_sensitivity": (C.c_int, [C.c_void_p, C.c_int, H, C.c_double]),
        "lbm_topopt_set_sensitivity_host": (C.c_int, [C.c_void_p, C.c_int, dp, C.c_double]),
        "lbm_topopt_get_design_sensitivity": (C.c_int, [C.c_void_p, C.c_int, dp]),
        "lbm_topopt_update": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), dp]),
        "lbm_wang_recompute_count": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int64)]),
        "lbm_schedule_count": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int64),
                                         C.POINTER(C.c_int64)]),
        "lbm_gradient_schedule": (C.c_int, [H, C.c_int, C.c_int, C.c_int, dp, dp,
                                            C.POINTER(CGradStats)]),
        "lbm_batch_gradient_schedule": (C.c_int, [H, C.c_int, C.c_int, C.c_int, C.c_int, dp,
                                                  C.POINTER(dp), C.POINTER(CGradStats)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _ptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_double))


def select_device(ordinal: int) -> None:
    """Use GPU `ordinal` for handles created afterwards by this thread."""
    lib = load_library()
    rc = lib.lbm_select_device(int(ordinal))
    if rc:
        raise LBMError(rc, lib.lbm_last_error(None).decode())


def schedule_count(nsteps: int, nsnapshots: int, schedule: int = SCHEDULE_DYNAMIC):
    """(recomputed steps, states kept by the forward sweep) of a checkpoint schedule."""
    lib = load_library()
    rec, saved = C.c_int64(), C.c_int64()
    rc = lib.lbm_schedule_count(int(nsteps), int(nsnapshots), int(schedule), C.byref(rec),
                                C.byref(saved))
    if rc:
        raise LBMError(rc, lib.lbm_last_error(None).decode())
    return rec.value, saved.value


def _io_check(lib, rc):
    if rc:
        raise LBMError(rc, lib.lbm_last_error(None).decode())


def write_petsc_vec(path: str, v) -> None:
    """PETSc binary Vec file (writeVectorToBinary)."""
    lib = load_library()
    v = np.ascontiguousarray(v, dtype=np.float64)
    _io_check(lib, lib.lbm_write_petsc_vec(path.encode(), _ptr(v), v.size))


def read_petsc_vec(path: str) -> np.ndarray:
    """PETSc binary Vec file (loadVectorFromBinary)."""
    lib = load_library()
    n = C.c_int64()
    _io_check(lib, lib.lbm_read_petsc_vec(path.encode(), None, 0, C.byref(n)))
    v = np.empty(n.value)
    _io_check(lib, lib.lbm_read_petsc_vec(path.encode(), _ptr(v), v.size, C.byref(n)))
    return v


def write_vts(path: str, dims, fields) -> None:
    """VTK XML StructuredGrid of point fields: fields = {name: array of
    ncells * ncomp values} (ncomp inferred)."""
    lib = load_library()
    nx, ny, nz = (list(dims) + [1, 1])[:3]
    ncell = nx * ny * nz
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in fields.values()]
    names = (C.c_char_p * len(arrs))(*[k.encode() for k in fields])
    comps = (C.c_int * len(arrs))(*[a.size // ncell for a in arrs])
    ptrs = (C.POINTER(C.c_double) * len(arrs))(*[_ptr(a) for a in arrs])
    _io_check(lib, lib.lbm_write_vts_fields(path.encode(), nx, ny, nz, len(arrs), names, comps, ptrs))


def wang_recompute_count(nsteps: int, nsnapshots: int) -> int:
    lib = load_library()
    out = C.c_int64()
    rc = lib.lbm_wang_recompute_count(nsteps, nsnapshots, C.byref(out))
    if rc:
        raise LBMError(rc, lib.lbm_last_error(None).decode())
    return out.value


class Handle:
    """Owns one lbm_handle (device-resident lattice)."""

    def __init__(self, cfg: Config):
        self.lib = load_library()
        self.cfg = cfg
        self._c = cfg.to_c()
        h = C.c_void_p()
        rc = self.lib.lbm_create(C.byref(self._c), C.byref(h))
        if rc:
            raise LBMError(rc, self.lib.lbm_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.lbm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int):
        if rc:
            raise LBMError(rc, self.lib.lbm_last_error(self.h).decode())

    # -- forward ---------------------------------------------------------------
    def set_bc_profile(self, k: int, table):
        """Table of boundary k (configured with PROFILE_TABLE): shape (nt, npos)
        for a factor, (nt, npos, dim) for a velocity vector; row t mod nt is used
        at time step t (lbm_set_bc_profile)."""
        a = np.ascontiguousarray(table, dtype=np.float64)
        if a.ndim == 2:
            nt, ncomp = a.shape[0], 1
        elif a.ndim == 3:
            nt, ncomp = a.shape[0], a.shape[2]
        else:
            raise ValueError("table must be (nt, npos) or (nt, npos, ncomp)")
        self._check(self.lib.lbm_set_bc_profile(self.h, int(k), int(nt), int(ncomp), _ptr(a)))

    def set_design(self, gamma: np.ndarray):
        g = np.ascontiguousarray(gamma, dtype=np.float64).ravel()
        if g.size != self.cfg.ncells:
            raise ValueError("gamma has %d values, expected %d" % (g.size, self.cfg.ncells))
        self._check(self.lib.lbm_set_design(self.h, _ptr(g)))

    def init_equilibrium(self, macros: Optional[np.ndarray] = None):
        m = None if macros is None else np.ascontiguousarray(macros, dtype=np.float64).ravel()
        self._check(self.lib.lbm_init_equilibrium(self.h, _ptr(m)))

    def forward(self, nsteps: int, per_step: bool = False):
        js = np.zeros(max(nsteps, 1)) if per_step else None
        tot = np.zeros(1)
        self._check(self.lib.lbm_forward(self.h, int(nsteps), _ptr(js), _ptr(tot)))
        return (float(tot[0]), js[:nsteps]) if per_step else float(tot[0])

    def time(self) -> int:
        t = C.c_int()
        self._check(self.lib.lbm_get_time(self.h, C.byref(t)))
        return t.value

    def populations(self) -> np.ndarray:
        f = np.empty(self.cfg.ncells * self.cfg.npop)
        self._check(self.lib.lbm_get_populations(self.h, _ptr(f)))
        return f

    def set_populations(self, f: np.ndarray, t: int):
        a = np.ascontiguousarray(f, dtype=np.float64).ravel()
        if a.size != self.cfg.ncells * self.cfg.npop:
            raise ValueError("wrong population count")
        self._check(self.lib.lbm_set_populations(self.h, _ptr(a), int(t)))

    def macros(self) -> np.ndarray:
        m = np.empty(self.cfg.ncells * self.cfg.nmac)
        self._check(self.lib.lbm_get_macros(self.h, _ptr(m)))
        return m

    # -- adjoint ---------------------------------------------------------------
    def adjoint_reset(self):
        self._check(self.lib.lbm_adjoint_reset(self.h))

    def adjoint_step(self):
        self._check(self.lib.lbm_adjoint_step(self.h))

    def adjoint(self) -> np.ndarray:
        a = np.empty(self.cfg.ncells * self.cfg.npop)
        self._check(self.lib.lbm_get_adjoint(self.h, _ptr(a)))
        return a

    def sensitivity(self) -> np.ndarray:
        s = np.empty(self.cfg.ncells)
        self._check(self.lib.lbm_get_sensitivity(self.h, _ptr(s)))
        return s

    def gradient(self, nsteps: int, nsnapshots: int, schedule: int = SCHEDULE_DYNAMIC):
        J = np.zeros(1)
        s = np.empty(self.cfg.ncells)
        st = CGradStats()
        self._check(self.lib.lbm_gradient_schedule(self.h, int(nsteps), int(nsnapshots),
                                                   int(schedule), _ptr(J), _ptr(s), C.byref(st)))
        return float(J[0]), s, st

    def gradient_steady(self, max_steady: int, check_every: int, tol: float, n_unsteady: int,
                        nsnapshots: int):
        """lbm_gradient_steady: (J, dJ/dgamma, stats, steady steps)."""
        J = np.zeros(1)
        s = np.empty(self.cfg.ncells)
        st = CGradStats()
        S = C.c_int()
        self._check(self.lib.lbm_gradient_steady(self.h, int(max_steady), int(check_every),
                                                 float(tol), int(n_unsteady), int(nsnapshots),
                                                 C.byref(S), _ptr(J), _ptr(s), C.byref(st)))
        return float(J[0]), s, st, S.value

    def time_steps(self, which: int, nsteps: int) -> float:
        ms = C.c_float()
        self._check(self.lib.lbm_time_steps(self.h, int(which), int(nsteps), C.byref(ms)))
        return ms.value

    def autotune(self, nsteps: int = 5):
        """Pick the fastest thread-block shapes for the step kernels."""
        self._check(self.lib.lbm_autotune(self.h, int(nsteps)))
        return self.launch_shape(0), self.launch_shape(1)

    def launch_shape(self, which: int):
        bx, by = C.c_int(), C.c_int()
        self._check(self.lib.lbm_get_launch_shape(self.h, int(which), C.byref(bx), C.byref(by)))
        return bx.value, by.value

    def dims(self):
        d = (C.c_int * 3)()
        self._check(self.lib.lbm_get_dims(self.h, d))
        return tuple(d)

    def write_vts(self, path: str, gamma=None):
        """Macros of the current state (and gamma) as a .vts file."""
        g = None if gamma is None else np.ascontiguousarray(gamma, dtype=np.float64)
        self._check(self.lib.lbm_write_vts(self.h, path.encode(), _ptr(g)))

    def forward_steady(self, max_steps: int, check_every: int = 100, tol: float = 1e-6):
        """Advance until max |f_t - f_{t-1}| < tol (tested every check_every
        steps) or max_steps; returns (steps taken, last change)."""
        n, ch = C.c_int(), C.c_double()
        self._check(self.lib.lbm_forward_steady(self.h, int(max_steps), int(check_every),
                                                float(tol), C.byref(n), C.byref(ch)))
        return n.value, ch.value

    def set_launch_shape(self, which: int, bx: int, by: int):
        self._check(self.lib.lbm_set_launch_shape(self.h, int(which), int(bx), int(by)))

    def set_reverse_variant(self, lean: int):
        """0: default register budget of the reverse step, 1: the register-lean
        variant (one more resident block per SM); same results."""
        self._check(self.lib.lbm_set_reverse_variant(self.h, int(lean)))

    @property
    def reverse_variant(self) -> int:
        r = self.lib.lbm_get_reverse_variant(self.h)
        self._check(min(r, 0))
        return r

    def launch_count(self) -> int:
        n = C.c_int64()
        self._check(self.lib.lbm_get_launch_count(self.h, C.byref(n)))
        return n.value


class _View(Handle):
    """A lattice owned by a Batch (not destroyed on its own)."""

    def __init__(self, lib, cfg, h):  # noqa: D401 - plain holder
        self.lib, self.cfg, self.h = lib, cfg, h

    def close(self):
        self.h = None


class Batch:
    """Several lattices advanced by one launch per time step (lbm_batch_*)."""

    def __init__(self, cfgs: Sequence[Config]):
        self.lib = load_library()
        self.cfgs = list(cfgs)
        arr = (CConfig * len(self.cfgs))(*[c.to_c() for c in self.cfgs])
        self._arr = arr
        b = C.c_void_p()
        rc = self.lib.lbm_batch_create(arr, len(self.cfgs), C.byref(b))
        if rc:
            raise LBMError(rc, self.lib.lbm_batch_last_error(None).decode())
        self.b = b
        self.views = []
        for i, cfg in enumerate(self.cfgs):
            h = C.c_void_p()
            self._check(self.lib.lbm_batch_handle(self.b, i, C.byref(h)))
            self.views.append(_View(self.lib, cfg, h))

    def _check(self, rc):
        if rc:
            raise LBMError(rc, self.lib.lbm_batch_last_error(self.b).decode())

    def close(self):
        if getattr(self, "b", None):
            for v in self.views:
                v.h = None
            self.lib.lbm_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __getitem__(self, i) -> Handle:
        return self.views[i]

    def __len__(self):
        return len(self.views)

    def autotune(self, nsteps: int = 3):
        """Tune the block shapes; returns the forward one (reverse_shape()
        gives the other)."""
        self._check(self.lib.lbm_batch_autotune(self.b, int(nsteps)))
        bx, by = C.c_int(), C.c_int()
        self._check(self.lib.lbm_batch_get_launch_shape(self.b, C.byref(bx), C.byref(by)))
        return bx.value, by.value

    def reverse_shape(self):
        bx, by = C.c_int(), C.c_int()
        self._check(self.lib.lbm_batch_get_reverse_shape(self.b, C.byref(bx), C.byref(by)))
        return bx.value, by.value

    def set_launch_shape(self, which: int, bx: int, by: int):
        """Block shape of the batched forward (which=0) or reverse (which=1)
        step: one of the autotuner's shapes."""
        self._check(self.lib.lbm_batch_set_launch_shape(self.b, int(which), int(bx), int(by)))

    def set_reverse_variant(self, lean: int):
        self._check(self.lib.lbm_batch_set_reverse_variant(self.b, int(lean)))

    @property
    def reverse_variant(self) -> int:
        r = self.lib.lbm_batch_get_reverse_variant(self.b)
        self._check(min(r, 0))
        return r

    def forward(self, nsteps: int):
        J = np.zeros(len(self))
        self._check(self.lib.lbm_batch_forward(self.b, int(nsteps), _ptr(J)))
        return J

    def gradient(self, nsteps: int, nsnapshots: int, use_graph: bool = True,
                 schedule: int = SCHEDULE_DYNAMIC):
        J = np.zeros(len(self))
        sens = [np.empty(c.ncells) for c in self.cfgs]
        ptrs = (C.POINTER(C.c_double) * len(self))(*[_ptr(a) for a in sens])
        st = CGradStats()
        self._check(self.lib.lbm_batch_gradient_schedule(
            self.b, int(nsteps), int(nsnapshots), int(schedule), int(bool(use_graph)), _ptr(J),
            ptrs, C.byref(st)))
        return J, sens, st

    def time_steps(self, which: int, nsteps: int) -> float:
        ms = C.c_float()
        self._check(self.lib.lbm_batch_time_steps(self.b, int(which), int(nsteps), C.byref(ms)))
        return ms.value

    def launch_count(self) -> int:
        n = C.c_int64()
        self._check(self.lib.lbm_batch_get_launch_count(self.b, C.byref(n)))
        return n.value


# -- reference-style facades -----------------------------------------------------

# -- design update on the device --------------------------------------------------

VOLUME_NONE, VOLUME_FLUID, VOLUME_MATERIAL = 0, 1, 2
MAX_STAGES, MAX_REALISATIONS = 2, 8


class CTopOptConfig(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("design_box", C.c_int * 6), ("nstages", C.c_int),
                ("radius", C.c_int * MAX_STAGES), ("filter_box", C.c_int * 6),
                ("project", C.c_int * MAX_STAGES), ("beta", C.c_double * MAX_STAGES),
                ("eta", C.c_double * MAX_STAGES), ("nreal", C.c_int),
                ("real_eta", C.c_double * MAX_REALISATIONS), ("volume_type", C.c_int),
                ("volume", C.c_double), ("volume_real", C.c_int), ("move_limit", C.c_double),
                ("magic", C.c_double)]


class TopOpt:
    """The design update of the optimisation loop on the device (lbm_topopt_*):
    design variables on a box, up to two density-filter + tanh-projection
    stages to the physical gamma, their transposes, a volume constraint and
    MMA.  stages: list of (radius, project, beta, eta)."""

    def __init__(self, nx, ny, nz, design_box, stages=((2, True, 1.0, 0.5),), filter_box=None,
                 nreal=1, real_eta=None, volume_type=VOLUME_FLUID, volume=0.5, volume_real=0,
                 move_limit=0.1, magic=5.0, background=None, x0=None):
        self.lib = load_library()
        lib = self.lib
        c = CTopOptConfig()
        lib.lbm_topopt_config_default(C.byref(c))
        c.nx, c.ny, c.nz = int(nx), int(ny), int(nz)
        c.design_box[:] = [int(v) for v in design_box]
        c.filter_box[:] = [int(v) for v in (filter_box if filter_box is not None else design_box)]
        c.nstages = len(stages)
        for k, (r, proj, beta, eta) in enumerate(stages):
            c.radius[k], c.project[k], c.beta[k], c.eta[k] = int(r), int(bool(proj)), beta, eta
        c.nreal = int(nreal)
        for r, e in enumerate(real_eta or []):
            c.real_eta[r] = e
        c.volume_type, c.volume, c.volume_real = int(volume_type), float(volume), int(volume_real)
        c.move_limit, c.magic = float(move_limit), float(magic)
        self.cfg = c
        self.ncells = int(nx) * int(ny) * int(nz)
        self.t = C.c_void_p()
        bg = None if background is None else np.ascontiguousarray(background, dtype=np.float64)
        xx = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
        rc = lib.lbm_topopt_create(C.byref(c), _ptr(bg), _ptr(xx), C.byref(self.t))
        if rc:
            raise LBMError(rc, lib.lbm_last_error(None).decode())
        n = C.c_int64()
        self._check(lib.lbm_topopt_num_variables(self.t, C.byref(n)))
        self.n = n.value
        self.nreal = int(nreal)

    def _check(self, rc):
        if rc:
            raise LBMError(rc, self.lib.lbm_topopt_last_error(self.t).decode())

    def close(self):
        if self.t:
            self.lib.lbm_topopt_destroy(self.t)
            self.t = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_variables(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        assert x.size == self.n
        self._check(self.lib.lbm_topopt_set_variables(self.t, _ptr(x)))

    def variables(self):
        x = np.empty(self.n)
        self._check(self.lib.lbm_topopt_get_variables(self.t, _ptr(x)))
        return x

    def set_beta(self, stage, beta):
        self._check(self.lib.lbm_topopt_set_beta(self.t, int(stage), float(beta)))

    def physical(self, r=0):
        g = np.empty(self.ncells)
        self._check(self.lib.lbm_topopt_physical(self.t, int(r), _ptr(g)))
        return g

    def apply(self, r, handle):
        self._check(self.lib.lbm_topopt_apply(self.t, int(r), handle.h))

    def set_sensitivity(self, r, handle, J):
        self._check(self.lib.lbm_topopt_set_sensitivity(self.t, int(r), handle.h, float(J)))

    def set_sensitivity_host(self, r, dJdgamma, J):
        s = np.ascontiguousarray(dJdgamma, dtype=np.float64)
        assert s.size == self.ncells
        self._check(self.lib.lbm_topopt_set_sensitivity_host(self.t, int(r), _ptr(s), float(J)))

    def design_sensitivity(self, r=0):
        d = np.empty(self.n)
        self._check(self.lib.lbm_topopt_get_design_sensitivity(self.t, int(r), _ptr(d)))
        return d

    def update(self):
        """One volume-constraint + MMA step; returns (change, constraint values)."""
        ch = C.c_double()
        g = np.zeros(MAX_REALISATIONS + 1)
        self._check(self.lib.lbm_topopt_update(self.t, C.byref(ch), _ptr(g)))
        m = (self.nreal if self.nreal > 1 else 0) + (1 if self.cfg.volume_type else 0)
        return ch.value, g[:m].copy()


class IsothermalLBSolver:
    """Mirror of IsothermalLBSolver2d/3d (latticeBoltzmann/isothermalLBSolver2d.hh:20-110)."""

    def __init__(self, cfg: Config):
        self.handle = Handle(cfg)

    def setFieldFromDesignVec(self, gamma):
        self.handle.set_design(gamma)

    def initializeAtEquilibrium(self, macros=None):
        self.handle.init_equilibrium(macros)

    def collideAndStream(self, nsteps: int = 1) -> float:
        return self.handle.forward(nsteps)

    def getDistributions(self):
        return self.handle.populations()

    def setDistributions(self, f, t):
        self.handle.set_populations(f, t)

    def getCurrentTimestep(self) -> int:
        return self.handle.time()


class AdjointLBSolver:
    """Mirror of AdjointLBSolver (adjointLatticeBoltzmann/adjointLBSolver.hh:11-46)."""

    def __init__(self, solver: IsothermalLBSolver):
        self.handle = solver.handle

    def resetAdjoints(self):
        self.handle.adjoint_reset()

    def adjointStep(self):
        self.handle.adjoint_step()

    def getSensitivities(self):
        return self.handle.sensitivity()


class LBDynamicCheckpointing:
    """Checkpointed forward+adjoint with Wang et al. dynamic checkpointing
    (topOpt/LBCheckpointing.cc:37-65) and nsnapshots device slots."""

    schedule = SCHEDULE_DYNAMIC

    def __init__(self, nsnapshots: int, solver: IsothermalLBSolver):
        self.k = int(nsnapshots)
        self.solver = solver

    def gradient(self, nsteps: int):
        return self.solver.handle.gradient(nsteps, self.k, self.schedule)


class LBStaticCheckpointing(LBDynamicCheckpointing):
    """LBStaticCheckpointing (topOpt/LBCheckpointing.cc:4-35): the checkpoint
    placement is planned before the forward sweep; same gradient."""

    schedule = SCHEDULE_STATIC
