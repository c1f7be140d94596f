"""ctypes access to the CPU oracles: the C restatement (oracle/liblbmoracle.so)
and, where it was built, the reference's own operators (oracle/_ref/libref.so).
Test infrastructure only."""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "lbm-topopt_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)

from lbmgpu import CConfig, Config  # noqa: E402

ORACLE_SO = os.path.join(ROOT, "oracle", "liblbmoracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libref.so")

_dp = C.POINTER(C.c_double)


def _bind(lib, prefix):
    cp = C.POINTER(CConfig)
    sig = {
        "forward": (C.c_int, [cp, _dp, _dp, C.c_int, _dp, _dp, _dp]),
        "gradient": (C.c_int, [cp, _dp, _dp, C.c_int, _dp, _dp]),
        "adjoint_step": (C.c_int, [cp, _dp, _dp, C.c_int, _dp, _dp]),
        "collide_cell": (C.c_int, [cp, _dp, C.c_double, _dp, _dp]),
        "reverse_cell": (C.c_int, [cp, _dp, C.c_double, _dp, _dp, _dp]),
    }
    for k, (r, a) in sig.items():
        fn = getattr(lib, prefix + k)
        fn.restype, fn.argtypes = r, a
    fn = getattr(lib, prefix + "set_bc_profile")
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64 if prefix == "orc_" else C.c_longlong, _dp]
    if prefix == "orc_":
        lib.orc_wang_count.restype = C.c_int
        lib.orc_wang_count.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int)]
        lib.orc_static_count.restype = C.c_int
        lib.orc_static_count.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int64),
                                         C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.orc_forward_from.restype = C.c_int
        lib.orc_forward_from.argtypes = [cp, _dp, _dp, C.c_int, C.c_int, _dp, _dp]
        lib.orc_init.restype = C.c_int
        lib.orc_init.argtypes = [cp, _dp, _dp]
        lib.orc_macros.restype = C.c_int
        lib.orc_macros.argtypes = [cp, _dp, _dp]
        lib.orc_objective.restype = C.c_int
        lib.orc_objective.argtypes = [cp, _dp, _dp, _dp]
        lib.orc_apply_bcs.restype = C.c_int
        lib.orc_apply_bcs.argtypes = [cp, C.c_int, _dp]
        lib.orc_gradient_steady.restype = C.c_int
        lib.orc_gradient_steady.argtypes = [cp, _dp, _dp, C.c_int, C.c_int, C.c_double, C.c_int,
                                            _dp, _dp, C.POINTER(C.c_int)]
        lib.orc_set_phase.restype = C.c_int
        lib.orc_set_phase.argtypes = [C.c_int, C.c_int]
    else:
        lib.ref_wang_count.restype = C.c_int
        lib.ref_wang_count.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_longlong),
                                       C.POINTER(C.c_int)]
        lib.ref_static_count.restype = C.c_int
        lib.ref_static_count.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_longlong),
                                         C.POINTER(C.c_int), C.POINTER(C.c_int)]
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


class OracleLib:
    """Same calls for both libraries."""

    def __init__(self, path: str, prefix: str):
        self.lib = _bind(C.CDLL(path), prefix)
        self.prefix = prefix

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def set_tables(self, tables=None):
        """Tables of LBM_PROFILE_TABLE boundaries, {slot: (nt, npos) or (nt, npos,
        ncomp) array}, as the library's lbm_set_bc_profile takes them; None
        clears every slot."""
        for k in range(8):
            self._fn("set_bc_profile")(k, 0, 0, 0, None)
        for k, t in (tables or {}).items():
            a = np.ascontiguousarray(t, dtype=np.float64)
            ncomp = 1 if a.ndim == 2 else a.shape[2]
            rc = self._fn("set_bc_profile")(int(k), a.shape[0], ncomp, a.shape[1], _p(a))
            if rc:
                raise RuntimeError("set_bc_profile failed: %d" % rc)

    def forward(self, cfg: Config, gamma, nsteps, macros=None):
        c = cfg.to_c()
        g = np.ascontiguousarray(gamma, dtype=np.float64)
        f = np.zeros(cfg.ncells * cfg.npop)
        js = np.zeros(max(nsteps, 1))
        tot = np.zeros(1)
        m = None if macros is None else np.ascontiguousarray(macros, dtype=np.float64)
        rc = self._fn("forward")(C.byref(c), _p(g), _p(m), int(nsteps), _p(f), _p(js), _p(tot))
        if rc:
            raise RuntimeError("%sforward failed: %d" % (self.prefix, rc))
        return f, js[:nsteps], float(tot[0])

    def gradient(self, cfg: Config, gamma, nsteps, macros=None):
        c = cfg.to_c()
        g = np.ascontiguousarray(gamma, dtype=np.float64)
        s = np.zeros(cfg.ncells)
        tot = np.zeros(1)
        m = None if macros is None else np.ascontiguousarray(macros, dtype=np.float64)
        rc = self._fn("gradient")(C.byref(c), _p(g), _p(m), int(nsteps), _p(tot), _p(s))
        if rc:
            raise RuntimeError("%sgradient failed: %d" % (self.prefix, rc))
        return float(tot[0]), s

    def adjoint_step(self, cfg: Config, gamma, f_t, t, lam, sens):
        c = cfg.to_c()
        g = np.ascontiguousarray(gamma, dtype=np.float64)
        f = np.ascontiguousarray(f_t, dtype=np.float64)
        lam = np.array(lam, dtype=np.float64)
        sens = np.array(sens, dtype=np.float64)
        rc = self._fn("adjoint_step")(C.byref(c), _p(g), _p(f), int(t), _p(lam), _p(sens))
        if rc:
            raise RuntimeError("adjoint_step failed: %d" % rc)
        return lam, sens

    def collide_cell(self, cfg: Config, fin, gamma):
        c = cfg.to_c()
        fin = np.ascontiguousarray(fin, dtype=np.float64)
        fout = np.zeros(cfg.npop)
        mac = np.zeros(4)
        rc = self._fn("collide_cell")(C.byref(c), _p(fin), float(gamma), _p(fout), _p(mac))
        if rc:
            raise RuntimeError("collide_cell failed: %d" % rc)
        return fout, mac[:cfg.nmac]

    def reverse_cell(self, cfg: Config, fin, gamma, lam_out):
        c = cfg.to_c()
        fin = np.ascontiguousarray(fin, dtype=np.float64)
        lo = np.ascontiguousarray(lam_out, dtype=np.float64)
        li = np.zeros(cfg.npop)
        dg = np.zeros(1)
        rc = self._fn("reverse_cell")(C.byref(c), _p(fin), float(gamma), _p(lo), _p(li), _p(dg))
        if rc:
            raise RuntimeError("reverse_cell failed: %d" % rc)
        return li, float(dg[0])

    def objective(self, cfg: Config, f, gamma):
        """weight * F of the populations f (FP64 AoS) as given (oracle only)."""
        c = cfg.to_c()
        f = np.ascontiguousarray(f, dtype=np.float64)
        g = np.ascontiguousarray(gamma, dtype=np.float64)
        J = C.c_double()
        rc = self.lib.orc_objective(C.byref(c), _p(f), _p(g), C.byref(J))
        if rc:
            raise RuntimeError("objective failed: %d" % rc)
        return J.value

    def apply_bcs(self, cfg: Config, f, t):
        """The boundary conditions of step t applied to a copy of f (oracle only)."""
        c = cfg.to_c()
        f = np.array(f, dtype=np.float64)
        rc = self.lib.orc_apply_bcs(C.byref(c), int(t), _p(f))
        if rc:
            raise RuntimeError("apply_bcs failed: %d" % rc)
        return f

    def gradient_steady(self, cfg: Config, gamma, max_steady, check_every, tol, n_unsteady,
                        macros=None):
        """Steady phase, then n_unsteady objective steps; (J, dJ/dgamma, steady steps)."""
        c = cfg.to_c()
        g = np.ascontiguousarray(gamma, dtype=np.float64)
        s = np.zeros(cfg.ncells)
        tot = np.zeros(1)
        S = C.c_int()
        m = None if macros is None else np.ascontiguousarray(macros, dtype=np.float64)
        rc = self.lib.orc_gradient_steady(C.byref(c), _p(g), _p(m), int(max_steady),
                                          int(check_every), float(tol), int(n_unsteady), _p(tot),
                                          _p(s), C.byref(S))
        if rc:
            raise RuntimeError("gradient_steady failed: %d" % rc)
        return float(tot[0]), s, S.value

    def set_phase(self, t_phase=2147483647, obj_from=1):
        """Ramps start after step t_phase; the objective counts steps >= obj_from."""
        self.lib.orc_set_phase(int(t_phase), int(obj_from))

    def wang_count(self, nsteps, nsnap):
        if self.prefix == "orc_":
            r, ok = C.c_int64(), C.c_int()
        else:
            r, ok = C.c_longlong(), C.c_int()
        rc = self._fn("wang_count")(int(nsteps), int(nsnap), C.byref(r), C.byref(ok))
        if rc:
            raise RuntimeError("wang_count failed: %d" % rc)
        return int(r.value), bool(ok.value)

    def static_count(self, nsteps, nsnap):
        """StaticCheckpointing(nsnap, nsteps + 1): (recomputed, reversal exact, states kept)."""
        r = C.c_int64() if self.prefix == "orc_" else C.c_longlong()
        ok, saved = C.c_int(), C.c_int()
        rc = self._fn("static_count")(int(nsteps), int(nsnap), C.byref(r), C.byref(ok),
                                      C.byref(saved))
        if rc:
            raise RuntimeError("static_count failed: %d" % rc)
        return int(r.value), bool(ok.value), int(saved.value)


def oracle() -> OracleLib:
    return OracleLib(ORACLE_SO, "orc_")


def reference():
    """The reference build, or None where it was not built (no reference tree)."""
    if not os.path.exists(REF_SO):
        return None
    return OracleLib(REF_SO, "ref_")
