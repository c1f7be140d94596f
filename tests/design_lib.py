"""ctypes access to the CPU oracles of the design update: the oracle's density
filter, projection and MMA (oracle/design_oracle.c) and, where it was built,
the reference's own MMA (topOpt/MMA.cc in oracle/_ref/libref.so).  Also the
seeded MMA test problems the golden trajectories are made from.  Test
infrastructure only."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from oracle_lib import ORACLE_SO, REF_SO

_dp = C.POINTER(C.c_double)


def _p(a):
    return None if a is None else np.ascontiguousarray(a).ctypes.data_as(_dp)


class Stage(C.Structure):
    _fields_ = [("radius", C.c_int), ("box", C.c_int * 6), ("project", C.c_int),
                ("beta", C.c_double), ("eta", C.c_double)]


class Chain(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("nstages", C.c_int),
                ("stage", Stage * 2)]


def make_chain(nx, ny, nz, stages):
    """stages: list of (radius, box, project, beta, eta)"""
    ch = Chain()
    ch.nx, ch.ny, ch.nz, ch.nstages = nx, ny, nz, len(stages)
    for k, (r, box, proj, beta, eta) in enumerate(stages):
        ch.stage[k].radius = r
        ch.stage[k].box[:] = list(box)
        ch.stage[k].project = int(proj)
        ch.stage[k].beta = beta
        ch.stage[k].eta = eta
    return ch


_orc = None


def _oracle():
    global _orc
    if _orc is None:
        lib = C.CDLL(ORACLE_SO)
        cp = C.POINTER(Chain)
        lib.dsg_filter_forward.argtypes = [cp, _dp, _dp]
        lib.dsg_filter_transpose.argtypes = [cp, _dp, _dp]
        lib.dsg_mma_create.restype = C.c_void_p
        lib.dsg_mma_create.argtypes = [C.c_int, C.c_int, _dp, _dp]
        lib.dsg_mma_destroy.argtypes = [C.c_void_p]
        lib.dsg_mma_update.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, C.c_double,
                                       C.POINTER(C.c_int), _dp]
        _orc = lib
    return _orc


def filter_forward(ch, xfull):
    out = np.empty(ch.nx * ch.ny * ch.nz)
    assert _oracle().dsg_filter_forward(C.byref(ch), _p(np.asarray(xfull, float)), _p(out)) == 0
    return out


def filter_transpose(ch, xfull, s):
    s = np.array(s, dtype=float)
    assert _oracle().dsg_filter_transpose(C.byref(ch), _p(np.asarray(xfull, float)), _p(s)) == 0
    return s


class OracleMMA:
    """The oracle's MMA: x <- update(x, df0, g, dg, movlim)."""

    def __init__(self, n, m, x0, a=None):
        self.n, self.m = n, m
        self.lib = _oracle()
        self.h = self.lib.dsg_mma_create(n, m, _p(np.asarray(x0, float)), _p(a))

    def update(self, x, df0, g, dg, movlim):
        x = np.array(x, dtype=float)
        it, ch = C.c_int(), C.c_double()
        self.lib.dsg_mma_update(self.h, _p(x), _p(df0), _p(np.asarray(g, float)),
                                _p(np.ascontiguousarray(dg, dtype=float)), movlim,
                                C.byref(it), C.byref(ch))
        return x, ch.value, it.value

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.dsg_mma_destroy(self.h)
            self.h = None


class ReferenceMMA:
    """The reference's MMA (topOpt/MMA.cc) built in oracle/_ref."""

    def __init__(self, n, m, x0, a=None):
        lib = C.CDLL(REF_SO)
        lib.ref_mma_create.restype = C.c_void_p
        lib.ref_mma_create.argtypes = [C.c_int, C.c_int, _dp, _dp]
        lib.ref_mma_update.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, C.c_double, _dp]
        lib.ref_mma_destroy.argtypes = [C.c_void_p]
        self.lib, self.n, self.m = lib, n, m
        self.h = lib.ref_mma_create(n, m, _p(np.asarray(x0, float)), _p(a))

    def update(self, x, df0, g, dg, movlim):
        x = np.array(x, dtype=float)
        ch = C.c_double()
        self.lib.ref_mma_update(self.h, _p(x), _p(df0), _p(np.asarray(g, float)),
                                _p(np.ascontiguousarray(dg, dtype=float)), movlim, C.byref(ch))
        return x, ch.value, 0

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_mma_destroy(self.h)
            self.h = None


def reference_mma_available():
    return os.path.exists(REF_SO)


def mma_problem(kind, n, seed):
    """Seeded test problems.  'plain': min sum w (x - t)^2 s.t. mean(x) <= 0.4.
    'minmax': min max_k J_k, J_k = sum w_k (x - t_k)^2 / n, written as the
    reference's robust form (objective sensitivity 0, constraints J_k + 5 - z,
    a = 1) with mean(x) <= 0.5.  Returns (m, a, evaluate(x) -> df0, g, dg)."""
    rng = np.random.default_rng(seed)
    t = rng.uniform(0, 1, (3, n))
    w = rng.uniform(0.5, 2, (3, n))
    if kind == "plain":
        def ev(x):
            return 2 * w[0] * (x - t[0]), np.array([x.mean() - 0.4]), np.full((1, n), 1.0 / n)
        return 1, None, ev
    a = np.array([1., 1., 1., 0.])

    def ev(x):
        J = [np.sum(w[k] * (x - t[k]) ** 2) / n for k in range(3)]
        dJ = [2 * w[k] * (x - t[k]) / n for k in range(3)]
        g = np.array([J[0] + 5, J[1] + 5, J[2] + 5, x.mean() - 0.5])
        return np.zeros(n), g, np.vstack(dJ + [np.full(n, 1.0 / n)])
    return 4, a, ev


def mma_trajectory(solver_cls, kind, n=300, seed=3, iters=30, movlim=0.1):
    m, a, ev = mma_problem(kind, n, seed)
    x = np.full(n, 0.5)
    s = solver_cls(n, m, x, a)
    xs, chs = [], []
    for _ in range(iters):
        df0, g, dg = ev(x)
        x, ch, _ = s.update(x, df0, g, dg, movlim)
        xs.append(x.copy())
        chs.append(ch)
    return np.array(xs), np.array(chs)
