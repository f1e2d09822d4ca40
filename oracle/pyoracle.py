"""ctypes binding of the oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of bench.py as the checker; never by the product library.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build_oracle import build_oracle

_dp = C.POINTER(C.c_double)


class OracleParams(C.Structure):
    _fields_ = [
        ("pre_smooth", C.c_int), ("post_smooth", C.c_int),
        ("smooth_damp", C.c_double), ("alpha", C.c_double), ("beta", C.c_double),
        ("project_pressure", C.c_int),
        ("restart", C.c_int), ("maxit", C.c_int), ("minit", C.c_int),
        ("red_factor", C.c_double), ("res_norm_min", C.c_double), ("div_factor", C.c_double),
        ("vanka_mode", C.c_int), ("reuse_factors", C.c_int), ("nthreads", C.c_int),
    ]


VANKA_SEQ, VANKA_COLOUR = 0, 1
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle()
        L = C.CDLL(str(path))
        L.oracle_default_params.argtypes = [C.POINTER(OracleParams)]
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.c_void_p, C.c_int, C.POINTER(OracleParams)]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_ndof.argtypes = [C.c_void_p, C.c_int]
        L.oracle_coupled_defect.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_int]
        L.oracle_matvec.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        L.oracle_level_defect.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp]
        L.oracle_cell_vanka.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_int]
        L.oracle_restrict.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        L.oracle_prolongate.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        L.oracle_solve_exact.argtypes = [C.c_void_p, _dp, _dp]
        L.oracle_vcycle.argtypes = [C.c_void_p, _dp, _dp]
        L.oracle_fgmres.restype = C.c_int
        L.oracle_fgmres.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.oracle_lu_solve.argtypes = [_dp, _dp, C.c_int]
        L.oracle_local_system.restype = C.c_int
        L.oracle_local_system.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    """FP64 CPU restatement of the reference solver over a problem's levels.

    The level descriptors' arrays must outlive the oracle (keep the problem
    alive)."""

    def __init__(self, problem, **params):
        L = lib()
        p = OracleParams()
        L.oracle_default_params(C.byref(p))
        for k, v in params.items():
            if k == "vanka_mode" and isinstance(v, str):
                v = {"seq": VANKA_SEQ, "colour": VANKA_COLOUR}[v]
            setattr(p, k, v)
        self.params = p
        self.problem = problem
        self._h = L.oracle_create(C.cast(problem.descs, C.c_void_p), problem.n_levels, C.byref(p))
        self._L = L

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.oracle_destroy(self._h)
            self._h = None

    def ndof(self, level=-1):
        return self._L.oracle_ndof(self._h, level % self.problem.n_levels)

    def coupled_defect(self, level, x, b, project=True):
        x, b = _f(x), _f(b)
        r = np.empty_like(x)
        self._L.oracle_coupled_defect(self._h, level, _p(x), _p(b), _p(r), int(project))
        return r

    def matvec(self, level, x):
        x = _f(x)
        y = np.empty_like(x)
        self._L.oracle_matvec(self._h, level, _p(x), _p(y))
        return y

    def defect(self, level, u, f):
        u, f = _f(u), _f(f)
        d = np.empty_like(u)
        res = C.c_double()
        self._L.oracle_level_defect(self._h, level, _p(u), _p(f), _p(d), C.byref(res))
        return d, res.value

    def cell_vanka(self, level, u, rhs, sweeps=1):
        u = _f(u).copy()
        rhs = _f(rhs)
        self._L.oracle_cell_vanka(self._h, level, _p(u), _p(rhs), sweeps)
        return u

    def restrict(self, level, fine):
        fine = _f(fine)
        coarse = np.empty(self.ndof(level - 1))
        self._L.oracle_restrict(self._h, level, _p(fine), _p(coarse))
        return coarse

    def prolongate(self, level, coarse):
        coarse = _f(coarse)
        fine = np.empty(self.ndof(level))
        self._L.oracle_prolongate(self._h, level, _p(coarse), _p(fine))
        return fine

    def solve_exact(self, rhs):
        rhs = _f(rhs)
        u = np.empty_like(rhs)
        self._L.oracle_solve_exact(self._h, _p(rhs), _p(u))
        return u

    def vcycle(self, v):
        v = _f(v)
        z = np.empty_like(v)
        self._L.oracle_vcycle(self._h, _p(z), _p(v))
        return z

    def iterate(self, sol, rhs):
        sol = _f(sol).copy()
        rhs = _f(rhs)
        out = np.zeros(3)
        it = self._L.oracle_fgmres(self._h, _p(sol), _p(rhs), _p(out))
        return sol, {"iterations": abs(it), "diverged": it < 0, "res0": out[0], "res": out[1],
                     "true_res": out[2]}

    def local_system(self, level, cell, u, rhs):
        u, rhs = _f(u), _f(rhs)
        n = 3 * self.problem.desc(level).n_ulocal + 4  # 85 (Q2) or 49 (P2+bubble)
        S = np.zeros(n * n)
        R = np.zeros(n)
        self._L.oracle_local_system(self._h, level, cell, _p(u), _p(rhs), _p(S), _p(R))
        return S.reshape(n, n).T.copy(), R  # row-major A[row, col]


def lu_solve(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """dgetrf+dgetrs restatement on a row-major square matrix."""
    n = a.shape[0]
    colmajor = np.asfortranarray(a, dtype=np.float64).ravel(order="F").copy()
    x = _f(b).copy()
    lib().oracle_lu_solve(_p(colmajor), _p(x), n)
    return x
