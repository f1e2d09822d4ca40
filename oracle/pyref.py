"""ctypes front end of oracle/_ref/libref_harness.so: the reference's own
Defect_NSE4 / MatVect_NSE4 / IntoL20Vector3D (src/FE/MGComponents3D.C:3210,
:3030, :1756) and flexible FGMRES (TFgmresIte::Iterate, src/FE/FgmresIte.C:250)
and cell Vanka (TNSE_MGLevel4::CellVanka, src/FE/NSE_MGLevel4.C:1653) run on
one level of a problem built here; and (oracle/_ref/libref_transfer.so) the
grid transfers Prolongate / DefectRestriction between two levels and the
multigrid cycle driver (TMultiGridIte::Iterate, TNSE_MultiGrid::Cycle) over
all levels of a problem, which the harnessed FGMRES can take as its
preconditioner (the whole reference solver).  TEST INFRASTRUCTURE ONLY — it exists where the reference tree does (see
build_ref_harness, build_ref_transfer).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build_oracle import build_ref_harness, build_ref_hybrid, build_ref_transfer

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_dpp = C.POINTER(_dp)
_LIB = None


def ref_harness_lib():
    """The loaded harness, or None when the reference tree is absent."""
    global _LIB
    if _LIB is None:
        path = build_ref_harness()
        if path is None:
            return None
        _LIB = _declare(C.CDLL(str(path)))
    return _LIB


_HLIB = None


def ref_hybrid_lib():
    """The harness in the reference's colour-parallel build (its OpenMP
    colour loop of CellVanka), or None when the reference tree is absent."""
    global _HLIB
    if _HLIB is None:
        path = build_ref_hybrid()
        if path is None:
            return None
        L = _declare(C.CDLL(str(path)))
        L.ref_vanka_set_colours.argtypes = [C.c_void_p, C.c_int, _ip, _ip, C.c_int, C.c_int]
        L.ref_vanka_set_colours.restype = C.c_int
        _HLIB = L
    return _HLIB


def _declare(L):
    """ctypes signatures of the harness entry points (both builds)."""
    L.ref_level_create.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _ip, _dpp, _ip, _ip, _dpp,
                                   _ip, _ip, _dpp]
    L.ref_level_create.restype = C.c_void_p
    L.ref_level_destroy.argtypes = [C.c_void_p]
    L.ref_level_destroy.restype = None
    L.ref_defect.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_int, C.c_int]
    L.ref_defect.restype = None
    L.ref_matvec.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_int]
    L.ref_matvec.restype = None
    L.ref_fgmres.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double,
                             C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p,
                             C.c_int]
    L.ref_fgmres.restype = C.c_int
    L.ref_into_l20.argtypes = [_dp, C.c_int, C.c_int]
    L.ref_into_l20.restype = None
    L.ref_vanka_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _ip, _ip,
                                   _ip, _ip, _dpp, _ip, _ip, _dpp, _ip, _ip, _dpp,
                                   C.c_double]
    L.ref_vanka_create.restype = C.c_void_p
    L.ref_vanka2_create.argtypes = L.ref_vanka_create.argtypes
    L.ref_vanka2_create.restype = C.c_void_p
    L.ref_vanka_destroy.argtypes = [C.c_void_p]
    L.ref_vanka_destroy.restype = None
    L.ref_vanka_sweeps.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_double]
    L.ref_vanka_sweeps.restype = None
    L.ref_vanka_solve_exact.argtypes = [C.c_void_p, _dp, _dp, C.c_int]
    L.ref_vanka_solve_exact.restype = None
    return L


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_ip)


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


class RefLevel:
    """One level (the dict of ``OseenProblem.arrays``) built as the
    reference's matrix objects (copied once; freed with this object)."""

    def __init__(self, arrays: dict, threads: int = 1):
        L = ref_harness_lib()
        if L is None:
            raise RuntimeError("reference tree not present: the reference harness is not built")
        self._L = L
        self._h = None
        self.threads = threads
        self.n_u, self.n_p = int(arrays["n_udof"]), int(arrays["n_pdof"])
        self.n_active = int(arrays["n_active"])
        keep = []

        def ip(a):
            a, p = _i(a)
            keep.append(a)
            return p

        def dpp(arrs):
            ptrs = (_dp * len(arrs))()
            for k, a in enumerate(arrs):
                a, p = _d(a)
                keep.append(a)
                ptrs[k] = p
            keep.append(ptrs)
            return C.cast(ptrs, _dpp)

        self._h = L.ref_level_create(
            self.n_u, self.n_active, self.n_p,
            ip(arrays["a_rowptr"]), ip(arrays["a_col"]), dpp(arrays["a"]),
            ip(arrays["b_rowptr"]), ip(arrays["b_col"]), dpp(arrays["b"]),
            ip(arrays["bt_rowptr"]), ip(arrays["bt_col"]), dpp(arrays["bt"]))

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.ref_level_destroy(self._h)
            self._h = None

    @property
    def ndof(self) -> int:
        return 3 * self.n_u + self.n_p

    def _defect(self, nstype, x, b, project):
        x, xp = _d(x)
        b, bp = _d(b)
        assert x.size == self.ndof and b.size == self.ndof
        r = np.empty(self.ndof)
        self._L.ref_defect(self._h, nstype, xp, bp, r.ctypes.data_as(_dp), int(project),
                           self.threads)
        return r

    def _matvec(self, nstype, x):
        x, xp = _d(x)
        assert x.size == self.ndof
        y = np.empty(self.ndof)
        self._L.ref_matvec(self._h, nstype, xp, y.ctypes.data_as(_dp), self.threads)
        return y

    def defect(self, x, b, project: bool) -> np.ndarray:
        """r = b - K x through Defect_NSE4; the pressure part projected into
        L2_0 (P1disc) when ``project``, as under INTERNAL_PROJECT_PRESSURE."""
        return self._defect(4, x, b, project)

    def matvec(self, x) -> np.ndarray:
        """y = K x through MatVect_NSE4."""
        return self._matvec(4, x)

    def defect_nse2(self, x, b, project: bool) -> np.ndarray:
        """Defect_NSE2: the one-block (NSTYPE-2) defect with A11 as the A
        matrix of every velocity component."""
        return self._defect(2, x, b, project)

    def matvec_nse2(self, x) -> np.ndarray:
        """MatVect_NSE2 with A11 as the one A matrix."""
        return self._matvec(2, x)

    def fgmres_with_oracle_vcycle(self, oracle, sol, rhs) -> tuple[np.ndarray, int]:
        """The reference's FGMRES on this level (which must be the oracle's
        finest), preconditioned by the oracle's V-cycle (``oracle_vcycle``
        called directly as the harness's C preconditioner), with the
        oracle's restart / maxit / minit / red_factor / res_norm_min /
        div_factor / project_pressure.  Returns (solution, iterations)."""
        assert self.ndof == oracle.ndof(-1)
        fn = C.cast(oracle._L.oracle_vcycle, C.c_void_p)
        return self.fgmres(fn, C.c_void_p(oracle._h), oracle.params, sol, rhs)

    def fgmres_with_reference_cycle(self, cycle, params, sol, rhs) -> tuple[np.ndarray, int]:
        """The whole reference solver: its FGMRES on this level (the
        cycle's finest) preconditioned by its own cycle driver (``cycle``, a
        RefCycle), with the smoothing and FGMRES parameters of ``params``
        (an oracle's OracleParams).  Returns (solution, iterations)."""
        assert self.ndof == cycle.nf
        fn, ctx = cycle.preconditioner(params.pre_smooth, params.post_smooth, params.smooth_damp)
        return self.fgmres(fn, ctx, params, sol, rhs)

    def fgmres(self, fn, ctx, p, sol, rhs) -> tuple[np.ndarray, int]:
        """ref_fgmres with the C preconditioner ``fn(ctx, z, v)`` and the
        FGMRES parameters of ``p`` (an OracleParams)."""
        sol = np.array(sol, dtype=np.float64, copy=True)
        rhs, rp = _d(rhs)
        assert sol.size == self.ndof == rhs.size
        it = self._L.ref_fgmres(self._h, sol.ctypes.data_as(_dp), rp, p.restart, p.maxit,
                                p.minit, p.red_factor, p.res_norm_min, p.div_factor,
                                p.project_pressure, fn, ctx, self.threads)
        if it < 0:
            raise ValueError("ref_fgmres refused the parameters (div_factor < 1)")
        return sol, it


class RefVankaLevel:
    """One level (the dict of ``OseenProblem.arrays``) as the reference's
    TNSE_MGLevel4, for its cell Vanka (run by oracle/ref_vanka.cpp): the
    sequential build's cell loop (src/FE/NSE_MGLevel4.C:1653-2087), or, with
    ``colours`` (one colour per cell, no two cells of a colour sharing a
    DOF), the colour-parallel build's OpenMP colour loop (:603-1651) over
    those colours in increasing order, cells of a colour in index order, on
    ``threads`` threads.  With ``one_block`` the level is an NSTYPE-2
    TNSE_MGLevel2 (src/FE/NSE_MGLevel2.C) built on a[0] alone, its CellVanka
    :336-700 (no colour-parallel variant)."""

    def __init__(self, arrays: dict, alpha: float = 1.0, colours=None, threads: int = 4,
                 one_block: bool = False):
        assert not (one_block and colours is not None)
        L = ref_harness_lib() if colours is None else ref_hybrid_lib()
        if L is None:
            raise RuntimeError("reference tree not present: the reference harness is not built")
        self._L = L
        self._h = None
        self.n_u, self.n_p = int(arrays["n_udof"]), int(arrays["n_pdof"])
        udofs = np.ascontiguousarray(arrays["cell_udofs"], dtype=np.int32)
        pdofs = np.ascontiguousarray(arrays["cell_pdofs"], dtype=np.int32)
        n_cells, nu_loc = udofs.shape
        keep = [udofs, pdofs]

        def ip(a):
            a, p = _i(a)
            keep.append(a)
            return p

        def dpp(arrs):
            ptrs = (_dp * len(arrs))()
            for k, a in enumerate(arrs):
                a, p = _d(a)
                keep.append(a)
                ptrs[k] = p
            keep.append(ptrs)
            return C.cast(ptrs, _dpp)

        create = L.ref_vanka2_create if one_block else L.ref_vanka_create
        self._h = create(
            self.n_u, int(arrays["n_active"]), self.n_p, n_cells, nu_loc,
            udofs.ctypes.data_as(_ip), pdofs.ctypes.data_as(_ip),
            ip(arrays["a_rowptr"]), ip(arrays["a_col"]),
            dpp(arrays["a"][:1] if one_block else arrays["a"]),
            ip(arrays["b_rowptr"]), ip(arrays["b_col"]), dpp(arrays["b"]),
            ip(arrays["bt_rowptr"]), ip(arrays["bt_col"]), dpp(arrays["bt"]), float(alpha))
        if not self._h:
            raise ValueError(f"unsupported local velocity size {nu_loc}")
        if colours is not None:
            assert len(colours) == n_cells
            ptr, order = colour_lists(colours)
            if L.ref_vanka_set_colours(self._h, len(ptr) - 1, ptr.ctypes.data_as(_ip),
                                       order.ctypes.data_as(_ip), n_cells, threads) != 0:
                raise ValueError("inconsistent colouring")

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.ref_vanka_destroy(self._h)
            self._h = None

    def cell_vanka(self, u, rhs, sweeps: int = 1, damp: float = 1.0) -> np.ndarray:
        """``sweeps`` reference CellVanka sweeps from ``u`` (a copy is
        returned) with damping ``damp``."""
        u = np.array(u, dtype=np.float64, copy=True)
        rhs, rp = _d(rhs)
        assert u.size == rhs.size == 3 * self.n_u + self.n_p
        self._L.ref_vanka_sweeps(self._h, u.ctypes.data_as(_dp), rp, sweeps, damp)
        return u

    def solve_exact(self, rhs, pin_pressure: bool = True) -> np.ndarray:
        """TNSE_MGLevel4::SolveExact: the dense solve of the level's system,
        the first pressure equation replaced by p_0 = 0 when
        ``pin_pressure`` (INTERNAL_PROJECT_PRESSURE)."""
        rhs, rp = _d(rhs)
        assert rhs.size == 3 * self.n_u + self.n_p
        u = np.zeros(rhs.size)
        self._L.ref_vanka_solve_exact(self._h, u.ctypes.data_as(_dp), rp, int(pin_pressure))
        return u


_TLIB = {}


def ref_transfer_lib(hybrid: bool = False):
    """The loaded transfer harness (with ``hybrid``: its colour-parallel
    build), or None when the reference tree is absent."""
    if hybrid not in _TLIB:
        path = build_ref_transfer(hybrid=hybrid)
        if path is None:
            return None
        L = C.CDLL(str(path))
        L.ref_transfer_create.argtypes = [C.c_int] * 4 + [_ip, _ip] + [C.c_int] * 4 + [_ip] * 4
        L.ref_transfer_create.restype = C.c_void_p
        L.ref_transfer_destroy.argtypes = [C.c_void_p]
        L.ref_transfer_destroy.restype = None
        L.ref_transfer_prolongate.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_transfer_prolongate.restype = None
        L.ref_transfer_restrict.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_transfer_restrict.restype = None
        _ipp = C.POINTER(_ip)
        L.ref_cycle_create.argtypes = ([C.c_int] + [_ip] * 4 + [_ipp] * 4
                                       + [C.c_int, _ipp, _ipp, _dpp, _ipp, _ipp, _dpp, _ipp,
                                          _ipp, _dpp, C.c_double, C.c_double])
        L.ref_cycle_create.restype = C.c_void_p
        L.ref_cycle_destroy.argtypes = [C.c_void_p]
        L.ref_cycle_destroy.restype = None
        L.ref_cycle_vcycle.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_int, C.c_double]
        L.ref_cycle_vcycle.restype = None
        L.ref_cycle_configure.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double]
        L.ref_cycle_configure.restype = None
        if hybrid:
            L.ref_cycle_set_colours.argtypes = [C.c_void_p, C.c_int, C.c_int, _ip, _ip, C.c_int,
                                                C.c_int]
            L.ref_cycle_set_colours.restype = C.c_int
        _TLIB[hybrid] = L
    return _TLIB[hybrid]


def colour_lists(colours):
    """(colour_ptr, cell_order) of a per-cell colour array: the colours in
    increasing order, each with its cells in index order."""
    col = np.asarray(colours, dtype=np.int64)
    assert col.ndim == 1 and col.size and col.min() >= 0
    order = np.argsort(col, kind="stable").astype(np.int32)
    counts = np.bincount(col)
    ptr = np.concatenate([[0], np.cumsum(counts[counts > 0])]).astype(np.int32)
    return ptr, order


class RefTransfer:
    """The reference's Prolongate / DefectRestriction between level ``level``
    of a hexahedral Q2/P1disc problem and the next coarser one
    (src/FE/MGComponents3D.C, run by oracle/ref_transfer.cpp)."""

    def __init__(self, problem, level: int):
        L = ref_transfer_lib()
        if L is None:
            raise RuntimeError("reference tree not present: the transfer harness is not built")
        self._L = L
        self._h = None
        c, f = problem.arrays(level - 1), problem.arrays(level)
        self.nc = 3 * c["n_udof"] + c["n_pdof"]
        self.nf = 3 * f["n_udof"] + f["n_pdof"]
        keep = [np.ascontiguousarray(a, dtype=np.int32) for a in
                (c["cell_udofs"], c["cell_pdofs"], f["cell_udofs"], f["cell_pdofs"],
                 f["cell_parent"], f["cell_child"])]
        ptr = [a.ctypes.data_as(_ip) for a in keep]
        self._h = L.ref_transfer_create(c["n_cells"], c["n_udof"], c["n_active"], c["n_pdof"],
                                        ptr[0], ptr[1], f["n_cells"], f["n_udof"],
                                        f["n_active"], f["n_pdof"], *ptr[2:])
        if not self._h:
            raise ValueError("the levels are not a regular refinement (8 children per cell)")

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.ref_transfer_destroy(self._h)
            self._h = None

    def prolongate(self, coarse) -> np.ndarray:
        coarse, cp = _d(coarse)
        assert coarse.size == self.nc
        fine = np.empty(self.nf)
        self._L.ref_transfer_prolongate(self._h, cp, fine.ctypes.data_as(_dp))
        return fine

    def restrict(self, fine) -> np.ndarray:
        fine, fp = _d(fine)
        assert fine.size == self.nf
        coarse = np.empty(self.nc)
        self._L.ref_transfer_restrict(self._h, fp, coarse.ctypes.data_as(_dp))
        return coarse


class RefCycle:
    """The reference's multigrid preconditioner call, TMultiGridIte::Iterate
    (src/FE/MultiGridIte.C:76-132) with TNSE_MultiGrid::Cycle
    (src/FE/NSE_MultiGrid.C:434-1779), over every level of a hexahedral
    Q2/P1disc problem (run by oracle/ref_transfer.cpp): cell Vanka on each
    level above the coarsest, the exact solve on the coarsest one.  The
    sequential build's cell loop, or with ``colours`` the colour-parallel
    build's OpenMP colour loop over every smoothed level's own colouring
    (its cell_colour), on ``threads`` threads."""

    def __init__(self, problem, alpha: float = 1.0, beta: float = 1.0, colours: bool = False,
                 threads: int = 4):
        L = ref_transfer_lib(hybrid=colours)
        if L is None:
            raise RuntimeError("reference tree not present: the transfer harness is not built")
        self._L = L
        self._h = None
        lv = [problem.arrays(l) for l in range(problem.n_levels)]
        top = lv[-1]
        self.nf = 3 * top["n_udof"] + top["n_pdof"]
        keep = []

        def ints(vals):
            v = np.ascontiguousarray(vals, dtype=np.int32)
            keep.append(v)
            return v.ctypes.data_as(_ip)

        def iarr(arrs):  # one int array per entry; None -> null
            v = [None if a is None else np.ascontiguousarray(a, dtype=np.int32) for a in arrs]
            keep.extend(x for x in v if x is not None)
            return (_ip * len(v))(*[_ip() if x is None else x.ctypes.data_as(_ip) for x in v])

        def darr(arrs):
            v = [np.ascontiguousarray(a, dtype=np.float64) for a in arrs]
            keep.extend(v)
            return (_dp * len(v))(*[a.ctypes.data_as(_dp) for a in v])

        n_blocks = len(lv[0]["a"])
        assert all(len(d["a"]) == n_blocks for d in lv)

        def cat(key):
            return [m for d in lv for m in d[key]]

        self._keep = keep
        self._h = L.ref_cycle_create(
            len(lv), ints([d["n_cells"] for d in lv]), ints([d["n_udof"] for d in lv]),
            ints([d["n_active"] for d in lv]), ints([d["n_pdof"] for d in lv]),
            iarr([d["cell_udofs"] for d in lv]), iarr([d["cell_pdofs"] for d in lv]),
            iarr([None] + [d["cell_parent"] for d in lv[1:]]),
            iarr([None] + [d["cell_child"] for d in lv[1:]]), n_blocks,
            iarr([d["a_rowptr"] for d in lv]), iarr([d["a_col"] for d in lv]),
            darr(cat("a") if n_blocks == 9 else
                 [m for d in lv for m in list(d["a"]) + [d["a"][0]] * 8]),
            iarr([d["b_rowptr"] for d in lv]), iarr([d["b_col"] for d in lv]), darr(cat("b")),
            iarr([d["bt_rowptr"] for d in lv]), iarr([d["bt_col"] for d in lv]), darr(cat("bt")),
            alpha, beta)
        if not self._h:
            raise ValueError("the levels are not a regular refinement (8 children per cell)")
        if colours:
            for l in range(1, len(lv)):
                ptr, order = colour_lists(lv[l]["cell_colour"])
                if L.ref_cycle_set_colours(self._h, l, len(ptr) - 1, ptr.ctypes.data_as(_ip),
                                           order.ctypes.data_as(_ip), lv[l]["n_cells"],
                                           threads) != 0:
                    raise ValueError(f"inconsistent colouring on level {l}")

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.ref_cycle_destroy(self._h)
            self._h = None

    def vcycle(self, v, pre: int = 2, post: int = 2, damp: float = 1.0) -> np.ndarray:
        v, vp = _d(v)
        assert v.size == self.nf
        z = np.zeros(self.nf)
        self._L.ref_cycle_vcycle(self._h, vp, z.ctypes.data_as(_dp), pre, post, damp)
        return z

    def preconditioner(self, pre: int = 2, post: int = 2, damp: float = 1.0):
        """(C function pointer, context) of this cycle as the preconditioner
        callback of RefLevel.fgmres, with the given smoothing."""
        self._L.ref_cycle_configure(self._h, pre, post, damp)
        return C.cast(self._L.ref_cycle_precond, C.c_void_p), C.c_void_p(self._h)


def ref_into_l20(v, order: int = -11) -> np.ndarray:
    """IntoL20Vector3D on a copy of ``v``."""
    L = ref_harness_lib()
    if L is None:
        raise RuntimeError("reference tree not present: the reference harness is not built")
    v = np.array(v, dtype=np.float64, copy=True)
    L.ref_into_l20(v.ctypes.data_as(_dp), v.size, order)
    return v
