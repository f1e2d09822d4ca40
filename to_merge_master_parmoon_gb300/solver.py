"""Python handle on libpmgpu (include/pmgpu.h).

``PmSolver`` mirrors the objects the reference builds for
SC_SOLVER_SADDLE=16 / SC_PRECONDITIONER_SADDLE=5 / SC_SMOOTHER_SADDLE=2:
``add_level`` is TNSE_MultiGrid::AddLevel, ``defect`` TNSE_MGLevel4::Defect,
``coupled_defect`` Defect_NSE4, ``matvec`` MatVect_NSE4, ``cell_vanka``
TNSE_MGLevel4::CellVanka, ``restrict``/``prolongate`` DefectRestriction /
Prolongate, ``solve_exact`` TNSE_MGLevel4::SolveExact, ``vcycle``
TMultiGridIte::Iterate and ``iterate`` TFgmresIte::Iterate.  Every call goes
through the C ABI into CUDA kernels; a missing library or device raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import PM_STATUS, PmLevelDesc, PmOptions, PmResult, gpu_lib

OPTION_NAMES = [f for f, _ in PmOptions._fields_]


class PmError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{PM_STATUS.get(status, status)}: {msg}")
        self.status = status


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class PmSolver:
    def __init__(self, levels=None, **options):
        self._lib = gpu_lib()
        opt = PmOptions()
        self._lib.pm_default_options(C.byref(opt))
        for k, v in options.items():
            if k == "precision" and isinstance(v, str):
                v = {"fp64": 0, "mixed": 1}[v]
            if k not in OPTION_NAMES:
                raise KeyError(f"unknown option {k}")
            setattr(opt, k, v)
        self.options = opt
        h = C.c_void_p()
        st = self._lib.pm_create(C.byref(h), C.byref(opt))
        if st != 0:
            raise PmError(st, "pm_create failed")
        self._h = h
        self._ndof = []
        if levels is not None:
            for d in levels:
                self.add_level(d)
            self.setup()

    # ---------------------------------------------------------------- admin
    def _check(self, st: int, what: str) -> int:
        if st not in (0,):
            msg = self._lib.pm_last_error(self._h)
            raise PmError(st, f"{what}: {msg.decode() if msg else ''}")
        return st

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pm_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def add_level(self, desc):
        self._check(self._lib.pm_add_level(self._h, C.byref(desc)), "pm_add_level")
        self._ndof.append(3 * desc.n_udof + desc.n_pdof)

    def setup(self):
        self._check(self._lib.pm_setup(self._h), "pm_setup")

    def update_matrices(self, descs):
        self._check(self._lib.pm_update_matrices(self._h, descs, len(descs)), "pm_update_matrices")

    def refactor(self) -> float:
        ms = C.c_double()
        self._check(self._lib.pm_refactor(self._h, C.byref(ms)), "pm_refactor")
        return ms.value

    @property
    def n_levels(self) -> int:
        return self._lib.pm_n_levels(self._h)

    def level_decoupled(self, level: int) -> int:
        """How a nine-block level runs: 0 nine blocks and the 85x85 LU; 1
        A12..A32 zero (three diagonal blocks, block elimination); 2 also
        A11 = A22 = A33 (one block read, one inverse per cell)."""
        return self._lib.pm_level_decoupled(self._h, level)

    def ndof(self, level: int = -1) -> int:
        return self._ndof[level]

    @property
    def kernel_launches(self) -> int:
        return self._lib.pm_kernel_launches(self._h)

    @property
    def device_bytes(self) -> int:
        return self._lib.pm_device_bytes(self._h)

    def profile(self, enable: bool = True):
        self._check(self._lib.pm_profile_enable(self._h, int(enable)), "pm_profile_enable")

    def profile_read(self) -> dict:
        """Totals of the two Vanka sweep kernels since profile(True):
        {"residual": {...}, "apply": {...}} with ms, launches, bytes."""
        out = {}
        for k, name in enumerate(("residual", "apply")):
            ms, n, b = C.c_double(), C.c_longlong(), C.c_double()
            self._check(self._lib.pm_profile_read(self._h, k, C.byref(ms), C.byref(n), C.byref(b)),
                        "pm_profile_read")
            out[name] = {"ms": ms.value, "launches": n.value, "bytes": b.value}
        return out

    def assemble_level(self, level, cell_h, conv, nu):
        """pm_assemble_level: Galerkin Oseen blocks of one level on the device
        from cell sizes (n_cells x 3) and nodal convection [b1|b2|b3]."""
        cell_h, conv = _f64(cell_h), _f64(conv)
        self._check(self._lib.pm_assemble_level(self._h, level, _dp(cell_h), _dp(conv), float(nu)),
                    "pm_assemble_level")

    def assemble_level_device(self, level, d_cell_h: int, d_conv: int, nu):
        """pm_assemble_level_device: the same from device arrays (addresses)."""
        self._check(self._lib.pm_assemble_level_device(self._h, level, C.c_void_p(d_cell_h),
                                                       C.c_void_p(d_conv), float(nu)),
                    "pm_assemble_level_device")

    def assemble_system_level_device(self, level, d_cell_h: int, d_conv: int, nu, c_mass, c_a,
                                     b_scale=1.0, bt_scale=1.0):
        """pm_assemble_system_level_device: the theta-scheme system from device arrays."""
        self._check(self._lib.pm_assemble_system_level_device(
            self._h, level, C.c_void_p(d_cell_h), C.c_void_p(d_conv), float(nu), float(c_mass),
            float(c_a), float(b_scale), float(bt_scale)), "pm_assemble_system_level_device")

    def assemble_system_level(self, level, cell_h, conv, nu, c_mass, c_a, b_scale=1.0,
                              bt_scale=1.0):
        """pm_assemble_system_level: c_mass M + c_a A in the velocity blocks,
        scaled B and BT (theta-scheme system of TSystemTNSE3D)."""
        cell_h, conv = _f64(cell_h), _f64(conv)
        self._check(self._lib.pm_assemble_system_level(self._h, level, _dp(cell_h), _dp(conv),
                                                       float(nu), float(c_mass), float(c_a),
                                                       float(b_scale), float(bt_scale)),
                    "pm_assemble_system_level")

    def system_rhs(self, old_rhs, rhs, sol, c_old, c_new, c2):
        """pm_system_rhs: working right-hand side of the theta scheme."""
        old_rhs, rhs, sol = _f64(old_rhs), _f64(rhs), _f64(sol)
        out = np.empty_like(rhs)
        self._check(self._lib.pm_system_rhs(self._h, _dp(old_rhs), _dp(rhs), _dp(sol), float(c_old),
                                            float(c_new), float(c2), _dp(out)), "pm_system_rhs")
        return out

    def system_rhs_device(self, d_old: int, d_rhs: int, d_sol: int, c_old, c_new, c2, d_out: int):
        """pm_system_rhs_device: the same on device vectors (addresses)."""
        self._check(self._lib.pm_system_rhs_device(self._h, C.c_void_p(d_old), C.c_void_p(d_rhs),
                                                   C.c_void_p(d_sol), float(c_old), float(c_new),
                                                   float(c2), C.c_void_p(d_out)),
                    "pm_system_rhs_device")

    def interpolate_coarse(self, level, d_fine: int, d_coarse: int):
        """pm_interpolate_coarse: velocity nodal values of `level` at the nodes
        of level-1 (device addresses)."""
        self._check(self._lib.pm_interpolate_coarse(self._h, level, C.c_void_p(d_fine),
                                                    C.c_void_p(d_coarse)),
                    "pm_interpolate_coarse")

    # ------------------------------------------------------------ level ops
    def coupled_defect(self, level, x, b, project=True):
        x, b = _f64(x), _f64(b)
        r = np.empty_like(x)
        self._check(self._lib.pm_coupled_defect(self._h, level, _dp(x), _dp(b), _dp(r), int(project)),
                    "pm_coupled_defect")
        return r

    def defect(self, level, u, f):
        u, f = _f64(u), _f64(f)
        d = np.empty_like(u)
        res = C.c_double()
        self._check(self._lib.pm_defect(self._h, level, _dp(u), _dp(f), _dp(d), C.byref(res)),
                    "pm_defect")
        return d, res.value

    def matvec(self, level, x):
        x = _f64(x)
        y = np.empty_like(x)
        self._check(self._lib.pm_matvec(self._h, level, _dp(x), _dp(y)), "pm_matvec")
        return y

    def cell_vanka(self, level, u, rhs, sweeps=1):
        u = _f64(u).copy()
        rhs = _f64(rhs)
        self._check(self._lib.pm_cell_vanka(self._h, level, _dp(u), _dp(rhs), sweeps), "pm_cell_vanka")
        return u

    def restrict(self, level, fine):
        fine = _f64(fine)
        coarse = np.empty(self._ndof[level - 1])
        self._check(self._lib.pm_restrict(self._h, level, _dp(fine), _dp(coarse)), "pm_restrict")
        return coarse

    def prolongate(self, level, coarse):
        coarse = _f64(coarse)
        fine = np.empty(self._ndof[level])
        self._check(self._lib.pm_prolongate(self._h, level, _dp(coarse), _dp(fine)), "pm_prolongate")
        return fine

    def solve_exact(self, rhs):
        rhs = _f64(rhs)
        u = np.empty_like(rhs)
        self._check(self._lib.pm_solve_exact(self._h, _dp(rhs), _dp(u)), "pm_solve_exact")
        return u

    def vcycle(self, v):
        v = _f64(v)
        z = np.empty_like(v)
        self._check(self._lib.pm_vcycle(self._h, _dp(z), _dp(v)), "pm_vcycle")
        return z

    # ------------------------------------------------------ learned smoother
    def attach_learned(self, mlp, omega=1.0, fallback_ratio=0.5):
        """Insert the network as an extra post-smoothing step on every level
        (None detaches)."""
        self._check(self._lib.pm_learned_attach(self._h, mlp._h if mlp is not None else None,
                                                omega, fallback_ratio), "pm_learned_attach")
        self._mlp = mlp

    def learned_status(self):
        on, fb = C.c_int(), C.c_int()
        self._check(self._lib.pm_learned_status(self._h, C.byref(on), C.byref(fb)),
                    "pm_learned_status")
        return {"enabled": on.value, "fallbacks": fb.value}

    def harvest(self, sol_exact, rhs, n_cycles, d_X_ptr, d_T_ptr, capacity, n_pairs):
        """(residual, error) training pairs of the plain V-cycle iteration on
        the finest level; returns the new row count."""
        sol_exact, rhs = _f64(sol_exact), _f64(rhs)
        n = C.c_longlong(n_pairs)
        self._check(self._lib.pm_learned_harvest(self._h, _dp(sol_exact), _dp(rhs), n_cycles,
                                                 C.c_void_p(d_X_ptr), C.c_void_p(d_T_ptr),
                                                 capacity, C.byref(n)), "pm_learned_harvest")
        return n.value

    # ---------------------------------------------------------------- solve
    def iterate(self, sol, rhs, allow=(0,)):
        """TFgmresIte::Iterate on host vectors; returns (solution, result dict)."""
        sol = _f64(sol).copy()
        rhs = _f64(rhs)
        r = PmResult()
        st = self._lib.pm_solve(self._h, _dp(sol), _dp(rhs), C.byref(r))
        if st not in allow:
            self._check(st, "pm_solve")
        out = r.as_dict()
        out["status_name"] = PM_STATUS.get(st, str(st))
        return sol, out

    def iterate_device(self, d_sol_ptr: int, d_rhs_ptr: int, allow=(0,)):
        """TFgmresIte::Iterate on device vectors (raw CUDA pointers)."""
        r = PmResult()
        st = self._lib.pm_solve_device(self._h, C.c_void_p(d_sol_ptr), C.c_void_p(d_rhs_ptr), C.byref(r))
        if st not in allow:
            self._check(st, "pm_solve_device")
        out = r.as_dict()
        out["status_name"] = PM_STATUS.get(st, str(st))
        return out


def device_count() -> int:
    return gpu_lib().pm_device_count()


def solve_batch(solvers, sols, rhss, nthreads=0, allow=(0,)):
    """pm_solve_batch: independent systems, one set-up PmSolver each, solved
    concurrently (each handle's stream overlaps the others on the GPU).
    Returns (solutions, list of result dicts)."""
    n = len(solvers)
    lib = solvers[0]._lib
    sols = [_f64(x).copy() for x in sols]
    rhss = [_f64(b) for b in rhss]
    H = (C.c_void_p * n)(*[S._h for S in solvers])
    X = (C.POINTER(C.c_double) * n)(*[_dp(x) for x in sols])
    B = (C.POINTER(C.c_double) * n)(*[_dp(b) for b in rhss])
    R = (PmResult * n)()
    st = lib.pm_solve_batch(H, n, X, B, R, nthreads)
    if st not in allow:
        raise PmError(st, "pm_solve_batch")
    return sols, [R[i].as_dict() for i in range(n)]



class PmFusedSolver(PmSolver):
    """Independent systems on one mesh stacked into one block-diagonal
    hierarchy (pm_add_level_batch): every V-cycle and FGMRES kernel covers all
    of them in one launch, while each system keeps its own Arnoldi process,
    Givens rotations, coarse inverse, L2_0 projection and stopping test.
    ``systems[s][l]`` is the level-l descriptor of system s (equal sizes
    across systems on every level)."""

    def __init__(self, systems, **options):
        super().__init__(None, **options)
        G = len(systems)
        L = len(systems[0])
        if any(len(d) != L for d in systems):
            raise ValueError("every stacked system needs the same number of levels")
        for lev in range(L):
            arr = (PmLevelDesc * G)(*[systems[s][lev] for s in range(G)])
            self._check(self._lib.pm_add_level_batch(self._h, arr, G), "pm_add_level_batch")
            d = systems[0][lev]
            self._ndof.append(G * (3 * d.n_udof + d.n_pdof))
        self.setup()
        self.n_systems = G
        self.ndof_sys = 3 * systems[0][-1].n_udof + systems[0][-1].n_pdof

    def solve(self, sols, rhss, allow=(0,)):
        """pm_solve_fused on host vectors (one per system, own layout);
        returns (solutions, list of per-system result dicts)."""
        G = self.n_systems
        sols = [_f64(x).copy() for x in sols]
        rhss = [_f64(b) for b in rhss]
        X = (C.POINTER(C.c_double) * G)(*[_dp(x) for x in sols])
        B = (C.POINTER(C.c_double) * G)(*[_dp(b) for b in rhss])
        R = (PmResult * G)()
        st = self._lib.pm_solve_fused(self._h, X, B, R)
        if st not in allow:
            self._check(st, "pm_solve_fused")
        out = [R[i].as_dict() for i in range(G)]
        for o in out:
            o["status_name"] = PM_STATUS.get(o["status"], str(o["status"]))
        return sols, out


def solve_fused_groups(groups, sols, rhss, allow=(0,)):
    """Several PmFusedSolver groups at once, one host thread per group (the
    groups' streams overlap on the GPU).  sols[g] / rhss[g]: lists of the
    group's vectors.  Returns (solutions, results) nested like the input."""
    import threading
    out = [None] * len(groups)
    err = []

    def run(g):
        try:
            out[g] = groups[g].solve(sols[g], rhss[g], allow=allow)
        except Exception as e:  # reported after the join
            err.append(e)

    threads = [threading.Thread(target=run, args=(g,)) for g in range(len(groups))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if err:
        raise err[0]
    return [o[0] for o in out], [o[1] for o in out]
