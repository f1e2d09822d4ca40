"""GPU parity of one-block (NSTYPE-2) levels and of coupled NSTYPE-4 blocks.

One-block levels pass a[0] only (TNSE_MGLevel2's single A matrix,
src/FE/NSE_MGLevel2.C:54-110) and are smoothed by the exact block solve of
the cell system (A^{-1} and the 4x4 Schur complement) instead of the 85x85
LU.  The oracle runs the same problem as nine blocks with the 85x85 LU
(NSE_MGLevel4.C:1653-2087), so the two agree to rounding: 1e-12 for the
operator, 1e-9 for FP64 sweeps, 5e-4 for the FP32 V-cycle, 1e-6 for the
FGMRES solution.

The coupled test gives A12..A32 seeded nonzero entries on the active rows
(as a Newton or deformation-tensor linearisation has them) and keeps the
builder's values on the Dirichlet rows, which the reference ignores there
(MGComponents3D.C:3143-3162, NSE_MGLevel4.C:1853-1854)."""
import ctypes as C

import numpy as np
import pytest

from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def normalise_p(v, nu):
    v = v.copy()
    v[3 * nu::4] -= v[3 * nu::4].mean()
    return v


@pytest.fixture(scope="module")
def P(problems):
    return problems(3, 1e-2, 0)


@pytest.fixture(scope="module")
def oracle(P):
    return Oracle(P)


@pytest.fixture(scope="module")
def one64(P):
    from to_merge_master_parmoon_gb300 import PmSolver
    return PmSolver(P.descs_one_block(), precision="fp64")


@pytest.fixture(scope="module")
def one32(P):
    from to_merge_master_parmoon_gb300 import PmSolver
    return PmSolver(P.descs_one_block(), precision="mixed")


def rand(P, level, seed):
    return np.random.default_rng(seed).standard_normal(P.ndof(level))


def test_levels_are_one_block(P, one64):
    from to_merge_master_parmoon_gb300 import PmSolver
    assert P.is_one_block()
    assert [one64._lib.pm_level_blocks(one64._h, l) for l in range(3)] == [1, 1, 1]
    S9 = PmSolver(P.descs)
    assert [S9._lib.pm_level_blocks(S9._h, l) for l in range(3)] == [9, 9, 9]


@pytest.mark.parametrize("level", [0, 1, 2])
def test_one_block_operator(P, one64, oracle, level):
    x, b = rand(P, level, 1), rand(P, level, 2)
    assert rel(one64.coupled_defect(level, x, b), oracle.coupled_defect(level, x, b)) < 1e-12
    assert rel(one64.matvec(level, x), oracle.matvec(level, x)) < 1e-12
    d_g, r_g = one64.defect(level, x, b)
    d_o, r_o = oracle.defect(level, x, b)
    assert rel(d_g, d_o) < 1e-12 and abs(r_g - r_o) < 1e-12 * r_o


def test_one_block_coarse(P, one64, oracle):
    b = rand(P, 0, 5)
    assert rel(one64.solve_exact(b), oracle.solve_exact(b)) < 1e-10


@pytest.mark.parametrize("level", [1, 2])
def test_one_block_vanka(P, one64, one32, oracle, level):
    u, f = 0.1 * rand(P, level, 6), rand(P, level, 7)
    for sweeps in (1, 2):
        ref = oracle.cell_vanka(level, u, f, sweeps)
        assert rel(one64.cell_vanka(level, u, f, sweeps), ref) < 1e-9
        assert rel(one32.cell_vanka(level, u, f, sweeps), ref) < 5e-4


def test_one_block_vcycle(P, one64, one32, oracle):
    v = rand(P, 2, 8)
    z_o = oracle.vcycle(v)
    assert rel(one64.vcycle(v), z_o) < 1e-9
    assert rel(one32.vcycle(v), z_o) < 5e-4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_one_block_fgmres(P, oracle, precision):
    from to_merge_master_parmoon_gb300 import PmSolver
    b = P.rhs()
    x0 = np.zeros_like(b)
    tol = 1e-10 * np.linalg.norm(oracle.coupled_defect(2, x0, b))
    xo, io = Oracle(P, restart=20, maxit=60, res_norm_min=tol).iterate(x0, b)
    S = PmSolver(P.descs_one_block(), precision=precision, restart=20, maxit=60, res_norm_min=tol)
    xg, ig = S.iterate(x0, b)
    nu = P.desc(2).n_udof
    assert ig["true_res"] <= 1.05 * tol
    assert rel(normalise_p(xg, nu), normalise_p(xo, nu)) < 1e-6
    if precision == "fp64":
        assert abs(ig["iterations"] - io["iterations"]) <= 1


def test_one_block_known_answer(problems):
    from to_merge_master_parmoon_gb300 import PmSolver
    Pq = problems(3, 1.0, 0, "quadlin_oseen")
    b, ex = Pq.rhs(), Pq.exact()
    r0 = np.linalg.norm(PmSolver(Pq.descs).coupled_defect(2, np.zeros_like(b), b))
    S = PmSolver(Pq.descs_one_block(), precision="mixed", restart=20, maxit=60,
                 res_norm_min=1e-12 * r0)
    x, _ = S.iterate(np.zeros_like(b), b)
    n3 = 3 * Pq.desc(2).n_udof
    assert np.abs(x[:n3] - ex[:n3]).max() < 1e-8
    dp = x[n3:] - ex[n3:]
    dp[0::4] -= dp[0::4].mean()
    assert np.abs(dp).max() < 1e-6


def test_block_count_errors(P):
    from to_merge_master_parmoon_gb300 import PmSolver
    from to_merge_master_parmoon_gb300.solver import PmError
    from to_merge_master_parmoon_gb300._lib import PmLevelDesc
    bad = (PmLevelDesc * P.n_levels)()
    for l in range(P.n_levels):
        C.pointer(bad[l])[0] = P.desc(l)
    bad[0].a[2] = None  # eight of nine blocks
    with pytest.raises(PmError, match="PM_BADARG"):
        PmSolver(bad)
    S = PmSolver(P.descs_one_block())
    with pytest.raises(PmError, match="PM_BADARG"):
        S.update_matrices(P.descs)  # nine blocks on one-block levels
    S.update_matrices(P.descs_one_block())


class Coupled:
    """The problem's levels with seeded coupling blocks A12..A32 on the
    active rows; everything else shared with the problem."""

    def __init__(self, P, eps, seed):
        from to_merge_master_parmoon_gb300._lib import PmLevelDesc
        rng = np.random.default_rng(seed)
        self.n_levels = P.n_levels
        self.descs = (PmLevelDesc * P.n_levels)()
        self._keep = [P]
        for l in range(P.n_levels):
            d = P.arrays(l)
            C.pointer(self.descs[l])[0] = P.desc(l)
            act = np.repeat(np.arange(d["n_udof"]) < d["n_active"], np.diff(d["a_rowptr"]))
            scale = np.abs(d["a"][0][act]).max()  # active rows (Dirichlet rows hold 1)
            for k in (1, 2, 3, 5, 6, 7):
                v = np.where(act, eps * scale * rng.standard_normal(act.size), d["a"][k])
                v = np.ascontiguousarray(v)
                self._keep.append(v)
                self.descs[l].a[k] = v.ctypes.data_as(C.POINTER(C.c_double))
        self._P = P

    def ndof(self, level=-1):
        return self._P.ndof(level)


def test_coupled_blocks(P):
    from to_merge_master_parmoon_gb300 import PmSolver
    Q = Coupled(P, 0.02, 11)
    O = Oracle(Q)
    S64 = PmSolver(Q.descs, precision="fp64")
    S32 = PmSolver(Q.descs, precision="mixed")
    for level in (0, 1, 2):
        x, b = rand(P, level, 21), rand(P, level, 22)
        assert rel(S64.coupled_defect(level, x, b), O.coupled_defect(level, x, b)) < 1e-12
        assert rel(S64.matvec(level, x), O.matvec(level, x)) < 1e-12
    b0 = rand(P, 0, 23)
    assert rel(S64.solve_exact(b0), O.solve_exact(b0)) < 1e-10
    for level in (1, 2):
        u, f = 0.1 * rand(P, level, 24), rand(P, level, 25)
        ref = O.cell_vanka(level, u, f, 1)
        assert rel(S64.cell_vanka(level, u, f, 1), ref) < 1e-9
        assert rel(S32.cell_vanka(level, u, f, 1), ref) < 5e-4
    v = rand(P, 2, 26)
    z = O.vcycle(v)
    assert rel(S64.vcycle(v), z) < 1e-9
    assert rel(S32.vcycle(v), z) < 5e-4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_coupled_blocks_fgmres(P, precision):
    from to_merge_master_parmoon_gb300 import PmSolver
    Q = Coupled(P, 0.01, 11)
    b = P.rhs()
    x0 = np.zeros_like(b)
    O = Oracle(Q)
    tol = 1e-10 * np.linalg.norm(O.coupled_defect(2, x0, b))
    xo, io = Oracle(Q, restart=20, maxit=80, res_norm_min=tol).iterate(x0, b)
    S = PmSolver(Q.descs, precision=precision, restart=20, maxit=80, res_norm_min=tol)
    xg, ig = S.iterate(x0, b)
    nu = P.desc(2).n_udof
    assert ig["true_res"] <= 1.05 * tol
    assert rel(normalise_p(xg, nu), normalise_p(xo, nu)) < 1e-6
    if precision == "fp64":
        assert ig["iterations"] == io["iterations"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_upload_by_host_reads_matches_copies(P, precision):
    """upload_mode=1 (the SMs read the caller's arrays, FP32 copies and the
    Dirichlet-row zeroing of A12..A32 in the same pass) stores exactly what
    the copy-engine path stores: identical operator, sweeps and V-cycle."""
    from to_merge_master_parmoon_gb300 import PmSolver
    Q = Coupled(P, 0.01, 11)
    for descs in (Q.descs, P.descs_one_block()):
        S0 = PmSolver(descs, precision=precision, upload_mode=0)
        S1 = PmSolver(descs, precision=precision, upload_mode=1)
        for level in (0, 1, 2):
            x = rand(P, level, 31)
            assert np.array_equal(S0.matvec(level, x), S1.matvec(level, x))
        u, f = 0.1 * rand(P, 2, 32), rand(P, 2, 33)
        assert np.array_equal(S0.cell_vanka(2, u, f, 1), S1.cell_vanka(2, u, f, 1))
        v = rand(P, 2, 34)
        assert np.array_equal(S0.vcycle(v), S1.vcycle(v))
        S1.update_matrices(descs)
        assert np.array_equal(S0.vcycle(v), S1.vcycle(v))
