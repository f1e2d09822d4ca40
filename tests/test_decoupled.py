"""Nine-block levels whose off-diagonal velocity blocks vanish run decoupled:
their defects and sweeps read the diagonal blocks only and each cell's 85x85
system is solved by exact block elimination (27x27 inverses and the 4x4
pressure Schur complement) instead of the LU of the reference's CellVanka
(src/FE/NSE_MGLevel4.C:1784-2031).  Mode 1: A11, A22, A33 differ (three
arrays, three inverses); mode 2: A11 = A22 = A33, as in the Galerkin Oseen
form (src/FE/NSE3D_FixPo.C:1919-2071): one array, one inverse.  The local
solution is the same, so the sweeps match the oracle's LU sweeps to the FP64
tolerance of the other Vanka tests (1e-9), the mixed ones to 5e-4, and
FGMRES reaches the same solution (1e-6 after L2_0 normalisation) in the same
FP64 iteration count.

A level whose A12..A32 hold nonzero entries keeps the 85x85 LU and all nine
blocks (mode 0); pm_update_matrices re-checks after every upload and
switches.
"""
import numpy as np
import pytest

from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu

OFFDIAG = (1, 2, 3, 5, 6, 7)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def normalise_p(v, nu):
    v = v.copy()
    v[3 * nu::4] -= v[3 * nu::4].mean()
    return v


def couple(P, eps):
    """Velocity coupling A12 = A21 = eps A11 on every level (active rows: the
    off-diagonal blocks of Dirichlet rows are ignored), in place."""
    for level in range(P.n_levels):
        a = P.arrays(level)
        a["a"][1][:] = eps * a["a"][0]
        a["a"][3][:] = eps * a["a"][0]


def uncouple(P):
    for level in range(P.n_levels):
        a = P.arrays(level)
        for k in OFFDIAG:
            a["a"][k][:] = 0.0


def distinct_diagonal(P):
    """A22 = 1.5 A11, A33 = 0.75 A11 (still uncoupled), in place."""
    for level in range(P.n_levels):
        a = P.arrays(level)
        a["a"][4][:] = 1.5 * a["a"][0]
        a["a"][8][:] = 0.75 * a["a"][0]


def fgmres_parity(P, S, oracle_params=None):
    b = P.rhs()
    x0 = np.zeros_like(b)
    L = P.n_levels
    r0 = np.linalg.norm(Oracle(P).coupled_defect(L - 1, x0, b))
    tol = 1e-10 * r0
    xo, io = Oracle(P, restart=20, maxit=80, res_norm_min=tol).iterate(x0, b)
    xg, ig = S.iterate(x0, b)
    nu = P.desc(L - 1).n_udof
    return rel(normalise_p(xg, nu), normalise_p(xo, nu)), ig, io, tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_galerkin_levels_run_decoupled(problems, precision):
    from to_merge_master_parmoon_gb300 import PmSolver
    P = problems(3, 1e-2, 0)
    S = PmSolver(P.descs, precision=precision, restart=20, maxit=80)
    assert [S.level_decoupled(l) for l in range(3)] == [2, 2, 2]
    S0 = PmSolver(P.descs, precision=precision, decouple=0)
    assert [S0.level_decoupled(l) for l in range(3)] == [0, 0, 0]
    O = Oracle(P)
    rng = np.random.default_rng(3)
    tol = 1e-9 if precision == "fp64" else 5e-4
    for level in (1, 2):
        u = 0.1 * rng.standard_normal(P.ndof(level))
        f = rng.standard_normal(P.ndof(level))
        want = O.cell_vanka(level, u, f, 2)
        assert rel(S.cell_vanka(level, u, f, 2), want) < tol
        assert rel(S0.cell_vanka(level, u, f, 2), want) < tol
        x, b = rng.standard_normal(P.ndof(level)), rng.standard_normal(P.ndof(level))
        assert rel(S.coupled_defect(level, x, b), O.coupled_defect(level, x, b)) < (
            1e-12 if precision == "fp64" else 1e-12)
    S0.close()
    S.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_decoupled_fgmres_matches_oracle(problems, precision):
    from to_merge_master_parmoon_gb300 import PmSolver
    P = problems(3, 1e-2, 0)
    b = P.rhs()
    r0 = np.linalg.norm(Oracle(P).coupled_defect(2, np.zeros_like(b), b))
    S = PmSolver(P.descs, precision=precision, restart=20, maxit=80, res_norm_min=1e-10 * r0)
    d, ig, io, tol = fgmres_parity(P, S)
    assert ig["true_res"] <= 1.05 * tol and d < 1e-6
    if precision == "fp64":
        assert ig["iterations"] == io["iterations"]
    S.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_distinct_diagonal_blocks(precision):
    """Uncoupled levels with A11, A22, A33 all different run in mode 1 (three
    arrays, three inverses per cell) and match the oracle's LU sweeps and
    FGMRES."""
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    P = OseenProblem(n_levels=3, nu=1e-2, seed=4)
    distinct_diagonal(P)
    b = P.rhs()
    r0 = np.linalg.norm(Oracle(P).coupled_defect(2, np.zeros_like(b), b))
    S = PmSolver(P.descs, precision=precision, restart=20, maxit=80, res_norm_min=1e-10 * r0)
    assert [S.level_decoupled(l) for l in range(3)] == [1, 1, 1]
    O = Oracle(P)
    rng = np.random.default_rng(8)
    tol = 1e-9 if precision == "fp64" else 5e-4
    for level in (1, 2):
        u = 0.1 * rng.standard_normal(P.ndof(level))
        f = rng.standard_normal(P.ndof(level))
        assert rel(S.cell_vanka(level, u, f, 2), O.cell_vanka(level, u, f, 2)) < tol
    d, ig, io, tol = fgmres_parity(P, S)
    assert ig["true_res"] <= 1.05 * tol and d < 1e-6
    if precision == "fp64":
        assert ig["iterations"] == io["iterations"]
    S.close()


def test_coupled_blocks_keep_the_lu_and_update_switches():
    """Set up on Galerkin values (mode 2 on every level), then
    pm_update_matrices with A12 = A21 = 0.05 A11 switches every level to the
    85x85 LU and the nine blocks (mode 0: its factor storage grows), then
    uncoupled with distinct diagonal blocks to mode 1; each time FGMRES
    matches the oracle's."""
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    P = OseenProblem(n_levels=3, nu=1e-2, seed=5)
    b = P.rhs()
    r0 = np.linalg.norm(Oracle(P).coupled_defect(2, np.zeros_like(b), b))
    S = PmSolver(P.descs, precision="fp64", restart=20, maxit=80, res_norm_min=1e-10 * r0)
    assert [S.level_decoupled(l) for l in range(3)] == [2, 2, 2]
    d, ig, io, tol = fgmres_parity(P, S)
    assert d < 1e-6 and ig["iterations"] == io["iterations"]
    couple(P, 0.05)
    S.update_matrices(P.descs)
    assert [S.level_decoupled(l) for l in range(3)] == [0, 0, 0]
    d, ig, io, tol = fgmres_parity(P, S)
    assert d < 1e-6 and ig["iterations"] == io["iterations"]
    uncouple(P)
    distinct_diagonal(P)
    S.update_matrices(P.descs)
    assert [S.level_decoupled(l) for l in range(3)] == [1, 1, 1]
    d, ig, io, tol = fgmres_parity(P, S)
    assert d < 1e-6 and ig["iterations"] == io["iterations"]
    S.close()


@pytest.mark.parametrize("variant", [1, 2, -1])
@pytest.mark.parametrize("mode", [2, 1])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_residual_kernels_on_decoupled_levels(precision, mode, variant):
    """Every local-residual kernel on decoupled levels (1 row groups, 2
    flattened stream, -1 the tuner's choice) gives the oracle's sweeps;
    mode 2 reads one A block, mode 1 three."""
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    P = OseenProblem(n_levels=3, nu=1e-2, seed=6)
    if mode == 1:
        distinct_diagonal(P)
    S = PmSolver(P.descs, precision=precision, residual_variant=variant)
    assert [S.level_decoupled(l) for l in range(3)] == [mode] * 3
    res = [S._lib.pm_level_variant(S._h, l) % 2 for l in (1, 2)]
    if variant in (1, 2):
        assert res == [variant - 1] * 2
    O = Oracle(P)
    rng = np.random.default_rng(9)
    tol = 1e-9 if precision == "fp64" else 5e-4
    for level in (1, 2):
        u = 0.1 * rng.standard_normal(P.ndof(level))
        f = rng.standard_normal(P.ndof(level))
        assert rel(S.cell_vanka(level, u, f, 2), O.cell_vanka(level, u, f, 2)) < tol
    S.close()


@pytest.mark.parametrize("diagonal", ["equal", "distinct"])
def test_fp32_block_elimination(diagonal):
    """Mixed precision eliminates every decoupled cell in FP32 by default
    (factor_fp32 = -1; the stored factors are FP32 either way);
    factor_fp32 = 0 eliminates in FP64.  The FP32 sweeps stay within the
    mixed tolerance of the oracle's LU sweeps, and FGMRES reaches the same
    solution (1e-6 after L2_0 normalisation) in at most one iteration more
    than with FP64 elimination."""
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    P = OseenProblem(n_levels=3, nu=1e-2, seed=4)
    if diagonal == "distinct":
        distinct_diagonal(P)
    b = P.rhs()
    r0 = np.linalg.norm(Oracle(P).coupled_defect(2, np.zeros_like(b), b))
    kw = dict(precision="mixed", restart=20, maxit=80, res_norm_min=1e-10 * r0)
    S = PmSolver(P.descs, **kw)
    assert S.options.factor_fp32 == -1
    mode = 2 if diagonal == "equal" else 1
    assert [S.level_decoupled(l) for l in range(3)] == [mode] * 3
    O = Oracle(P)
    rng = np.random.default_rng(11)
    for level in (1, 2):
        u = 0.1 * rng.standard_normal(P.ndof(level))
        f = rng.standard_normal(P.ndof(level))
        assert rel(S.cell_vanka(level, u, f, 2), O.cell_vanka(level, u, f, 2)) < 5e-4
    d, ig, io, tol = fgmres_parity(P, S)
    S64 = PmSolver(P.descs, factor_fp32=0, **kw)
    _, i64, _, _ = fgmres_parity(P, S64)
    print(f"FP32 elimination ({diagonal} diagonal): {ig['iterations']} iterations "
          f"(FP64 elimination {i64['iterations']}), error vs oracle {d:.2e}")
    assert ig["status"] == 0
    assert ig["true_res"] <= 1.05 * tol and d < 1e-6
    assert ig["iterations"] <= i64["iterations"] + 1
    S.close()
    S64.close()
