"""Tetrahedral P2+bubble/P1disc systems (ParMooN's C_B2_3D_T_A / D_P1_3D_T
pair, 15 + 4 local DOFs, 49 x 49 Vanka blocks) on cubes split into 6 Kuhn
tetrahedra.

CPU: the builder's basis against the reference's own tables (golden fixture
made from include/FE3D/BF_C_T_B2_3D.h and BF_D_T_P1_3D.h), the
AnsatzQuadLin known answer (quadratic u, linear p lie in the discrete
spaces) by a sparse direct solve, exactness of the handed-over prolongation
on coarse-space functions, and the layout invariants (distinct cell DOFs, a
valid colouring, sorted patterns), and the oracle's FGMRES + GMG.
GPU: defects, mat-vecs, transfers, coarse solve, Vanka sweeps and V-cycles
against the oracle (FP64 1e-9, mixed 5e-4), FGMRES to 1e-10 with the
solution within 1e-6 and, in FP64, the same iteration count; the known
answer on the GPU; hexahedra-only features refuse tetrahedral levels."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

GOLD = Path(__file__).parent / "golden" / "basis_tet_b2_p1.json"
_cache = {}


def tetra(n_levels=2, example="quadlin_oseen", nu=1.0, seed=0):
    from to_merge_master_parmoon_gb300 import OseenProblem
    key = (n_levels, example, nu, seed)
    if key not in _cache:
        _cache[key] = OseenProblem(n_levels=n_levels, nu=nu, seed=seed, example=example,
                                   element="tetra")
    return _cache[key]


def test_tet_basis_matches_reference_tables():
    from to_merge_master_parmoon_gb300._lib import host_lib
    g = json.loads(GOLD.read_text())
    lib = host_lib()
    v, d = (C.c_double * 15)(), (C.c_double * 45)()
    pv, pd = (C.c_double * 4)(), (C.c_double * 12)()
    for pt, ref in zip(g["points"], g["values"]):
        lib.pmh_b2_basis(pt[0], pt[1], pt[2], v, d)
        lib.pmh_p1t_basis(pt[0], pt[1], pt[2], pv, pd)
        D, PD = np.array(d[:]).reshape(15, 3), np.array(pd[:]).reshape(4, 3)
        np.testing.assert_allclose(v[:], ref["b2"], rtol=0, atol=1e-13)
        for c, name in enumerate(("xi", "eta", "zeta")):
            np.testing.assert_allclose(D[:, c], ref["b2_" + name], rtol=0, atol=1e-12)
            np.testing.assert_allclose(PD[:, c], ref["p1_" + name], rtol=0, atol=1e-14)
        np.testing.assert_allclose(pv[:], ref["p1"], rtol=0, atol=1e-14)


def direct_solve(P, level, pin_value):
    K = P.scipy_matrix(level).tolil()
    b = P.rhs().copy()
    r = 3 * P.desc(level).n_udof
    K[r, :] = 0.0
    K[r, r] = 1.0
    b[r] = pin_value
    return spl.splu(K.tocsc()).solve(b)


@pytest.mark.parametrize("example,nu", [("quadlin_stokes", 1.0), ("quadlin_oseen", 1.0),
                                        ("quadlin_oseen", 1e-2)])
def test_tet_known_answer_direct(example, nu):
    P = tetra(example=example, nu=nu)
    ex = P.exact()
    n3 = 3 * P.desc(1).n_udof
    x = direct_solve(P, 1, ex[n3])
    assert np.abs(x[:n3] - ex[:n3]).max() < 1e-9
    assert np.abs(x[n3:] - ex[n3:]).max() < 1e-7


def test_tet_prolongation_is_exact_on_coarse_functions():
    P = tetra(n_levels=3)
    for level in (1, 2):
        a, c = P.arrays(level), P.desc(level - 1)
        Pu = sp.csr_matrix((a["pu_val"], a["pu_col"], a["pu_rowptr"]),
                           shape=(a["n_udof"], c.n_udof))
        cf = P.convection_nodal(level - 1).reshape(3, -1)  # quadratic: in P2 on both levels
        ff = P.convection_nodal(level).reshape(3, -1)
        for k in range(3):
            assert np.abs(Pu @ cf[k] - ff[k]).max() < 1e-12
    # pressure: the P1disc coefficients of the linear exact pressure on level 1
    # (finest level of the 2-level problem) map to those on level 2
    a = P.arrays(2)
    Pp = sp.csr_matrix((a["pp_val"], a["pp_col"], a["pp_rowptr"]),
                       shape=(a["n_pdof"], P.desc(1).n_pdof))
    e2, e3 = tetra(n_levels=2).exact(), P.exact()
    p2, p3 = e2[3 * P.desc(1).n_udof:], e3[3 * P.desc(2).n_udof:]
    assert np.abs(Pp @ p2 - p3).max() < 1e-12


def test_tet_layout_invariants():
    P = tetra(n_levels=2)
    for level in range(P.n_levels):
        a = P.arrays(level)
        assert a["cell_udofs"].shape[1] == 15
        assert all(len(set(c)) == 15 for c in a["cell_udofs"])
        for colour in np.unique(a["cell_colour"]):
            cells = a["cell_udofs"][a["cell_colour"] == colour]
            assert len(np.unique(cells)) == cells.size  # no shared DOF in a colour
        for r in range(a["n_active"]):
            cols = a["a_col"][a["a_rowptr"][r]:a["a_rowptr"][r + 1]]
            assert np.all(np.diff(cols) > 0)
        # Dirichlet rows hold the diagonal only
        for r in range(a["n_active"], a["n_udof"]):
            assert list(a["a_col"][a["a_rowptr"][r]:a["a_rowptr"][r + 1]]) == [r]


@pytest.mark.parametrize("element", ["hexa", "tetra"])
def test_host_reassembly_reproduces_the_build(element):
    """pmh_reassemble (the host timing of a re-assembly) rewrites every
    level's values with the build's cell loop: bit-identical arrays."""
    from to_merge_master_parmoon_gb300 import OseenProblem
    P = OseenProblem(n_levels=2, nu=1e-2, seed=5, element=element)
    before = [{k: [v.copy() for v in P.arrays(l)[k]] for k in ("a", "b", "bt")}
              for l in range(P.n_levels)]
    rhs = P.rhs()
    P.reassemble()
    for l in range(P.n_levels):
        a = P.arrays(l)
        for k in ("a", "b", "bt"):
            assert all(np.array_equal(x, y) for x, y in zip(before[l][k], a[k]))
    assert np.array_equal(rhs, P.rhs())


@pytest.mark.parametrize("example,nu", [("quadlin_oseen", 1.0), ("random", 1e-2)])
def test_oracle_fgmres_on_tetrahedra(example, nu):
    """The oracle's FGMRES + V(2,2) with 49 x 49 cell Vanka (colour order) and
    the handed-over transfers converges and agrees with a direct solve."""
    from oracle.pyoracle import Oracle
    P = tetra(n_levels=2, example=example, nu=nu)
    b = P.rhs()
    r0 = np.linalg.norm(Oracle(P).coupled_defect(1, np.zeros_like(b), b))
    x, info = Oracle(P, restart=20, maxit=60, res_norm_min=1e-11 * r0).iterate(np.zeros_like(b), b)
    assert info["true_res"] <= 1.05e-11 * r0 and info["iterations"] <= 30
    n3 = 3 * P.desc(1).n_udof
    xd = direct_solve(P, 1, x[n3])
    assert np.linalg.norm(x - xd) <= 1e-8 * np.linalg.norm(xd)


# ------------------------------------------------------------------ GPU ----
# Every operator of the path through the C ABI on tetrahedral levels against
# the oracle (same tolerances as the hexahedral parity tests), nine-block and
# one-block descriptors, both precisions.

def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def rnd(P, level, seed):
    return np.random.default_rng(seed).standard_normal(P.ndof(level))


def tet_solvers(one_block):
    from oracle.pyoracle import Oracle
    from to_merge_master_parmoon_gb300 import PmSolver
    P = tetra(n_levels=3, example="random", nu=1e-2)
    descs = P.descs_one_block() if one_block else P.descs
    return P, PmSolver(descs, precision="fp64"), PmSolver(descs, precision="mixed"), Oracle(P)


@pytest.mark.gpu
@pytest.mark.parametrize("one_block", [False, True])
def test_tet_gpu_operators_match_oracle(one_block):
    P, g64, g32, O = tet_solvers(one_block)
    for level in range(3):
        x, b = rnd(P, level, 1), rnd(P, level, 2)
        assert rel(g64.coupled_defect(level, x, b, True), O.coupled_defect(level, x, b, True)) < 1e-12
        assert rel(g64.matvec(level, x), O.matvec(level, x)) < 1e-12
    for level in (1, 2):
        xf, xc = rnd(P, level, 3), rnd(P, level - 1, 4)
        assert rel(g64.restrict(level, xf), O.restrict(level, xf)) < 1e-13
        assert rel(g64.prolongate(level, xc), O.prolongate(level, xc)) < 1e-13
        u, f = 0.1 * rnd(P, level, 6), rnd(P, level, 7)
        assert rel(g64.cell_vanka(level, u, f, 2), O.cell_vanka(level, u, f, 2)) < 1e-9
        assert rel(g32.cell_vanka(level, u, f, 2), O.cell_vanka(level, u, f, 2)) < 5e-4
    b0 = rnd(P, 0, 5)
    assert rel(g64.solve_exact(b0), O.solve_exact(b0)) < 1e-10
    v = rnd(P, 2, 8)
    z = O.vcycle(v)
    assert rel(g64.vcycle(v), z) < 1e-9
    assert rel(g32.vcycle(v), z) < 5e-4


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("apply_variant", [0, 2])
def test_tet_gpu_fgmres_matches_oracle(precision, apply_variant):
    from oracle.pyoracle import Oracle
    from to_merge_master_parmoon_gb300 import PmSolver
    P = tetra(n_levels=3, example="random", nu=1e-2)
    b = P.rhs()
    x0 = np.zeros_like(b)
    O = Oracle(P)
    r0 = np.linalg.norm(O.coupled_defect(2, x0, b))
    tol = 1e-10 * r0
    xo, io = Oracle(P, restart=20, maxit=60, res_norm_min=tol).iterate(x0, b)
    S = PmSolver(P.descs, precision=precision, restart=20, maxit=60, res_norm_min=tol,
                 apply_variant=apply_variant)
    xg, ig = S.iterate(x0, b)
    n = P.desc(2).n_udof
    pg, po = xg.copy(), xo.copy()
    pg[3 * n::4] -= pg[3 * n::4].mean()
    po[3 * n::4] -= po[3 * n::4].mean()
    assert ig["true_res"] <= 1.05 * tol
    assert rel(pg, po) < 1e-6
    if precision == "fp64":
        assert ig["iterations"] == io["iterations"]


@pytest.mark.gpu
def test_tet_known_answer_on_gpu():
    from to_merge_master_parmoon_gb300 import PmSolver
    P = tetra(n_levels=3, example="quadlin_oseen", nu=1.0)
    b, ex = P.rhs(), P.exact()
    r0 = np.linalg.norm(PmSolver(P.descs).coupled_defect(2, np.zeros_like(b), b))
    n3 = 3 * P.desc(2).n_udof
    for precision in ("fp64", "mixed"):
        S = PmSolver(P.descs, precision=precision, restart=20, maxit=60, res_norm_min=1e-12 * r0)
        x, info = S.iterate(np.zeros_like(b), b)
        assert np.abs(x[:n3] - ex[:n3]).max() < 1e-8
        dp = x[n3:] - ex[n3:]
        dp[0::4] -= dp[0::4].mean()
        assert np.abs(dp).max() < 1e-6


@pytest.mark.gpu
def test_tet_hexahedral_only_features_refuse():
    from to_merge_master_parmoon_gb300 import PmError, PmSolver
    P = tetra(n_levels=2, example="random", nu=1e-2)
    with pytest.raises(PmError):
        PmSolver(P.descs, precision="mixed", vanka_inverse=1)
    S = PmSolver(P.descs, precision="fp64")
    with pytest.raises(PmError):
        S.assemble_level(1, np.ones((P.desc(1).n_cells, 3)), np.zeros(3 * P.desc(1).n_udof), 1.0)
