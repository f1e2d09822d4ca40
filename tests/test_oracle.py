"""CPU tests: the oracle (FP64 restatement of the reference solver) pinned
against the reference's own basis tables, its known-answer fixture and
scipy, plus the problem builder's layout invariants."""
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.linalg as sla
import scipy.sparse.linalg as spla

from oracle.pyoracle import Oracle, lu_solve

GOLD = Path(__file__).parent / "golden" / "basis_q2_p1.json"


def test_q2_p1_basis_matches_reference_tables():
    """pmh_q2_basis (used by assembly and transfers) equals the reference's
    C_H_Q2_3D_* / D_H_P1_3D_* at the golden points."""
    import ctypes as C
    from to_merge_master_parmoon_gb300._lib import host_lib
    g = json.loads(GOLD.read_text())
    lib = host_lib()
    v = (C.c_double * 27)()
    d = (C.c_double * 81)()
    for pt, ref in zip(g["points"], g["values"]):
        lib.pmh_q2_basis(pt[0], pt[1], pt[2], v, d)
        vals = np.array(v[:])
        der = np.array(d[:]).reshape(27, 3)
        np.testing.assert_allclose(vals, ref["q2"], rtol=0, atol=1e-14)
        np.testing.assert_allclose(der[:, 0], ref["q2_xi"], rtol=0, atol=1e-14)
        np.testing.assert_allclose(der[:, 1], ref["q2_eta"], rtol=0, atol=1e-14)
        np.testing.assert_allclose(der[:, 2], ref["q2_zeta"], rtol=0, atol=1e-14)
        np.testing.assert_allclose(ref["p1"], [1.0, *pt], rtol=0, atol=1e-15)


def test_lu_restatement_matches_scipy():
    rng = np.random.default_rng(3)
    for n in (5, 85, 120):
        a = rng.standard_normal((n, n)) + n * 0.1 * np.eye(n)
        b = rng.standard_normal(n)
        x = lu_solve(a, b)
        np.testing.assert_allclose(x, sla.lu_solve(sla.lu_factor(a), b), rtol=1e-10, atol=1e-12)


def test_local_vanka_block_solve(problems):
    """Local 85x85 blocks: the restated LU solves them like scipy does."""
    P = problems(3, 1e-2, 0)
    O = Oracle(P)
    rng = np.random.default_rng(0)
    u = rng.standard_normal(P.ndof(2))
    f = rng.standard_normal(P.ndof(2))
    for cell in (0, 17, 255, 511):
        A, r = O.local_system(2, cell, u, f)
        x = lu_solve(A, r)
        assert np.linalg.norm(A @ x - r) / np.linalg.norm(r) < 1e-13
        np.testing.assert_allclose(x, np.linalg.solve(A, r), rtol=1e-9, atol=1e-11)


def test_layout_matches_reference_conventions(problems):
    P = problems(3, 1e-2, 0)
    for level in range(P.n_levels):
        a = P.arrays(level)
        nu, na = a["n_udof"], a["n_active"]
        rp = a["a_rowptr"]
        # Dirichlet rows hold only the diagonal, value 1 in every block
        assert np.all(np.diff(rp)[na:] == 1)
        assert np.all(a["a_col"][rp[na:-1]] == np.arange(na, nu))
        for k in range(9):
            assert np.all(a["a"][k][rp[na:-1]] == 1.0)
        # columns sorted within rows
        for i in range(0, nu, max(1, nu // 50)):
            c = a["a_col"][rp[i]:rp[i + 1]]
            assert np.all(np.diff(c) > 0)
        # B: 27 per row; BT = B^T on active rows
        assert np.all(np.diff(a["b_rowptr"]) == 27)
        n = 3 * nu + a["n_pdof"]
        K = P.scipy_matrix(level).toarray() if n < 3000 else None
        if K is not None:
            B = K[3 * nu:, :3 * nu]
            BT = K[:3 * nu, 3 * nu:]
            act = np.r_[np.arange(na), nu + np.arange(na), 2 * nu + np.arange(na)]
            np.testing.assert_allclose(BT[act], B.T[act], atol=1e-14)


@pytest.mark.parametrize("example,nu", [("quadlin_stokes", 1.0), ("quadlin_stokes", 1e-2),
                                        ("quadlin_oseen", 1.0)])
def test_known_answer_ansatz_quadlin(problems, example, nu):
    """Examples/NSE_3D/AnsatzQuadLin.h: u in Q2, p in P1, so the discrete
    solution is the interpolant; the oracle's FGMRES+GMG must recover it."""
    P = problems(3, nu, 0, example)
    b, ex = P.rhs(), P.exact()
    O = Oracle(P, res_norm_min=0.0)
    assert np.linalg.norm(O.coupled_defect(2, ex, b, project=False)) < 1e-11 * np.linalg.norm(b)
    r0 = np.linalg.norm(O.coupled_defect(2, np.zeros_like(b), b))
    O = Oracle(P, restart=20, maxit=60, res_norm_min=1e-12 * r0)
    sol, info = O.iterate(np.zeros_like(b), b)
    assert info["true_res"] < 2e-12 * r0
    n3 = 3 * P.desc(2).n_udof
    assert np.abs(sol[:n3] - ex[:n3]).max() < 1e-8
    dp = sol[n3:] - ex[n3:]
    dp[0::4] -= dp[0::4].mean()
    assert np.abs(dp).max() < 1e-6


def test_fgmres_matches_direct_solve(problems):
    """Oracle FGMRES+V-cycle solution equals a sparse direct solve of the
    same system (pressure fixed by the L2_0 condition)."""
    P = problems(3, 1e-2, 0)
    b = P.rhs()
    K = P.scipy_matrix(-1).tolil()
    n = K.shape[0]
    nu3 = 3 * P.desc(2).n_udof
    # replace first pressure equation by the zero-mean condition on constant modes
    K[nu3, :] = 0
    for c in range(0, n - nu3, 4):
        K[nu3, nu3 + c] = 1.0
    bb = b.copy()
    bb[nu3] = 0.0
    xd = spla.spsolve(K.tocsc(), bb)
    O = Oracle(P, res_norm_min=0.0)
    r0 = np.linalg.norm(O.coupled_defect(2, np.zeros_like(b), b))
    O = Oracle(P, restart=20, maxit=60, res_norm_min=1e-11 * r0)
    sol, info = O.iterate(np.zeros_like(b), b)
    for v in (sol, xd):  # same L2_0 normalisation of the pressure
        v[nu3::4] -= v[nu3::4].mean()
    rel = np.linalg.norm(sol - xd) / np.linalg.norm(xd)
    assert rel < 1e-7, rel


def test_transfers_are_transposes(problems):
    """Restriction is the transpose of prolongation (DefectRestriction
    divides by the same multiplicity Prolongate averages with)."""
    P = problems(3, 1e-2, 0)
    O = Oracle(P)
    rng = np.random.default_rng(1)
    for level in (1, 2):
        xf = rng.standard_normal(P.ndof(level))
        xc = rng.standard_normal(P.ndof(level - 1))
        lhs = xf @ O.prolongate(level, xc)
        rhs = O.restrict(level, xf) @ xc
        assert abs(lhs - rhs) < 1e-10 * abs(lhs)


def test_prolongation_reproduces_q2_and_p1(problems):
    """Nodal interpolation: prolongating the interpolant of a Q2 field (and
    a P1 pressure) gives the fine interpolant exactly."""
    P = problems(3, 1.0, 0, "quadlin_stokes")
    Pc = problems(2, 1.0, 0, "quadlin_stokes")
    O = Oracle(P)
    fine = O.prolongate(2, Pc.exact())
    ex = P.exact()
    n3 = 3 * P.desc(2).n_udof
    np.testing.assert_allclose(fine[:n3], ex[:n3], atol=1e-12)
    np.testing.assert_allclose(fine[n3:], ex[n3:], atol=1e-12)


def test_colour_and_seq_vanka_converge_to_same_solution(problems):
    P = problems(3, 1e-2, 0)
    b = P.rhs()
    out = []
    for mode in ("seq", "colour"):
        O = Oracle(P, vanka_mode=mode, res_norm_min=0.0)
        r0 = np.linalg.norm(O.coupled_defect(2, np.zeros_like(b), b))
        O = Oracle(P, vanka_mode=mode, restart=20, maxit=60, res_norm_min=1e-11 * r0)
        sol, info = O.iterate(np.zeros_like(b), b)
        n3 = 3 * P.desc(2).n_udof
        sol[n3::4] -= sol[n3::4].mean()
        out.append(sol)
    assert np.linalg.norm(out[0] - out[1]) / np.linalg.norm(out[1]) < 1e-7
