"""Theta-scheme system operations on the device (the steps of
TSystemTNSE3D::AssembleSystMat, src/System/SystemTNSE3D.C:1118-1274, and its
working right-hand side) against host restatements with the host builder's
Oseen blocks and a host Q2 mass matrix (4-point Gauss rule):
* pm_assemble_system_level: K = [[c_mass M + c_a A, bt_scale BT], [b_scale B, 0]]
  on every level (mat-vec, 1e-13 relative);
* pm_system_rhs: c_old old + c_new rhs + (M - c2 A) sol on active rows,
  rhs on Dirichlet rows, 0 on pressure rows (1e-13);
* three Crank-Nicolson steps with the device system: every step's solution
  satisfies the host-assembled system to the solver tolerance.
Each on nine-block (NSTYPE 4) and one-block (NSTYPE 2) levels: the theta
system keeps A11 = A22 = A33 and A12..A32 = 0."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

GP = np.array([-0.86113631159405257522, -0.33998104358485626480,
               0.33998104358485626480, 0.86113631159405257522])
GW = np.array([0.34785484513745385737, 0.65214515486254614263,
               0.65214515486254614263, 0.34785484513745385737])


def mass_ref():
    from to_merge_master_parmoon_gb300._lib import host_lib
    lib = host_lib()
    M = np.zeros((27, 27))
    v = np.empty(27)
    d = np.empty(81)
    for qc in range(4):
        for qb in range(4):
            for qa in range(4):
                lib.pmh_q2_basis(GP[qa], GP[qb], GP[qc], v.ctypes.data_as(C.POINTER(C.c_double)),
                                 d.ctypes.data_as(C.POINTER(C.c_double)))
                M += GW[qa] * GW[qb] * GW[qc] * np.outer(v, v)
    return M


def host_mass(P, level):
    a = P.arrays(level)
    h = P.cell_sizes(level)
    Mr = mass_ref()
    ud = a["cell_udofs"]
    det = h.prod(axis=1) / 8.0
    rows = np.repeat(ud, 27, axis=1).ravel()
    cols = np.tile(ud, (1, 27)).ravel()
    vals = (det[:, None, None] * Mr[None]).reshape(-1)
    n = a["n_udof"]
    M = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    keep = sp.diags((np.arange(n) < a["n_active"]).astype(float))
    return (keep @ M).tocsr()


def host_blocks(P, level):
    a = P.arrays(level)
    n, npp, na = a["n_udof"], a["n_pdof"], a["n_active"]
    rows = np.repeat(np.arange(n), np.diff(a["a_rowptr"]))
    A = sp.csr_matrix((a["a"][0], (rows, a["a_col"])), shape=(n, n))
    act = sp.diags((np.arange(n) < na).astype(float))
    brow = np.repeat(np.arange(npp), np.diff(a["b_rowptr"]))
    B = [sp.csr_matrix((a["b"][k], (brow, a["b_col"])), shape=(npp, n)) for k in range(3)]
    trow = np.repeat(np.arange(n), np.diff(a["bt_rowptr"]))
    BT = [sp.csr_matrix((a["bt"][k], (trow, a["bt_col"])), shape=(n, npp)) for k in range(3)]
    return (act @ A).tocsr(), B, BT, na


def host_system(P, level, c_mass, c_a, b_scale, bt_scale):
    A, B, BT, na = host_blocks(P, level)
    M = host_mass(P, level)
    n = A.shape[0]
    V = c_mass * M + c_a * A
    dirich = sp.diags((np.arange(n) >= na).astype(float))
    V = (V + dirich).tocsr()
    Z = sp.csr_matrix((n, n))
    top = sp.bmat([[V, Z, Z, bt_scale * BT[0]], [Z, V, Z, bt_scale * BT[1]],
                   [Z, Z, V, bt_scale * BT[2]]])
    bot = sp.hstack([b_scale * B[0], b_scale * B[1], b_scale * B[2],
                     sp.csr_matrix((B[0].shape[0], B[0].shape[0]))])
    return sp.vstack([top, bot]).tocsr()


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def assemble_system(S, P, c_mass, c_a, b_scale, bt_scale):
    for level in range(P.n_levels):
        S.assemble_system_level(level, P.cell_sizes(level), P.convection_nodal(level), P.nu,
                                c_mass, c_a, b_scale, bt_scale)
    S.refactor()


@pytest.mark.parametrize("one_block", [False, True])
def test_system_operator_and_rhs(problems, one_block):
    from to_merge_master_parmoon_gb300 import PmSolver
    P = problems(3, 1e-2, 0)
    tau, theta = 1e-2, 0.5
    S = PmSolver(P.descs_one_block() if one_block else P.descs, precision="fp64")
    assemble_system(S, P, 1.0, tau * theta, 1.0, tau)
    rng = np.random.default_rng(9)
    for level in range(P.n_levels):
        x = rng.standard_normal(P.ndof(level))
        K = host_system(P, level, 1.0, tau * theta, 1.0, tau)
        assert rel(S.matvec(level, x), K @ x) < 1e-13
    A, B, BT, na = host_blocks(P, 2)
    M = host_mass(P, 2)
    n = A.shape[0]
    old, rhs, sol = (rng.standard_normal(P.ndof(2)) for _ in range(3))
    out = S.system_rhs(old, rhs, sol, tau * theta, tau * theta, tau * (1 - theta))
    want = np.zeros_like(rhs)
    W = (M - tau * (1 - theta) * A).tocsr()
    for c in range(3):
        sl = slice(c * n, (c + 1) * n)
        w = tau * theta * old[sl] + tau * theta * rhs[sl] + W @ sol[sl]
        w[na:] = rhs[sl][na:]
        want[sl] = w
    assert rel(out, want) < 1e-13
    torch = pytest.importorskip("torch")
    d_old, d_rhs, d_sol = (torch.from_numpy(v).cuda() for v in (old, rhs, sol))
    d_out = torch.empty_like(d_rhs)
    S.system_rhs_device(d_old.data_ptr(), d_rhs.data_ptr(), d_sol.data_ptr(), tau * theta,
                        tau * theta, tau * (1 - theta), d_out.data_ptr())
    assert np.array_equal(d_out.cpu().numpy(), out)


@pytest.mark.parametrize("one_block", [False, True])
def test_crank_nicolson_steps(problems, one_block):
    from to_merge_master_parmoon_gb300 import PmSolver
    P = problems(3, 1e-2, 0)
    tau, theta = 1e-2, 0.5
    f = P.rhs()                      # forcing (Dirichlet rows carry the boundary values)
    S = PmSolver(P.descs_one_block() if one_block else P.descs, precision="mixed", restart=20, maxit=80, res_norm_min=1e-30,
                 red_factor=1e-10)
    assemble_system(S, P, 1.0, tau * theta, 1.0, tau)
    K = host_system(P, 2, 1.0, tau * theta, 1.0, tau)
    u = np.zeros_like(f)
    for step in range(3):
        w = S.system_rhs(f, f, u, tau * (1 - theta), tau * theta, tau * (1 - theta))
        u_new, info = S.iterate(u, w)
        r = w - K @ u_new
        n3 = 3 * P.desc(2).n_udof
        r[n3::4] -= r[n3::4].mean()  # L2_0 projection of the pressure defect
        assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(w), step
        assert not np.allclose(u_new[:n3], u[:n3])
        u = u_new
