"""Device assembly of the Galerkin Oseen blocks (pm_assemble_level) against
the host builder's CSR values: the operator of every level (mat-vec through
the C ABI) within 1e-13 relative in FP64 (only the order of the quadrature
sums differs), 1e-6 in mixed precision (FP32 copies of the values), and the
FGMRES solution within 1e-10.  Assembling with another viscosity into the
same pattern reproduces the host builder's system for that viscosity."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def assemble_all(S, P, nu):
    for level in range(P.n_levels):
        S.assemble_level(level, P.cell_sizes(level), P.convection_nodal(level), nu)
    S.refactor()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("one_block", [False, True])
def test_device_assembly_matches_host_builder(problems, precision, one_block):
    from to_merge_master_parmoon_gb300 import PmSolver
    P = problems(3, 1e-2, 0)
    descs = P.descs_one_block() if one_block else P.descs
    S_host = PmSolver(descs, precision=precision)
    S_dev = PmSolver(descs, precision=precision)
    assemble_all(S_dev, P, P.nu)
    tol = 1e-13 if precision == "fp64" else 1e-6
    rng = np.random.default_rng(5)
    for level in range(P.n_levels):
        x = rng.standard_normal(P.ndof(level))
        assert rel(S_dev.matvec(level, x), S_host.matvec(level, x)) < tol
    b = P.rhs()
    x0 = np.zeros_like(b)
    r0 = np.linalg.norm(S_host.coupled_defect(2, x0, b))
    kw = dict(precision=precision, restart=20, maxit=60, res_norm_min=1e-10 * r0)
    xh, ih = PmSolver(descs, **kw).iterate(x0, b)
    Sd = PmSolver(descs, **kw)
    assemble_all(Sd, P, P.nu)
    xd, idev = Sd.iterate(x0, b)
    assert idev["true_res"] <= 1.05e-10 * r0
    assert rel(xd, xh) < 1e-8


def test_device_assembly_replaces_values(problems):
    from to_merge_master_parmoon_gb300 import PmSolver
    P1 = problems(3, 1e-2, 0)
    P3 = problems(3, 3e-2, 0)   # same convection field (same seed), other viscosity
    S = PmSolver(P1.descs, precision="fp64")
    assemble_all(S, P1, 3e-2)
    ref = PmSolver(P3.descs, precision="fp64")
    rng = np.random.default_rng(6)
    for level in range(P1.n_levels):
        x = rng.standard_normal(P1.ndof(level))
        assert rel(S.matvec(level, x), ref.matvec(level, x)) < 1e-13
