"""Fused batch of independent Oseen systems (pm_add_level_batch +
pm_solve_fused): systems on one mesh stacked into one block-diagonal
hierarchy, every V-cycle and FGMRES kernel one launch over all of them, one
Arnoldi process, Givens sequence and stopping test per system
(TFgmresIte::Iterate, src/FE/FgmresIte.C:250-677, per system).  Each fused
result must match the same system solved alone by pm_solve: identical FP64
iteration counts and solutions within 1e-9 (the per-system sums run in
another order), the mixed-precision ones within 1e-6 of it after the L2_0
normalisation; a system that stops early (converged, or at maxit) must not
disturb the others; and one system against the oracle (the reference's
algorithm on the CPU) to 1e-6."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tol(P, b, rel):
    nu3 = 3 * P.desc(P.n_levels - 1).n_udof
    bp = b.copy()
    bp[nu3::4] -= bp[nu3::4].mean()
    return rel * np.linalg.norm(bp)


def _l20(P, x):
    nu3 = 3 * P.desc(P.n_levels - 1).n_udof
    y = x.copy()
    y[nu3::4] -= y[nu3::4].mean()
    return y


def _rel(P, a, b):
    a, b = _l20(P, a), _l20(P, b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fused_equals_individual_solves(problems, precision):
    from to_merge_master_parmoon_gb300 import PmFusedSolver, PmSolver
    # nu = 3e-3 needs about 19 iterations: with maxit 14 it stops at maxit,
    # after a restart, while the others converge in 7-9, so the sweeps drop
    # systems in the middle of the solve
    specs = [(3, 1e-2, 200), (3, 1e-1, 201), (3, 3e-3, 202), (3, 3e-2, 203)]
    Ps = [problems(lv, nu, seed) for lv, nu, seed in specs]
    bs = [P.rhs() for P in Ps]
    tol = min(_tol(P, b, 1e-10) for P, b in zip(Ps, bs))
    kw = dict(precision=precision, restart=10, maxit=14, res_norm_min=tol)
    alone = []
    for P, b in zip(Ps, bs):
        S = PmSolver(P.descs, **kw)
        alone.append(S.iterate(np.zeros_like(b), b, allow=(0, 1)))
        S.close()
    F = PmFusedSolver([P.descs for P in Ps], **kw)
    assert F.n_systems == len(Ps)
    xs, infos = F.solve([np.zeros_like(b) for b in bs], bs, allow=(0, 1))
    F.close()
    statuses = [ib["status"] for ib in infos]
    assert 1 in statuses and 0 in statuses, statuses  # one at maxit, others converged
    for P, (xa, ia), xf, ib in zip(Ps, alone, xs, infos):
        assert ib["status"] == ia["status_name"].startswith("PM_MAXIT") * 1
        if precision == "fp64":
            assert ib["iterations"] == ia["iterations"]
            assert _rel(P, xf, xa) <= 1e-9
        else:
            # FP32 V-cycles: the fused level may run other kernel variants
            # (other FP32 summation orders); converged solutions agree to
            # 1e-6, the one stopped at maxit (residual ~1e-8) more loosely
            assert abs(ib["iterations"] - ia["iterations"]) <= 1
            assert _rel(P, xf, xa) <= (1e-6 if ib["status"] == 0 else 1e-4)
        if ib["status"] == 0:
            assert ib["true_res"] <= 1.05 * tol


def test_fused_matches_oracle(problems):
    from oracle.pyoracle import Oracle
    from to_merge_master_parmoon_gb300 import PmFusedSolver
    Ps = [problems(3, 1e-2, 210), problems(3, 2e-2, 211)]
    bs = [P.rhs() for P in Ps]
    tol = min(_tol(P, b, 1e-10) for P, b in zip(Ps, bs))
    F = PmFusedSolver([P.descs for P in Ps], precision="fp64", restart=20, maxit=60,
                      res_norm_min=tol)
    xs, infos = F.solve([np.zeros_like(b) for b in bs], bs)
    F.close()
    for P, b, xf, ib in zip(Ps, bs, xs, infos):
        O = Oracle(P, restart=20, maxit=60, res_norm_min=tol)
        xo, io = O.iterate(np.zeros_like(b), b)
        assert ib["iterations"] == io["iterations"]
        assert _rel(P, xf, xo) <= 1e-6


def test_fused_tetrahedra(problems):
    """Tetrahedral P2+bubble/P1disc systems: the handed-over prolongations are
    stacked with the matrices."""
    from to_merge_master_parmoon_gb300 import OseenProblem, PmFusedSolver, PmSolver
    Ps = [OseenProblem(n_levels=2, nu=nu, seed=seed, element="tetra")
          for nu, seed in ((1e-2, 220), (5e-2, 221))]
    bs = [P.rhs() for P in Ps]
    tol = min(_tol(P, b, 1e-10) for P, b in zip(Ps, bs))
    kw = dict(precision="fp64", restart=20, maxit=80, res_norm_min=tol)
    F = PmFusedSolver([P.descs for P in Ps], **kw)
    xs, infos = F.solve([np.zeros_like(b) for b in bs], bs)
    F.close()
    for P, b, xf, ib in zip(Ps, bs, xs, infos):
        S = PmSolver(P.descs, **kw)
        xa, ia = S.iterate(np.zeros_like(b), b)
        S.close()
        assert ib["iterations"] == ia["iterations"]
        assert _rel(P, xf, xa) <= 1e-9


def test_fused_refuses_mixed_sizes_and_single_system_calls(problems):
    from to_merge_master_parmoon_gb300 import PmFusedSolver
    from to_merge_master_parmoon_gb300.solver import PmError
    with pytest.raises(PmError, match="PM_BADARG"):
        PmFusedSolver([problems(3, 1e-2, 230).descs, problems(3, 1e-2, 231).descs[:2]
                       + [problems(4, 1e-2, 231).descs[3]]])
    P = problems(3, 1e-2, 230)
    F = PmFusedSolver([P.descs, P.descs], precision="fp64")
    with pytest.raises(PmError, match="PM_BADARG"):
        F.iterate(np.zeros(F.ndof()), np.zeros(F.ndof()))
    F.close()
