"""Batched solves of independent Oseen systems of uneven size (the batch of
independent systems the reference solves one after another, each with its own
FGMRES + GMG): pm_solve_batch runs them concurrently from host threads, one
handle and stream per system.  Every batched result must equal the system
solved alone, bit for bit (same kernels in the same order on its own stream,
deterministic reductions), and reach the tolerance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_equals_individual_solves(problems):
    from to_merge_master_parmoon_gb300 import PmSolver, solve_batch
    specs = [(3, 1e-2, 100), (4, 3e-2, 101), (3, 1e-1, 102), (4, 1e-2, 103),
             (3, 5e-2, 104), (4, 2e-2, 105)]
    Ps = [problems(lv, nu, seed) for lv, nu, seed in specs]
    solvers, rhss, tols = [], [], []
    for k, P in enumerate(Ps):
        b = P.rhs()
        nu3 = 3 * P.desc(P.n_levels - 1).n_udof
        bp = b.copy()
        bp[nu3::4] -= bp[nu3::4].mean()
        tol = 1e-10 * np.linalg.norm(bp)
        prec = "mixed" if k % 2 == 0 else "fp64"
        solvers.append(PmSolver(P.descs, precision=prec, restart=20, maxit=80, res_norm_min=tol))
        rhss.append(b)
        tols.append(tol)
    alone = [S.iterate(np.zeros_like(b), b) for S, b in zip(solvers, rhss)]
    xs, infos = solve_batch(solvers, [np.zeros_like(b) for b in rhss], rhss, nthreads=4)
    for (xa, ia), xb, ib, tol in zip(alone, xs, infos, tols):
        assert np.array_equal(xa, xb)
        assert ia["iterations"] == ib["iterations"]
        assert ib["true_res"] <= 1.05 * tol
    # a handle may appear only once in a batch
    from to_merge_master_parmoon_gb300.solver import PmError
    with pytest.raises(PmError, match="PM_BADARG"):
        solve_batch([solvers[0], solvers[0]], [np.zeros_like(rhss[0])] * 2, [rhss[0]] * 2)
    for S in solvers:
        S.close()
