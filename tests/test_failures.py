"""Failure paths of the solver: each is produced on the host (a non-finite
input, a tolerance, a memory cap, a wait limit) and must come back as a
status code, with the GPU context still usable afterwards.  The reference
ends the program instead (exit(4711) on FGMRES divergence,
src/FE/FgmresIte.C:564-566; on a diverging coarse smoother,
src/FE/NSE_MultiGrid.C:629-633).

No test here faults, traps or hangs a GPU: the timeout test lets a bounded
wait of the bulk-copy apply give up after one poll; the kernel then waits
(with its normal bound) for the copies it has in flight and returns.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PM_OK, PM_DIVERGED, PM_NAN, PM_TIMEOUT, PM_OOM = 0, 2, 3, 4, 5


def clean_solve_ok(P, **options):
    """A fresh handle on the same problem solves to 1e-10 (the context and
    the device are fine after the failure)."""
    from to_merge_master_parmoon_gb300 import PmSolver
    b = P.rhs()
    S = PmSolver(P.descs, restart=20, maxit=80, res_norm_min=1e-10 * np.linalg.norm(b), **options)
    _, info = S.iterate(np.zeros_like(b), b)
    S.close()
    return info["status"] == PM_OK


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_in_rhs_gives_pm_nan(problems, precision):
    from to_merge_master_parmoon_gb300 import PmSolver
    P = problems(3, 1e-2, 0)
    S = PmSolver(P.descs, precision=precision)
    b = P.rhs()
    b[7] = np.nan
    _, info = S.iterate(np.zeros_like(b), b, allow=(PM_NAN,))
    assert info["status"] == PM_NAN
    # the same handle solves a finite system afterwards
    b = P.rhs()
    S2 = PmSolver(P.descs, precision=precision, restart=20, maxit=80,
                  res_norm_min=1e-10 * np.linalg.norm(b))
    _, info = S2.iterate(np.zeros_like(b), b)
    assert info["status"] == PM_OK
    S.close()
    S2.close()


def test_nan_in_a_matrix_value_gives_pm_nan():
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    P = OseenProblem(n_levels=3, nu=1e-2, seed=0)
    P.arrays(2)["a"][0][1234] = np.nan
    S = PmSolver(P.descs, precision="mixed")
    b = P.rhs()
    _, info = S.iterate(np.zeros_like(b), b, allow=(PM_NAN,))
    assert info["status"] == PM_NAN
    S.close()


def test_small_div_factor_gives_pm_diverged(problems):
    """SC_DIV_FACTOR: the solve stops as soon as the residual exceeds
    div_factor * res0 (here after the first iteration, which reduces the
    residual by far less than 1e-3)."""
    from to_merge_master_parmoon_gb300 import PmSolver
    P = problems(3, 1e-2, 0)
    S = PmSolver(P.descs, div_factor=1e-3, res_norm_min=0.0)
    b = P.rhs()
    _, info = S.iterate(np.zeros_like(b), b, allow=(PM_DIVERGED,))
    assert info["status"] == PM_DIVERGED
    assert info["iterations"] == 1
    assert info["res"] > 1e-3 * info["res0"]
    S.close()


def test_device_memory_cap_gives_pm_oom(problems):
    from to_merge_master_parmoon_gb300 import PmError, PmSolver
    P = problems(3, 1e-2, 0)
    # too small for the first level's arrays
    with pytest.raises(PmError) as e:
        PmSolver(P.descs, max_device_bytes=1 << 16)
    assert e.value.status == PM_OOM
    # large enough for every level, too small for pm_setup's buffers
    S = PmSolver(None)
    for d in P.descs:
        S.add_level(d)
    added = S.device_bytes
    S.setup()
    full = S.device_bytes
    S.close()
    S = PmSolver(None, max_device_bytes=added + (full - added) // 2)
    for d in P.descs:
        S.add_level(d)
    with pytest.raises(PmError) as e:
        S.setup()
    assert e.value.status == PM_OOM
    S.close()
    assert clean_solve_ok(P)


def test_bulk_copy_wait_limit_gives_pm_timeout(problems):
    """The bulk-copy apply (mixed precision, LU levels, apply_variant 1) with
    its factor waits limited to one poll: the copies just issued cannot have
    landed, every warp gives up its first wait, drains its copies and
    returns; the host reports PM_TIMEOUT.  A handle with the default limit
    then sweeps and solves normally."""
    from to_merge_master_parmoon_gb300 import PmError, PmSolver
    P = problems(3, 1e-2, 0)
    S = PmSolver(P.descs, precision="mixed", decouple=0, apply_variant=1, wait_limit=1)
    assert S._lib.pm_level_variant(S._h, 2) // 2 == 1  # the bulk-copy apply
    rng = np.random.default_rng(1)
    u, f = 0.1 * rng.standard_normal(P.ndof(2)), rng.standard_normal(P.ndof(2))
    with pytest.raises(PmError) as e:
        S.cell_vanka(2, u, f, 1)
    assert e.value.status == PM_TIMEOUT
    S.close()
    assert clean_solve_ok(P, precision="mixed", decouple=0, apply_variant=1)


def test_update_with_a_changed_pattern_is_refused():
    """pm_update_matrices takes new values for the set-up's patterns only:
    a column index moved within the same nnz is refused (PM_BADARG), the
    original pattern is accepted again."""
    from to_merge_master_parmoon_gb300 import OseenProblem, PmError, PmSolver
    P = OseenProblem(n_levels=3, nu=1e-2, seed=0)
    S = PmSolver(P.descs)
    col = P.arrays(2)["a_col"]
    old = int(col[61])
    col[61] = col[62]  # a sampled position: same nnz, different pattern
    with pytest.raises(PmError) as e:
        S.update_matrices(P.descs)
    assert e.value.status == 6
    col[61] = old
    S.update_matrices(P.descs)
    S.close()
