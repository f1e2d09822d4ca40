"""Parity at the configured problem size of the CPU-runnable case: the steady
Oseen problem on 16^3 cells (4 levels from 2^3, Q2/P1disc, 124,195 DOF,
nu = 1e-2, seed 0), FGMRES(20) + one V(2,2) cell-Vanka cycle, relative
residual 1e-10.

The oracle's FGMRES (src/FE/FgmresIte.C:250-677 over the cycle of
src/FE/NSE_MultiGrid.C:434-1779) is the reference answer; where the
reference tree is present, the reference's own solver (its FGMRES over its
own cycle driver, compiled where they lie; sequential and colour-parallel
cell Vanka) is run on the same problem and the oracle checked against it.  Bars, as the
path's correctness target states them: the GPU solution reaches 1e-10
relative residual, its velocity and its pressure each differ from the
oracle's by at most 1e-6 relative L2 (pressures compared after the same
L2_0 normalisation, the reference's IntoL20FEFunction3D), and the FP64 path
takes the oracle's iteration count.  The errors are printed with the result.
"""
import numpy as np
import pytest

from oracle.pyoracle import Oracle

LEVELS, NU, SEED, RTOL = 4, 1e-2, 0, 1e-10


def split_error(x, ref, nu):
    """Relative L2 differences of the velocity and of the L2_0-normalised
    pressure (constant P1disc modes, every 4th pressure entry)."""
    n3 = 3 * nu
    xp, rp = x[n3:].copy(), ref[n3:].copy()
    xp[0::4] -= xp[0::4].mean()
    rp[0::4] -= rp[0::4].mean()
    eu = np.linalg.norm(x[:n3] - ref[:n3]) / np.linalg.norm(ref[:n3])
    ep = np.linalg.norm(xp - rp) / np.linalg.norm(rp)
    return float(eu), float(ep)


@pytest.fixture(scope="module")
def config0(problems):
    P = problems(LEVELS, NU, SEED)
    b = P.rhs()
    x0 = np.zeros_like(b)
    r0 = float(np.linalg.norm(Oracle(P).coupled_defect(LEVELS - 1, x0, b)))
    # factors reused across sweeps: the same blocks and pivots as refactoring
    # in every sweep (bit-identical, test_oracle_factor_reuse_is_exact)
    O = Oracle(P, restart=20, maxit=100, res_norm_min=RTOL * r0, reuse_factors=1)
    xo, io = O.iterate(x0, b)
    return P, b, r0, xo, io


def test_oracle_factor_reuse_is_exact(config0):
    """The oracle with per-sweep refactorisation (the reference's cell Vanka,
    src/FE/NSE_MGLevel4.C:1784-2031) and with factors kept across sweeps give
    the same solution bit for bit at 16^3."""
    P, b, r0, xo, io = config0
    O = Oracle(P, restart=20, maxit=100, res_norm_min=RTOL * r0, reuse_factors=0)
    x, i = O.iterate(np.zeros_like(b), b)
    assert i["iterations"] == io["iterations"]
    assert np.array_equal(x, xo)
    assert io["true_res"] <= RTOL * r0


def test_oracle_equals_the_whole_reference_solver(config0):
    """The reference's own solver on this problem, compiled where it lies
    (single thread, sequential build): its flexible FGMRES
    (TFgmresIte::Iterate, src/FE/FgmresIte.C:250-677, run by
    oracle/ref_harness.cpp) preconditioned by its own cycle driver
    (TMultiGridIte::Iterate with TNSE_MultiGrid::Cycle over four
    TNSE_MGLevel4 levels, run by oracle/ref_transfer.cpp).  The oracle with
    the sequential cell loop takes the same iterations and agrees to
    rounding; the colour-ordered oracle the GPU is compared with is within
    the solve tolerance of it."""
    from oracle.pyref import ref_harness_lib, ref_transfer_lib
    if ref_harness_lib() is None or ref_transfer_lib() is None:
        pytest.skip("reference tree not present: the harnesses are not built")
    from oracle.pyref import RefCycle, RefLevel
    P, b, r0, xo, io = config0
    x0 = np.zeros_like(b)
    O = Oracle(P, restart=20, maxit=100, res_norm_min=RTOL * r0, vanka_mode="seq",
               reuse_factors=1)
    xs, i_s = O.iterate(x0, b)
    xr, it = RefLevel(P.arrays(LEVELS - 1), threads=1).fgmres_with_reference_cycle(
        RefCycle(P), O.params, x0, b)
    nu = P.desc(LEVELS - 1).n_udof
    eu, ep = split_error(xo, xr, nu)
    print(f"config 0 reference solver: {it} iterations (oracle sequential "
          f"{i_s['iterations']}, colour-ordered {io['iterations']}); colour-ordered oracle vs "
          f"reference u {eu:.2e} p {ep:.2e}")
    assert it == i_s["iterations"]
    assert np.linalg.norm(xs - xr) <= 1e-13 * np.linalg.norm(xr)
    assert eu <= 1e-7 and ep <= 1e-7


def test_colour_oracle_equals_the_colour_parallel_reference_solver(config0):
    """The colour-ordered oracle the GPU is compared with, against the
    reference's own solver in its colour-parallel build (CellVanka's OpenMP
    colour loop, src/FE/NSE_MGLevel4.C:603-1651, over every level's own
    colouring, inside its cycle driver and FGMRES): the same iterations and
    the same solution to rounding."""
    from oracle.pyref import ref_harness_lib, ref_transfer_lib
    if ref_harness_lib() is None or ref_transfer_lib(hybrid=True) is None:
        pytest.skip("reference tree not present: the harnesses are not built")
    from oracle.pyref import RefCycle, RefLevel
    P, b, r0, xo, io = config0
    x0 = np.zeros_like(b)
    O = Oracle(P, restart=20, maxit=100, res_norm_min=RTOL * r0)
    xr, it = RefLevel(P.arrays(LEVELS - 1), threads=4).fgmres_with_reference_cycle(
        RefCycle(P, colours=True, threads=4), O.params, x0, b)
    print(f"config 0 colour-parallel reference solver: {it} iterations "
          f"(oracle {io['iterations']}), rel. difference "
          f"{np.linalg.norm(xo - xr) / np.linalg.norm(xr):.2e}")
    assert it == io["iterations"]
    assert np.linalg.norm(xo - xr) <= 1e-13 * np.linalg.norm(xr)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_config0_solution_vs_oracle(config0, precision):
    from to_merge_master_parmoon_gb300 import PmSolver
    P, b, r0, xo, io = config0
    S = PmSolver(P.descs, precision=precision, restart=20, maxit=100, res_norm_min=RTOL * r0)
    xg, ig = S.iterate(np.zeros_like(b), b)
    S.close()
    nu = P.desc(LEVELS - 1).n_udof
    eu, ep = split_error(xg, xo, nu)
    print(f"config 0 {precision}: iterations {ig['iterations']} (oracle {io['iterations']}), "
          f"rel. residual {ig['true_res'] / r0:.2e}, error vs oracle u {eu:.2e} p {ep:.2e}")
    assert ig["status"] == 0
    assert ig["true_res"] <= 1.05 * RTOL * r0
    assert eu <= 1e-6 and ep <= 1e-6
    if precision == "fp64":
        assert ig["iterations"] == io["iterations"]
