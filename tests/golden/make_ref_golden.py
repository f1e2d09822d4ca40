"""Regenerate the reference's golden vectors on levels built by the problem
builder, run through oracle/ref_harness.cpp and oracle/ref_vanka.cpp, which
oracle/build_oracle.py compiles with the reference sources where they lie:
* tests/golden/ref_defect_*.npz: Defect_NSE4 (with and without the P1disc
  pressure projection) and MatVect_NSE4 (src/FE/MGComponents3D.C:3210, :3030);
* tests/golden/ref_transfer_*.npz: Prolongate of x and DefectRestriction
  of b between a level and the next coarser one (src/FE/MGComponents3D.C:468,
  :996 and the scalar versions for the pressure);
* tests/golden/ref_coarse_*.npz: the coarse solve TNSE_MGLevel4::SolveExact
  (src/FE/NSE_MGLevel4.C:5728-5847, first pressure equation p_0 = 0) of b
  on the coarsest level;
* tests/golden/ref_vanka_*.npz: one and two sweeps of the cell Vanka
  TNSE_MGLevel4::CellVanka (src/FE/NSE_MGLevel4.C:1653-2087, sequential
  build, damping 1, no relaxation) from u = x with right-hand side b;
* tests/golden/ref_vanka_nse2_*.npz: the same sweeps by the reference's
  NSTYPE-2 level (TNSE_MGLevel2::CellVanka, src/FE/NSE_MGLevel2.C:336-700)
  built on the one velocity block A11 of these one-block problems;
* tests/golden/ref_vanka_colour_*.npz: the same sweeps by the reference's
  colour-parallel build (-D_HYBRID: CellVanka's OpenMP colour loop,
  src/FE/NSE_MGLevel4.C:603-1651) over the level's own colouring, and two
  sweeps with damping 0.8 and relaxation 0.7;
* tests/golden/ref_cycle_*.npz: one V(2,2) cycle from zero on b, the
  preconditioner call TMultiGridIte::Iterate (src/FE/MultiGridIte.C:76-132)
  with TNSE_MultiGrid::Cycle (src/FE/NSE_MultiGrid.C:434-1779) over two or
  three TNSE_MGLevel4 levels: cell Vanka on the levels above the coarsest
  (sequential build), SolveExact on the coarsest, the reference's transfers
  between them;
* tests/golden/ref_cycle_colour_*.npz, ref_solve_colour_*.npz: the same
  cycle and whole solver in the reference's colour-parallel build (every
  smoothed level swept by the OpenMP colour loop over its own colouring);
* tests/golden/ref_solve_*.npz: the whole reference solver, its flexible
  FGMRES (TFgmresIte::Iterate, src/FE/FgmresIte.C:250-677) preconditioned by
  that cycle driver, from zero on the problem's right-hand side (stored with
  the solution and the iteration count).
Needs the reference tree; the fixtures are committed so the tests do not.
``python make_ref_golden.py cycle`` writes the cycle fixtures only,
``python make_ref_golden.py solve`` the whole-solver ones,
``python make_ref_golden.py colour`` the colour-parallel Vanka, cycle and
solver ones.

Inputs are exact binary fractions of the DOF index (``golden_inputs``), so
every platform forms the same x and b without a random generator.
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

HERE = Path(__file__).resolve().parent

# name -> (OseenProblem keyword arguments, level)
CASES = {
    "hexa": (dict(n_levels=2, nu=1e-2, seed=0), 1),
    "channel": (dict(n_levels=2, nu=1e-2, seed=0, example="channel", periodic="xz",
                     stretch_y=1.5, box=[0.0, 6.0, -1.0, 1.0, 0.0, 3.0]), 1),
    "tetra": (dict(n_levels=2, nu=1.0, seed=0, example="quadlin_oseen", element="tetra"), 0),
}


def golden_inputs(n: int):
    i = np.arange(n, dtype=np.int64)
    x = ((i * 7919 + 13) % 2003 - 1001).astype(np.float64) / 512.0
    b = ((i * 104729 + 7) % 1999 - 999).astype(np.float64) / 256.0
    return x, b


def build_problem(kwargs: dict):
    from to_merge_master_parmoon_gb300 import OseenProblem
    kw = dict(kwargs)
    if "box" in kw:
        kw["box"] = tuple(kw["box"])
    return OseenProblem(**kw)


# name -> (OseenProblem keyword arguments, level) of the Vanka fixtures: a
# level above the coarsest (which the library solves exactly) and small
# enough that one colour per cell stays within the library's colour limit
VANKA_CASES = {
    "hexa": (CASES["hexa"][0], 1),
    "tetra": (dict(n_levels=2, nu=1.0, seed=0, example="quadlin_oseen", element="tetra",
                   nx0=1, ny0=1, nz0=1), 1),
}


# name -> (OseenProblem keyword arguments, level) of the colour-parallel Vanka
# fixtures: the reference's OpenMP colour loop over the level's own colouring
# (cell_colour of the problem), which is also what the library sweeps by
COLOUR_VANKA_CASES = {
    "hexa": (dict(CASES["hexa"][0], n_levels=3), 2),
    "channel": (CASES["channel"][0], 1),
    "tetra": VANKA_CASES["tetra"],
}
# (damping, relaxation alpha) of the second pair of colour-parallel sweeps
COLOUR_VANKA_DAMPED = (0.8, 0.7)


def write_colour_vanka_fixtures() -> None:
    from oracle.pyref import RefVankaLevel
    damp, alpha = COLOUR_VANKA_DAMPED
    for name, (kwargs, level) in COLOUR_VANKA_CASES.items():
        P = build_problem(kwargs)
        a = P.arrays(level)
        x, b = golden_inputs(P.ndof(level))
        V = RefVankaLevel(a, colours=a["cell_colour"])
        W = RefVankaLevel(a, alpha=alpha, colours=a["cell_colour"])
        np.savez_compressed(
            HERE / f"ref_vanka_colour_{name}.npz",
            problem=json.dumps(kwargs), level=level, n_cells=a["n_cells"],
            colours=np.asarray(a["cell_colour"], dtype=np.int32),
            u_sweep1=V.cell_vanka(x, b, 1), u_sweep2=V.cell_vanka(x, b, 2),
            u_damped2=W.cell_vanka(x, b, 2, damp), damp=damp, alpha=alpha,
            source=("reference src/FE/NSE_MGLevel4.C TNSE_MGLevel4::CellVanka (_HYBRID: "
                    "the OpenMP colour loop) run by oracle/ref_vanka.cpp"))
        print("wrote colour vanka", name, "level", level, "ndof", P.ndof(level))


# name -> (OseenProblem keyword arguments, fine level) of the transfer fixtures
TRANSFER_CASES = {
    "hexa": (CASES["hexa"][0], 1),
    "channel": (CASES["channel"][0], 1),
}


# name -> OseenProblem keyword arguments of the cycle fixtures: two levels
# (the V-cycle of the fine level over the exactly solved coarse one) and
# three (cell Vanka on the middle level too, its cells and the finest ones in
# composed child frames)
CYCLE_CASES = {
    "hexa": CASES["hexa"][0],
    "channel": CASES["channel"][0],
    "hexa3": dict(CASES["hexa"][0], n_levels=3),
    "channel3": dict(CASES["channel"][0], n_levels=3),
}


def write_cycle_fixtures() -> None:
    from oracle.pyref import RefCycle
    for name, kwargs in CYCLE_CASES.items():
        P = build_problem(kwargs)
        _, b = golden_inputs(P.ndof(-1))
        np.savez_compressed(
            HERE / f"ref_cycle_{name}.npz", problem=json.dumps(kwargs), level=P.n_levels - 1,
            vcycle=RefCycle(P).vcycle(b, pre=2, post=2, damp=1.0),
            source=("reference src/FE/MultiGridIte.C TMultiGridIte::Iterate with "
                    "src/FE/NSE_MultiGrid.C TNSE_MultiGrid::Cycle (V(2,2), cell Vanka _SEQ, "
                    "SolveExact) run by oracle/ref_transfer.cpp"))
        print("wrote cycle", name, "ndof", P.ndof(-1))


# name -> (OseenProblem keyword arguments, FGMRES parameters) of the fixtures
# of the whole reference solver: its FGMRES over its own cycle driver on
# every level of the problem, from zero on the problem's right-hand side
SOLVE_CASES = {
    "hexa3": (dict(CASES["hexa"][0], n_levels=3),
              dict(restart=20, maxit=100, red_factor=1e-10, res_norm_min=1e-30)),
}


def write_solve_fixtures() -> None:
    from oracle.pyoracle import Oracle
    from oracle.pyref import RefCycle, RefLevel
    for name, (kwargs, fgmres) in SOLVE_CASES.items():
        P = build_problem(kwargs)
        b = P.rhs()
        params = Oracle(P, vanka_mode="seq", **fgmres).params
        x, it = RefLevel(P.arrays(P.n_levels - 1), threads=1).fgmres_with_reference_cycle(
            RefCycle(P), params, np.zeros_like(b), b)
        np.savez_compressed(
            HERE / f"ref_solve_{name}.npz", problem=json.dumps(kwargs), level=P.n_levels - 1,
            fgmres=json.dumps(fgmres), rhs=b, solution=x, iterations=it,
            source=("reference src/FE/FgmresIte.C TFgmresIte::Iterate (run by "
                    "oracle/ref_harness.cpp) preconditioned by src/FE/MultiGridIte.C "
                    "TMultiGridIte::Iterate with src/FE/NSE_MultiGrid.C TNSE_MultiGrid::Cycle "
                    "(V(2,2), cell Vanka _SEQ, SolveExact; run by oracle/ref_transfer.cpp)"))
        print("wrote solve", name, "iterations", it, "ndof", b.size)


# the cycle and whole-solver fixtures of the reference's colour-parallel
# build: every smoothed level swept by CellVanka's OpenMP colour loop over the
# level's own colouring (its cell_colour)
COLOUR_CYCLE_CASES = ("hexa3", "channel3")
COLOUR_SOLVE_CASES = ("hexa3",)


def write_colour_cycle_fixtures() -> None:
    from oracle.pyoracle import Oracle
    from oracle.pyref import RefCycle, RefLevel
    for name in COLOUR_CYCLE_CASES:
        kwargs = CYCLE_CASES[name]
        P = build_problem(kwargs)
        _, b = golden_inputs(P.ndof(-1))
        np.savez_compressed(
            HERE / f"ref_cycle_colour_{name}.npz", problem=json.dumps(kwargs),
            level=P.n_levels - 1, vcycle=RefCycle(P, colours=True).vcycle(b, pre=2, post=2,
                                                                          damp=1.0),
            source=("reference src/FE/MultiGridIte.C TMultiGridIte::Iterate with "
                    "src/FE/NSE_MultiGrid.C TNSE_MultiGrid::Cycle (V(2,2), cell Vanka _HYBRID "
                    "colour loop over the levels' cell_colour, SolveExact) run by "
                    "oracle/ref_transfer.cpp"))
        print("wrote colour cycle", name, "ndof", P.ndof(-1))
    for name in COLOUR_SOLVE_CASES:
        kwargs, fgmres = SOLVE_CASES[name]
        P = build_problem(kwargs)
        b = P.rhs()
        params = Oracle(P, vanka_mode="colour", **fgmres).params
        x, it = RefLevel(P.arrays(P.n_levels - 1), threads=1).fgmres_with_reference_cycle(
            RefCycle(P, colours=True), params, np.zeros_like(b), b)
        np.savez_compressed(
            HERE / f"ref_solve_colour_{name}.npz", problem=json.dumps(kwargs),
            level=P.n_levels - 1, fgmres=json.dumps(fgmres), solution=x, iterations=it,
            source=("reference src/FE/FgmresIte.C TFgmresIte::Iterate (run by "
                    "oracle/ref_harness.cpp) preconditioned by the colour-parallel cycle of "
                    "ref_cycle_colour_*; right-hand side: that of ref_solve_" + name + ".npz"))
        print("wrote colour solve", name, "iterations", it)


def main() -> None:
    from oracle.pyref import RefLevel, RefTransfer, RefVankaLevel, ref_harness_lib
    if ref_harness_lib() is None:
        raise SystemExit("reference tree not found; cannot regenerate the defect golden files")
    if sys.argv[1:] == ["cycle"]:
        write_cycle_fixtures()
        return
    if sys.argv[1:] == ["solve"]:
        write_solve_fixtures()
        return
    if sys.argv[1:] == ["colour"]:
        write_colour_vanka_fixtures()
        write_colour_cycle_fixtures()
        return
    for name, (kwargs, level) in CASES.items():
        P = build_problem(kwargs)
        R = RefLevel(P.arrays(level), threads=1)
        x, b = golden_inputs(R.ndof)
        np.savez_compressed(
            HERE / f"ref_defect_{name}.npz",
            problem=json.dumps(kwargs), level=level, n_udof=R.n_u, n_pdof=R.n_p,
            r_project=R.defect(x, b, True), r_plain=R.defect(x, b, False), y=R.matvec(x),
            source=("reference src/FE/MGComponents3D.C Defect_NSE4 / MatVect_NSE4 "
                    "run by oracle/ref_harness.cpp"))
        print("wrote", name, "level", level, "ndof", R.ndof)
    for name, (kwargs, level) in VANKA_CASES.items():
        P = build_problem(kwargs)
        V = RefVankaLevel(P.arrays(level))
        x, b = golden_inputs(P.ndof(level))
        np.savez_compressed(
            HERE / f"ref_vanka_{name}.npz",
            problem=json.dumps(kwargs), level=level, n_cells=P.arrays(level)["n_cells"],
            u_sweep1=V.cell_vanka(x, b, 1), u_sweep2=V.cell_vanka(x, b, 2),
            source=("reference src/FE/NSE_MGLevel4.C TNSE_MGLevel4::CellVanka (_SEQ) "
                    "run by oracle/ref_vanka.cpp"))
        print("wrote vanka", name, "level", level, "ndof", P.ndof(level))
    for name, (kwargs, level) in VANKA_CASES.items():
        P = build_problem(kwargs)
        V = RefVankaLevel(P.arrays(level), one_block=True)
        x, b = golden_inputs(P.ndof(level))
        np.savez_compressed(
            HERE / f"ref_vanka_nse2_{name}.npz",
            problem=json.dumps(kwargs), level=level, n_cells=P.arrays(level)["n_cells"],
            u_sweep1=V.cell_vanka(x, b, 1), u_sweep2=V.cell_vanka(x, b, 2),
            source=("reference src/FE/NSE_MGLevel2.C TNSE_MGLevel2::CellVanka (NSTYPE 2, "
                    "the one velocity block A11) run by oracle/ref_vanka.cpp"))
        print("wrote NSTYPE-2 vanka", name, "level", level, "ndof", P.ndof(level))
    for name, (kwargs, _) in CASES.items():
        P = build_problem(kwargs)
        V = RefVankaLevel(P.arrays(0))
        _, b = golden_inputs(P.ndof(0))
        np.savez_compressed(
            HERE / f"ref_coarse_{name}.npz", problem=json.dumps(kwargs), level=0,
            n_cells=P.arrays(0)["n_cells"], solution=V.solve_exact(b),
            source=("reference src/FE/NSE_MGLevel4.C TNSE_MGLevel4::SolveExact "
                    "run by oracle/ref_vanka.cpp"))
        print("wrote coarse", name, "ndof", P.ndof(0))
    for name, (kwargs, level) in TRANSFER_CASES.items():
        P = build_problem(kwargs)
        T = RefTransfer(P, level)
        xc, _ = golden_inputs(P.ndof(level - 1))
        _, bf = golden_inputs(P.ndof(level))
        np.savez_compressed(
            HERE / f"ref_transfer_{name}.npz",
            problem=json.dumps(kwargs), level=level, prolongated=T.prolongate(xc),
            restricted=T.restrict(bf),
            source=("reference src/FE/MGComponents3D.C Prolongate / DefectRestriction "
                    "run by oracle/ref_transfer.cpp"))
        print("wrote transfer", name, "level", level)
    write_cycle_fixtures()


if __name__ == "__main__":
    main()
