"""Benchmark: time-to-1e-8 relative residual of the 3D Oseen saddle-point
solve (Q2/P1disc, 64^3 cells, 6 levels from 2^3, nu = 1e-2) on one GB300.

One step = one complete linear solve with the matrices already resident in
HBM: factor every local 85x85 Vanka block and the coarse system, then
FGMRES(20) preconditioned by one V(2,2) cycle with cell Vanka until
||b - K x|| <= 1e-8 ||b||.  ``value`` is the mean step time (CUDA events on
the library's stream) of the mixed-precision path; the plain FP64 GPU path
is timed beside it.  ``e2e`` times the same solve through the C ABI with
host buffers: per step the matrix values are copied host->device
(pm_update_matrices), refactored, and the rhs/solution travel through
pm_solve.

``--impl reference`` times the CPU restatement of the reference solver
(oracle/, FP64, every Vanka block refactored in every sweep as in
src/FE/NSE_MGLevel4.C:1653-2087) on all host cores: one complete solve to
1e-8 (its measured wall time is the value), then one FGMRES iteration per
step as the bounded per-step sample.

The same oracle solve at the full size is ``cpu_baseline`` of the default
run, and its solution is the answer every GPU variant's ``error_vs_oracle``
(relative L2 of velocity and of the L2_0-normalised pressure) is taken
against.  ``cpu_runs_16cube`` adds the three CPU settings of the
CPU-runnable case (16^3, rtol 1e-10): one thread with the reference's
cell-by-cell Vanka, all cores with colour-parallel Vanka, and all cores
with the local factors kept across sweeps.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "3D Oseen time-to-1e-8 residual: mixed+learned vs plain FP64 GMG on one GB300"
RTOL = 1e-8


# FP64 flops of k_assemble_cells<false> per cell: scaled nodal convection
# (81 x 2), the diffusion/mass y-z factors (81 x 13), the z and y contractions
# of the convection integrals (243 x 3 and 243 x 9 FMA), the x contraction
# with diffusion per A entry (729 x 8 FMA) and its addition into the CSR
# value (729), the B/BT entries (108 x 15)
ASSEMBLY_FLOP_PER_CELL = 81 * 2 + 81 * 13 + 2 * (243 * 3 + 243 * 9) + 729 * 16 + 729 + 108 * 15


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--levels", type=int, default=6)
    ap.add_argument("--nu", type=float, default=1e-2)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-systems", type=int, default=48)
    ap.add_argument("--no-assembly", action="store_true")
    ap.add_argument("--no-channel", action="store_true")
    ap.add_argument("--only-mlp", type=int, default=0, metavar="ROWS",
                    help="forward passes of the learned smoother's MLP on ROWS random "
                         "feature rows only (warm-up + steps): the case profiled for "
                         "k_mlp_layer_tc")
    ap.add_argument("--only-factor", action="store_true",
                    help="refactorisation of every level only (nine-block mixed levels, "
                         "warm-up + steps passes): the case profiled for the factor kernels")
    ap.add_argument("--only-sweep", default="", choices=["", "mixed", "fp64"],
                    help="cell-Vanka sweeps of the finest level only (pm_cell_vanka, warm-up "
                         "+ steps sweeps) in the given precision: the case profiled for the "
                         "local-residual and apply kernels")
    ap.add_argument("--residual-variant", type=int, default=0,
                    help="pm_options.residual_variant of the --only-sweep case")
    ap.add_argument("--factor-fp32", type=int, default=-1, choices=[-1, 0, 1],
                    help="pm_options.factor_fp32 of the --only-factor case (-1: FP32 block "
                         "elimination, FP64 85x85 LU; 0: both FP64; 1: both FP32)")
    ap.add_argument("--decouple", type=int, default=1,
                    help="pm_options.decouple of the --only-sweep / --only-factor cases (0: the "
                         "85x85 LU and all nine blocks on every level)")
    ap.add_argument("--channel-steps", type=int, default=10,
                    help="timed Crank-Nicolson steps per variant of the channel run "
                         "(a bounded sample of its 200 steps)")
    ap.add_argument("--channel-variants", default="fp64,mixed,mixed_learned,mixed_scaled_divergence",
                    help="comma-separated channel variants to run")
    ap.add_argument("--only-channel", action="store_true",
                    help="the time-dependent channel run only (the learned variant is skipped): "
                         "e.g. all 200 steps of one variant")
    ap.add_argument("--only-batch", action="store_true",
                    help="the batch of independent systems only (concurrent handles, one "
                         "after another, and fused groups)")
    ap.add_argument("--only-assembly", action="store_true",
                    help="device assembly of every level only (one-block FP64 levels, "
                         "warm-up + steps passes): the case profiled for k_assemble_cells")
    ap.add_argument("--train-problems", type=int, default=8)
    ap.add_argument("--no-nu-study", action="store_true",
                    help="skip the nu = 1e-3 leg (64^3 FP64 / mixed / mixed + learned, and the "
                         "oracle against the GPU FP64 path at 16^3 and 32^3)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def max_over_ranks(x: float, world: int) -> float:
    """The largest x over the ranks of the process group (the replicas' step
    time); a CUDA tensor with NCCL, a host tensor otherwise (gloo)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.seek(0)
        sm, mx, reasons = [], None, set()
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


# DRAM bytes (read + write) per cell of one local-residual launch of the
# headline kernel (k_vanka_residual_rows<float,1,1,8,27,true,true>: FP32, one
# A block, interleaved velocity) from one ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum = 136.83 + 2.90 MB) of a 32^3 colour launch of 4,096 cells:
#   ncu --set full --clock-control none -k regex:'k_vanka_residual|k_schur_apply' -s 32 -c 2 \
#       python bench.py --only-sweep mixed --levels 5 --warmup 1 --steps 2
# Traffic grows with the cells a launch processes (every cell reads its own
# 27 rows), so it scales to a launch of any size.
RESIDUAL_DRAM_BYTES_PER_CELL = 34114


# the FP32 sweep kernels by level mode (0 nine blocks + LU, 1 three diagonal
# blocks, 2 one block A11 = A22 = A33)
def residual_kernel_name(mode, variant):
    """The FP32 local-residual kernel a level runs: level mode (0 nine blocks
    + LU, 1 three diagonal blocks, 2 one block A11 = A22 = A33) and residual
    kernel (0 row groups, 1 flattened stream)."""
    blocks = {0: "nine A blocks", 1: "A11, A22, A33", 2: "one A block (A11 = A22 = A33)"}[mode]
    if variant == 1:
        return ("k_vanka_residual<float,4,1> (cell-local residuals over full CSR rows of one "
                f"colour, flattened entry stream; {blocks}, BT, B)")
    if mode == 2:
        return ("k_vanka_residual_rows<float,1,1,8,27,true,true> (cell-local residuals over full "
                "CSR rows of one colour, 8 lanes per row, A and BT rows of a step loaded "
                f"together, velocity gathered from its interleaved copy; {blocks}, BT, B)")
    kind = {0: 0, 1: 2}[mode]
    vec, ur = {0: (4, 1), 2: (1, 8)}[kind]
    return (f"k_vanka_residual_rows<float,{vec},{kind},{ur},27> (cell-local "
            f"residuals over full CSR rows of one colour, 8 lanes per row; {blocks}, BT, B)")


APPLY_KERNEL = {
    0: "k_vanka_apply<float,27> (stored FP32 LU, one cell per warp, columns prefetched in "
       "registers and L2; substitution + update)",
    1: "k_schur_apply<float,3> (stored FP32 block elimination: three 27x27 inverses, B, A^-1 BT, "
       "4x4 Schur inverse; one cell per warp, GEMVs + update)",
    2: "k_schur_apply<float,1,true> (stored FP32 block elimination: one 27x27 inverse, B, "
       "A^-1 BT, 4x4 Schur inverse; one cell per warp, GEMVs + update of the interleaved "
       "velocity)"}


def ncu_traffic(P):
    """DRAM bytes per average residual launch of this workload: the measured
    per-cell traffic times the average cells per residual launch (all
    smoothed cells / (8 colours x smoothed levels)); None when unmeasured."""
    if RESIDUAL_DRAM_BYTES_PER_CELL is None:
        return None
    cells = [P.desc(l).n_cells for l in range(1, P.n_levels)]
    return RESIDUAL_DRAM_BYTES_PER_CELL * sum(cells) / (8 * len(cells))


def split_error(x, ref, nu):
    """Relative L2 differences of the velocity [u1|u2|u3] and of the pressure
    after the same L2_0 normalisation of both (the constant P1disc modes,
    every 4th pressure entry, as IntoL20FEFunction3D)."""
    import numpy as np
    n3 = 3 * nu
    xp, rp = x[n3:].copy(), ref[n3:].copy()
    xp[0::4] -= xp[0::4].mean()
    rp[0::4] -= rp[0::4].mean()
    return {"u": float(np.linalg.norm(x[:n3] - ref[:n3]) / np.linalg.norm(ref[:n3])),
            "p": float(np.linalg.norm(xp - rp) / np.linalg.norm(rp))}


def oracle_solve(P, b, tol, threads, maxit=200, **params):
    """The oracle's FGMRES(20) + V(2,2) from x0 = 0 to ||b - K x|| <= tol on
    `threads` host threads; returns (solution, result, wall seconds)."""
    import numpy as np
    from oracle.pyoracle import Oracle
    O = Oracle(P, restart=20, maxit=maxit, res_norm_min=tol, nthreads=threads, **params)
    t = time.perf_counter()
    x, info = O.iterate(np.zeros_like(b), b)
    return x, info, time.perf_counter() - t


def pressure_projected_norm(P, b):
    """||b - K 0|| with the pressure part projected (Defect_NSE4 of x0 = 0)."""
    import numpy as np
    bp = b.copy()
    nu3 = 3 * P.desc(P.n_levels - 1).n_udof
    bp[nu3::4] -= bp[nu3::4].mean()
    return float(np.linalg.norm(bp))


def cpu_runs_16cube(threads, device):
    """The CPU-runnable case (16^3 cells, 4 levels, nu = 1e-2, seed 0,
    FGMRES(20) + V(2,2), rtol 1e-10) in the three CPU settings: (1) one
    thread, the reference's cell-by-cell Vanka (_SEQ,
    src/FE/NSE_MGLevel4.C:1653-2087) refactoring every block in every sweep;
    (2) all cores, colour-parallel Vanka (the _HYBRID colour loop,
    :807-820), refactoring every sweep; (3) as (2) with the local factors
    kept across sweeps (separates the algorithmic gain of factor reuse from
    the GPU's).  Beside them the GPU FP64 and mixed solves of the same
    system; every result with its error against setting (2)."""
    import numpy as np
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    P = OseenProblem(n_levels=4, nu=1e-2, seed=0, nthreads=threads)
    b = P.rhs()
    tol = 1e-10 * pressure_projected_norm(P, b)
    nu = P.desc(3).n_udof
    runs = {}
    x2, i2, t2 = oracle_solve(P, b, tol, threads)
    for name, th, params in (("run1_one_thread_seq", 1, {"vanka_mode": "seq"}),
                             ("run2_all_cores", threads, {}),
                             ("run3_all_cores_factor_reuse", threads, {"reuse_factors": 1})):
        if name == "run2_all_cores":
            x, i, t = x2, i2, t2
        else:
            x, i, t = oracle_solve(P, b, tol, th, **params)
        runs[name] = {"s": t, "threads": th, "iterations": i["iterations"],
                      "rel_res": i["true_res"] / i["res0"], "error_vs_oracle": split_error(x, x2, nu)}
    for prec in ("fp64", "mixed"):
        S = PmSolver(P.descs, precision=prec, device=device, restart=20, maxit=200,
                     res_norm_min=tol)
        S.iterate(np.zeros_like(b), b)  # untimed: graph capture
        f_ms = S.refactor()
        t = time.perf_counter()
        x, i = S.iterate(np.zeros_like(b), b)
        t = time.perf_counter() - t
        runs[f"gpu_{prec}"] = {"s": t + f_ms * 1e-3, "factor_ms": f_ms, "solve_ms": i["solve_ms"],
                               "iterations": i["iterations"], "rel_res": i["true_res"] / i["res0"],
                               "error_vs_oracle": split_error(x, x2, nu)}
        S.close()
    return {"workload": "steady 3D Oseen, Q2/P1disc, 16^3 cells, 4 levels from 2^3, nu=0.01, "
                        "seed 0, FGMRES(20)+V(2,2), rtol 1e-10", "ndof": P.ndof(-1),
            "timer": "wall clock (time.perf_counter) around the solve, set-up excluded; GPU "
                     "rows: refactorisation + solve with host vectors", **runs}


def solve_bytes(P, s, iterations, mode=0, pre=2, post=2, restart=20):
    """Algorithmic (unique) bytes of one FGMRES solve of `iterations`
    iterations: per iteration one V(pre,post) cycle in value size `s` (8
    FP64, 4 FP32), one FP64 mat-vec on the finest level and the modified
    Gram-Schmidt vector traffic.  Per level with cells, matrix bytes
    mat = nblk s nnzA + 4 nnzA + 4 (N_U+1) + (3 s + 4)(nnzB + nnzBT)
    + 4 (N_P+1) + 4 (N_U+1) with nblk = 9 A arrays (mode 0), 3 on
    decoupled levels with distinct diagonal blocks (mode 1) or 1 when
    A11 = A22 = A33 (mode 2); defect = mat + 3 s DOF; Vanka sweep = mat +
    3 s DOF + the stored local solve per cell: 85^2 s + 85 (LU and pivots),
    2851 s (mode 1: three 27x27 inverses, B, A^-1 BT, the 4x4 Schur
    inverse) or 1393 s (mode 2: one inverse); transfers s (2 DOF_f +
    2 DOF_c); the coarse dense solve reads its inverse (FP64).  Arnoldi step
    k of a restart cycle: (k+1) x (2 + 3) x 8 DOF."""
    nblk = {0: 9, 1: 3, 2: 1}[mode]
    L = P.n_levels
    nbytes = 0.0

    def mat(d, sv, nb):
        return (nb * sv * d.a_nnz + 4.0 * d.a_nnz + 4.0 * (d.n_udof + 1)
                + (3 * sv + 4.0) * (d.b_nnz + d.bt_nnz) + 4.0 * (d.n_pdof + 1)
                + 4.0 * (d.n_udof + 1))

    for l in range(1, L):
        d = P.desc(l)
        dof = 3 * d.n_udof + d.n_pdof
        nloc = 3 * d.n_ulocal + d.n_plocal
        m = mat(d, s, nblk)
        local = {0: nloc * nloc * s + nloc, 1: 2851 * s, 2: 1393 * s}[mode]
        sweep = m + 3 * s * dof + d.n_cells * local
        dc = P.desc(l - 1)
        dof_c = 3 * dc.n_udof + dc.n_pdof
        nbytes += (pre + post) * sweep + (m + 3 * s * dof) + s * (2 * dof + 2 * dof_c)
    d0 = P.desc(0)
    n0 = 3 * d0.n_udof + d0.n_pdof
    nbytes += 8.0 * n0 * n0
    df = P.desc(L - 1)
    dof_f = 3 * df.n_udof + df.n_pdof
    per_it_fixed = nbytes + mat(df, 8, nblk) + 2 * 8.0 * dof_f
    total = 0.0
    for j in range(iterations):
        k = j % restart
        total += per_it_fixed + (k + 1) * 5 * 8.0 * dof_f
    return total


def residual_fma(P, nblk):
    """FMA of the cell-local residual kernel for one sweep of every level with
    cells: per cell, every entry of its 27 velocity rows' A rows (nblk FMA:
    9 with nine blocks, 3 decoupled), of their BT rows on active rows (3) and
    of its 4 pressure rows' B rows (3).  Returns {level: FMA per sweep}."""
    import numpy as np
    out = {}
    for l in range(1, P.n_levels):
        a = P.arrays(l)
        la = np.diff(a["a_rowptr"]).astype(np.int64)
        lbt = np.diff(a["bt_rowptr"]).astype(np.int64)
        lbt[a["n_active"]:] = 0
        lb = np.diff(a["b_rowptr"]).astype(np.int64)
        ud, pd = a["cell_udofs"], a["cell_pdofs"]
        out[l] = int(nblk * la[ud].sum() + 3 * lbt[ud].sum() + 3 * lb[pd].sum())
    return out


# FMA of one cell's block-elimination factorisation (k_schur_factor<NB>):
# NB = 3 (distinct diagonal blocks): per component a Gauss-Jordan on
# [A_c | I | G_c] (27 x 58: sum over k of 26 rows x (57 - k) columns) and its
# share of the 4x4 Schur complement (16 x 27); NB = 1 (A11 = A22 = A33): one
# Gauss-Jordan on [A | I | G1 G2 G3] (27 x 66) and the Schur complement
# (16 x 27 x 3)
SCHUR_FMA_PER_CELL = {1: 3 * (26 * sum(57 - k for k in range(27)) + 16 * 27),
                      2: 26 * sum(65 - k for k in range(27)) + 16 * 27 * 3}


def run_reference(args):
    """The reference arm: the oracle (the reference's algorithm restated on
    the CPU, FP64, every local block refactored in every sweep) on all host
    threads, on rank 0 only.  One complete solve to 1e-8 is timed first; its
    wall time is the value (time to tolerance).  Then warm-up + steps bounded
    samples of one FGMRES iteration each (V(2,2) + mat-vec + MGS) give the
    per-step time."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    from oracle.pyoracle import Oracle
    from to_merge_master_parmoon_gb300 import OseenProblem
    threads = os.cpu_count() or 1
    P = OseenProblem(n_levels=args.levels, nu=args.nu, seed=args.seed, nthreads=threads)
    b = P.rhs()
    tol = RTOL * pressure_projected_norm(P, b)
    _, info, t_full = oracle_solve(P, b, tol, threads)
    O = Oracle(P, restart=20, maxit=1, res_norm_min=0.0, nthreads=threads)
    times = []
    for s in range(args.warmup + args.steps):
        t = time.perf_counter()
        O.iterate(np.zeros_like(b), b)
        dt = time.perf_counter() - t
        if s >= args.warmup:
            times.append(dt)
    per_it = sum(times) / len(times)
    value = t_full
    n = args.levels
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_it * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded divergence-free Fourier convection, smooth forcing)",
        "config": {"workload": f"steady 3D Oseen, Q2/P1disc, {2 ** n}^3 cells, {n} levels from 2^3, "
                               f"nu={args.nu}, FGMRES(20)+V(2,2) cell Vanka, rtol 1e-8",
                   "ndof": P.ndof(-1)},
        "iterations": info["iterations"], "rel_res": info["true_res"] / info["res0"],
        "per_iteration_s": per_it,
        "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port",
                         "sample": f"one complete solve to 1e-8 at the full size, timed once "
                                   f"({info['iterations']} FGMRES iterations); each step: one "
                                   f"FGMRES iteration (V(2,2) + mat-vec + MGS)"},
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def assembly_run(P, S, args, threads, S1=None):
    """Device re-assembly of the Galerkin Oseen blocks of every level
    (pm_assemble_level_device from device cell sizes and nodal convection)
    against the host builder's assembly of the same levels on all host
    threads, then Crank-Nicolson steps (tau = 1e-2) of the time-dependent
    Oseen system with the convection field held fixed, every step on the
    device: the system M + tau/2 A, B, tau BT on every level, the
    refactorisation, the working right-hand side and the FGMRES solve; on
    one-block (NSTYPE-2) levels when the problem has them (S1), as the theta
    system keeps A11 = A22 = A33 and A12..A32 = 0, and on the nine-block
    levels of S."""
    import numpy as np
    import torch
    dev = [(torch.from_numpy(P.cell_sizes(l)).cuda(),
            torch.from_numpy(P.convection_nodal(l)).cuda()) for l in range(P.n_levels)]
    cells = [P.desc(l).n_cells for l in range(P.n_levels)]

    def assemble_all():
        t0 = time.perf_counter()
        for l, (h, c) in enumerate(dev):
            S.assemble_level_device(l, h.data_ptr(), c.data_ptr(), P.nu)
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        assemble_all()
    gpu = [assemble_all() for _ in range(args.steps)]
    cpu = []
    for _ in range(2):
        t0 = time.perf_counter()
        P.reassemble()
        cpu.append(time.perf_counter() - t0)
    # the device-assembled levels solve as the host-built ones do
    n = P.ndof(-1)
    d_b = torch.from_numpy(P.rhs()).cuda()
    d_x = torch.zeros(n, dtype=torch.float64, device="cuda")
    f0 = S.refactor()
    info0 = S.iterate_device(d_x.data_ptr(), d_b.data_ptr())

    tau, theta = 1e-2, 0.5
    sysm = (1.0, tau * theta, 1.0, tau)

    def theta_steps(T):
        d_u = torch.zeros(n, dtype=torch.float64, device="cuda")
        d_w = torch.empty_like(d_u)
        d_v = torch.empty_like(d_u)
        rows = []
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            for l, (h, c) in enumerate(dev):
                T.assemble_system_level_device(l, h.data_ptr(), c.data_ptr(), P.nu, *sysm)
            t_asm = time.perf_counter() - t0
            f_ms = T.refactor()
            t0 = time.perf_counter()
            T.system_rhs_device(d_b.data_ptr(), d_b.data_ptr(), d_u.data_ptr(), tau * (1 - theta),
                                tau * theta, tau * (1 - theta), d_w.data_ptr())
            t_rhs = time.perf_counter() - t0
            d_v.copy_(d_u)
            torch.cuda.synchronize()
            info = T.iterate_device(d_v.data_ptr(), d_w.data_ptr())
            d_u.copy_(d_v)
            torch.cuda.synchronize()
            rows.append({"assembly_ms": t_asm * 1e3, "factor_ms": f_ms, "rhs_ms": t_rhs * 1e3,
                         "solve_ms": info["solve_ms"], "iterations": info["iterations"],
                         "rel_res": info["true_res"] / max(float(torch.linalg.norm(d_w)), 1e-300)})
        rows = rows[args.warmup:]

        def mean(key):
            return sum(r[key] for r in rows) / len(rows)

        out = {k: mean(k) for k in ("assembly_ms", "factor_ms", "rhs_ms", "solve_ms",
                                    "iterations")}
        out["step_ms"] = sum(out[k] for k in ("assembly_ms", "factor_ms", "rhs_ms", "solve_ms"))
        out["max_rel_res"] = max(r["rel_res"] for r in rows)
        out["steps"] = len(rows)
        return out

    g = sum(gpu) / len(gpu)
    return {
        "cells": sum(cells), "levels": P.n_levels,
        "gpu_ms": g * 1e3, "cpu_ms": min(cpu) * 1e3, "cpu_threads": threads,
        "speedup": min(cpu) / g,
        "fp64_gflops": ASSEMBLY_FLOP_PER_CELL * sum(cells) / g / 1e9,
        "iterations_after": info0["iterations"], "factor_ms_after": f0,
        "theta_steps": {"tau": tau, "theta": theta, "convection": "fixed (time-dependent Oseen)",
                        "nine_block": theta_steps(S),
                        "one_block": theta_steps(S1) if S1 is not None else None},
    }


def channel_run(args, threads, net):
    """Time-dependent channel (TNSE3D): box [0, 2pi] x [-1, 1] x [0, pi],
    64 x 64 x 32 hexahedra (5 levels from 4 x 4 x 2), periodic in x and z,
    no-slip at y = +-1, y = tanh(2.5 eta)/tanh(2.5), Q2/P1disc, nu = 1/180,
    body force 2 nu e_x, initial velocity 1 - y^2 plus a 5 % seeded
    divergence-free perturbation; Crank-Nicolson (theta = 1/2), dt = 1e-3,
    one Oseen linearisation per step on the current velocity, solved to a
    1e-8 residual reduction.  Every step on the device: the velocity at the
    coarse nodes (pm_interpolate_coarse), the system M + dt/2 A(u), B, dt BT
    on every level (pm_assemble_system_level_device), the refactorisation,
    the working right-hand side (pm_system_rhs_device) and the FGMRES solve
    from u.  NSTYPE-2 levels (the system keeps A11 = A22 = A33, A12..A32 = 0).
    Variants: FP64, mixed, mixed + learned smoother, and mixed with the
    divergence constraint scaled by dt (SCALE_DIVERGENCE_CONSTRAINT = 1); 2
    untimed steps, then args.channel_steps timed steps from the same initial
    state each."""
    import numpy as np
    import torch
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    from to_merge_master_parmoon_gb300.solver import PmError
    P = OseenProblem(n_levels=5, nu=1.0 / 180.0, seed=args.seed, example="channel", nx0=4, ny0=4,
                     nz0=2, box=(0.0, 2 * np.pi, -1.0, 1.0, 0.0, np.pi), periodic="xz",
                     stretch_y=2.5, perturb=0.05, nthreads=threads)
    L = P.n_levels
    D1 = P.descs_one_block()
    tau, theta = 1e-3, 0.5
    n3 = 3 * P.desc(L - 1).n_udof
    d_h = [torch.from_numpy(P.cell_sizes(l)).cuda() for l in range(L)]
    d_conv = [torch.empty(3 * P.desc(l).n_udof, dtype=torch.float64, device="cuda")
              for l in range(L - 1)]
    d_f = torch.from_numpy(P.rhs()).cuda()
    u0 = torch.zeros_like(d_f)
    u0[:n3] = torch.from_numpy(P.convection_nodal(L - 1)).cuda()
    d_w = torch.empty_like(d_f)
    out = {"workload": "channel 64x64x32 (tanh 2.5 in y), periodic x/z, Q2/P1disc, nu=1/180, "
                       "CN dt=1e-3, one Oseen linearisation per step to 1e-8 reduction",
           "ndof": P.ndof(-1), "levels": L, "timed_steps": args.channel_steps}
    # B unscaled as with the reference's default SCALE_DIVERGENCE_CONSTRAINT = -1;
    # the last variant sets it to 1 (B scaled by dt as well,
    # src/System/SystemTNSE3D.C:1248-1264)
    wanted = set(args.channel_variants.split(","))
    for name, prec, learned, b_scale in (("fp64", "fp64", False, 1.0),
                                         ("mixed", "mixed", False, 1.0),
                                         ("mixed_learned", "mixed", True, 1.0),
                                         ("mixed_scaled_divergence", "mixed", False, tau)):
        if name not in wanted or (learned and net is None):
            continue
        kw = dict(precision=prec, restart=20, maxit=100, res_norm_min=1e-300, red_factor=1e-8,
                  red_initial=1)
        try:
            S = PmSolver(D1, upload_mode=1, **kw)
        except PmError:
            S = PmSolver(D1, upload_mode=0, **kw)
        if learned:
            S.attach_learned(net, omega=1.0, fallback_ratio=0.5)
        d_u = u0.clone()
        rows = []
        for k in range(2 + args.channel_steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            conv = [None] * L
            conv[L - 1] = d_u[:n3]
            for l in range(L - 1, 0, -1):
                S.interpolate_coarse(l, conv[l].data_ptr(), d_conv[l - 1].data_ptr())
                conv[l - 1] = d_conv[l - 1]
            for l in range(L):
                S.assemble_system_level_device(l, d_h[l].data_ptr(), conv[l].data_ptr(), P.nu,
                                               1.0, tau * theta, b_scale, tau)
            t1 = time.perf_counter()
            f_ms = S.refactor()
            t2 = time.perf_counter()
            S.system_rhs_device(d_f.data_ptr(), d_f.data_ptr(), d_u.data_ptr(), tau * (1 - theta),
                                tau * theta, tau * (1 - theta), d_w.data_ptr())
            info = S.iterate_device(d_u.data_ptr(), d_w.data_ptr(), allow=(0, 1))
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            rows.append({"assembly_ms": (t1 - t0) * 1e3, "factor_ms": f_ms,
                         "solve_ms": (t3 - t2) * 1e3, "step_ms": (t3 - t0) * 1e3,
                         "iterations": info["iterations"],
                         "reduction": info["true_res"] / max(info["res0"], 1e-300)})
        rows = rows[2:]
        mean = lambda key: sum(r[key] for r in rows) / len(rows)
        out[name] = {k: mean(k) for k in ("step_ms", "assembly_ms", "factor_ms", "solve_ms",
                                           "iterations")}
        out[name]["max_reduction"] = max(r["reduction"] for r in rows)
        out[name]["s_timed_steps"] = sum(r["step_ms"] for r in rows) / 1e3
        out[name]["s_per_200_steps"] = mean("step_ms") * 200 / 1e3
        out[name]["s_per_200_steps_measured"] = len(rows) >= 200
        if learned:
            out[name]["learned_status"] = S.learned_status()
        umax = float(d_u[:n3].abs().max())
        out[name]["max_abs_u"] = umax
        S.close()
    return out


def only_mlp(args):
    """MLP forward (397 -> 256 -> 256 -> 85, BF16 on tcgen05, FP32 accumulate)
    on args.only_mlp rows of seeded random features; prints the mean time of
    a pass and the flop rate (3.78e5 flop per row)."""
    import torch
    from to_merge_master_parmoon_gb300.learned import Mlp
    m = args.only_mlp
    net = Mlp(device=0, seed=0, max_batch=m)
    g = torch.Generator(device="cuda").manual_seed(0)
    X = torch.randn(m, 397, device="cuda", generator=g)
    ts = []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        net.forward(X)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    t = sum(ts[args.warmup:]) / args.steps
    flop = 2.0 * (397 * 256 + 256 * 256 + 256 * 85) * m
    print(json.dumps({"only_mlp": True, "rows": m, "ms_per_pass": t * 1e3,
                      "tflops": flop / t / 1e12}), flush=True)


def only_factor(args):
    """pm_refactor of nine-block mixed levels, args.warmup + args.steps times;
    prints the mean factorisation time (the library's CUDA events)."""
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    P = OseenProblem(n_levels=args.levels, nu=args.nu, seed=args.seed, nthreads=os.cpu_count() or 1)
    S = PmSolver(P.descs, precision="mixed", decouple=args.decouple,
                 factor_fp32=args.factor_fp32)
    ms = [S.refactor() for _ in range(args.warmup + args.steps)][args.warmup:]
    print(json.dumps({"only_factor": True, "levels": P.n_levels,
                      "factor_fp32": args.factor_fp32,
                      "cells": sum(P.desc(l).n_cells for l in range(1, P.n_levels)),
                      "factor_ms": sum(ms) / len(ms)}), flush=True)


def only_sweep(args):
    """pm_cell_vanka on the finest level of a nine-block problem (args.levels
    levels from 2^3, seed args.seed), one sweep per call, args.warmup +
    args.steps calls in the precision args.only_sweep; prints the kernels a
    sweep launches and the mean device time of the local-residual and apply
    kernels per sweep (profiling events around every launch).  A sweep is 8
    colours x (residual + apply) between two Dirichlet updates, so under a
    profiler the residual launch of colour k of sweep s is number
    8 s + k of its kernel."""
    import numpy as np
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    P = OseenProblem(n_levels=args.levels, nu=args.nu, seed=args.seed, nthreads=os.cpu_count() or 1)
    S = PmSolver(P.descs, precision=args.only_sweep, decouple=args.decouple,
                 residual_variant=args.residual_variant)
    L = P.n_levels
    rng = np.random.default_rng(0)
    u = 0.1 * rng.standard_normal(P.ndof(L - 1))
    f = rng.standard_normal(P.ndof(L - 1))
    for _ in range(args.warmup):
        u = S.cell_vanka(L - 1, u, f, 1)
    S.profile(True)
    n0 = S.kernel_launches
    for _ in range(args.steps):
        u = S.cell_vanka(L - 1, u, f, 1)
    launches = (S.kernel_launches - n0) // args.steps
    prof = S.profile_read()
    S.profile(False)
    out = {"only_sweep": args.only_sweep, "levels": L, "decoupled": S.level_decoupled(L - 1),
           "residual_kernel": S._lib.pm_level_variant(S._h, L - 1) % 2,
           "cells": P.desc(L - 1).n_cells, "kernel_launches_per_sweep": launches}
    for k, v in prof.items():
        out[k] = {"ms_per_sweep": v["ms"] / args.steps, "launches": v["launches"],
                  "avg_launch_ms": v["ms"] / max(v["launches"], 1),
                  "bytes_per_launch": v["bytes"] / max(v["launches"], 1),
                  "achieved_gbs": v["bytes"] / (v["ms"] * 1e-3) / 1e9 if v["ms"] else None}
    print(json.dumps(out), flush=True)
    S.close()


def only_assembly(args):
    """pm_assemble_level_device on every level of one-block FP64 levels,
    args.warmup + args.steps passes; prints the mean time of a pass."""
    import torch
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    P = OseenProblem(n_levels=args.levels, nu=args.nu, seed=args.seed, nthreads=os.cpu_count() or 1)
    S = PmSolver(P.descs_one_block() if P.is_one_block() else P.descs, precision="fp64")
    dev = [(torch.from_numpy(P.cell_sizes(l)).cuda(),
            torch.from_numpy(P.convection_nodal(l)).cuda()) for l in range(P.n_levels)]
    times = []
    for k in range(args.warmup + args.steps):
        n0 = S.kernel_launches
        t0 = time.perf_counter()
        for l, (h, c) in enumerate(dev):
            S.assemble_level_device(l, h.data_ptr(), c.data_ptr(), P.nu)
        times.append(time.perf_counter() - t0)
        launches = S.kernel_launches - n0
    times = times[args.warmup:]
    print(json.dumps({"only_assembly": True, "levels": P.n_levels,
                      "cells": sum(P.desc(l).n_cells for l in range(P.n_levels)),
                      "ms_per_pass": 1e3 * sum(times) / len(times),
                      "kernel_launches_per_pass": launches}), flush=True)


def train_network(device, args, log=None):
    """The learned smoother's network (learned.STANDARD_CONFIG: pairs
    harvested from plain FP64 solves of 32^3 problems with nu log-uniform in
    [1e-3, 1e-1], AdamW lr 1e-3, 20 epochs, all on the GPU), cached in the
    package's build folder keyed by the training configuration."""
    from to_merge_master_parmoon_gb300.learned import standard_network
    return standard_network(device, problems=args.train_problems,
                            cache_dir=ROOT / "to_merge_master_parmoon_gb300" / "_build", log=log)


def nu_study(args, device, net, threads, log=None):
    """The convection-dominated case nu = 1e-3 (mesh Peclet number |b| h /
    2 nu up to 7.8 at 64^3 on the unstabilised Galerkin form): the 64^3
    problem (6 levels, seed 2) solved from zero by FP64, mixed and mixed +
    learned, at most 200 FGMRES(20) iterations toward 1e-8, each with its
    time, iterations, final relative residual and status; and the same
    method on the oracle (the reference's algorithm on the CPU) against the
    GPU FP64 path at 16^3 (to 1e-8, at most 200 iterations) and 32^3 (40
    iterations): same iteration counts, or the same residual reached, show
    that what the GPU does at nu = 1e-3 is the method's behaviour."""
    import numpy as np
    import torch
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    nu = 1e-3
    out = {"nu": nu}
    P = OseenProblem(n_levels=args.levels, nu=nu, seed=2, nthreads=threads)
    b = P.rhs()
    r0 = pressure_projected_norm(P, b)
    d_b = torch.from_numpy(b).cuda()
    d_x = torch.zeros_like(d_b)
    for name, prec, learned in (("fp64", "fp64", False), ("mixed", "mixed", False),
                                ("mixed_learned", "mixed", True)):
        S = PmSolver(P.descs, precision=prec, device=device, restart=20, maxit=200,
                     res_norm_min=RTOL * r0, upload_mode=1)
        if learned:
            S.attach_learned(net, omega=1.0, fallback_ratio=0.5)
        f_ms = S.refactor()
        d_x.zero_()
        torch.cuda.synchronize()
        info = S.iterate_device(d_x.data_ptr(), d_b.data_ptr(), allow=(0, 1, 2, 3))
        row = {"factor_ms": f_ms, "solve_ms": info["solve_ms"], "iterations": info["iterations"],
               "rel_res": info["true_res"] / r0, "status": info["status_name"]}
        if learned:
            row["learned_status"] = S.learned_status()
        out[f"{2 ** args.levels}cube_{name}"] = row
        if log:
            log(f"nu=1e-3 {name}: {row}")
        S.close()
    del d_b, d_x
    # the oracle against the GPU FP64 path on smaller meshes
    for levels, maxit in ((4, 200), (5, 40)):
        Q = OseenProblem(n_levels=levels, nu=nu, seed=2, nthreads=threads)
        bq = Q.rhs()
        tol = RTOL * pressure_projected_norm(Q, bq)
        xo, io, t_or = oracle_solve(Q, bq, tol, threads, maxit=maxit)
        S = PmSolver(Q.descs, precision="fp64", device=device, restart=20, maxit=maxit,
                     res_norm_min=tol)
        xg, ig = S.iterate(np.zeros_like(bq), bq, allow=(0, 1, 2, 3))
        S.close()
        rq = pressure_projected_norm(Q, bq)
        out[f"{2 ** levels}cube_oracle_vs_gpu_fp64"] = {
            "maxit": maxit, "oracle_iterations": io["iterations"],
            "oracle_rel_res": io["true_res"] / rq, "oracle_s": t_or,
            "gpu_iterations": ig["iterations"], "gpu_rel_res": ig["true_res"] / rq,
            "gpu_status": ig["status_name"],
            "error_vs_oracle": split_error(xg, xo, Q.desc(levels - 1).n_udof)}
        if log:
            log(f"nu=1e-3 {2 ** levels}^3: {out[f'{2 ** levels}cube_oracle_vs_gpu_fp64']}")
    return out


def batch_run(args, device, log=None):
    """Batched independent systems of uneven size: sizes drawn uniformly from
    {8^3, 16^3, 32^3} cubes, nu log-uniform in [1e-3, 1e-1], seeds 100+s;
    every fourth system (12 of 48) tetrahedral (6 Kuhn tetrahedra per cube,
    P2+bubble/P1disc, 49-DOF Vanka blocks), the others Q2/P1disc hexahedra;
    mixed precision, FGMRES(20)+V(2,2) to 1e-8 (at most 100 iterations).
    Timed once through pm_solve_batch (host vectors, concurrent host threads,
    one stream per system) and once as the same pm_solve calls one after
    another; both after one untimed pass."""
    import numpy as np
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver, solve_batch
    rng = np.random.default_rng(2)
    probs, solvers, rhss = [], [], []
    t0 = time.perf_counter()
    for k in range(args.batch_systems):
        levels = int(rng.integers(3, 6))
        nu = float(10 ** rng.uniform(-3, -1))
        element = "tetra" if k % 4 == 3 else "hexa"
        P = OseenProblem(n_levels=levels, nu=nu, seed=100 + k, nthreads=os.cpu_count() or 1,
                         element=element)
        b = P.rhs()
        nu3 = 3 * P.desc(levels - 1).n_udof
        bp = b.copy()
        bp[nu3::4] -= bp[nu3::4].mean()
        solvers.append(PmSolver(P.descs, precision="mixed", device=device, restart=20, maxit=100,
                                res_norm_min=RTOL * float(np.linalg.norm(bp))))
        probs.append(P)
        rhss.append(b)
    build_s = time.perf_counter() - t0
    zeros = [np.zeros_like(b) for b in rhss]
    solve_batch(solvers, zeros, rhss, allow=(0, 1, 2, 3))  # untimed pass
    t = time.perf_counter()
    _, infos = solve_batch(solvers, zeros, rhss, allow=(0, 1, 2, 3))
    t_batch = time.perf_counter() - t
    t = time.perf_counter()
    for S, b in zip(solvers, rhss):
        S.iterate(np.zeros_like(b), b, allow=(0, 1, 2, 3))
    t_seq = time.perf_counter() - t
    conv = sum(1 for i in infos if i["status"] == 0)
    dofs = sum(P.ndof(-1) for P in probs)
    if log:
        log(f"batch: {len(solvers)} systems, {conv} converged, batch {t_batch:.3f} s, "
            f"one after another {t_seq:.3f} s")
    xs_batch = solve_batch(solvers, zeros, rhss, allow=(0, 1, 2, 3))[0]
    for S in solvers:
        S.close()
    solvers = []
    fused = fused_batch_run(probs, rhss, xs_batch, infos, device, log)
    tet = [P.element == "tetra" for P in probs]
    out = {"systems": len(probs), "tetrahedral_systems": sum(tet),
           "converged_to_1e-8": conv, "total_dof": dofs,
           "tetrahedral_dof": sum(P.ndof(-1) for P, t in zip(probs, tet) if t),
           "cells": sorted({P.desc(P.n_levels - 1).n_cells for P in probs}),
           "iterations": [i["iterations"] for i in infos],
           "iterations_tetrahedral": [i["iterations"] for i, t in zip(infos, tet) if t],
           "batch_s": t_batch, "sequential_s": t_seq, "speedup": t_seq / t_batch,
           "build_s": build_s, "fused": fused}
    return out


def fused_batch_run(probs, rhss, xs_ref, infos_ref, device, log=None):
    """The same systems as fused groups: systems of one mesh (same element
    and size) stacked into one PmFusedSolver each, every kernel one launch
    over the group; the groups run concurrently (one host thread and stream
    each).  Timed after one untimed pass; per system the iterations and the
    relative L2 difference to the pm_solve_batch solution (L2_0-normalised
    pressure)."""
    import numpy as np
    from to_merge_master_parmoon_gb300 import PmFusedSolver, solve_fused_groups
    keys = sorted({(P.element, P.n_levels) for P in probs})
    members = {k: [i for i, P in enumerate(probs) if (P.element, P.n_levels) == k] for k in keys}
    t0 = time.perf_counter()
    groups = []
    for k in keys:
        idx = members[k]
        # each system to 1e-8 of its own initial residual (x0 = 0: the same
        # test as res_norm_min = 1e-8 ||b|| of the single-system solves)
        groups.append(PmFusedSolver([probs[i].descs for i in idx], precision="mixed",
                                    device=device, restart=20, maxit=100, res_norm_min=0.0,
                                    red_factor=RTOL, red_initial=1))
    setup_s = time.perf_counter() - t0
    zs = [[np.zeros_like(rhss[i]) for i in members[k]] for k in keys]
    bs = [[rhss[i] for i in members[k]] for k in keys]
    solve_fused_groups(groups, zs, bs, allow=(0, 1, 2, 3))  # untimed pass
    t = time.perf_counter()
    xs, infos = solve_fused_groups(groups, zs, bs, allow=(0, 1, 2, 3))
    t_fused = time.perf_counter() - t
    per_group = []
    diffs = [0.0] * len(probs)
    its = [0] * len(probs)
    for g, k in enumerate(keys):
        t = time.perf_counter()
        groups[g].solve(zs[g], bs[g], allow=(0, 1, 2, 3))
        t_alone = time.perf_counter() - t
        for q, i in enumerate(members[k]):
            P = probs[i]
            nu3 = 3 * P.desc(P.n_levels - 1).n_udof
            a, r = xs[g][q].copy(), xs_ref[i].copy()
            a[nu3::4] -= a[nu3::4].mean()
            r[nu3::4] -= r[nu3::4].mean()
            diffs[i] = float(np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-300))
            its[i] = infos[g][q]["iterations"]
        per_group.append({"element": k[0], "cells": probs[members[k][0]].desc(k[1] - 1).n_cells,
                          "systems": len(members[k]), "solve_s": t_alone,
                          "max_iterations": max(infos[g][q]["iterations"]
                                                for q in range(len(members[k]))),
                          "kernel_launches": groups[g].kernel_launches,
                          # kernels the tuner chose per smoothed level of the
                          # stacked hierarchy (pm_level_variant: residual
                          # kernel + 2 * apply kernel)
                          "level_variants": [groups[g]._lib.pm_level_variant(groups[g]._h, lv)
                                             for lv in range(1, k[1])]})
    conv = sum(1 for grp in infos for i in grp if i["status"] == 0)
    if log:
        log(f"fused batch: {len(keys)} groups, {conv} converged, {t_fused:.3f} s "
            f"(groups concurrently), set-up {setup_s:.2f} s")
    for G in groups:
        G.close()
    return {"groups": per_group, "fused_s": t_fused, "setup_s": setup_s,
            "converged_to_1e-8": conv, "iterations": its,
            "max_rel_diff_vs_batch_converged": max(
                (d for d, i in zip(diffs, infos_ref) if i["status"] == 0), default=None),
            "rel_diff_vs_batch": diffs}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.only_assembly:
        only_assembly(args)
        return
    if args.only_batch:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"only_batch": batch_run(args, 0, log=lambda *a: print(*a, file=sys.stderr))}),
              flush=True)
        return
    if args.only_factor:
        only_factor(args)
        return
    if args.only_sweep:
        only_sweep(args)
        return
    if args.only_channel:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"only_channel": channel_run(args, os.cpu_count() or 1, None)}),
              flush=True)
        return
    if args.only_mlp > 0:
        only_mlp(args)
        return
    rank, world, local = dist_env()
    import numpy as np
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    from to_merge_master_parmoon_gb300.solver import PmError

    threads = os.cpu_count() or 1
    P = OseenProblem(n_levels=args.levels, nu=args.nu, seed=args.seed + rank, nthreads=threads)
    b = P.rhs()
    n = P.ndof(-1)
    d_b = torch.from_numpy(b).cuda()
    d_x = torch.zeros(n, dtype=torch.float64, device="cuda")

    r0 = pressure_projected_norm(P, b)
    # learned smoother: trained once (harvest on 32^3 problems, GPU training),
    # outside the timed region; cached by configuration in the build folder
    net, learned_info = train_network(local, args, log=lambda *a: print(*a, file=sys.stderr))
    # matrix values move by SM loads of the caller's (pageable) arrays where
    # the GPU can read host memory (Grace-coupled), else by copy-engine
    # copies.  The arrays are not page-locked: on the GB300 machine copies from
    # cudaHostRegister'ed memory fell to 5-10 GB/s after sustained GPU load
    # while pageable memory kept 175-190 GB/s.
    def make(descs, prec, **extra):
        kw = dict(precision=prec, device=local, restart=20, maxit=200, res_norm_min=RTOL * r0,
                  **extra)
        try:
            return PmSolver(descs, upload_mode=1, **kw)
        except PmError:
            return PmSolver(descs, upload_mode=0, **kw)

    solvers, setup_s = {}, {}
    # the Galerkin levels have A12..A32 = 0: by default they run decoupled
    # (A11, A22, A33 only, block-elimination cell solve); the *_lu variants
    # keep the reference's 85x85 LU and all nine blocks (decouple=0)
    for name, prec, extra in (("mixed_learned", "mixed", {}), ("mixed", "mixed", {}),
                              ("fp64", "fp64", {}), ("mixed_lu", "mixed", {"decouple": 0}),
                              ("fp64_lu", "fp64", {"decouple": 0})):
        # set-up: upload, colouring, transfers, local factorisation, coarse LU
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solvers[name] = make(P.descs, prec, **extra)
        setup_s[name] = time.perf_counter() - t0
    solvers["mixed_learned"].attach_learned(net, omega=1.0, fallback_ratio=0.5)
    # how the finest level runs per variant: 0 nine blocks + 85x85 LU, 1
    # three diagonal blocks, 2 one block (A11 = A22 = A33)
    modes = {k: S.level_decoupled(args.levels - 1) for k, S in solvers.items()}
    res_variants = {k: S._lib.pm_level_variant(S._h, args.levels - 1) % 2
                    for k, S in solvers.items()}
    # the same system as NSTYPE-2 levels (one velocity block; the Galerkin
    # Oseen form has A12..A32 = 0 and A11 = A22 = A33), smoothed by the exact
    # block solve of the cell systems: reported beside the headline
    one_block = P.is_one_block()
    D1 = P.descs_one_block() if one_block else None
    if one_block:
        for name, prec in (("mixed_one_block", "mixed"), ("fp64_one_block", "fp64")):
            solvers[name] = make(D1, prec)

    def step(S):
        d_x.zero_()
        torch.cuda.synchronize()
        fms = S.refactor()
        info = S.iterate_device(d_x.data_ptr(), d_b.data_ptr())
        return fms, info

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    results, solutions = {}, {}
    for prec, S in solvers.items():
        for _ in range(args.warmup):
            step(S)
        barrier()
        profile = True
        if profile:
            S.profile(True)
        launches0 = S.kernel_launches
        t_dev = []
        iters = []
        with Clocks(local) as clk:
            # NVTX range "timed_<variant>": lets a profiler select the timed steps
            torch.cuda.nvtx.range_push(f"timed_{prec}")
            t0 = time.perf_counter()
            for _ in range(args.steps):
                fms, info = step(S)
                t_dev.append(fms + info["solve_ms"])
                iters.append(info["iterations"])
            barrier()
            wall = time.perf_counter() - t0
            torch.cuda.nvtx.range_pop()
        solutions[prec] = d_x.cpu().numpy()
        results[prec] = {
            "ms": sum(t_dev) / len(t_dev), "wall_ms": wall * 1e3 / args.steps,
            "factor_ms": fms, "solve_ms": info["solve_ms"], "iterations": iters[-1],
            "rel_res": info["true_res"] / info["res0"], "launches": S.kernel_launches - launches0,
            "clocks": clk.summary(),
            # each FGMRES iteration applies one V-cycle
            "vcycles_per_s": iters[-1] / (info["solve_ms"] * 1e-3),
            "dof_iterations_per_s": n * iters[-1] / (info["solve_ms"] * 1e-3),
            "setup_s": setup_s.get(prec),
        }
        if profile:
            results[prec]["profile"] = S.profile_read()
            S.profile(False)
        if prec == "mixed_learned":
            results[prec]["learned"] = S.learned_status()
        # variants the later legs do not use give their device memory back
        if prec in ("fp64", "fp64_lu", "mixed_lu", "fp64_one_block"):
            S.close()

    # reduce: max over ranks
    ms = max_over_ranks(results["mixed_learned"]["ms"], world)

    # end to end through the C ABI with host buffers: every step uploads the
    # level matrices (pm_update_matrices, which refactors) and solves from
    # host vectors (pm_solve copies b in and x out)
    def e2e_run(S, descs, nblk):
        x = np.zeros(n)
        h2d = 0
        for lv in range(P.n_levels):
            d = P.desc(lv)
            h2d += 8 * (nblk * d.a_nnz + 3 * d.b_nnz + 3 * d.bt_nnz)
        h2d += 16 * n
        times, t_upd = [], []
        for s in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            S.update_matrices(descs)
            t1 = time.perf_counter()
            xs, info = S.iterate(x, b)
            times.append(time.perf_counter() - t)
            t_upd.append(t1 - t)
        times, t_upd = times[args.warmup:], t_upd[args.warmup:]
        return {"value": sum(times) / len(times), "unit": "s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 8 * n,
                "update_matrices_s": sum(t_upd) / len(t_upd),
                "upload_mode": S.options.upload_mode}

    e2e = e2e1 = None
    if not args.no_e2e:
        e2e = e2e_run(solvers["mixed_learned"], P.descs, 9)
        if one_block:
            e2e1 = e2e_run(solvers["mixed_one_block"], D1, 1)

    batch = None
    if not args.no_batch and rank == 0:
        batch = batch_run(args, local, log=lambda *a: print(*a, file=sys.stderr))

    assembly = None
    if not args.no_assembly and rank == 0:
        assembly = assembly_run(P, solvers["mixed"], args, threads,
                                solvers.get("mixed_one_block"))

    channel = None
    if not args.no_channel and rank == 0:
        channel = channel_run(args, threads, net)

    low_nu = None
    if not args.no_nu_study and rank == 0:
        low_nu = nu_study(args, local, net, threads, log=lambda *a: print(*a, file=sys.stderr))

    if rank != 0:
        return
    cpu = cpu16 = None
    errors = {}
    if not args.no_cpu_baseline:
        # the oracle's complete solve at the full size: the CPU baseline's
        # time to tolerance and the answer every GPU variant is checked against
        xo, io, t_or = oracle_solve(P, b, RTOL * r0, threads)
        cpu = {"value": t_or, "unit": "s", "cores": threads, "kind": "port",
               "sample": f"oracle FGMRES(20)+V(2,2) solve to 1e-8 at the full size, timed once "
                         f"({io['iterations']} iterations, colour-parallel cell Vanka refactoring "
                         f"every local block in every sweep)",
               "iterations": io["iterations"], "rel_res": io["true_res"] / io["res0"]}
        nu_f = P.desc(args.levels - 1).n_udof
        errors = {k: split_error(x, xo, nu_f) for k, x in solutions.items()}
        del xo
        cpu16 = cpu_runs_16cube(threads, local)
    peak, peak_kind = measured_peaks()
    prof = results["mixed"].get("profile", {})

    def kernel_roof(d):
        if not d or not d.get("ms"):
            return None, None, None
        return (d["bytes"] / (d["ms"] * 1e-3) / 1e9, d["ms"] / d["launches"],
                d["bytes"] / d["launches"])

    achieved, avg_ms, per_launch = kernel_roof(prof.get("residual"))
    a_ach, a_ms, a_bytes = kernel_roof(prof.get("apply"))
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "traffic": ncu_traffic(P),
            "kernel": residual_kernel_name(modes["mixed"], res_variants["mixed"]),
            "peak_kind": peak_kind, "avg_launch_ms": avg_ms, "bytes_per_launch": per_launch,
            "apply_kernel": {"name": APPLY_KERNEL[modes["mixed"]],
                             "achieved": a_ach, "frac": (a_ach / peak) if a_ach else None,
                             "avg_launch_ms": a_ms, "bytes_per_launch": a_bytes}}
    def whole_solve(name, s_val):
        r = results[name]
        nb = solve_bytes(P, s_val, r["iterations"], mode=modes[name])
        gbs = nb / (r["solve_ms"] * 1e-3) / 1e9
        return {"algorithmic_gb": nb / 1e9, "achieved_gbs": gbs, "frac": gbs / peak,
                "note": "unique bytes of the whole FGMRES solve (V-cycles, FP64 mat-vecs, "
                        "Gram-Schmidt) / solve time; peak = measured HBM copy bandwidth"}

    # FP64 pipe: the measured FMA rate of this GPU (a kernel of the library)
    # against the FP64 residual kernel and the factorisation
    fp64_roof = None
    import ctypes as C
    from to_merge_master_parmoon_gb300._lib import gpu_lib
    rate = C.c_double()
    if gpu_lib().pm_measure_fp64_fma(local, C.byref(rate)) == 0 and rate.value > 0:
        r64 = results["fp64"]
        pr = r64.get("profile", {}).get("residual")
        sweeps = r64["iterations"] * 4
        fma = residual_fma(P, 3)
        res = None
        if pr and pr["ms"]:
            t = pr["ms"] * 1e-3 / args.steps
            fl = 2.0 * sum(fma.values()) * sweeps
            by = pr["bytes"] / args.steps
            res = {"flop_per_solve": fl, "achieved_tflops": fl / t / 1e12,
                   "fp64_frac": fl / t / rate.value, "hbm_frac": by / t / 1e9 / peak,
                   "flop_per_algorithmic_byte": fl / by,
                   "balance_flop_per_byte": rate.value / (peak * 1e9)}
            res["bound"] = "fp64" if res["fp64_frac"] > res["hbm_frac"] else "hbm"
        cells = sum(P.desc(l).n_cells for l in range(1, P.n_levels))
        fac_fl = 2.0 * SCHUR_FMA_PER_CELL.get(modes["fp64"], 0) * cells
        fp64_roof = {"fp64_rate_tflops": rate.value / 1e12,
                     "how": "pm_measure_fp64_fma: 8 independent FMA chains per thread, 16 CTAs "
                            "of 256 threads per SM, CUDA events, 2 flop per FMA",
                     "fp64_residual": res,
                     "factor": {"flop": fac_fl, "ms": r64["factor_ms"],
                                "achieved_tflops": fac_fl / (r64["factor_ms"] * 1e-3) / 1e12,
                                "fp64_frac": fac_fl / (r64["factor_ms"] * 1e-3) / rate.value,
                                "note": "block elimination of every decoupled cell, Gauss-Jordan "
                                        "FMA counted in full (zero multipliers are skipped)"}}
    whole = {"fp64": whole_solve("fp64", 8), "mixed": whole_solve("mixed", 4),
             "fp64_lu": whole_solve("fp64_lu", 8), "mixed_lu": whole_solve("mixed_lu", 4)}
    lu = {"note": "the same nine-block system with decouple=0: every cell solved by the "
                  "85x85 LU of the reference's CellVanka and all nine A blocks read"}
    for name in ("mixed_lu", "fp64_lu"):
        r = results[name]
        lu[name] = {"value": r["ms"] * 1e-3,
                    **{k: r[k] for k in ("factor_ms", "solve_ms", "iterations", "rel_res",
                                         "vcycles_per_s", "dof_iterations_per_s", "setup_s")},
                    "error_vs_oracle": errors.get(name),
                    "sweep_kernels": {
                        k: {"ms_total": v["ms"], "launches": v["launches"],
                            "achieved_gbs": kernel_roof(v)[0],
                            "frac": (kernel_roof(v)[0] / peak) if v["ms"] else None}
                        for k, v in r.get("profile", {}).items()}}
    one = None
    if one_block:
        one = {"note": "same system as NSTYPE-2 levels (a[0] only); exact block solve of the "
                       "cell systems (A^-1 + 4x4 Schur complement, 1393 stored values per cell); "
                       "byte counts of its own (1 A array, 1393 values per cell)"}
        for name in ("mixed_one_block", "fp64_one_block"):
            r = results[name]
            one[name] = {"value": r["ms"] * 1e-3,
                         **{k: r[k] for k in ("factor_ms", "solve_ms", "iterations", "rel_res")},
                         "error_vs_oracle": errors.get(name),
                         "sweep_kernels": {
                             k: {"ms_total": v["ms"], "launches": v["launches"],
                                 "achieved_gbs": kernel_roof(v)[0],
                                 "frac": (kernel_roof(v)[0] / peak) if v["ms"] else None}
                             for k, v in r.get("profile", {}).items()}}
        one["e2e"] = e2e1
    nlev = args.levels
    line = {
        "metric": METRIC, "value": ms * 1e-3, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded divergence-free Fourier convection, smooth forcing)",
        "config": {"workload": f"steady 3D Oseen, Q2/P1disc, {2 ** nlev}^3 cells, {nlev} levels "
                               f"from 2^3, nu={args.nu}, FGMRES(20)+V(2,2) cell Vanka, rtol 1e-8",
                   "ndof": n, "precision": "mixed: FP32 V-cycle + FP32 local block "
                                           "elimination, FP64 FGMRES/coarse; "
                                           "learned: BF16 MLP (tcgen05) post-smoothing step "
                                           "on the finest level",
                   "l2": "inputs (11.7 GB of matrices) larger than L2", "parallelism": "replicas"},
        "fp64": {"value": results["fp64"]["ms"] * 1e-3, "iterations": results["fp64"]["iterations"],
                 "vcycles_per_s": results["fp64"]["vcycles_per_s"],
                 "dof_iterations_per_s": results["fp64"]["dof_iterations_per_s"],
                 "setup_s": results["fp64"]["setup_s"],
                 "factor_ms": results["fp64"]["factor_ms"], "solve_ms": results["fp64"]["solve_ms"],
                 "rel_res": results["fp64"]["rel_res"],
                 "error_vs_oracle": errors.get("fp64"),
                 "sweep_kernels": {k: {"ms_total": v["ms"], "launches": v["launches"],
                                       "achieved_gbs": (v["bytes"] / (v["ms"] * 1e-3) / 1e9) if v["ms"] else None}
                                   for k, v in results["fp64"].get("profile", {}).items()}},
        "mixed": {"value": results["mixed"]["ms"] * 1e-3,
                  **{k: results["mixed"][k] for k in ("factor_ms", "solve_ms", "iterations", "rel_res",
                                                      "vcycles_per_s", "dof_iterations_per_s",
                                                      "setup_s")},
                  "error_vs_oracle": errors.get("mixed")},
        "mixed_learned": {**{k: results["mixed_learned"][k]
                             for k in ("factor_ms", "solve_ms", "iterations", "rel_res", "wall_ms",
                                       "vcycles_per_s", "dof_iterations_per_s", "setup_s")},
                          "learned_status": results["mixed_learned"].get("learned"),
                          "error_vs_oracle": errors.get("mixed_learned"),
                          "training": learned_info},
        "speedup_vs_fp64": results["fp64"]["ms"] / results["mixed_learned"]["ms"],
        "speedup_mixed_vs_fp64": results["fp64"]["ms"] / results["mixed"]["ms"],
        "roofline": roof,
        "whole_solve_roofline": whole,
        "fp64_roofline": fp64_roof,
        "nine_block_lu": lu,
        "one_block": one,
        "batch": batch,
        "assembly": assembly,
        "channel": channel,
        "nu_1e-3": low_nu,
        "cpu_baseline": cpu,
        "cpu_runs_16cube": cpu16,
        "e2e": e2e,
        "gpu_launches": results["mixed_learned"]["launches"],
        "clocks": {k: results["mixed_learned"]["clocks"][k] for k in ("sm_mhz", "sm_max_mhz", "reasons")},
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
