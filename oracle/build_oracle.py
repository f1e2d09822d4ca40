"""Build recipe of the oracle (test infrastructure only).

* ``oracle/_build/liboracle.so`` — the FP64 CPU restatement (oracle.cpp).
* ``oracle/_ref/ref_basis_pin``  — the reference's own basis-function headers
  compiled where they lie under the reference tree (only when that tree is
  present; its output is committed as tests/golden/basis_q2_p1.json).
* ``oracle/_ref/libref_harness.so`` — the reference's coupled-system kernels,
  its flexible FGMRES and its cell Vanka (the translation units of
  REF_HARNESS_TUS below) compiled where they lie, driven by ref_harness.cpp
  and ref_vanka.cpp (only when the tree is present; the defect outputs are
  committed as tests/golden/ref_defect_*.npz).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
what this builds.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE = Path(os.environ.get("PM_REFERENCE_TREE", "/root/reference"))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)


def build_oracle() -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    out = BUILD / "liboracle.so"
    srcs = [HERE / "oracle.cpp"]
    deps = srcs + [HERE / "oracle.h", ROOT / "include" / "pmgpu.h", Path(__file__)]
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return out
    _run(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared",
          f"-I{ROOT / 'include'}",
          f"-I{HERE}", *map(str, srcs), "-o", str(out)])
    return out


def build_ref_pin() -> Path | None:
    hdr = REFERENCE / "include" / "FE3D"
    if not (hdr / "BF_C_H_Q2_3D.h").exists():
        return None
    REF_OUT.mkdir(parents=True, exist_ok=True)
    out = REF_OUT / "ref_basis_pin"
    _run(["g++", "-O0", "-std=c++17", f"-I{hdr}", str(HERE / "ref_basis_pin.cpp"), "-o", str(out)])
    return out


# reference translation units of the harness, compiled where they lie
REF_HARNESS_TUS = ("FE/MGComponents3D", "FE/FgmresIte", "FE/ItMethod", "FE/Matrix",
                   "FE/SquareMatrix", "FE/Structure", "FE/SquareStructure", "FE/Blas1",
                   "FE/NSE_MGLevel4", "FE/NSE_MGLevel", "FE/LinAlg", "FE/FESpace",
                   "FE/FESpace3D", "FE/FE3D", "FE/Structure3D", "FE/SquareStructure3D",
                   "FE/SquareMatrix3D", "FE/Matrix3D", "Geometry/Collection")
REF_INCLUDE_DIRS = ("General", "FE", "Geometry", "FE3D", "FE2D", "FE1D", "System",
                    "QuadFormulas", "Parallel", "AMG")


def build_ref_harness() -> Path | None:
    """Compile the reference's coupled defect / mat-vec code with
    ref_harness.cpp into oracle/_ref/libref_harness.so.  The reference objects
    are built with hidden symbols and function sections so that the link
    (``--gc-sections``) keeps only what the harness reaches, and ``-z defs``
    proves nothing it keeps is unresolved.  Returns None without the tree."""
    src = REFERENCE / "src"
    if not all((src / f"{t}.C").exists() for t in REF_HARNESS_TUS):
        return None
    objdir = REF_OUT / "harness_obj"
    objdir.mkdir(parents=True, exist_ok=True)
    out = REF_OUT / "libref_harness.so"
    mine = [HERE / "ref_harness.cpp", HERE / "ref_vanka.cpp", Path(__file__),
            *sorted((HERE / "ref_stubs").glob("*.h"))]
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in mine):
        return out
    # _SEQ: the reference's sequential build, whose cell Vanka the oracle restates
    inc = ["-D__3D__", "-D_SEQ", f"-I{HERE / 'ref_stubs'}"]
    inc += [f"-I{REFERENCE / 'include' / d}" for d in REF_INCLUDE_DIRS]
    # include/FE/NSE_MGLevel.h (reached from FgmresIte.C and NSE_MGLevel4.C)
    # includes the CUDA runtime headers; declarations only, nothing of them
    # is linked
    cuda_inc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
    inc += ["-isystem", str(cuda_inc)]
    flags = ["g++", "-O2", "-std=c++11", "-fPIC", "-fopenmp", "-w", "-ffp-contract=off",
             "-ffunction-sections", "-fdata-sections", "-fvisibility=hidden"]
    jobs = [(src / f"{t}.C", objdir / f"{Path(t).name}.o") for t in REF_HARNESS_TUS]
    jobs.append((HERE / "ref_harness.cpp", objdir / "ref_harness.o"))
    jobs.append((HERE / "ref_vanka.cpp", objdir / "ref_vanka.o"))
    procs = [(subprocess.Popen([*flags, *inc, "-c", str(s), "-o", str(o)], stdout=subprocess.PIPE,
                               stderr=subprocess.STDOUT, text=True), s) for s, o in jobs]
    for pr, s in procs:
        log = pr.communicate()[0]
        if pr.returncode != 0:
            raise RuntimeError(f"reference harness: compiling {s} failed:\n{log}")
    _run(["g++", "-shared", "-fopenmp", "-Wl,--gc-sections", "-Wl,-z,defs",
          *[str(o) for _, o in jobs], "-o", str(out)])
    return out


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref_pin())
    print(build_ref_harness())
