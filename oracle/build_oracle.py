"""Build recipe of the oracle (test infrastructure only).

* ``oracle/_build/liboracle.so`` — the FP64 CPU restatement (oracle.cpp).
* ``oracle/_ref/ref_basis_pin``  — the reference's own basis-function headers
  compiled where they lie under the reference tree (only when that tree is
  present; its output is committed as tests/golden/basis_q2_p1.json).
* ``oracle/_ref/libref_harness.so`` — the reference's coupled-system kernels,
  its flexible FGMRES and its cell Vanka (the translation units of
  REF_HARNESS_TUS below) compiled where they lie, driven by ref_harness.cpp
  and ref_vanka.cpp (only when the tree is present; the defect and Vanka
  outputs are committed as tests/golden/ref_defect_*.npz, ref_vanka_*.npz).
* ``oracle/_ref/libref_hybrid.so`` — the same with the reference's
  colour-parallel build of its cell Vanka (-D_HYBRID; only when the tree is
  present; its sweeps are committed as tests/golden/ref_vanka_colour_*.npz).
* ``oracle/_ref/libref_transfer.so`` — the reference's grid transfers with
  the FE and geometry databases they read, and its multigrid cycle driver
  (TMultiGridIte, TNSE_MultiGrid) over one TNSE_MGLevel4 per level
  (REF_TRANSFER_TUS), driven by ref_transfer.cpp (only when the tree is
  present; its outputs are committed as tests/golden/ref_transfer_*.npz and
  tests/golden/ref_cycle_*.npz, and with libref_harness.so's FGMRES as
  tests/golden/ref_solve_*.npz).
* ``oracle/_ref/libref_transfer_hybrid.so`` — the same in the reference's
  colour-parallel build (-D_HYBRID), whose levels smooth with the OpenMP
  colour loop of CellVanka (only when the tree is present; committed as
  tests/golden/ref_cycle_colour_*.npz and ref_solve_colour_*.npz).
* ``oracle/_ref/libref_facade.so`` — include/pmgpu_parmoon.h (the solver as a
  ParMooN TItMethod) compiled against the reference's headers and matrix
  classes in ref_facade.cpp, linked with libpmgpu.so (only when the tree is
  present).

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
                   "FE/NSE_MGLevel4", "FE/NSE_MGLevel2", "FE/NSE_MGLevel", "FE/LinAlg",
                   "FE/FESpace",
                   "FE/FESpace3D", "FE/FE3D", "FE/Structure3D", "FE/SquareStructure3D",
                   "FE/SquareMatrix3D", "FE/Matrix3D", "Geometry/Collection")
REF_INCLUDE_DIRS = ("General", "FE", "Geometry", "FE3D", "FE2D", "FE1D", "System",
                    "QuadFormulas", "Parallel", "AMG", "Refinement")


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
    mine = [HERE / "ref_harness.cpp", HERE / "ref_vanka.cpp", *_ref_deps()]
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in mine):
        return out
    jobs = [(src / f"{t}.C", objdir / f"{Path(t).name}.o") for t in REF_HARNESS_TUS]
    jobs.append((HERE / "ref_harness.cpp", objdir / "ref_harness.o"))
    jobs.append((HERE / "ref_vanka.cpp", objdir / "ref_vanka.o"))
    _compile(jobs, _ref_flags())
    _run(["g++", "-shared", "-fopenmp", "-Wl,--gc-sections", "-Wl,-z,defs",
          *[str(o) for _, o in jobs], "-o", str(out)])
    return out


def build_ref_hybrid() -> Path | None:
    """The same translation units and harness as build_ref_harness, with the
    reference's colour-parallel build (-D_HYBRID instead of -D_SEQ: the
    OpenMP colour loop of TNSE_MGLevel4::CellVanka), into
    oracle/_ref/libref_hybrid.so.  ref_hybrid_mapper.h is force-included and
    stands for the constructor's TParFEMapper3D (parMapper_P).  Returns None
    without the tree."""
    src = REFERENCE / "src"
    if not all((src / f"{t}.C").exists() for t in REF_HARNESS_TUS):
        return None
    objdir = REF_OUT / "hybrid_obj"
    objdir.mkdir(parents=True, exist_ok=True)
    out = REF_OUT / "libref_hybrid.so"
    mine = [HERE / "ref_harness.cpp", HERE / "ref_vanka.cpp", HERE / "ref_hybrid_mapper.h",
            *_ref_deps()]
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in mine):
        return out
    jobs = [(src / f"{t}.C", objdir / f"{Path(t).name}.o") for t in REF_HARNESS_TUS]
    jobs.append((HERE / "ref_harness.cpp", objdir / "ref_harness.o"))
    jobs.append((HERE / "ref_vanka.cpp", objdir / "ref_vanka.o"))
    _compile(jobs, _hybrid_flags(), extra_deps=[HERE / "ref_hybrid_mapper.h"])
    _run(["g++", "-shared", "-fopenmp", "-Wl,--gc-sections", "-Wl,-z,defs",
          *[str(o) for _, o in jobs], "-o", str(out)])
    return out


# reference translation units of the facade check: the TItMethod base and
# the matrix and structure classes the adapter reads
REF_FACADE_TUS = ("FE/ItMethod", "FE/Matrix", "FE/SquareMatrix", "FE/Structure",
                  "FE/SquareStructure", "FE/Blas1")


def build_ref_facade() -> Path | None:
    """Compile include/pmgpu_parmoon.h (the library as a ParMooN TItMethod)
    against the reference's own headers in ref_facade.cpp, with the
    reference's matrix classes, into oracle/_ref/libref_facade.so, linked
    with the package's libpmgpu.so.  Returns None without the tree or
    without libpmgpu.so."""
    src = REFERENCE / "src"
    gpu = ROOT / "to_merge_master_parmoon_gb300" / "_build" / "libpmgpu.so"
    if not gpu.exists() or not all((src / f"{t}.C").exists() for t in REF_FACADE_TUS):
        return None
    objdir = REF_OUT / "facade_obj"
    objdir.mkdir(parents=True, exist_ok=True)
    out = REF_OUT / "libref_facade.so"
    mine = [HERE / "ref_facade.cpp", ROOT / "include" / "pmgpu_parmoon.h",
            ROOT / "include" / "pmgpu_facade.h", ROOT / "include" / "pmgpu.h", gpu, *_ref_deps()]
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in mine):
        return out
    jobs = [(src / f"{t}.C", objdir / f"{Path(t).name}.o") for t in REF_FACADE_TUS]
    jobs.append((HERE / "ref_facade.cpp", objdir / "ref_facade.o"))
    flags = _ref_flags() + [f"-I{ROOT / 'include'}"]
    _compile(jobs, [f if f != "-std=c++11" else "-std=c++17" for f in flags])
    _run(["g++", "-shared", "-fopenmp", "-Wl,--gc-sections", "-Wl,-z,defs",
          *[str(o) for _, o in jobs], f"-L{gpu.parent}", "-lpmgpu",
          f"-Wl,-rpath,{gpu.parent}", "-o", str(out)])
    return out


def _ref_deps():
    """Files every reference-harness object depends on besides its source."""
    return [HERE / "ref_level_space.h", HERE / "ref_lapack.h", Path(__file__),
            *sorted((HERE / "ref_stubs").glob("*.h"))]


def _compile(jobs, cmd, extra_deps=()):
    """Compile (source, object) pairs with ``cmd``, os.cpu_count() at a time,
    skipping objects newer than their source, _ref_deps() and extra_deps."""
    from concurrent.futures import ThreadPoolExecutor

    newest_dep = max(d.stat().st_mtime for d in [*_ref_deps(), *extra_deps])

    def one(job):
        src, obj = job
        if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, newest_dep):
            return None
        r = subprocess.run([*cmd, "-c", str(src), "-o", str(obj)], capture_output=True, text=True)
        return None if r.returncode == 0 else f"compiling {src} failed:\n{r.stdout}{r.stderr}"

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as pool:
        errors = [e for e in pool.map(one, jobs) if e]
    if errors:
        raise RuntimeError("reference harness: " + errors[0])


def _ref_flags():
    """The reference's 3D sequential build (-D_SEQ: its cell Vanka is the
    sequential one the oracle restates), the stubs of oracle/ref_stubs/, and
    the reference's own include directories."""
    inc = ["-D__3D__", "-D_SEQ", f"-I{HERE / 'ref_stubs'}", f"-I{HERE}"]
    inc += [f"-I{REFERENCE / 'include' / d}" for d in REF_INCLUDE_DIRS]
    # include/FE/NSE_MGLevel.h (reached from FgmresIte.C and NSE_MGLevel4.C)
    # includes the CUDA runtime headers; declarations only, nothing of them
    # is linked
    cuda_inc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
    inc += ["-isystem", str(cuda_inc)]
    return ["g++", "-O2", "-std=c++11", "-fPIC", "-fopenmp", "-w", "-ffp-contract=off",
            "-ffunction-sections", "-fdata-sections", "-fvisibility=hidden", *inc]


# The reference translation units of the transfer harness: what the link of
# ref_transfer.cpp pulls from the reference's src/ (the TDatabase and
# TFEDatabase3D constructors register every descriptor and element, so their
# closure is wide).  Linked from a static archive, so that only needed
# members enter and the 2D twins of some 3D helpers do not collide.
REF_TRANSFER_TUS = {
    "FE": ("AuxParam3D", "BaseFunct1D", "BaseFunct2D", "BaseFunct3D", "Blas1", "ConvDiff",
          "Convolution", "FE1D", "FE2D", "FE2DMapper", "FE2DMapper1Reg", "FE3D", "FE3DMapper",
          "FE3DMapper1Reg", "FEDatabase2D", "FEDatabase3D", "FEDesc1D", "FEDesc2D", "FEDesc3D",
          "FEFunction3D", "FESpace", "FESpace3D", "HNDesc", "HangingNode", "HexaAffin",
          "HexaIsoparametric", "HexaTrilinear", "LinAlg", "LineAffin", "MGComponents3D",
          "NodalFunctional1D", "NodalFunctional2D", "NodalFunctional3D", "QuadAffin",
          "QuadBilinear", "QuadIsoparametric", "RefTrans3D", "TNSE3D_FixPo", "TetraAffin",
          "TetraIsoparametric", "TriaAffin", "TriaIsoparametric",
          # the cycle driver and what it runs: TMultiGridIte, TNSE_MultiGrid,
          # the TNSE_MGLevel4 levels and their matrix classes
          "ItMethod", "MultiGridIte", "FgmresIte", "NSE_MultiGrid", "NSE_MGLevel",
          "NSE_MGLevel4", "NSE_MGLevel5",
          "Matrix", "SquareMatrix", "Structure", "SquareStructure", "Matrix3D",
          "SquareMatrix3D", "Structure3D", "SquareStructure3D"),
    "General": ("Database", "MainUtilities", "MooNMD_Io", "Utilities", "Vector"),
    "Geometry": ("BaseCell", "BdPlane", "BoundComp", "BoundComp3D", "BoundEdge", "BoundFace", "Brick",
          "Collection", "GridCell", "Hexahedron", "InterfaceJoint3D", "It_Between", "It_EQ",
          "It_EQLevel", "It_Finest", "It_LE", "It_LELevel", "It_OCAF", "It_Search", "Joint",
          "JointCollection", "JointEqN", "Line", "Mapper", "Parallelogram", "Quadrangle",
          "Rectangle", "RefDesc", "Tetrahedron", "Triangle", "Vertex"),
    "QuadFormulas": ("QuadFormula", "QuadFormula1D", "QuadFormula2D", "QuadFormula3D", "QuadFormulaHexa",
          "QuadFormulaQuad", "QuadFormulaTetra", "QuadFormulaTria"),
    "Refinement": ("RefHexaRegDesc", "RefLineDesc", "RefNoRef", "RefQuad1Conf0Desc", "RefQuad1Conf1Desc",
          "RefQuad1Conf2Desc", "RefQuad1Conf3Desc", "RefQuad2Conf0Desc", "RefQuad2Conf1Desc",
          "RefQuad2Conf2Desc", "RefQuad2Conf3Desc", "RefQuadBis0Desc", "RefQuadBis1Desc",
          "RefQuadRegDesc", "RefQuadToTri0Desc", "RefQuadToTri1Desc", "RefTetraBis01Desc",
          "RefTetraBis02Desc", "RefTetraBis03Desc", "RefTetraBis04Desc", "RefTetraBis05Desc",
          "RefTetraBis0Desc", "RefTetraBis10Desc", "RefTetraBis12Desc", "RefTetraBis13Desc",
          "RefTetraBis14Desc", "RefTetraBis15Desc", "RefTetraBis1Desc", "RefTetraBis20Desc",
          "RefTetraBis21Desc", "RefTetraBis23Desc", "RefTetraBis24Desc", "RefTetraBis25Desc",
          "RefTetraBis2Desc", "RefTetraBis30Desc", "RefTetraBis32Desc", "RefTetraBis34Desc",
          "RefTetraBis35Desc", "RefTetraBis3Desc", "RefTetraBis40Desc", "RefTetraBis41Desc",
          "RefTetraBis43Desc", "RefTetraBis45Desc", "RefTetraBis4Desc", "RefTetraBis51Desc",
          "RefTetraBis52Desc", "RefTetraBis53Desc", "RefTetraBis54Desc", "RefTetraBis5Desc",
          "RefTetraQuad0Desc", "RefTetraQuad1Desc", "RefTetraQuad2Desc", "RefTetraQuad3Desc",
          "RefTetraReg0Desc", "RefTetraReg1Desc", "RefTetraReg2Desc", "RefTetraRegDesc",
          "RefTriBis01Desc", "RefTriBis02Desc", "RefTriBis0Desc", "RefTriBis10Desc",
          "RefTriBis12Desc", "RefTriBis1Desc", "RefTriBis20Desc", "RefTriBis21Desc",
          "RefTriBis2Desc", "RefTriRegDesc", "Refinement"),
}


def _hybrid_flags():
    """_ref_flags() for the reference's colour-parallel build: -D_HYBRID
    instead of -D_SEQ, with ref_hybrid_mapper.h standing for the
    constructor's TParFEMapper3D."""
    return [f for f in _ref_flags() if f != "-D_SEQ"] + [
        "-D_HYBRID", "-include", str(HERE / "ref_hybrid_mapper.h"),
        "-DparMapper_P=ref_hybrid_mapper()"]


def build_ref_transfer(hybrid: bool = False) -> Path | None:
    """Compile the reference's grid transfers (Prolongate, DefectRestriction,
    GetProlongationMatrix3D) and the databases they read, and its cycle
    driver, with ref_transfer.cpp, into oracle/_ref/libref_transfer.so, or
    with ``hybrid`` in the reference's colour-parallel build into
    oracle/_ref/libref_transfer_hybrid.so.  Returns None without the tree."""
    srcs = [REFERENCE / "src" / d / f"{t}.C" for d, ts in REF_TRANSFER_TUS.items() for t in ts]
    if not all(s.exists() for s in srcs):
        return None
    tag = "transfer_hybrid" if hybrid else "transfer"
    objdir = REF_OUT / f"{tag}_obj"
    objdir.mkdir(parents=True, exist_ok=True)
    out = REF_OUT / f"libref_{tag}.so"
    extra = [HERE / "ref_hybrid_mapper.h"] if hybrid else []
    mine = [HERE / "ref_transfer.cpp", *extra, *_ref_deps()]
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in mine):
        return out
    flags = _hybrid_flags() if hybrid else _ref_flags()
    jobs = [(s, objdir / f"{s.parent.name}_{s.stem}.o") for s in srcs]
    _compile(jobs, flags, extra_deps=extra)
    own = objdir / "ref_transfer.o"
    _compile([(HERE / "ref_transfer.cpp", own)], flags, extra_deps=extra)
    archive = objdir / "libref_transfer_tus.a"
    if archive.exists():
        archive.unlink()
    _run(["ar", "rcs", str(archive), *[str(o) for _, o in jobs]])
    # -Bsymbolic: the reference objects call this library's own operator new
    # (zero-filling, see ref_transfer.cpp), whatever was loaded before it
    _run(["g++", "-shared", "-fopenmp", "-Wl,--gc-sections", "-Wl,-z,defs", "-Wl,-Bsymbolic",
          str(own), str(archive), "-o", str(out)])
    return out


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref_pin())
    print(build_ref_harness())
    print(build_ref_hybrid())
    print(build_ref_transfer())
    print(build_ref_transfer(hybrid=True))
    print(build_ref_facade())
