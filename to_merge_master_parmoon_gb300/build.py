"""Build the native parts of the package in-tree.

* ``_build/libpmgpu.so``  — the sm_103a solver library behind include/pmgpu.h
  (nvcc, ``-gencode arch=compute_103a,code=sm_103a``).
* ``_build/libpmhost.so`` — the host-only Oseen problem builder (g++/OpenMP).

Translation units are compiled in parallel; nothing is rebuilt when the
outputs are newer than every source.  No cmake, no -march=native: the same
recipe runs on x86_64 (cross-compiling the device code) and on aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-O3,-fopenmp", f"-I{INCLUDE}", f"-I{CSRC}"]
GXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", f"-I{INCLUDE}", f"-I{CSRC}"]

GPU_CU = ["pm_api.cu", "pm_sparse.cu", "pm_vanka.cu", "pm_vanka_schur.cu", "pm_vanka_tma.cu",
          "pm_batch.cu",
          "pm_learned.cu", "pm_mlp_tc.cu", "pm_assemble.cu",
          "pm_noalloc.cu", "pm_diag.cu"]
GPU_CPP = ["pm_setup_host.cpp"]
HOST_CPP = ["oseen_problem.cpp", "oseen_tet.cpp"]
HEADERS = [INCLUDE / "pmgpu.h", CSRC / "pm_kernels.h", CSRC / "pm_setup_host.h",
           CSRC / "oseen_problem.h", CSRC / "oseen_internal.h", CSRC / "pm_learned.h"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpmgpu.so")


def _stale(out: Path, srcs) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in list(srcs) + HEADERS)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r


def build_gpu(verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    out = BUILD / "libpmgpu.so"
    srcs = [CSRC / f for f in GPU_CU + GPU_CPP]
    if not _stale(out, srcs):
        return out
    nvcc = nvcc_path()
    jobs = []
    objs = []
    for f in GPU_CU:
        o = BUILD / (f + ".o")
        objs.append(o)
        jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(CSRC / f), "-o", str(o)])
    for f in GPU_CPP:
        o = BUILD / (f + ".o")
        objs.append(o)
        jobs.append(["g++", *GXX_FLAGS, "-c", str(CSRC / f), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr, file=sys.stderr)
    _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fopenmp", *map(str, objs), "-o", str(out),
          "-lcudart", "-lgomp"])
    return out


def build_host() -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    out = BUILD / "libpmhost.so"
    srcs = [CSRC / f for f in HOST_CPP]
    if not _stale(out, srcs):
        return out
    _run(["g++", *GXX_FLAGS, "-shared", *map(str, srcs), "-o", str(out)])
    return out


def build_all(verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        fg = ex.submit(build_gpu, verbose)
        fh = ex.submit(build_host)
        fg.result()
        fh.result()


if __name__ == "__main__":
    build_all(verbose=True)
    print("built", sorted(p.name for p in BUILD.glob("*.so")))
