"""The solver behind the reference's own class interface.

* CPU, where the reference tree is present: include/pmgpu_parmoon.h
  (TFgmresIteGPU, a TItMethod of include/FE/ItMethod.h:45-172 with
  TFgmresIte's constructor, include/FE/FgmresIte.h:86-97) compiles against
  the reference's headers and matrix classes (oracle/ref_facade.cpp) and
  links with libpmgpu.so.  Its descriptor filler turns the reference's
  TSquareMatrix / TMatrix objects and the spaces' GlobalNumbers /
  BeginIndex into the exact level descriptors of pmgpu.h, and
  Iterate(A, B, sol, rhs) through a TItMethod pointer reaches pm_solve:
  without a GPU it returns -1 with PM_NO_DEVICE (no fallback).
* GPU: the façade's core (include/pmgpu_facade.h) driven by
  tests/facade_driver.cpp solves like the oracle's FGMRES (FP64: same
  iteration count; both precisions 1e-6 after L2_0 normalisation), and a
  second Iterate after the caller changed its matrices in place uploads
  them again and solves the changed system.
"""
import ctypes as C
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PM_NO_DEVICE = 9


def test_parmoon_adapter_compiles_and_reaches_the_library(problems):
    from oracle import build_oracle
    from to_merge_master_parmoon_gb300._lib import gpu_lib
    path = build_oracle.build_ref_facade()
    if path is None:
        pytest.skip("reference tree not present: the adapter needs ParMooN's headers")
    lib = C.CDLL(str(path))
    lib.ref_facade_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                   C.c_void_p, C.c_void_p, C.c_void_p]
    P = problems(3, 1e-2, 0)
    b = P.rhs()
    x = np.zeros_like(b)
    out = (C.c_int * 3)()
    lib.ref_facade_run(C.cast(P.descs, C.c_void_p), P.n_levels, 1, 80, 1e-10 * np.linalg.norm(b),
                       x.ctypes.data, b.ctypes.data, out)
    iterations, status, mismatch = list(out)
    assert mismatch == 0  # every filled descriptor equals its level
    if gpu_lib().pm_device_count() == 0:
        assert (iterations, status) == (-1, PM_NO_DEVICE)
    else:
        assert status == 0 and iterations > 0


def _driver(tmp_path):
    from oracle import build_oracle
    from to_merge_master_parmoon_gb300 import build as pkg_build
    gpu = pkg_build.BUILD
    oracle_so = build_oracle.build_oracle()
    exe = tmp_path / "facade_driver"
    cmd = ["g++", "-O2", "-std=c++17", f"-I{ROOT / 'include'}", f"-I{pkg_build.CSRC}",
           f"-I{ROOT / 'oracle'}", str(ROOT / "tests" / "facade_driver.cpp"),
           f"-L{gpu}", "-lpmgpu", "-lpmhost", f"-L{oracle_so.parent}", "-loracle",
           f"-Wl,-rpath,{gpu}", f"-Wl,-rpath,{oracle_so.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_facade_core_solves_and_reuploads(tmp_path, precision):
    exe = _driver(tmp_path)
    r = subprocess.run([str(exe), str(precision)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    print(out)
    assert out["status"] == 0 and out["status_after_update"] == 0
    assert out["rel_res"] <= 1.05e-10
    assert out["error_vs_oracle"] <= 1e-6
    assert out["error_vs_oracle_after_update"] <= 1e-6
    assert out["error_vs_half_pressure"] <= 1e-6
    if precision == 0:
        assert out["iterations"] == out["oracle_iterations"]
        assert out["iterations_after_update"] == out["oracle_iterations_after_update"]
