"""Build recipe of the oracle (test infrastructure only).

* ``oracle/_build/liboracle.so`` — the FP64 CPU restatement (oracle.cpp).
* ``oracle/_ref/ref_basis_pin``  — the reference's own basis-function headers
  compiled where they lie under the reference tree (only when that tree is
  present; its output is committed as tests/golden/basis_q2_p1.json).

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
    deps = srcs + [HERE / "oracle.h", ROOT / "include" / "pmgpu.h"]
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return out
    _run(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-shared", f"-I{ROOT / 'include'}",
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


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref_pin())
