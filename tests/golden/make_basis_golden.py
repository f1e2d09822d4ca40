"""Regenerate tests/golden/basis_q2_p1.json and basis_tet_b2_p1.json from the
reference's own basis function headers (include/FE3D/BF_C_H_Q2_3D.h,
BF_D_H_P1_3D.h, BF_C_T_B2_3D.h, BF_D_T_P1_3D.h), compiled where they lie by
oracle/build_oracle.py.  Needs the reference tree; the fixtures are committed
so the tests do not."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.build_oracle import build_ref_pin  # noqa: E402


def main() -> None:
    exe = build_ref_pin()
    if exe is None:
        raise SystemExit("reference tree not found; cannot regenerate the basis golden file")
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    data = json.loads(out)
    data["source"] = ("reference include/FE3D/BF_C_H_Q2_3D.h and include/FE3D/BF_D_H_P1_3D.h "
                      "compiled by oracle/ref_basis_pin.cpp")
    (Path(__file__).parent / "basis_q2_p1.json").write_text(json.dumps(data, indent=1) + "\n")
    print("wrote", len(data["points"]), "points")
    out = subprocess.run([str(exe), "tet"], capture_output=True, text=True, check=True).stdout
    data = json.loads(out)
    data["source"] = ("reference include/FE3D/BF_C_T_B2_3D.h and include/FE3D/BF_D_T_P1_3D.h "
                      "compiled by oracle/ref_basis_pin.cpp (argument tet)")
    (Path(__file__).parent / "basis_tet_b2_p1.json").write_text(json.dumps(data, indent=1) + "\n")
    print("wrote", len(data["points"]), "tetrahedron points")


if __name__ == "__main__":
    main()
