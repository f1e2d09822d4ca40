"""CPU tests of the boundary: libpmgpu.so builds for sm_103a, loads, and
exports every entry point include/pmgpu.h declares (no compute calls)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "pmgpu.h").read_text()
    return sorted(set(re.findall(r"\b(pm_[a-z_0-9]+)\s*\(", text)))


def test_header_and_binding_agree():
    from to_merge_master_parmoon_gb300._lib import GPU_SYMBOLS
    assert declared_symbols() == sorted(GPU_SYMBOLS)


def test_library_exports_every_declared_symbol():
    from to_merge_master_parmoon_gb300._lib import gpu_lib
    lib = gpu_lib()
    for sym in declared_symbols():
        assert hasattr(lib, sym), sym


def test_library_is_built_for_sm_103a():
    import subprocess
    so = ROOT / "to_merge_master_parmoon_gb300" / "_build" / "libpmgpu.so"
    assert so.exists()
    out = subprocess.run(["cuobjdump", "--list-elf", str(so)], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    assert "sm_103a" in out.stdout


def test_options_defaults_mirror_reference_database():
    """Defaults of pm_default_options are the TDatabase::ParamDB defaults
    (src/General/Database.C:640-871) that the path uses."""
    from to_merge_master_parmoon_gb300._lib import PmOptions, gpu_lib
    o = PmOptions()
    gpu_lib().pm_default_options(C.byref(o))
    assert (o.pre_smooth, o.post_smooth) == (2, 2)
    assert o.smooth_damp == 1.0 and o.beta == 1.0 and o.alpha == 1.0
    assert o.red_factor == 0.0 and o.res_norm_min == 1e-10 and o.div_factor == 1e10
    assert o.project_pressure == 1
    # not a database entry: mixed precision eliminates decoupled cells in
    # FP32 and factors coupled ones (85x85 LU) in FP64
    assert o.factor_fp32 == -1


def test_no_device_is_reported_not_faked(monkeypatch):
    """Without a GPU the library refuses to create a handle (no CPU fallback)."""
    from to_merge_master_parmoon_gb300._lib import gpu_lib
    lib = gpu_lib()
    if lib.pm_device_count() > 0:
        pytest.skip("a GPU is present")
    from to_merge_master_parmoon_gb300 import PmError, PmSolver
    with pytest.raises(PmError) as e:
        PmSolver()
    assert e.value.status == 9  # PM_NO_DEVICE


@pytest.mark.parametrize("opts,status", [
    (dict(factor_fp32=2), 6),                        # PM_BADARG: not -1, 0 or 1
    (dict(precision="fp64", factor_fp32=1), 6),      # PM_BADARG: FP32 factors need mixed
    (dict(precision="fp64", factor_fp32=-1), 9),     # the default: valid in both precisions
    (dict(precision="mixed", factor_fp32=0), 9),
])
def test_factor_precision_option_is_validated_before_the_device(opts, status):
    """pm_create checks factor_fp32 (-1 default: FP32 block elimination and
    FP64 85x85 LU in mixed precision; 0 all FP64; 1 all FP32, mixed only)
    before it looks for a device, so on a host without a GPU a valid
    setting reports PM_NO_DEVICE and an invalid one PM_BADARG."""
    from to_merge_master_parmoon_gb300._lib import gpu_lib
    if gpu_lib().pm_device_count() > 0:
        pytest.skip("a GPU is present")
    from to_merge_master_parmoon_gb300 import PmError, PmSolver
    with pytest.raises(PmError) as e:
        PmSolver(**opts)
    assert e.value.status == status
