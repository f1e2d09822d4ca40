"""ctypes declarations of the package's two native libraries.

``libpmgpu.so`` exports the solver C ABI of include/pmgpu.h; ``libpmhost.so``
exports the host-side Oseen problem builder.  Both are built in-tree by
``to_merge_master_parmoon_gb300.build``.  Loading fails loudly when a library
is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

BUILD = Path(__file__).resolve().parent / "_build"

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)


class PmLevelDesc(C.Structure):
    _fields_ = [
        ("n_udof", C.c_int), ("n_pdof", C.c_int), ("n_active", C.c_int),
        ("hanging_bound", C.c_int), ("n_dirichlet", C.c_int),
        ("a_nnz", C.c_int), ("a_rowptr", c_int_p), ("a_col", c_int_p), ("a", c_double_p * 9),
        ("b_nnz", C.c_int), ("b_rowptr", c_int_p), ("b_col", c_int_p), ("b", c_double_p * 3),
        ("bt_nnz", C.c_int), ("bt_rowptr", c_int_p), ("bt_col", c_int_p), ("bt", c_double_p * 3),
        ("n_cells", C.c_int), ("n_ulocal", C.c_int), ("n_plocal", C.c_int),
        ("cell_udofs", c_int_p), ("cell_pdofs", c_int_p),
        ("cell_parent", c_int_p), ("cell_child", c_int_p), ("cell_colour", c_int_p),
        ("pu_nnz", C.c_int), ("pu_rowptr", c_int_p), ("pu_col", c_int_p), ("pu_val", c_double_p),
        ("pp_nnz", C.c_int), ("pp_rowptr", c_int_p), ("pp_col", c_int_p), ("pp_val", c_double_p),
    ]


class PmOptions(C.Structure):
    _fields_ = [
        ("precision", C.c_int), ("factor_fp32", C.c_int),
        ("pre_smooth", C.c_int), ("post_smooth", C.c_int),
        ("smooth_damp", C.c_double), ("alpha", C.c_double), ("beta", C.c_double),
        ("project_pressure", C.c_int),
        ("restart", C.c_int), ("maxit", C.c_int), ("minit", C.c_int),
        ("red_factor", C.c_double), ("res_norm_min", C.c_double), ("div_factor", C.c_double),
        ("device", C.c_int), ("use_graphs", C.c_int), ("verbose", C.c_int),
        ("pin_host", C.c_int), ("vanka_inverse", C.c_int), ("residual_variant", C.c_int),
        ("apply_variant", C.c_int), ("upload_mode", C.c_int), ("red_initial", C.c_int),
        ("decouple", C.c_int), ("wait_limit", C.c_int), ("max_device_bytes", C.c_longlong),
        ("learned_levels", C.c_int),
    ]


class PmResult(C.Structure):
    _fields_ = [
        ("iterations", C.c_int), ("res0", C.c_double), ("res", C.c_double),
        ("true_res", C.c_double), ("setup_ms", C.c_double), ("solve_ms", C.c_double),
        ("vcycles", C.c_int), ("status", C.c_int),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class PmhParams(C.Structure):
    _fields_ = [
        ("nx0", C.c_int), ("ny0", C.c_int), ("nz0", C.c_int), ("n_levels", C.c_int),
        ("x0", C.c_double), ("x1", C.c_double), ("y0", C.c_double), ("y1", C.c_double),
        ("z0", C.c_double), ("z1", C.c_double), ("nu", C.c_double), ("seed", C.c_uint64),
        ("example", C.c_int), ("n_modes", C.c_int), ("nthreads", C.c_int),
        ("periodic", C.c_int), ("stretch_y", C.c_double), ("perturb", C.c_double),
        ("element", C.c_int),
    ]


PM_STATUS = {0: "PM_OK", 1: "PM_MAXIT", 2: "PM_DIVERGED", 3: "PM_NAN", 4: "PM_TIMEOUT",
             5: "PM_OOM", 6: "PM_BADARG", 7: "PM_CUDA_ERROR", 8: "PM_NOT_SETUP",
             9: "PM_NO_DEVICE"}

# every symbol include/pmgpu.h declares, with (restype, argtypes)
_P = C.c_void_p
GPU_SYMBOLS = {
    "pm_default_options": (None, [C.POINTER(PmOptions)]),
    "pm_status_string": (C.c_char_p, [C.c_int]),
    "pm_last_error": (C.c_char_p, [_P]),
    "pm_device_count": (C.c_int, []),
    "pm_create": (C.c_int, [C.POINTER(_P), C.POINTER(PmOptions)]),
    "pm_add_level": (C.c_int, [_P, C.POINTER(PmLevelDesc)]),
    "pm_setup": (C.c_int, [_P]),
    "pm_update_matrices": (C.c_int, [_P, C.POINTER(PmLevelDesc), C.c_int]),
    "pm_destroy": (C.c_int, [_P]),
    "pm_n_levels": (C.c_int, [_P]),
    "pm_level_ndof": (C.c_int, [_P, C.c_int]),
    "pm_level_blocks": (C.c_int, [_P, C.c_int]),
    "pm_level_decoupled": (C.c_int, [_P, C.c_int]),
    "pm_set_tolerances": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                    C.c_double]),
    "pm_measure_fp64_fma": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    "pm_level_variant": (C.c_int, [_P, C.c_int]),
    "pm_coupled_defect": (C.c_int, [_P, C.c_int, c_double_p, c_double_p, c_double_p, C.c_int]),
    "pm_defect": (C.c_int, [_P, C.c_int, c_double_p, c_double_p, c_double_p, c_double_p]),
    "pm_matvec": (C.c_int, [_P, C.c_int, c_double_p, c_double_p]),
    "pm_cell_vanka": (C.c_int, [_P, C.c_int, c_double_p, c_double_p, C.c_int]),
    "pm_restrict": (C.c_int, [_P, C.c_int, c_double_p, c_double_p]),
    "pm_prolongate": (C.c_int, [_P, C.c_int, c_double_p, c_double_p]),
    "pm_solve_exact": (C.c_int, [_P, c_double_p, c_double_p]),
    "pm_vcycle": (C.c_int, [_P, c_double_p, c_double_p]),
    "pm_solve": (C.c_int, [_P, c_double_p, c_double_p, C.POINTER(PmResult)]),
    "pm_solve_device": (C.c_int, [_P, C.c_void_p, C.c_void_p, C.POINTER(PmResult)]),
    "pm_assemble_level": (C.c_int, [_P, C.c_int, c_double_p, c_double_p, C.c_double]),
    "pm_assemble_level_device": (C.c_int, [_P, C.c_int, C.c_void_p, C.c_void_p, C.c_double]),
    "pm_assemble_system_level": (C.c_int, [_P, C.c_int, c_double_p, c_double_p, C.c_double,
                                           C.c_double, C.c_double, C.c_double, C.c_double]),
    "pm_assemble_system_level_device": (C.c_int, [_P, C.c_int, C.c_void_p, C.c_void_p, C.c_double,
                                                  C.c_double, C.c_double, C.c_double,
                                                  C.c_double]),
    "pm_system_rhs": (C.c_int, [_P, c_double_p, c_double_p, c_double_p, C.c_double, C.c_double,
                                C.c_double, c_double_p]),
    "pm_system_rhs_device": (C.c_int, [_P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                       C.c_double, C.c_double, C.c_void_p]),
    "pm_interpolate_coarse": (C.c_int, [_P, C.c_int, C.c_void_p, C.c_void_p]),
    "pm_solve_batch": (C.c_int, [C.POINTER(_P), C.c_int, C.POINTER(c_double_p),
                                 C.POINTER(c_double_p), C.POINTER(PmResult), C.c_int]),
    "pm_add_level_batch": (C.c_int, [_P, C.POINTER(PmLevelDesc), C.c_int]),
    "pm_solve_fused": (C.c_int, [_P, C.POINTER(c_double_p), C.POINTER(c_double_p),
                                 C.POINTER(PmResult)]),
    "pm_n_systems": (C.c_int, [_P]),
    "pm_refactor": (C.c_int, [_P, c_double_p]),
    "pm_kernel_launches": (C.c_longlong, [_P]),
    "pm_device_bytes": (C.c_longlong, [_P]),
    "pm_pinned_bytes": (C.c_longlong, [_P]),
    "pm_profile_enable": (C.c_int, [_P, C.c_int]),
    "pm_profile_read": (C.c_int, [_P, C.c_int, c_double_p, C.POINTER(C.c_longlong), c_double_p]),
    "pm_l20_project_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "pm_mlp_create": (C.c_int, [C.POINTER(_P), C.c_int, C.c_ulonglong, C.c_int]),
    "pm_mlp_destroy": (C.c_int, [_P]),
    "pm_mlp_num_params": (C.c_longlong, []),
    "pm_mlp_get_params": (C.c_int, [_P, C.POINTER(C.c_float), C.c_longlong]),
    "pm_mlp_set_params": (C.c_int, [_P, C.POINTER(C.c_float), C.c_longlong]),
    "pm_mlp_forward": (C.c_int, [_P, C.c_void_p, C.c_int, C.c_void_p]),
    "pm_mlp_set_tensor_path": (C.c_int, [_P, C.c_int]),
    "pm_mlp_loss_grad": (C.c_int, [_P, C.c_void_p, C.c_void_p, C.c_int, c_double_p,
                                   C.POINTER(C.c_float)]),
    "pm_mlp_adamw_step": (C.c_int, [_P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float]),
    "pm_learned_attach": (C.c_int, [_P, _P, C.c_double, C.c_double]),
    "pm_learned_harvest": (C.c_int, [_P, c_double_p, c_double_p, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_longlong, C.POINTER(C.c_longlong)]),
    "pm_learned_status": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
}

HOST_SYMBOLS = {
    "pmh_default_params": (None, [C.POINTER(PmhParams)]),
    "pmh_build": (C.c_void_p, [C.POINTER(PmhParams)]),
    "pmh_free": (None, [C.c_void_p]),
    "pmh_n_levels": (C.c_int, [C.c_void_p]),
    "pmh_ndof": (C.c_int, [C.c_void_p, C.c_int]),
    "pmh_level_desc": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(PmLevelDesc)]),
    "pmh_rhs": (c_double_p, [C.c_void_p]),
    "pmh_exact": (c_double_p, [C.c_void_p]),
    "pmh_q2_basis": (None, [C.c_double, C.c_double, C.c_double, c_double_p, c_double_p]),
    "pmh_b2_basis": (None, [C.c_double, C.c_double, C.c_double, c_double_p, c_double_p]),
    "pmh_p1t_basis": (None, [C.c_double, C.c_double, C.c_double, c_double_p, c_double_p]),
    "pmh_max_convection": (C.c_double, [C.c_void_p]),
    "pmh_cell_sizes": (C.c_int, [C.c_void_p, C.c_int, c_double_p]),
    "pmh_convection_nodal": (C.c_int, [C.c_void_p, C.c_int, c_double_p]),
    "pmh_reassemble": (C.c_int, [C.c_void_p]),
}

_cache: dict[str, C.CDLL] = {}


def _load(name: str, symbols: dict) -> C.CDLL:
    if name in _cache:
        return _cache[name]
    path = BUILD / name
    if not path.exists():
        raise RuntimeError(
            f"{path} is missing: build the native library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(path))
    for sym, (res, args) in symbols.items():
        fn = getattr(lib, sym)
        fn.restype = res
        fn.argtypes = args
    _cache[name] = lib
    return lib


def gpu_lib() -> C.CDLL:
    return _load("libpmgpu.so", GPU_SYMBOLS)


def host_lib() -> C.CDLL:
    return _load("libpmhost.so", HOST_SYMBOLS)
