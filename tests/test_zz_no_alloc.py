"""pm_l20_project_noalloc: the allocation-free L2_0 pressure projection.

It exists for callers that cannot allocate device memory where they need the
projection (solvers inside an application-owned memory pool, MPI ranks with
pre-partitioned GPU memory); its reduction scratch is a file-scope device
array.  Checked through the C ABI against the projection
the existing entry point pm_coupled_defect applies, on two calls in a row,
within the FP64 tolerance of the other defect tests (1e-12 relative).

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_projection_matches_pm_coupled_defect(problems):
    import torch
    from to_merge_master_parmoon_gb300 import PmSolver
    from to_merge_master_parmoon_gb300._lib import gpu_lib

    lib = gpu_lib()
    P = problems(3, 1e-2, 0)
    S = PmSolver(P.descs, precision="fp64")
    level = 2
    nu, npp = P.desc(level).n_udof, P.desc(level).n_pdof
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream()
    for call in range(2):  # two calls in a row share the scratch array
        x = rng.standard_normal(P.ndof(level))
        b = rng.standard_normal(P.ndof(level)) + 3.0 * call
        r_plain = S.coupled_defect(level, x, b, project=False)
        r_proj = S.coupled_defect(level, x, b, project=True)  # existing entry point
        d_p = torch.from_numpy(r_plain[3 * nu:].copy()).cuda()
        st = lib.pm_l20_project_noalloc(C.c_void_p(d_p.data_ptr()), npp,
                                        C.c_void_p(stream.cuda_stream))
        assert st == 0
        torch.cuda.synchronize()
        got = d_p.cpu().numpy()
        want = r_proj[3 * nu:]
        assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
        assert abs(got[0::4].sum()) <= 1e-12 * np.abs(got[0::4]).sum()
    S.close()


def test_noalloc_projection_rejects_bad_sizes():
    import torch
    from to_merge_master_parmoon_gb300._lib import gpu_lib

    lib = gpu_lib()
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    ptr = C.c_void_p(d.data_ptr())
    assert lib.pm_l20_project_noalloc(ptr, 6, None) == 6          # not a multiple of 4
    assert lib.pm_l20_project_noalloc(ptr, 0, None) == 6
    assert lib.pm_l20_project_noalloc(ptr, 8_388_612, None) == 6  # beyond the scratch limit
    assert lib.pm_l20_project_noalloc(None, 8, None) == 6
