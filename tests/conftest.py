import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the native libraries once per session (no-op when up to date)."""
    from to_merge_master_parmoon_gb300 import build as pkg_build
    from oracle import build_oracle
    pkg_build.build_host()
    build_oracle.build_oracle()
    if os.environ.get("PM_SKIP_GPU_BUILD") != "1":
        try:
            pkg_build.build_gpu()
        except RuntimeError as e:  # nvcc missing: GPU tests will fail loudly
            print("libpmgpu build failed:", e)
    yield


@pytest.fixture(scope="session")
def problems():
    """Seeded problems shared across tests (kept alive for the oracle views)."""
    from to_merge_master_parmoon_gb300 import OseenProblem
    cache = {}

    def get(n_levels=3, nu=1e-2, seed=0, example="random"):
        key = (n_levels, nu, seed, example)
        if key not in cache:
            cache[key] = OseenProblem(n_levels=n_levels, nu=nu, seed=seed, example=example)
        return cache[key]

    return get
