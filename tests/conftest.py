import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def native_build():
    """Build libprk_gb300.so, the driver and the oracle libraries once when they are missing (nvcc
    cross-compiles for sm_103a without a GPU)."""
    lib = ROOT / "kernels_gb300" / "_build" / "libprk_gb300.so"
    if not lib.exists():
        from kernels_gb300 import build
        build.build()
    oracle_lib = ROOT / "oracle" / "_build" / "liboracle.so"
    if not oracle_lib.exists():
        import subprocess
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "all"], check=True)


@pytest.fixture(scope="session")
def golden():
    import json
    return json.loads((ROOT / "tests" / "golden" / "stencil_golden.json").read_text())


@pytest.fixture(scope="session")
def tiny_arrays():
    import numpy as np
    with np.load(ROOT / "tests" / "golden" / "tiny_out.npz") as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import kernels_gb300 as kg
    kg._lib.load()  # fails loudly if the library was not built
    return torch
