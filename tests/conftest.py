import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) and the built CUDA library")


def _has_gpu():
    try:
        import subprocess
        r = subprocess.run(["nvidia-smi", "-L"], capture_output=True, text=True, timeout=30)
        return r.returncode == 0 and "GPU" in r.stdout
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_ctx():
    import helios_gb300 as hx
    if not _has_gpu():
        pytest.fail("gpu test selected but no GPU is visible")
    ctx = hx.Context(0)
    yield ctx
    ctx.close()
