import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs on the GPU box")


def gpu_available() -> bool:
    try:
        import biwfa_gpu_pii2025_gb300 as pkg
        lib = pkg.load_library()
        ctx = lib.wfg_context_create(0)
        if ctx:
            lib.wfg_context_destroy(ctx)
            return True
    except Exception:
        return False
    return False


@pytest.fixture(scope="session")
def batch_aligner():
    import biwfa_gpu_pii2025_gb300 as pkg
    al = pkg.BatchAligner(0)
    yield al
    al.close()
