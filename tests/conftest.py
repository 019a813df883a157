import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 host)")


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / name) as z:
        return {k: z[k] for k in z.files}


def golden_scene_names() -> list[str]:
    return sorted(p.name for p in GOLDEN.glob("scene_*.npz"))


def f32_bits(a) -> np.ndarray:
    """Bit patterns of a float32 array (distinguishes -0 from +0, keeps NaN comparable)."""
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="session")
def port():
    import oracle

    return oracle.port()


@pytest.fixture(scope="session")
def ctx():
    from pipeline_gb300 import build, native

    build.build_all()
    c = native.Context(0)
    yield c
    c.close()
