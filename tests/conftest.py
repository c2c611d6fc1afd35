"""Shared fixtures.

Markers: `gpu` tests need a CUDA device and run the product path through
libwavey_cuda.so; everything else runs on the CPU (the oracle, the host
library, the C-ABI exports, host-side failure handling).
"""
from __future__ import annotations

import json
import math
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from wavey_gb300 import _build  # noqa: E402

# Speed of sound of Medium::default() (wavey-materials/src/medium.rs:22-24).
C_AIR = 331.3 * math.sqrt(1.0 + 20.0 / 273.15)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA path")
    config.addinivalue_line("markers", "slow: long CPU run")


def _has_cuda() -> bool:
    try:
        import torch  # noqa: F401

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session", autouse=True)
def native_libs():
    """Builds the host library always and the CUDA library where nvcc is."""
    return _build.build(cuda=True)


@pytest.fixture(scope="session")
def backend(native_libs):
    if not _has_cuda():
        pytest.skip("no CUDA device")
    from wavey_gb300.backend import CudaBackend

    b = CudaBackend(0)
    yield b
    b.close()


@pytest.fixture(scope="session")
def library():
    """Built-in materials used by the reference's FDTD tests
    (tests/golden/materials.json, written by tests/golden/make_materials.py)."""
    from wavey_gb300.materials import Material, Spectrum

    data = json.loads((ROOT / "tests" / "golden" / "materials.json").read_text())
    out = {}
    for mid, a in data.items():
        sp = Spectrum(float(a)) if isinstance(a, (int, float)) else Spectrum.bands(a["freqs_hz"], a["values"])
        out[mid] = Material(id=mid, absorption=sp, name=mid)
    return out
