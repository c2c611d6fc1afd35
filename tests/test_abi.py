"""The C-ABI libraries load and export every function their headers declare."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

from wavey_gb300 import _native

ROOT = Path(__file__).resolve().parents[1]


def declared(header: str):
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b((?:wavey_cuda|wh)_[a-z0-9_]+)\s*\(", text)))


@pytest.mark.parametrize("header,lib", [("wavey_cuda.h", "libwavey_cuda.so"), ("wavey_host.h", "libwavey_host.so")])
def test_every_declared_symbol_is_exported(header, lib):
    names = declared(header)
    assert len(names) > 5
    so = ctypes.CDLL(str(ROOT / "wavey_gb300" / "_lib" / lib))
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, f"{lib} lacks {missing}"


def test_bindings_cover_the_headers():
    """Every declared function has a ctypes signature in _native."""
    assert set(declared("wavey_host.h")) <= set(_native.host().__dict__) | {
        n for n in declared("wavey_host.h") if getattr(_native.host(), n).argtypes is not None}
    for n in declared("wavey_cuda.h"):
        assert getattr(_native.cuda(), n).argtypes is not None, n


def test_no_device_is_an_error_not_a_crash():
    """Without a usable device, creating a context returns an error code
    (there is no CPU fallback)."""
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a device is present")
    except ImportError:
        pass
    h = ctypes.c_void_p()
    st = _native.cuda().wavey_cuda_create(0, ctypes.byref(h))
    assert st == _native.WAVEY_E_CUDA
    assert not h.value


def test_backend_refuses_without_device():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a device is present")
    except ImportError:
        pass
    from wavey_gb300.backend import CudaBackend, WaveyError

    with pytest.raises(WaveyError):
        CudaBackend(0)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_native, "_LIB", tmp_path)
    monkeypatch.setattr(_native, "_cuda", None)
    with pytest.raises(RuntimeError, match="missing"):
        _native.cuda()
