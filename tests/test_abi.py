"""C-ABI library: it builds for sm_103a, loads without a GPU, and exports
every entry point that include/gridrt.h declares."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header: str):
    text = open(os.path.join(REPO, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rtg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = _declared("gridrt.h")
    assert "rtg_scene_build" in names and "rtg_trace_nearest" in names


def test_library_exports_all_declared(gridlib):
    L = ctypes.CDLL(gridlib.lib_path())
    missing = [n for n in _declared("gridrt.h") if not hasattr(L, n)]
    assert not missing, missing


def test_binding_covers_header(gridlib):
    assert set(_declared("gridrt.h")) <= set(gridlib.EXPORTS)


def test_version_without_gpu(gridlib):
    L = gridlib.load()
    assert b"sm_103a" in L.rtg_version()


def test_scene_create_without_gpu_fails_cleanly(gridlib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except ImportError:
        pass
    L = gridlib.load()
    h = ctypes.c_void_p()
    rc = L.rtg_scene_create(0, None, ctypes.byref(h))
    assert rc != 0 and not h.value
