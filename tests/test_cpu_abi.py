"""CPU-side checks of the C ABI library: it builds for sm_103a, loads without a GPU, and exports every entry point
declared in include/cssg.h; the Python front end refuses to run without a GPU (no CPU fallback)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "cssg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cssg_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from curvedspacesim_gb300 import _lib, build
    build.build()
    L = ctypes.CDLL(build.LIB_PATH)
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(_lib.EXPORTS) == names


def test_version_and_error_strings_without_gpu():
    from curvedspacesim_gb300 import _lib
    L = _lib.load()
    assert b"sm_103a" in L.cssg_version()
    assert L.cssg_mesh_create(None, 0, None, 0, 0, None) == 1  # CSSG_ERR_ARG, no device touched
    assert b"empty mesh" in L.cssg_last_error()


def test_no_cpu_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from curvedspacesim_gb300 import api
    with pytest.raises(Exception):
        api.Context(0)
