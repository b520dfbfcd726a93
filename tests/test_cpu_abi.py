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


def test_null_handles_are_argument_errors_without_gpu():
    """Every entry point rejects a null handle with CSSG_ERR_ARG and a message naming it, before touching a device;
    destroying a null handle is a no-op (CSSG_OK)."""
    from curvedspacesim_gb300 import _lib
    L = _lib.load()
    N = None
    calls = {
        "cssg_system_step": (N, 1, 1),
        "cssg_system_step_host": (N, 1, N, N, N, N, N, N, N, N),
        "cssg_system_set_state": (N, N, N, N, N),
        "cssg_system_get_state": (N, N, N, N, N),
        "cssg_system_compute_forces": (N,),
        "cssg_system_check": (N, N, N),
        "cssg_system_set_tuning": (N, 1.0, 8, 0, 0, 0, 1, 0),
        "cssg_system_autotune": (N, 1, N),
        "cssg_system_fire": (N, N, 0, N),
        "cssg_system_stress": (N, N),
        "cssg_system_kernels_per_step": (N, N),
        "cssg_transport_batch": (N, N, 0, N, N, N, N, 0, N, N),
        "cssg_distance_batch": (N, N, 1, N, N, N, N, N, 0, 1.0, N, 1.0, N, N, N, N, N),
        "cssg_distance_batch_noalloc": (N, N, 1, N, N, N, N, N, 0, 1.0, N, 1.0, N, N, N, N, N),
        "cssg_mesh_set_boundary": (N, 1),
        "cssg_system_create": (N, N, 0, N, N),
        "cssg_system_set_lanes": (N, 0),
        "cssg_system_lanes": (N, N),
        "cssg_system_set_lane_split": (N, 0),
        "cssg_system_lane_split": (N, N),
        "cssg_system_source_costs": (N, 0, N),
        "cssg_system_set_pass_groups": (N, 0, 0),
        "cssg_system_pass_groups": (N, N, N),
        "cssg_system_kernels_per_audit_step": (N, N),
        "cssg_system_set_work_caps": (N, 0, 0, 0),
        "cssg_system_set_screen_audit": (N, 0),
        "cssg_system_screen_audit_status": (N, N),
    }
    for name, args in calls.items():
        assert getattr(L, name)(*args) == 1, name  # CSSG_ERR_ARG
        assert name.encode() in L.cssg_last_error(), (name, L.cssg_last_error())
    for name in ("cssg_system_destroy", "cssg_mesh_destroy", "cssg_ctx_destroy"):
        assert getattr(L, name)(N) == 0, name


def test_pairs_to_neighbor_lists():
    """api.pairs_to_neighbor_lists groups pair records into simpleModel's lists (no GPU involved)."""
    import math

    import numpy as np

    from curvedspacesim_gb300 import api
    i = np.array([0, 0, 2, 2, 2])
    j = np.array([1, 2, 0, -2, 3])
    d = np.array([0.1, 0.2, 0.2, 0.9, math.inf])
    t = np.arange(15, dtype=np.float64)
    nb, nv, nd = api.pairs_to_neighbor_lists(4, i, j, d, t)
    assert nb == [[1, 2], [], [0, 1, 3], []]
    assert nd[0] == [0.1, 0.2] and nd[2][1] == math.inf and nd[2][2] == math.inf
    assert np.array_equal(nv[2][1], [9.0, 10.0, 11.0])
