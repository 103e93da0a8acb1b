"""C-ABI checks that need no GPU: the library loads, exports every entry point
declared in include/nbody_gb300.h, fills the reference defaults, and reports
errors (not crashes) without a device."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_entry_points():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:[\w\*]+\s+)+\**(nbody_\w+)\s*\(", src, re.M))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_entry_points()
    assert "nbody_create" in names and "nbody_step" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(nb):
    from nbody_gb300 import _lib
    L = C.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_entry_points() if not hasattr(L, n)]
    assert not missing, missing


def test_default_params_are_the_reference_defaults(nb):
    p = nb.params()
    assert p.precision == nb.PREC_FP32 and p.order == 1 and p.leaf_capacity == 8
    assert p.theta == 0.5 and p.eps == 0.01 and p.G == 1.0 and p.dt == 1e-3
    assert p.integrator == nb.INTEG_EULER and p.fixed_box == 1 and p.box_size == 1.0


def test_params_struct_layout_matches_header(nb):
    from nbody_gb300 import _lib
    # int x4, double x4, int x2, double[3], double, int  (natural alignment)
    assert C.sizeof(_lib.Params) == 96
    assert _lib.Params.box_min.offset == 56 and _lib.Params.device.offset == 88


def test_invalid_params_are_rejected_before_touching_a_device(nb):
    from nbody_gb300 import _lib
    L = _lib.load()
    for bad in ({"order": 0}, {"order": 9}, {"leaf_capacity": 0}, {"leaf_capacity": 65}, {"max_level": 22},
                {"theta": 0.0}, {"precision": 3}):
        p = nb.params(**bad)
        h = C.c_void_p()
        rc = L.nbody_create(C.byref(p), C.byref(h))
        assert rc == 1 and not h.value
        assert L.nbody_last_error(None)


def test_create_without_a_device_fails_cleanly(nb):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from nbody_gb300 import _lib
    L = _lib.load()
    p = nb.params()
    h = C.c_void_p()
    rc = L.nbody_create(C.byref(p), C.byref(h))
    assert rc == 6 and not h.value
    assert b"device" in L.nbody_last_error(None)
    with pytest.raises(nb.NbodyError):
        nb.CudaSimulation([1.0, 1.0, 1.0], [], 1e-3)


def test_null_context_is_refused_by_every_entry_point(nb):
    """Every call that takes a context returns NBODY_ERR_INVALID for NULL (no crash, no device)."""
    from nbody_gb300 import _lib
    L = _lib.load()
    d = C.c_double()
    i64 = C.c_int64()
    calls = {
        "nbody_set_state": (None, 0, None, None, None, None, None),
        "nbody_get_state": (None, 0, None, None, None, None, None, None),
        "nbody_step": (None, 1, C.byref(d)),
        "nbody_compute_forces": (None, None, None),
        "nbody_diagnostics": (None, None),
        "nbody_tree_info": (None, None, None, None, None),
        "nbody_get_tree": (None, None, None, None),
        "nbody_get_interactions": (None, 0, C.byref(i64), None),
        "nbody_set_timing": (None, 1),
        "nbody_get_time": (None, C.byref(d)),
        "nbody_device_memory": (None, None, None),
        "nbody_force_vjp": (None, None, None, None, None),
        "nbody_forward_checkpointed": (None, 1, 0, C.byref(d)),
        "nbody_backward": (None, None, None, None, None, None, None),
        "nbody_trajectory_open": (None, b"x.csv", 1, 0, 6),
        "nbody_trajectory_close": (None,),
        "nbody_set_timestep_control": (None, 1, 0.02, 0.0, 1e-6, 1e-2),
        "nbody_last_timestep": (None, C.byref(d)),
    }
    for name, args in calls.items():
        assert getattr(L, name)(*args) == 1, name
    assert L.nbody_stream(None) is None
    assert L.nbody_destroy(None) == 0


@pytest.mark.parametrize("src", ["drop_in_main.cpp", "adjoint_main.cpp"])
def test_cpp_drop_in_programs_compile_against_the_headers(src):
    """The C++ drop-in (include/nbody/cuda_simulation.h over the C ABI) compiles as the reference's
    C++14 code would use it, warnings as errors; linking and running need the GPU tests."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("no g++")
    r = subprocess.run(["g++", "-std=c++14", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only",
                        "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
