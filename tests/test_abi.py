"""CPU tests of the C-ABI boundary: the library loads, exports every entry
point include/mifgpu.h declares, and rejects invalid arguments before it
touches a device (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

from conftest import REPO


def declared_functions():
    src = open(os.path.join(REPO, "include", "mifgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mifgpu_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_the_binding_list(mifgpu_lib):
    assert declared_functions() == sorted(set(mifgpu_lib.EXPORTED))


def test_cpp_mirror_wraps_every_declared_function():
    hpp = open(os.path.join(REPO, "include", "mifgpu.hpp")).read()
    assert [f for f in declared_functions() if f not in hpp] == []


def test_cpp_mirror_compiles_and_links_against_the_library(tmp_path, mifgpu_lib):
    """Every mirror method is called once (tests/cpp/mirror_api_check.cpp);
    the program is compiled, linked with no undefined symbol, and not run."""
    import subprocess

    src = os.path.join(REPO, "tests", "cpp", "mirror_api_check.cpp")
    pkg = os.path.dirname(mifgpu_lib.__file__)
    out = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(REPO, "include"), "-o",
                          str(tmp_path / "mirror_api_check"), src, "-L", pkg, "-lmifgpu", "-Wl,--no-undefined"],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr


def test_library_exports_every_declared_symbol(mifgpu_lib):
    lib = mifgpu_lib.load_library()
    for name in declared_functions():
        assert hasattr(lib, name), name


def _params(mg, **kw):
    p = mg.Params()
    n = kw.get("n", (9, 9, 9))
    for d in range(3):
        p.n_global[d] = n[d]
        p.size[d] = 1.0
        p.periodic[d] = kw.get("periodic", (0, 0, 0))[d]
    p.Re = kw.get("Re", 100.0)
    p.dt = kw.get("dt", 1e-3)
    p.precision = kw.get("precision", 0)
    p.boundary_kind = kw.get("kind", 0)
    p.forcing = kw.get("forcing", 0)
    return p


@pytest.mark.parametrize("bad", [
    dict(n=(2, 9, 9)),          # fewer than 3 points on an axis
    dict(Re=0.0),
    dict(dt=-1.0),
    dict(precision=7),
    dict(kind=9),
    dict(forcing=-1),
    dict(n=(9, 9, 65535)),      # staggered z extent 65536: above grid z
    dict(n=(9, 9, 65534), periodic=(0, 0, 1)),  # periodic z: extent n + 2
    dict(n=(9, 262140, 9)),     # staggered y extent above 4 rows x 65535
    dict(n=(524280, 9, 9)),     # x above the face kernels' 8 x 65535
])
def test_create_rejects_invalid_parameters_without_a_device(mifgpu_lib, bad):
    lib = mifgpu_lib.load_library()
    p = _params(mifgpu_lib, **bad)
    h = C.c_void_p()
    assert lib.mifgpu_create(C.byref(p), C.byref(h)) == -1
    assert not h.value


@pytest.mark.parametrize("good", [
    dict(n=(9, 9, 65534)),                      # staggered z extent 65535
    dict(n=(9, 9, 65533), periodic=(0, 0, 1)),  # periodic z: 65533 + 2
    dict(n=(9, 262139, 9)),                     # staggered y extent 262140
])
def test_create_accepts_the_largest_grid_extents(mifgpu_lib, good):
    """At the grid limits the parameter check passes. What follows depends
    on the machine: without a device, create fails at the device query
    (MIFGPU_ECUDA). With one, the long Poisson lines are refused
    (MIFGPU_ENOTSUP) or the context is built. None of these is
    MIFGPU_EINVAL."""
    lib = mifgpu_lib.load_library()
    p = _params(mifgpu_lib, **good)
    h = C.c_void_p()
    rc = lib.mifgpu_create(C.byref(p), C.byref(h))
    if h.value:
        lib.mifgpu_destroy(h)
    assert rc != -1


def test_null_arguments_are_rejected(mifgpu_lib):
    lib = mifgpu_lib.load_library()
    assert lib.mifgpu_create(None, None) == -1
    assert lib.mifgpu_timestep(None, 0.0) == -1
    assert lib.mifgpu_run(None, 0.0, 1) == -1
    assert lib.mifgpu_upload(None, 0, None) == -1
    assert lib.mifgpu_download(None, 0, None) == -1
    assert lib.mifgpu_destroy(None) == -1
    assert lib.mifgpu_last_error(None) == b"null context"


def test_gpu_binding_fails_loudly_without_the_library(tmp_path, mifgpu_lib):
    import importlib

    mod = importlib.reload(mifgpu_lib)
    try:
        mod._LIB = None
        with pytest.raises(mod.MifGpuError):
            mod.load_library(str(tmp_path / "missing.so"))
    finally:
        importlib.reload(mifgpu_lib)
