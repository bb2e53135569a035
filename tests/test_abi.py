"""The C-ABI library: it builds, loads without a GPU, and exports every entry point
that include/psx.h declares.  No compute call is made here."""
import ctypes
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "psx.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    names = re.findall(r"\b(psx_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ("psx_scene_create", "psx_scene_simulate", "psx_scene_destroy", "psx_world_create", "psx_world_step"):
        assert n in names


@pytest.fixture(scope="module")
def libpsx():
    if shutil.which("nvcc") is None and not os.path.exists(os.path.join(ROOT, "physecs_gb300", "_lib", "libpsx.so")):
        pytest.skip("no nvcc to build the library")
    from physecs_gb300 import api
    return api.load()


def test_library_exports_every_declared_symbol(libpsx):
    missing = [n for n in declared_functions() if not hasattr(libpsx, n)]
    assert not missing, missing


def test_python_api_binds_exactly_the_header():
    from physecs_gb300 import api
    assert sorted(set(api.EXPORTS)) == declared_functions()


def test_errors_without_gpu_are_reported_not_raised(libpsx):
    """Creating a world on a machine without a usable device returns an error status
    and an error string rather than crashing."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from physecs_gb300 import api, scenes
    from physecs_gb300.desc import make_desc
    s = scenes.pyramid(rows=2)
    d = make_desc(s)
    out = ctypes.c_void_p()
    st = libpsx.psx_scene_create(ctypes.byref(d), ctypes.byref(out))
    assert st != 0
    assert libpsx.psx_last_error_string()
