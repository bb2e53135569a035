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


def struct_words(name):
    """4-byte words of `typedef struct name { ... } name;` in the header (fields of 4-byte
    scalar types, arrays included)."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, flags=re.S)
    assert m, name
    words = 0
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        typ, rest = decl.split(None, 1)
        assert typ in ("int32_t", "uint32_t", "float"), (name, decl)
        for var in rest.split(","):
            arr = re.search(r"\[(\d+)\]", var)
            words += int(arr.group(1)) if arr else 1
    return words


def test_record_layouts_match_the_python_packing():
    """The Python layer packs these records as flat 4-byte words; their widths follow the
    header."""
    expect = {"psx_body_delta": 17, "psx_character": 10, "psx_trigger_event": 9, "psx_trimesh_triangle": 20,
              "psx_trimesh_node": 8, "psx_ray": 8, "psx_ray_hit": 7, "psx_overlap_query": 14, "psx_overlap_hit": 3,
              "psx_overlap_mtd_hit": 7}
    for name, words in expect.items():
        assert struct_words(name) == words, name
    from physecs_gb300.api import pack_deltas
    assert pack_deltas([{"body": 0, "pos": [1, 2, 3], "kinematic": True}]).shape == (1, 17)


def test_ctypes_structures_match_the_header(tmp_path):
    """The option and descriptor structures the Python layer passes by pointer have the C
    compiler's size and field offsets (a field added on one side only shifts every later
    one)."""
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    import subprocess
    from physecs_gb300.api import PsxLaunchConfig, PsxSceneCarry, PsxServerOpts, PsxWorldOpts
    from physecs_gb300.desc import PsxSceneDesc
    structs = {"psx_launch_config": PsxLaunchConfig, "psx_world_opts": PsxWorldOpts,
               "psx_scene_carry": PsxSceneCarry, "psx_server_opts": PsxServerOpts, "psx_scene_desc": PsxSceneDesc}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "psx.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for field, _ in cls._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, field, cname, field))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, cls in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert got[(cname, field)] == getattr(cls, field).offset, (cname, field)
