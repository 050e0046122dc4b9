"""CPU tests of the C ABI: the library loads without a GPU, exports every entry point that
include/lucid_gb300.h declares, and its host-only helpers agree with the Python mirror."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

from lucid_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(lucid_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("lucid_create", "lucid_render", "lucid_quad_setup", "lucid_bin_count",
                 "lucid_bin_categorize", "lucid_bin_dispatch", "lucid_raster", "lucid_get_info"):
        assert must in names


def test_library_exports_every_declared_symbol(lucid_lib):
    missing = [n for n in declared_functions() if not hasattr(lucid_lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    from lucid_gb300 import _lib
    declared = set(declared_functions())
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert declared == bound, (declared - bound, bound - declared)


def test_status_strings_and_version(lucid_lib):
    assert lucid_lib.lucid_abi_version() == 1
    assert lucid_lib.lucid_status_string(0) == b"ok"
    assert lucid_lib.lucid_status_string(2) == b"capacity exceeded"


def test_default_options(lucid_lib):
    from lucid_gb300 import _lib
    o = _lib.Options()
    assert lucid_lib.lucid_default_options(ctypes.byref(o)) == 0
    assert o.bin_size == 32 and o.low_high_threshold == 1024 and o.max_instances == 65536


def test_invalid_arguments_without_gpu(lucid_lib):
    from lucid_gb300 import _lib
    o = _lib.Options()
    lucid_lib.lucid_default_options(ctypes.byref(o))
    o.bin_size = 48  # bins are 32 or 64 pixels
    h = ctypes.c_void_p()
    assert lucid_lib.lucid_create(ctypes.byref(o), 64, 64, ctypes.byref(h)) == _lib.NOT_SUPPORTED
    assert b"32x32 or 64x64" in lucid_lib.lucid_last_error_string()
    lucid_lib.lucid_default_options(ctypes.byref(o))
    assert lucid_lib.lucid_create(ctypes.byref(o), 0, 64, ctypes.byref(h)) == _lib.INVALID_ARG
    assert lucid_lib.lucid_bin_count(None, None) == _lib.INVALID_ARG
    assert lucid_lib.lucid_destroy(None) == 0


def test_build_instances_matches_reference_split(lucid_lib):
    from lucid_gb300 import _lib
    dcs = [(0, 2500, 1, 0xFFFFFFFF), (2500, 10, 1, 0x11223344), (2510, 0, 1, 0xFFFFFFFF),
           (2510, 1024, 5, 0xFFFFFFFF)]
    arr = (_lib.DrawCall * len(dcs))(*[_lib.DrawCall(*d) for d in dcs])
    out = np.zeros((16, 4), np.int32)
    cols = np.zeros(16, np.uint32)
    n, q = ctypes.c_int32(), ctypes.c_int32()
    st = lucid_lib.lucid_build_instances(arr, len(dcs), out.ctypes.data, cols.ctypes.data, 16,
                                         ctypes.byref(n), ctypes.byref(q))
    assert st == 0
    inst, icol, total = scenes.build_instances(dcs)
    assert n.value == len(inst) == 5 and q.value == total == 3534
    np.testing.assert_array_equal(out[:n.value], inst)
    np.testing.assert_array_equal(cols[:n.value], icol)
    assert inst[3, 3] & scenes.INST_HAS_COLOR  # non-white material colour
    # truncation like the reference's resize(max_instances)
    st = lucid_lib.lucid_build_instances(arr, len(dcs), out.ctypes.data, None, 2,
                                         ctypes.byref(n), ctypes.byref(q))
    assert st == _lib.CAPACITY_EXCEEDED and n.value == 2


@pytest.mark.parametrize("w,h,pos,fov", [(1280, 720, (0, 0, 0), 60.0), (333, 517, (1.5, -2.0, 7.0), 37.5)])
def test_make_config_matches_python(lucid_lib, w, h, pos, fov):
    from lucid_gb300 import _lib
    cam = scenes.Camera(position=pos, right=(0.6, 0.0, -0.8), up=(0.0, 1.0, 0.0),
                        forward=(-0.8, 0.0, -0.6), fov_y=math.radians(fov), near=0.1, far=90.0)
    py = scenes.make_config(cam, w, h, (0.1, 0.2, 0.3, 1.0), True)
    c = _lib.CameraC()
    c.position[:] = cam.position
    c.right[:] = cam.right
    c.up[:] = cam.up
    c.forward[:] = cam.forward
    c.fov_y_radians, c.near_plane, c.far_plane = cam.fov_y, cam.near, cam.far
    out = scenes.LucidConfig()
    bg = (ctypes.c_float * 4)(0.1, 0.2, 0.3, 1.0)
    assert lucid_lib.lucid_make_config(ctypes.byref(c), w, h, ctypes.cast(bg, ctypes.c_void_p), 1,
                                       ctypes.addressof(out)) == 0
    assert bytes(out) == bytes(py)


def test_info_struct_layout():
    from lucid_gb300 import _lib
    assert _lib.Info.temp.offset == (1152 - 64) * 4
    assert _lib.Info.error_code.offset == 1152 * 4
    assert ctypes.sizeof(_lib.Info) == 1216 * 4
    assert ctypes.sizeof(scenes.LucidConfig) == 352


def test_struct_sizes_match_header(tmp_path):
    """sizeof / offsetof of the public structs, compiled from include/lucid_gb300.h with the host
    C compiler, equal the ctypes mirrors."""
    import shutil
    import subprocess
    from lucid_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "sizes.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "lucid_gb300.h"\n'
        "int main(void) {\n"
        ' printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(lucid_options), sizeof(lucid_frame_inputs),'
        " sizeof(lucid_view), sizeof(lucid_tuning), sizeof(lucid_info), sizeof(lucid_camera),"
        " offsetof(lucid_options, grad_store_fragments), offsetof(lucid_view, out_rgba));\n"
        " return 0;\n}\n")
    exe = tmp_path / "sizes"
    subprocess.run([cc, "-I", os.path.join(root, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    want = [ctypes.sizeof(_lib.Options), ctypes.sizeof(_lib.FrameInputsC), ctypes.sizeof(_lib.ViewC),
            ctypes.sizeof(_lib.Tuning), ctypes.sizeof(_lib.Info), ctypes.sizeof(_lib.CameraC),
            _lib.Options.grad_store_fragments.offset, _lib.ViewC.out_rgba.offset]
    assert got == want
