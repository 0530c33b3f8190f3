"""C-ABI checks that need no GPU: the library builds for sm_103a, loads, exports every entry point
declared in include/gray_gb300.h, and the ctypes mirror has the C structs' exact layout."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gray_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(gray_[a-z_0-9]+)\s*\(", text, re.M)))


def test_header_declares_the_reference_methods():
    names = declared_functions()
    for want in ("gray_forward_pass", "gray_forward_pass_display", "gray_backward_pass", "gray_step",
                 "gray_update_bvh", "gray_rebuild_bvh", "gray_last_error"):
        assert want in names


def test_library_exports_every_declared_symbol(gray_lib):
    for name in declared_functions():
        assert hasattr(gray_lib, name), name
    assert gray_lib.gray_version().decode().startswith("gray_gb300")


def test_library_is_built_for_sm_103a(gray_lib):
    from gray_gb300 import _lib

    out = subprocess.run(["cuobjdump", "--list-elf", _lib.LIB_PATH], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    assert "sm_103a" in out.stdout


def test_errors_are_reported_without_a_gpu(gray_lib):
    from gray_gb300 import _lib

    p = _lib.ParamsC()  # zero render size: rejected before any CUDA call
    with pytest.raises(_lib.GrayError, match="render resolution"):
        _lib.call("gray_forward_pass", p, 0)
    with pytest.raises(_lib.GrayError):
        _lib.call("gray_rebuild_bvh", p, 0)


def _c_layout(tmp_path):
    from gray_gb300 import _lib

    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', 'int main(void) {']
    for cname, cls in (("gray_gaussians", _lib.GaussiansC), ("gray_camera", _lib.CameraC),
                       ("gray_config", _lib.ConfigC), ("gray_framebuffer", _lib.FramebufferC),
                       ("gray_metadata", _lib.MetadataC), ("gray_stats", _lib.StatsC),
                       ("gray_hitlist", _lib.HitlistC), ("gray_scene", _lib.SceneC),
                       ("gray_params", _lib.ParamsC)):
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return dict(line.rsplit(" ", 1) for line in out.strip().splitlines())


def test_ctypes_structs_match_c_layout(tmp_path):
    from gray_gb300 import _lib

    c = _c_layout(tmp_path)
    for cname, cls in (("gray_gaussians", _lib.GaussiansC), ("gray_camera", _lib.CameraC),
                       ("gray_config", _lib.ConfigC), ("gray_framebuffer", _lib.FramebufferC),
                       ("gray_metadata", _lib.MetadataC), ("gray_stats", _lib.StatsC),
                       ("gray_hitlist", _lib.HitlistC), ("gray_scene", _lib.SceneC),
                       ("gray_params", _lib.ParamsC)):
        assert int(c[f"{cname} size"]) == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(c[f"{cname}.{f}"]) == getattr(cls, f).offset, f"{cname}.{f}"
