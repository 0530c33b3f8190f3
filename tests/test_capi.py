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


def test_refit_without_visit_counters_is_refused(gray_lib):
    """A refit needs the caller's refit_flags (the static rebuild's scratch is its own): a NULL
    pointer is an argument error, raised before any launch."""
    from gray_gb300 import _lib

    p = _lib.ParamsC()
    p.image_width = p.image_height = p.render_width = p.render_height = 16
    p.gaussians.count = 100
    p.scene.bvh_valid = 1
    with pytest.raises(_lib.GrayError, match="refit_flags"):
        _lib.call("gray_update_bvh", p, 0)


def _structs():
    """(C struct name, ctypes mirror) of every struct the C ABI passes."""
    from gray_gb300 import _lib, batch

    return (("gray_gaussians", _lib.GaussiansC), ("gray_camera", _lib.CameraC), ("gray_config", _lib.ConfigC),
            ("gray_framebuffer", _lib.FramebufferC), ("gray_metadata", _lib.MetadataC), ("gray_stats", _lib.StatsC),
            ("gray_hitlist", _lib.HitlistC), ("gray_scene", _lib.SceneC), ("gray_params", _lib.ParamsC),
            ("gray_batch_scene", batch.BatchSceneC), ("gray_batch_view", batch.BatchViewC))


def _c_layout(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', 'int main(void) {']
    for cname, cls in _structs():
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
    c = _c_layout(tmp_path)
    for cname, cls in _structs():
        assert int(c[f"{cname} size"]) == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(c[f"{cname}.{f}"]) == getattr(cls, f).offset, f"{cname}.{f}"


def _ceil(a, b):
    return -(-a // b)


def test_frontier_and_batch_sizes(gray_lib):
    """Workspace sizing without a GPU: the frontier record length matches the header, a batch view's
    packet groups are its 2x2 packets, and a framebuffer's schedule holds the estimates, the order
    and a frontier per block tile for both packet shapes (8x16- and 16x8-pixel tiles)."""
    from gray_gb300 import batch

    L = batch._bind()
    m = re.search(r"#define GRAY_FRONTIER_WORDS (\d+)", open(HEADER).read())
    words = int(L.gray_frontier_words())
    assert m and words == int(m.group(1))
    header = 64
    for w, h in ((1, 1), (7, 5), (640, 480), (1600, 1040), (1920, 1080), (3840, 2160), (1001, 333)):
        for variant, (tw, th) in ((7, (4, 8)), (3, (8, 4))):
            packets = _ceil(w, tw) * _ceil(h, th)
            assert L.gray_batch_packets(w, h, variant) == packets
            assert L.gray_batch_groups(w, h, variant) == _ceil(_ceil(w, tw), 2) * _ceil(_ceil(h, th), 2)
            tiles = _ceil(w, 2 * tw) * _ceil(h, 2 * th)  # the forward's block tiles (2x2 packets)
            assert gray_lib.gray_schedule_words(w, h) >= header + tiles * (2 + words), (w, h, variant)


def test_copy_wait_selftest_checks_its_arguments(gray_lib):
    """The copy-wait self-test refuses a NULL status word and a limit above 2 s before any launch."""
    from gray_gb300 import _lib

    L = _lib.load()
    L.gray_selftest_copy_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    assert L.gray_selftest_copy_wait(None, 1000, None) == 1  # GRAY_ERR_INVALID_ARGUMENT
    assert b"status" in L.gray_last_error()
    assert L.gray_selftest_copy_wait(ctypes.c_void_p(16), 3_000_000_000, None) == 3  # GRAY_ERR_OUT_OF_RANGE
