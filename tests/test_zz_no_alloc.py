"""gray_rebuild_bvh_static: the BVH rebuild for callers that cannot allocate device memory.

Hosts that own the whole device budget (an engine or viewer plugin with a fixed reservation, or
code where the host's allocator must not be entered) cannot give the rebuild its transient
scratch (sort buffers, histograms, bounds, visit counters).  This entry point keeps that scratch
in a fixed device array inside the library (at most GRAY_STATIC_MAX_GAUSSIANS Gaussians) and must
produce exactly what gray_rebuild_bvh produces with caller-provided scratch.  The file is named so
that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

from gray_gb300 import _lib, classes, synthetic

STATIC_MAX = 262144  # GRAY_STATIC_MAX_GAUSSIANS in include/gray_gb300.h


def _static_rebuild(params, stream):
    L = _lib.load()
    f = L.gray_rebuild_bvh_static
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(_lib.ParamsC), ctypes.c_void_p]
    rc = f(ctypes.byref(params), ctypes.c_void_p(stream))
    if rc != 0:
        raise _lib.GrayError(L.gray_last_error().decode())


def test_static_rebuild_rejects_counts_above_its_maximum(gray_lib):
    p = _lib.ParamsC()
    p.gaussians.count = STATIC_MAX + 1
    with pytest.raises(_lib.GrayError, match="at most 262144 Gaussians"):
        _static_rebuild(p, 0)


@pytest.mark.gpu
def test_static_rebuild_matches_regular_rebuild_twice(gray_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tests import gpu_util as G

    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream().cuda_stream
    for seed, n in ((21, 120_000), (22, STATIC_MAX)):  # two calls in a row, the second at the maximum
        sc = synthetic.clustered_scene(n, seed=seed)
        rt = G.make_tracer(16, 16, sc.mean, sc.rotation, sc.scale, sc.opacity,
                           channels=np.zeros((sc.n, 3), np.float32))  # regular rebuild with caller scratch
        ref = rt.scene_workspace()
        out = classes._SceneWorkspace(sc.n, dev)
        for t in (out.nodes, out.geom, out.aabb):
            t.fill_(-1.0)
        params = rt._build_params()
        params.scene = out.struct()
        params.scene.sort_tmp = None   # no scratch from the caller
        params.scene.bounds = None
        params.scene.refit_flags = None
        _static_rebuild(params, stream)
        torch.cuda.synchronize()
        for name in ("geom", "l2w", "aabb", "visible", "nodes", "int_parent", "leaf_parent", "order", "codes",
                     "root_box"):
            assert torch.equal(getattr(out, name), getattr(ref, name)), (seed, name)
        rt.check_status()
