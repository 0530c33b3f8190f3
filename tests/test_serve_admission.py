"""Admission of the serving loop, on the CPU: requests are taken in arrival order while their
buffers (image, per-view colours, packet-group frontiers) fit in the free memory left above the
reserve, at most max_batch per launch; a request that does not fit alone waits."""
import pytest

from gray_gb300 import serve
from gray_gb300.camera import CameraInfo


class _Gaussians:
    def __init__(self, n):
        self.count = n


class _Tracer:
    def __init__(self, n):
        self._g = _Gaussians(n)

    def get_gaussians(self):
        return self._g


def _server(max_batch=8, reserve=0, counts=(1000, 50_000), ray_budget=None):
    srv = object.__new__(serve.RenderServer)  # no CUDA streams: only the host-side admission is used
    srv.tracers = [_Tracer(n) for n in counts]
    srv.max_batch = max_batch
    srv.ray_budget = ray_budget
    srv.reserve = reserve
    srv.queue = []
    srv._next = 0
    return srv


def _camera(w, h):
    return CameraInfo(image_width=w, image_height=h)


def _ceil(a, b):
    return -(-a // b)


def test_request_bytes_cover_image_colours_and_frontiers(gray_lib):
    srv = _server()
    r = srv.submit(1, _camera(1920, 1080), arrival=0.0)
    groups = max(_ceil(1920, 8) * _ceil(1080, 16), _ceil(1920, 16) * _ceil(1080, 8))
    words = int(gray_lib.gray_frontier_words())
    assert srv._request_bytes(r) == 12 * 1920 * 1080 + 12 * 50_000 + 4 * words * groups + 256


def test_admission_order_budget_and_batch_size(gray_lib):
    srv = _server(max_batch=3, reserve=1000)
    reqs = [srv.submit(i % 2, _camera(640, 480), arrival=float(i)) for i in range(5)]
    sizes = [srv._request_bytes(r) for r in reqs]
    # everything fits: at most max_batch, in arrival order
    batch, need = srv._admit(10 ** 12)
    assert [r.rid for r in batch] == [0, 1, 2] and need == sum(sizes[:3])
    # room for one more request only (free memory minus the reserve)
    batch, need = srv._admit(1000 + sizes[3] + sizes[4] - 1)
    assert [r.rid for r in batch] == [3] and need == sizes[3]
    # the last request alone does not fit: it waits, nothing is admitted
    batch, need = srv._admit(1000 + sizes[4] - 1)
    assert batch == [] and need == 0 and [r.rid for r in srv.queue] == [4]
    batch, _ = srv._admit(1000 + sizes[4])
    assert [r.rid for r in batch] == [4] and srv.queue == []


@pytest.mark.parametrize("rate", [50.0, 200.0])
def test_poisson_arrivals_are_seeded_and_increasing(rate):
    a = serve.poisson_arrivals(rate, 4000, seed=3)
    b = serve.poisson_arrivals(rate, 4000, seed=3)
    assert (a == b).all() and (a[1:] > a[:-1]).all()
    assert abs(a[-1] / 4000 - 1.0 / rate) < 0.1 / rate  # mean gap


def test_ray_budget_bounds_a_batch_but_always_admits_one(gray_lib):
    """With a ray budget, a batch takes requests in arrival order while their rays fit; a request
    larger than the budget still goes, alone."""
    srv = _server(max_batch=16, ray_budget=1920 * 1080 + 640 * 480)
    for w, h in ((3840, 2160), (640, 480), (1920, 1080), (640, 480), (640, 480)):
        srv.submit(0, _camera(w, h), arrival=0.0)
    big, _ = srv._admit(1 << 40)
    assert [r.camera.image_width for r in big] == [3840]
    nxt, _ = srv._admit(1 << 40)
    assert [r.camera.image_width for r in nxt] == [640, 1920]
    rest, _ = srv._admit(1 << 40)
    assert [r.camera.image_width for r in rest] == [640, 640]
