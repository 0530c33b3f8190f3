"""Scene IO and training cadence on the CPU: the safetensors reader/writer against the published
format (8-byte little-endian header length, JSON header, raw little-endian data), cameras.json
(gray/scene.py:156-170), and the train.py:217-287 cadence driven through a fake tracer."""
import json
import math
import struct

import numpy as np
import pytest
import torch

from gray_gb300 import TrainCadence, RaytracerConfig, load_cameras_json, look_at, save_cameras_json
from gray_gb300.safetensors_io import load_file, save_file


def _hand_built_file(path):
    """A file written from the format description: header keys in a different order than our
    writer's, a __metadata__ entry, no padding."""
    a = np.array([1.5, -2.0, 3.25], "<f4").tobytes()
    b = np.array([[7, -8]], "<i4").tobytes()
    h = np.array([1.0, 0.5], "<f2").tobytes()
    header = {"__metadata__": {"format": "pt"},
              "z_half": {"shape": [2], "data_offsets": [len(a) + len(b), len(a) + len(b) + len(h)], "dtype": "F16"},
              "a": {"data_offsets": [0, len(a)], "dtype": "F32", "shape": [3]},
              "b": {"dtype": "I32", "data_offsets": [len(a), len(a) + len(b)], "shape": [1, 2]},
              "empty": {"dtype": "F32", "shape": [0, 3], "data_offsets": [len(a) + len(b) + len(h)] * 2}}
    hj = json.dumps(header).encode()
    with open(path, "wb") as f:
        f.write(struct.pack("<Q", len(hj)) + hj + a + b + h)


def test_safetensors_reads_files_written_from_the_format(tmp_path):
    p = tmp_path / "x.safetensors"
    _hand_built_file(p)
    d = load_file(str(p))
    assert set(d) == {"a", "b", "z_half", "empty"}
    assert d["a"].dtype == torch.float32 and d["a"].tolist() == [1.5, -2.0, 3.25]
    assert d["b"].dtype == torch.int32 and d["b"].tolist() == [[7, -8]]
    assert d["z_half"].dtype == torch.float16 and d["z_half"].tolist() == [1.0, 0.5]
    assert tuple(d["empty"].shape) == (0, 3)


def test_safetensors_writer_layout_and_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    tensors = {"mean": torch.from_numpy(rng.standard_normal((5, 3)).astype(np.float32)),
               "sh_coeffs_rest": torch.from_numpy(rng.standard_normal((5, 15, 3)).astype(np.float16)),
               "current_sh_degree": torch.tensor([2], dtype=torch.int32),
               "flag": torch.tensor([True, False]), "nothing": torch.zeros(0, 4)}
    p = tmp_path / "y.safetensors"
    save_file(tensors, str(p), metadata={"iteration": 7})
    raw = p.read_bytes()
    (hlen,) = struct.unpack("<Q", raw[:8])
    assert (8 + hlen) % 8 == 0  # data section 8-byte aligned (header padded with spaces)
    header = json.loads(raw[8:8 + hlen])
    assert header["__metadata__"] == {"iteration": "7"}
    ends = sorted((v["data_offsets"] for k, v in header.items() if k != "__metadata__"))
    assert ends[0][0] == 0 and all(a[1] == b[0] for a, b in zip(ends, ends[1:]))
    assert ends[-1][1] == len(raw) - 8 - hlen
    m = header["mean"]
    b0, b1 = m["data_offsets"]
    np.testing.assert_array_equal(np.frombuffer(raw[8 + hlen + b0:8 + hlen + b1], "<f4").reshape(5, 3),
                                  tensors["mean"].numpy())
    back = load_file(str(p))
    for k, v in tensors.items():
        assert back[k].dtype == v.dtype and torch.equal(back[k], v), k


def test_cameras_json_round_trip_sorted_and_split(tmp_path):
    cams = []
    for i, name in enumerate(["c.png", "a.png", "b.png", "d.png"]):
        c = look_at((3.0 + i, -4.0, 1.0), (0, 0, 0), (0, 0, 1), 0.8 + 0.01 * i, 64 + i, 48, uid=i)
        c.image_name = name
        c.is_test = name == "b.png"
        cams.append(c)
    save_cameras_json(str(tmp_path), cams)
    model_file = tmp_path / "gaussians_00010.safetensors"
    model_file.write_bytes(b"")
    train, test = load_cameras_json(str(model_file))  # a file inside the model directory works too
    assert [c.image_name for c in train] == ["a.png", "c.png", "d.png"]
    assert [c.image_name for c in test] == ["b.png"]
    by_name = {c.image_name: c for c in cams}
    for c in train + test:
        o = by_name[c.image_name]
        np.testing.assert_array_equal(c.R, o.R)
        np.testing.assert_array_equal(c.origin, o.origin)
        assert c.fov_y == o.fov_y and c.image_width == o.image_width and c.uid == o.uid
        np.testing.assert_array_equal(c.rotation_c2w_blender(), o.rotation_c2w_blender())
    with pytest.raises(FileNotFoundError):
        load_cameras_json(str(tmp_path / "missing"))


class _FakeGaussians:
    def __init__(self, n):
        self.count = n
        self.scale = torch.zeros(n, 3)
        self.sh_increments = 0

    def increment_sh_degree(self):
        self.sh_increments += 1


class _FakeModule:
    def __init__(self, g):
        self.g = g
        self.rebuilds = []

    def get_gaussians(self):
        return self.g

    def rebuild_bvh(self):
        self.rebuilds.append(self.it)


class _FakeTracer:
    def __init__(self, n):
        self.cuda_module = _FakeModule(_FakeGaussians(n))
        self.prunes = []

    def prune(self, iteration):
        g = self.cuda_module.g
        self.prunes.append(iteration)
        g.count -= 1
        g.scale = g.scale[:-1]


def test_training_cadence_follows_train_py():
    cfg = RaytracerConfig(pruning_interval=100, pruning_from_iter=200, rebuild_interval=150,
                          sh_increment_interval=250, scale_decay=0.5)
    cad = TrainCadence(cfg)
    rt = _FakeTracer(10)
    events = []
    for it in range(1, 601):
        rt.cuda_module.it = it
        cad.before_iteration(rt, it)
        events.append(cad.after_step(rt, it))
    assert rt.prunes == [200, 300, 400, 500, 600]
    assert rt.cuda_module.rebuilds == [150, 200, 300, 400, 450, 500, 600]
    assert rt.cuda_module.g.sh_increments == 2
    assert sum(e.pruned for e in events) == 5 and rt.cuda_module.g.count == 5
    # log-scale decays by log(0.5) per iteration
    assert math.isclose(float(rt.cuda_module.g.scale[0, 0]), 600 * math.log(0.5), rel_tol=1e-5)
    # pruning off, no rebuild interval: nothing but the decay
    cad2 = TrainCadence(RaytracerConfig(pruning=False, rebuild_interval=0, scale_decay=1.0))
    rt2 = _FakeTracer(3)
    rt2.cuda_module.it = 0
    for it in range(1, 1001):
        assert cad2.after_step(rt2, it) == type(events[0])()
    assert float(rt2.cuda_module.g.scale.abs().sum()) == 0.0
