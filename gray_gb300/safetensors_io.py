"""Minimal reader/writer of the safetensors format (8-byte little-endian header length, JSON
header of {name: {dtype, shape, data_offsets}}, then the raw little-endian tensor bytes), so
scenes saved by the reference (gray/raytracer.py:422-438) load without the safetensors
package."""
from __future__ import annotations

import json
import struct

import numpy as np
import torch

_DT = {"F32": torch.float32, "F16": torch.float16, "BF16": torch.bfloat16, "F64": torch.float64,
       "I32": torch.int32, "I64": torch.int64, "I16": torch.int16, "I8": torch.int8, "U8": torch.uint8,
       "BOOL": torch.bool}
_RDT = {v: k for k, v in _DT.items()}


def load_file(path: str, device: str = "cpu") -> dict:
    with open(path, "rb") as f:
        data = f.read()
    (hlen,) = struct.unpack("<Q", data[:8])
    header = json.loads(data[8:8 + hlen])
    base = 8 + hlen
    out = {}
    for name, info in header.items():
        if name == "__metadata__":
            continue
        b, e = info["data_offsets"]
        dt = _DT[info["dtype"]]
        buf = bytearray(data[base + b:base + e])
        t = torch.frombuffer(buf, dtype=dt) if e > b else torch.zeros(0, dtype=dt)
        out[name] = t.reshape(info["shape"]).to(device)
    return out


def save_file(tensors: dict, path: str, metadata: dict | None = None):
    header, blobs, off = {}, [], 0
    for name in sorted(tensors):
        t = tensors[name].detach().contiguous().cpu()
        raw = t.view(torch.uint8).numpy().tobytes() if t.numel() else b""
        header[name] = {"dtype": _RDT[t.dtype], "shape": list(t.shape), "data_offsets": [off, off + len(raw)]}
        blobs.append(raw)
        off += len(raw)
    if metadata:
        header["__metadata__"] = {str(k): str(v) for k, v in metadata.items()}
    hj = json.dumps(header, separators=(",", ":")).encode()
    hj += b" " * ((8 - len(hj) % 8) % 8)
    with open(path, "wb") as f:
        f.write(struct.pack("<Q", len(hj)))
        f.write(hj)
        for b in blobs:
            f.write(b)
