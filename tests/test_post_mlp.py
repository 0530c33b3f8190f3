"""The post-processing MLP's input encoding (gray/mlp.py:218-262), on the CPU: the input channels,
then sin of every channel at frequencies 2^0 .. 2^(k-1) (channel-major), then the cosines."""
import math

import pytest
import torch

from gray_gb300 import mlp


@pytest.mark.parametrize("k", [0, 1, 3])
def test_positional_encoding_layout(k):
    g = torch.Generator().manual_seed(0)
    img = torch.randn(6, 3, 5, generator=g, dtype=torch.float64)
    enc = mlp.positional_encoding(img, k)
    assert enc.shape[0] == mlp.positional_encoding_size(6, k) == 6 + 12 * k
    assert torch.equal(enc[:6], img)
    for c in range(6):
        for f in range(k):
            assert torch.allclose(enc[6 + c * k + f], torch.sin(img[c] * 2.0 ** f))
            assert torch.allclose(enc[6 + 6 * k + c * k + f], torch.cos(img[c] * 2.0 ** f))
    vec = img.reshape(6, -1).T.contiguous()  # [N, C] form: the same values per row
    assert torch.allclose(mlp.positional_encoding(vec, k), enc.reshape(enc.shape[0], -1).T)


def test_positional_encoding_rejects_bad_input():
    with pytest.raises(ValueError):
        mlp.positional_encoding(torch.zeros(3), 1)
    with pytest.raises(ValueError):
        mlp.positional_encoding(torch.zeros(2, 3), -1)
