"""The learned proposal's FP64 oracle (oracle/cnn.py), pinned by the
mathematics: its backward pass equals central finite differences of its
forward pass and loss, col2im is the adjoint of im2col, and its parameter
layout is the library's (rv_cnn_param_count). No GPU needed."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import cnn  # noqa: E402


def test_param_count_matches_library(rv):
    assert cnn.param_count() == 231_873
    assert rv.rv_cnn_param_count() == cnn.param_count()


@pytest.mark.parametrize("layer", range(len(cnn.LAYERS)))
def test_col2im_is_the_adjoint_of_patches(layer):
    kh, kw, sh, sw, ph, pw, ci, co, relu = cnn.LAYERS[layer]
    shapes = {0: (2, 64, 256, 2), 1: (2, 16, 64, 64), 2: (2, 8, 32, 128), 3: (2, 4, 32, 128), 4: (2, 1, 32, 64)}
    rng = np.random.default_rng(layer)
    x = rng.standard_normal(shapes[layer])
    cols, _ = cnn.patches(x, kh, kw, sh, sw, ph, pw)
    g = rng.standard_normal(cols.shape)
    # <patches(x), g> == <x, col2im(g)>
    lhs = np.sum(cols * g)
    rhs = np.sum(x * cnn.col2im(g, x.shape, kh, kw, sh, sw, ph, pw))
    assert abs(lhs - rhs) <= 1e-9 * max(1.0, abs(lhs))


def test_backward_equals_central_differences():
    rng = np.random.default_rng(5)
    params = cnn.init_params(3)
    params[np.cumsum([w[0] * w[1] + b[0] for w, b in cnn.param_shapes()])[:-1] - 1] += 0.05  # non-zero biases
    tiles = rng.standard_normal((3, 64, 256, 2))
    labels = (rng.random((3, 32)) < 0.25).astype(np.float64)
    logits, cache = cnn.forward(params, tiles)
    loss, dz = cnn.bce(logits, labels, 3.0)
    grad = cnn.backward(params, cache, dz)
    # a few parameters of every layer, weights and biases
    offsets = np.concatenate([[0], np.cumsum([(w[0] * w[1], b[0]) for w, b in cnn.param_shapes()])])
    picks = []
    for lo, hi in zip(offsets[:-1], offsets[1:]):
        picks += list(rng.integers(lo, hi, size=3))
    h = 1e-6
    for i in picks:
        up = params.copy()
        up[i] += h
        down = params.copy()
        down[i] -= h
        fd = (cnn.bce(cnn.forward(up, tiles)[0], labels, 3.0)[0] - cnn.bce(cnn.forward(down, tiles)[0], labels, 3.0)[0]) / (
            2 * h)
        assert abs(fd - grad[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-8, (i, fd, grad[i])


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -2.5, 0.0])
    got = cnn.bf16_round(x)
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: to even (1.0); 1 + 3 * 2^-9
    # is above halfway: up
    assert list(got) == [1.0, 1.0, 1.0, 1.0 + 2 ** -7, -2.5, 0.0]
