"""The learned proposal's network on the GPU against its FP64 oracle
(oracle/cnn.py), all through the C ABI.

Tolerances (relative L2 norm of the difference):
- rv_gemm_bf16 against FP64 products of the same BF16-rounded operands:
  1e-5 of the product's magnitude (FP32 accumulation);
- logits against the oracle with BF16-rounded GEMM operands: 2e-3; against
  the oracle in full FP64: 2e-2;
- each layer's weight and bias gradient against the BF16-operand oracle:
  2e-2; against full FP64: 0.15 (BF16 operands alone move the deepest
  gradients by up to ~8 % on random tiles; the oracle measures that gap).
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

from revenant_gb300 import proposal
from revenant_gb300.library import lib

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import cnn as oracle_cnn  # noqa: E402

pytestmark = pytest.mark.gpu


def ok(status):
    assert status == 0, lib().rv_last_error().decode()


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def to_bf16_bits(x):
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def layer_slices():
    out, at = [], 0
    for (co, k), (cb,) in oracle_cnn.param_shapes():
        out.append(slice(at, at + co * k))
        at += co * k
        out.append(slice(at, at + cb))
        at += cb
    return out


@pytest.mark.parametrize("m,n,k", [(128, 16, 16), (300, 64, 100), (1000, 128, 640), (257, 33, 1000), (64, 200, 64)])
def test_gemm_against_fp64_of_bf16_operands(gpu, m, n, k):
    rng = np.random.default_rng(m * 7 + n + k)
    a = rng.standard_normal((m, k)).astype(np.float32)
    b = rng.standard_normal((n, k)).astype(np.float32)
    da, db, dd, st = gpu.array(a), gpu.array(b), gpu.zeros(m * n * 4), gpu.zeros(4)
    ok(lib().rv_gemm_bf16(gpu.stream, da.ptr, db.ptr, m, n, k, dd.ptr, st.ptr))
    gpu.synchronize()
    got = dd.download(np.float32, (m, n))
    assert st.download(np.uint32, (1,))[0] == 0
    want = oracle_cnn.bf16_round(a) @ oracle_cnn.bf16_round(b).T
    scale = np.abs(oracle_cnn.bf16_round(a)) @ np.abs(oracle_cnn.bf16_round(b)).T
    assert np.all(np.abs(got - want) <= 1e-5 * scale + 1e-30)


@pytest.fixture(scope="module")
def case():
    rng = np.random.default_rng(11)
    params = oracle_cnn.init_params(7)
    for s in layer_slices()[1::2]:
        params[s] = 0.05 * rng.standard_normal(s.stop - s.start)
    bits = to_bf16_bits(rng.standard_normal((4, 64, 256, 2)))
    tiles = oracle_cnn.bf16_to_f64(bits)
    labels = (rng.random((4, 32)) < 0.25).astype(np.float64)
    return params, bits, tiles, labels


def test_forward_matches_oracle(gpu, case):
    params, bits, tiles, labels = case
    net = proposal.Cnn(gpu, max_batch=8, seed=1)
    net.set_params(params)
    d_tiles = gpu.array(bits)
    d_logits = gpu.zeros(4 * 32 * 4)
    net.forward(d_tiles.address, 4, d_logits.address, 4 * 32)
    gpu.synchronize()
    got = d_logits.download(np.float32, (4, 32))
    want16, _ = oracle_cnn.forward(params, tiles, bf16=True)
    want64, _ = oracle_cnn.forward(params, tiles)
    assert rel(got, want16) < 2e-3, rel(got, want16)
    assert rel(got, want64) < 2e-2, rel(got, want64)
    assert net.status() == 0
    net.close()


def test_gradients_match_oracle(gpu, case):
    params, bits, tiles, labels = case
    net = proposal.Cnn(gpu, max_batch=8, seed=1)
    net.set_params(params)
    d_tiles = gpu.array(bits)
    net.forward(d_tiles.address, 4)
    logits16, cache16 = oracle_cnn.forward(params, tiles, bf16=True)
    _, dz = oracle_cnn.bce(logits16, labels, 3.0)
    d_dz = gpu.array(dz.astype(np.float32))
    net.backward(d_dz.address, dz.size)
    got = net.grads()
    want16 = oracle_cnn.backward(params, cache16, dz, bf16=True)
    logits64, cache64 = oracle_cnn.forward(params, tiles)
    want64 = oracle_cnn.backward(params, cache64, dz)
    for i, s in enumerate(layer_slices()):
        assert np.linalg.norm(want16[s]) > 0, i
        assert rel(got[s], want16[s]) < 2e-2, (i, rel(got[s], want16[s]))
        assert rel(got[s], want64[s]) < 0.15, (i, rel(got[s], want64[s]))
    assert net.status() == 0
    net.close()


def test_training_step_is_adam_on_the_oracle_gradient(gpu, case):
    """One rv_cnn_train_step: loss equals the oracle's, and the parameter
    update is Adam's first step, lr * sign(g) wherever the gradient is not
    tiny."""
    params, bits, tiles, labels = case
    net = proposal.Cnn(gpu, max_batch=8, seed=1)
    net.set_params(params)
    d_tiles, d_labels = gpu.array(bits), gpu.array(labels.astype(np.float32))
    lr = 1e-3
    loss = net.train_step(d_tiles.address, d_labels.address, 4, proposal.train_config(learning_rate=lr, pos_weight=3.0))
    logits16, cache16 = oracle_cnn.forward(params, tiles, bf16=True)
    want_loss, dz = oracle_cnn.bce(logits16, labels, 3.0)
    assert abs(loss - want_loss) <= 2e-3 * abs(want_loss)
    g = oracle_cnn.backward(params, cache16, dz, bf16=True)
    step = (net.params() - params.astype(np.float32)).astype(np.float64)
    for s in layer_slices():
        big = np.abs(g[s]) > 0.05 * np.abs(g[s]).max()
        np.testing.assert_allclose(step[s][big], -lr * np.sign(g[s][big]), rtol=2e-2, atol=1e-6)
    net.close()


def test_training_learns_a_marked_cell_task(gpu):
    """A few hundred Adam steps on tiles whose labelled cells carry a raised
    band: the loss falls by 10x and the labelled cells come out on top."""
    rng = np.random.default_rng(3)
    n = 64
    tiles = rng.standard_normal((n, 64, 256, 2)).astype(np.float32) * 0.3
    labels = np.zeros((n, 32), np.float32)
    for i in range(n):
        for c in rng.choice(32, size=rng.integers(0, 4), replace=False):
            labels[i, c] = 1
            tiles[i, :, 8 * c:8 * c + 8, :] += 0.8
    net = proposal.Cnn(gpu, max_batch=n, seed=2)
    d_tiles, d_labels = gpu.array(to_bf16_bits(tiles)), gpu.array(labels)
    cfg = proposal.train_config(learning_rate=2e-3, pos_weight=2.0)
    first = net.train_step(d_tiles.address, d_labels.address, n, cfg)
    for _ in range(300):
        last = net.train_step(d_tiles.address, d_labels.address, n, cfg, want_loss=False)
    last = net.train_step(d_tiles.address, d_labels.address, n, cfg)
    assert last < first / 10, (first, last)
    d_logits = gpu.zeros(n * 32 * 4)
    net.forward(d_tiles.address, n, d_logits.address, n * 32)
    gpu.synchronize()
    z = d_logits.download(np.float32, (n, 32))
    assert np.all((z > 0) == (labels > 0))
    assert net.status() == 0
    net.close()


def test_rejects_bad_batches(gpu):
    net = proposal.Cnn(gpu, max_batch=4, seed=1)
    buf = gpu.zeros(8 * 64 * 256 * 2 * 2)
    assert lib().rv_cnn_forward(net.handle, buf.ptr, 5, None, 0) != 0
    assert lib().rv_cnn_forward(net.handle, buf.ptr, 0, None, 0) != 0
    assert lib().rv_cnn_backward(net.handle, buf.ptr, 0) != 0
    net.close()
