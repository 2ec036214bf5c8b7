"""FP64 CPU restatement of the learned proposal's network: forward pass,
weighted binary cross-entropy and the exact backward pass.

TEST INFRASTRUCTURE ONLY. The product's network runs in
revenant_gb300/csrc/cnn.cu on the tensor cores; this module is the checker
its gradients are compared with (tests/test_cnn_oracle.py pins this module
itself against central finite differences, tests/test_gpu_cnn.py compares the
GPU with it). The reference has no learned detector: its detector is
core/detect/detector.cpp, whose candidates label the training tiles, so this
oracle is pinned by the mathematics (finite differences), not by reference
vectors.

The network (NHWC, weights [cout][kh][kw][cin] then biases, layer after
layer, the parameter order of rv_cnn_get_params):
  conv1 4x4 stride 4x4,           2 -> 64, ReLU
  conv2 2x2 stride 2x2,          64 -> 128, ReLU
  conv3 2x3 stride 2x1 pad 0x1, 128 -> 128, ReLU
  conv4 4x3 stride 4x1 pad 0x1, 128 -> 64, ReLU
  head  1x1,                     64 -> 1
on tiles of 64 frames x 256 bins x 2 channels; 32 logits per tile.

With bf16=True every GEMM operand is rounded to BF16 first (round to nearest
even), as the tensor cores see it, while sums stay FP64; the bias gradient is
summed from the unrounded values, as on the GPU.
"""
import numpy as np

LAYERS = [
    # (kh, kw, sh, sw, ph, pw, cin, cout, relu)
    (4, 4, 4, 4, 0, 0, 2, 64, True),
    (2, 2, 2, 2, 0, 0, 64, 128, True),
    (2, 3, 2, 1, 0, 1, 128, 128, True),
    (4, 3, 4, 1, 0, 1, 128, 64, True),
    (1, 1, 1, 1, 0, 0, 64, 1, False),
]


def param_shapes():
    return [((co, kh * kw * ci), (co,)) for kh, kw, sh, sw, ph, pw, ci, co, relu in LAYERS]


def param_count():
    return sum(w[0] * w[1] + b[0] for w, b in param_shapes())


def unpack(params):
    out, at = [], 0
    for (co, k), _ in param_shapes():
        w = params[at:at + co * k].reshape(co, k)
        at += co * k
        b = params[at:at + co]
        at += co
        out.append((w, b))
    return out


def bf16_round(x):
    """Round float64 values to the nearest BF16 (ties to even), via FP32."""
    f = np.asarray(x, np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_to_f64(raw_u16):
    """BF16 bit patterns (uint16) to float64."""
    return (np.asarray(raw_u16, np.uint16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def _out_size(n, k, s, p):
    return (n + 2 * p - k) // s + 1


def patches(x, kh, kw, sh, sw, ph, pw):
    """im2col of NHWC x: [B * HO * WO][kh * kw * C] in (kh, kw, c) order."""
    b, h, w, c = x.shape
    ho, wo = _out_size(h, kh, sh, ph), _out_size(w, kw, sw, pw)
    xp = np.pad(x, ((0, 0), (ph, ph), (pw, pw), (0, 0)))
    cols = np.empty((b, ho, wo, kh, kw, c), x.dtype)
    for i in range(kh):
        for j in range(kw):
            cols[:, :, :, i, j, :] = xp[:, i:i + sh * (ho - 1) + 1:sh, j:j + sw * (wo - 1) + 1:sw, :]
    return cols.reshape(b * ho * wo, kh * kw * c), (ho, wo)


def col2im(cols, shape, kh, kw, sh, sw, ph, pw):
    """Adjoint of patches(): sums patch gradients back onto NHWC `shape`."""
    b, h, w, c = shape
    ho, wo = _out_size(h, kh, sh, ph), _out_size(w, kw, sw, pw)
    g = cols.reshape(b, ho, wo, kh, kw, c)
    xp = np.zeros((b, h + 2 * ph, w + 2 * pw, c), cols.dtype)
    for i in range(kh):
        for j in range(kw):
            xp[:, i:i + sh * (ho - 1) + 1:sh, j:j + sw * (wo - 1) + 1:sw, :] += g[:, :, :, i, j, :]
    return xp[:, ph:ph + h, pw:pw + w, :]


def forward(params, tiles, bf16=False):
    """tiles: [B][64][256][2] float64. Returns (logits [B][32], cache)."""
    rnd = bf16_round if bf16 else (lambda v: v)
    x = np.asarray(tiles, np.float64)
    cache = []
    for (kh, kw, sh, sw, ph, pw, ci, co, relu), (w, b) in zip(LAYERS, unpack(params)):
        cols, (ho, wo) = patches(x, kh, kw, sh, sw, ph, pw)
        y = rnd(cols) @ rnd(w).T + b
        if relu:
            y = np.maximum(y, 0.0)
        cache.append((x.shape, cols))
        x = y.reshape(x.shape[0], ho, wo, co)
    logits = x.reshape(x.shape[0], -1)
    cache.append(logits)
    return logits, cache


def bce(logits, labels, pos_weight):
    """Mean weighted binary cross-entropy and its gradient w.r.t. the logits."""
    z = np.asarray(logits, np.float64)
    t = np.asarray(labels, np.float64)
    soft = np.log1p(np.exp(-np.abs(z)))
    loss = np.mean(pos_weight * t * (soft + np.maximum(-z, 0)) + (1 - t) * (soft + np.maximum(z, 0)))
    s = 1.0 / (1.0 + np.exp(-z))
    dz = (s * (pos_weight * t + 1 - t) - pos_weight * t) / z.size
    return loss, dz


def backward(params, cache, dlogits, bf16=False):
    """Gradient of sum(dlogits * logits) w.r.t. the parameters (flat)."""
    rnd = bf16_round if bf16 else (lambda v: v)
    layers = unpack(params)
    grads = [None] * len(LAYERS)
    dz = np.asarray(dlogits, np.float64).reshape(-1, 1)
    # each layer's post-activation output again, for the ReLU masks
    ys = []
    for li, ((kh, kw, sh, sw, ph, pw, ci, co, relu), (w, b)) in enumerate(zip(LAYERS, layers)):
        shape, cols = cache[li]
        y = rnd(cols) @ rnd(w).T + b
        ys.append(np.maximum(y, 0.0) if relu else y)
    for li in range(len(LAYERS) - 1, -1, -1):
        kh, kw, sh, sw, ph, pw, ci, co, relu = LAYERS[li]
        w, b = layers[li]
        shape, cols = cache[li]
        if relu:
            dz = dz * (ys[li] > 0)
        gw = rnd(dz).T @ rnd(cols)
        gb = dz.sum(axis=0)
        grads[li] = (gw, gb)
        if li > 0:
            dcols = rnd(dz) @ rnd(w)
            dx = col2im(dcols, shape, kh, kw, sh, sw, ph, pw)
            dz = dx.reshape(-1, shape[3])
    outs = []
    for gw, gb in grads:
        outs.append(gw.ravel())
        outs.append(gb.ravel())
    return np.concatenate(outs)


def init_params(seed):
    """He-normal weights, zero biases (numpy's generator; the GPU's own
    initialisation is tested only for its scale)."""
    rng = np.random.default_rng(seed)
    out = []
    for (co, k), (cb,) in param_shapes():
        out.append(rng.standard_normal(co * k) * np.sqrt(2.0 / k))
        out.append(np.zeros(cb))
    return np.concatenate(out)
