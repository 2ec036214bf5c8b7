"""Front-end DC and IQ-imbalance correction against the reference's twins.

The moments and correction kernels (core/dsp/front_end_correction_reference.cpp)
and the host estimator (FrontEndCorrector, core/dsp/front_end_correction.cpp)
must reproduce the reference bit for bit: chunk sums, corrected samples, the
estimate's doubles and the float correction parameters.
"""
import ctypes as C

import numpy as np
import pytest

from bindings import cf32, same_bits
from revenant_gb300 import abi
from revenant_gb300.library import lib


def impaired_ring(n, seed, dc=(0.031, -0.017), gain=1.12, phase_deg=4.0, noise=0.3):
    """A tone plus noise through a front end with DC offset and IQ imbalance."""
    rng = np.random.default_rng(seed)
    t = np.arange(n)
    z = 0.5 * np.exp(2j * np.pi * 0.0123 * t) + noise * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    ph = np.deg2rad(phase_deg)
    i = z.real
    q = gain * (z.imag * np.cos(ph) + z.real * np.sin(ph))
    out = np.zeros((n, 2), np.float32)
    out[:, 0] = (i + dc[0]).astype(np.float32)
    out[:, 1] = (q + dc[1]).astype(np.float32)
    return out


def chunk_sums(kind, ring, offset, count, mask):
    p = abi.IqMomentsParams(mask, offset, count)
    chunks = (count + 63) // 64
    sums = np.zeros(max(chunks * 5, 1), np.float32)
    assert kind.fn("iq_moments")(C.byref(p), ring.ctypes.data, ring.shape[0], sums.ctypes.data, sums.size) == 0
    return sums


@pytest.mark.parametrize("count,offset,log2", [(1, 0, 6), (63, 5, 8), (64, 0, 8), (1000, 900, 10), (65536, 12345, 17)])
def test_moments_and_correct_oracle_vs_reference(ora, ref, count, offset, log2):
    n = 1 << log2
    ring = impaired_ring(n, count + offset)
    mask = n - 1
    assert same_bits(chunk_sums(ora, ring, offset, count, mask), chunk_sums(ref, ring, offset, count, mask))
    p = abi.IqCorrectParams(mask, offset, count, np.float32(0.031), np.float32(-0.017), np.float32(-0.07),
                            np.float32(0.9))
    a, b = ring.copy(), ring.copy()
    assert ora.fn("iq_correct")(C.byref(p), ring.ctypes.data, n, a.ctypes.data, n) == 0
    assert ref.fn("iq_correct")(C.byref(p), ring.ctypes.data, n, b.ctypes.data, n) == 0
    assert same_bits(a, b)


def _sequence(blocks, counts, seed):
    rings, sums = [], []
    for b, count in enumerate(counts):
        ring = impaired_ring(1 << 16, seed + b)
        rings.append(ring)
        sums.append(chunk_sums_np(ring, count))
    stride = max(s.size for s in sums)
    packed = np.zeros((blocks, stride), np.float32)
    for b, s in enumerate(sums):
        packed[b, :s.size] = s
    return packed, stride


def chunk_sums_np(ring, count):
    from bindings import oracle
    return chunk_sums(oracle(), ring, 0, count, ring.shape[0] - 1)


@pytest.mark.parametrize("dc,iq", [(1, 1), (1, 0), (0, 1)])
def test_estimator_oracle_and_library_vs_reference(ora, ref, rv, dc, iq):
    counts = [4096, 65536, 1000, 65536, 32768, 7, 65536, 65536]
    blocks = len(counts)
    packed, stride = _sequence(blocks, counts, 40)
    rate = 2_400_000
    est = (abi.FrontEnd * blocks)()
    corr = (abi.IqCorrectParams * blocks)()
    cnt = np.array(counts, np.uint32)
    assert ref.fn("front_end_sequence")(packed.ctypes.data, stride, cnt.ctypes.data, blocks, rate, dc, iq, est, corr) == 0
    for impl, update, correction in [(ora, ora.lib.or_front_end_update, ora.lib.or_front_end_correction),
                                     (None, lib().rv_front_end_update, lib().rv_front_end_correction)]:
        st = abi.FrontEnd()
        assert lib().rv_front_end_init(C.byref(st)) == 0
        for b in range(blocks):
            row = np.ascontiguousarray(packed[b])
            assert update(C.byref(st), row.ctypes.data, stride, counts[b], rate) == 0
            for name in ("measured", "iq_plausible", "samples_seen", "dc_i", "dc_q", "gain", "sin_phase"):
                assert getattr(st, name) == getattr(est[b], name), (b, name, getattr(st, name), getattr(est[b], name))
            out = abi.IqCorrectParams()
            assert correction(C.byref(st), dc, iq, C.byref(out)) == 0
            for name in ("dc_i", "dc_q", "cross", "scale"):
                assert np.float32(getattr(out, name)).view(np.uint32) == np.float32(getattr(corr[b], name)).view(
                    np.uint32), (b, name)


@pytest.mark.gpu
@pytest.mark.parametrize("count,offset,log2", [(1, 0, 6), (1000, 900, 10), (65536, 12345, 17), (1 << 20, 77, 21)])
def test_gpu_moments_and_correct(gpu, ora, count, offset, log2):
    n = 1 << log2
    mask = n - 1
    ring = impaired_ring(n, count)
    want = chunk_sums(ora, ring, offset, count, mask)
    d_ring = gpu.array(ring)
    d_sums = gpu.zeros(want.nbytes)
    p = abi.IqMomentsParams(mask, offset, count)
    assert lib().rv_iq_moments(gpu.stream, C.byref(p), d_ring.ptr, n, d_sums.ptr, want.size) == 0
    gpu.synchronize()
    assert same_bits(d_sums.download(np.float32, want.shape), want)
    cp = abi.IqCorrectParams(mask, offset, count, np.float32(0.031), np.float32(-0.017), np.float32(-0.07),
                             np.float32(0.9))
    expect = ring.copy()
    assert ora.fn("iq_correct")(C.byref(cp), ring.ctypes.data, n, expect.ctypes.data, n) == 0
    assert lib().rv_iq_correct(gpu.stream, C.byref(cp), d_ring.ptr, n, d_ring.ptr, n) == 0  # in place
    gpu.synchronize()
    assert same_bits(d_ring.download(np.float32, (n, 2)), expect)
