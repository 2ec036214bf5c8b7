"""Fused coarse chain vs the oracle's three-stage chain, bit for bit.

The fused kernel reads the raw staging ring (cs16 or cu8) and writes the
channel ring; the oracle converts the whole ring to cf32, runs the branch
FIR and the FFT with the same offsets. Every word of the channel ring must
agree, including ring wrap, ragged block counts and 32-bit block-index wrap.
"""
import ctypes as C

import numpy as np
import pytest

from bindings import cf32, same_bits
from revenant_gb300 import abi
from revenant_gb300.library import lib

pytestmark = pytest.mark.gpu


def run(status):
    assert status == 0, lib().rv_last_error().decode()


def prototype(M, T, D):
    g = abi.GridParams(M, T, D)
    taps = np.zeros(M * T, np.float32)
    run(lib().rv_design_prototype(C.byref(g), 120.0, taps.ctypes.data, taps.size, None, None))
    tw = np.zeros((M, 2), np.float32)
    run(lib().rv_build_twiddles(M, tw.ctypes.data, M))
    return g, taps, tw


def raw_ring(seed, fmt, n):
    r = np.random.default_rng(seed)
    if fmt == abi.FORMAT_CS16:
        # a few tones plus noise, full 16-bit range exercised
        t = np.arange(n)
        z = 0.3 * np.exp(2j * np.pi * 0.0173 * t) + 0.2 * np.exp(-2j * np.pi * 0.31 * t)
        z = z + 0.05 * (r.standard_normal(n) + 1j * r.standard_normal(n))
        codes = np.empty(2 * n, np.int16)
        codes[0::2] = np.clip(np.round(z.real * 32767), -32768, 32767)
        codes[1::2] = np.clip(np.round(z.imag * 32767), -32768, 32767)
        return codes.view(np.uint8)
    return r.integers(0, 256, 2 * n, dtype=np.uint8)


def oracle_chain(ora, g, fmt, ring_log2, raw, p, taps, tw):
    n = 1 << ring_log2
    ring = cf32(n)
    cp = abi.ConvertParams(n - 1, 0, 0, n)
    assert ora.convert(fmt, cp, raw, ring) == 0
    # the first lead_zero samples of block 0's support read as zero
    start = (p.base_offset - (g.channels * g.taps_per_branch - 1)) & (n - 1)
    for k in range(p.lead_zero):
        ring[(start + k) & (n - 1)] = 0.0
    M = g.channels
    branch = cf32(max(p.block_count, 1) * M)
    bp = abi.PfbBranchParams(n - 1, p.base_offset, p.block_count)
    assert ora.pfb_branch(g, bp, taps, ring, branch[:p.block_count * M]) == 0
    fp = abi.PfbFftParams(M, g.decimation, int(np.log2(M)), p.block_base, p.block_count, p.out_ring_blocks,
                          p.out_ring_mask)
    out = cf32(M * p.out_ring_blocks)
    assert ora.pfb_fft(fp, branch, tw, out) == 0
    return out


CASES = [
    # (M, T, D, fmt, ring_log2, blocks, base_offset, block_base[, lead_zero])
    (64, 17, 32, abi.FORMAT_CS16, 16, 1, 5000, 0),
    (64, 17, 32, abi.FORMAT_CU8, 16, 300, 0, 0, 1087),
    (8, 17, 4, abi.FORMAT_CU8, 14, 500, 40, 10, 95),
    (64, 17, 32, abi.FORMAT_CS16, 16, 33, (1 << 16) - 40, 7),
    (64, 17, 32, abi.FORMAT_CS16, 18, 5000, 123456, 0xFFFFFF00),
    (64, 17, 32, abi.FORMAT_CU8, 18, 7000, 99, 3),
    (8, 17, 4, abi.FORMAT_CU8, 16, 9000, (1 << 16) - 3, 11),
    (8, 17, 4, abi.FORMAT_CS16, 14, 3000, 17, 0),
    (64, 17, 64, abi.FORMAT_CS16, 17, 1500, 4321, 5),
    # grids without a hand-instantiated kernel: the generic one (C2's grid first)
    (1024, 16, 512, abi.FORMAT_CS16, 18, 300, 777, 5),
    (1024, 16, 512, abi.FORMAT_CU8, 18, 257, (1 << 18) - 1000, 0xFFFFFFF0, 16383),
    (128, 17, 64, abi.FORMAT_CU8, 16, 500, 0, 0, 2175),
    (256, 16, 256, abi.FORMAT_CS16, 17, 203, 100, 3),
    (32, 17, 16, abi.FORMAT_CS16, 15, 1000, 9, 1),
]


def describe_mismatch(got, want):
    g, w = got.reshape(-1), want.reshape(-1)
    bad = np.nonzero(g.view(np.uint32) != w.view(np.uint32))[0]
    ulp = np.abs(g.view(np.int32).astype(np.int64) - w.view(np.int32).astype(np.int64))[bad]
    rel = np.abs(g[bad] - w[bad]) / np.maximum(np.abs(w).max(), 1e-30)
    return "%d of %d words differ; first %s; got %s want %s; ulp max %d median %d; rel-to-peak max %.3g" % (
        bad.size, g.size, bad[:4], g[bad[:4]], w[bad[:4]], ulp.max(), np.median(ulp), rel.max())


@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(map(str, c)))
def test_coarse_fused_matches_oracle(gpu, ora, case):
    M, T, D, fmt, ring_log2, blocks, base, block_base = case[:8]
    lead_zero = case[8] if len(case) > 8 else 0
    g, taps, tw = prototype(M, T, D)
    raw = raw_ring(blocks + M, fmt, 1 << ring_log2)
    ring_blocks = 1 << int(np.ceil(np.log2(blocks)))
    p = abi.CoarseParams((1 << ring_log2) - 1, base, blocks, block_base, ring_blocks, ring_blocks - 1, lead_zero)
    want = oracle_chain(ora, g, fmt, ring_log2, raw, p, taps, tw)
    d_raw, d_taps, d_tw = gpu.array(raw), gpu.array(taps), gpu.array(tw)
    d_out = gpu.zeros(M * ring_blocks * 8)
    run(lib().rv_coarse_fused(gpu.stream, C.byref(g), fmt, C.byref(p), d_raw.ptr, raw.nbytes, d_taps.ptr, taps.size,
                              d_tw.ptr, M, d_out.ptr, M * ring_blocks))
    gpu.synchronize()
    got = d_out.download(np.float32, want.shape)
    if not same_bits(got, want):
        # where does it start: compare the GPU plain chain too
        n = 1 << ring_log2
        d_ring, d_branch = gpu.zeros(n * 8), gpu.zeros(blocks * M * 8)
        run(lib().rv_convert(gpu.stream, fmt, C.byref(abi.ConvertParams(n - 1, 0, 0, n)), d_raw.ptr, raw.nbytes,
                             d_ring.ptr, n))
        run(lib().rv_pfb_branch(gpu.stream, C.byref(g), C.byref(abi.PfbBranchParams(n - 1, base, blocks)), d_taps.ptr,
                                taps.size, d_ring.ptr, n, d_branch.ptr, blocks * M))
        d_plain = gpu.zeros(M * ring_blocks * 8)
        fp = abi.PfbFftParams(M, D, int(np.log2(M)), block_base, blocks, ring_blocks, ring_blocks - 1)
        run(lib().rv_pfb_fft(gpu.stream, C.byref(fp), d_branch.ptr, blocks * M, d_tw.ptr, M, d_plain.ptr, M * ring_blocks))
        gpu.synchronize()
        plain = d_plain.download(np.float32, want.shape)
        pytest.fail("fused vs oracle: %s || plain-gpu vs oracle same: %s" % (
            describe_mismatch(got, want), same_bits(plain, want)))


def test_coarse_fused_rejects_and_reports(gpu):
    g, taps, tw = prototype(64, 17, 32)
    raw = np.zeros(4 << 12, np.uint8)
    p = abi.CoarseParams((1 << 12) - 1, 0, 200, 0, 256, 255)  # 200 blocks need more history than 4096
    d_raw, d_taps, d_tw, d_out = gpu.array(raw), gpu.array(taps), gpu.array(tw), gpu.zeros(64 * 256 * 8)
    st = lib().rv_coarse_fused(gpu.stream, C.byref(g), abi.FORMAT_CS16, C.byref(p), d_raw.ptr, raw.nbytes,
                               d_taps.ptr, taps.size, d_tw.ptr, 64, d_out.ptr, 64 * 256)
    assert st == abi.RV_ERR_INVALID and b"history" in lib().rv_last_error()
    # more channels than a CTA has threads: no fused kernel (checked on the
    # host before anything is launched)
    g2 = abi.GridParams(2048, 16, 1024)
    big = gpu.zeros(4 << 16)
    st = lib().rv_coarse_fused(gpu.stream, C.byref(g2), abi.FORMAT_CS16, C.byref(abi.CoarseParams((1 << 16) - 1, 0, 1, 0, 1, 0)),
                               big.ptr, 4 << 16, d_taps.ptr, 2048 * 16, d_tw.ptr, 2048, d_out.ptr, 2048)
    assert st == abi.RV_ERR_UNSUPPORTED


def test_context_outlived_by_buffers(gpu):
    from revenant_gb300.device import Device
    d = Device(0)
    b = d.buffer(1024)
    d.close()  # buffers made from it stay valid to free
    b.free()
