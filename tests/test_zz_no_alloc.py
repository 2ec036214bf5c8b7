"""The allocation-free channelizer entry point, against the allocating one.

rv_pfb_channelize_noalloc serves callers that may not allocate device memory
(per-block processing callbacks; plugins inside a device-memory budget they do
not own): it keeps the branch values in a fixed array inside the library.
Here it is called twice in a row through the C ABI, with different shapes and
inputs, and each result must equal rv_pfb_branch + rv_pfb_fft through a
caller-allocated buffer bit for bit (the same 0-ulp bar as every other GPU
test). This file is collected last, so a run that stops at the first failure
has run everything else first; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import cases
from bindings import same_bits
from revenant_gb300 import abi
from revenant_gb300.library import lib

pytestmark = pytest.mark.gpu


def ok(status):
    assert status == 0, lib().rv_last_error().decode()


def allocating_reference(gpu, g, bp, fp, d_taps, taps, d_ring, ring, d_tw, M, ring_blocks):
    d_branch = gpu.zeros(bp.block_count * M * 8)
    d_out = gpu.zeros(M * ring_blocks * 8)
    ok(lib().rv_pfb_branch(gpu.stream, C.byref(g), C.byref(bp), d_taps.ptr, taps.size, d_ring.ptr, ring.shape[0],
                           d_branch.ptr, bp.block_count * M))
    ok(lib().rv_pfb_fft(gpu.stream, C.byref(fp), d_branch.ptr, bp.block_count * M, d_tw.ptr, M, d_out.ptr,
                        M * ring_blocks))
    gpu.synchronize()
    return d_out.download(np.float32, (M * ring_blocks, 2))


@pytest.mark.parametrize("calls", [[(64, 17, 32, 300, 11), (64, 17, 32, 1000, 12)],
                                   [(8, 17, 4, 5000, 21), (1024, 16, 512, 700, 22)]])
def test_noalloc_matches_allocating_path_twice_in_a_row(gpu, calls):
    for M, T, D, blocks, seed in calls:
        g, bp, taps, ring = cases.branch_case(seed, M, T, D, blocks=blocks)
        tw = np.zeros((M, 2), np.float32)
        ok(lib().rv_build_twiddles(M, tw.ctypes.data, M))
        ring_blocks = 1 << int(np.ceil(np.log2(blocks)))
        fp = abi.PfbFftParams(M, D, int(np.log2(M)), seed * 977, blocks, ring_blocks, ring_blocks - 1)
        d_taps, d_ring, d_tw = gpu.array(taps), gpu.array(ring), gpu.array(tw)
        want = allocating_reference(gpu, g, bp, fp, d_taps, taps, d_ring, ring, d_tw, M, ring_blocks)
        d_out = gpu.zeros(M * ring_blocks * 8)
        ok(lib().rv_pfb_channelize_noalloc(gpu.stream, C.byref(g), C.byref(bp), C.byref(fp), d_taps.ptr, taps.size,
                                           d_ring.ptr, ring.shape[0], d_tw.ptr, M, d_out.ptr, M * ring_blocks))
        gpu.synchronize()
        got = d_out.download(np.float32, (M * ring_blocks, 2))
        assert np.abs(want).max() > 0
        assert same_bits(got, want), "M=%d blocks=%d" % (M, blocks)


@pytest.mark.parametrize("M,T,D,blocks,seed", [(64, 17, 32, 700, 31), (1024, 16, 512, 300, 32)])
def test_noalloc_matches_the_oracle(gpu, ora, M, T, D, blocks, seed):
    """The same calls against the oracle's branch filter and FFT (the CPU
    restatement pinned to the reference's twins), bit for bit."""
    from bindings import cf32
    g, bp, taps, ring = cases.branch_case(seed, M, T, D, blocks=blocks)
    tw = np.zeros((M, 2), np.float32)
    ok(lib().rv_build_twiddles(M, tw.ctypes.data, M))
    ring_blocks = 1 << int(np.ceil(np.log2(blocks)))
    fp = abi.PfbFftParams(M, D, int(np.log2(M)), seed * 131, blocks, ring_blocks, ring_blocks - 1)
    branch = cf32(blocks * M)
    assert ora.pfb_branch(g, bp, taps, ring, branch) == 0
    want = cf32(M * ring_blocks)
    assert ora.pfb_fft(fp, branch, tw, want) == 0
    d_taps, d_ring, d_tw = gpu.array(taps), gpu.array(ring), gpu.array(tw)
    d_out = gpu.zeros(M * ring_blocks * 8)
    for _ in range(2):
        ok(lib().rv_pfb_channelize_noalloc(gpu.stream, C.byref(g), C.byref(bp), C.byref(fp), d_taps.ptr, taps.size,
                                           d_ring.ptr, ring.shape[0], d_tw.ptr, M, d_out.ptr, M * ring_blocks))
        gpu.synchronize()
        assert same_bits(d_out.download(np.float32, (M * ring_blocks, 2)), want)


def test_noalloc_refuses_requests_beyond_its_scratch(gpu):
    M = 64
    g, bp, taps, ring = cases.branch_case(5, M, 17, 32, blocks=2)
    blocks = abi_max = (1 << 20) // M + 1
    bp = abi.PfbBranchParams(bp.ring_mask, bp.base_offset, blocks)
    fp = abi.PfbFftParams(M, 32, 6, 0, blocks, 1 << 15, (1 << 15) - 1)
    d_taps, d_ring = gpu.array(taps), gpu.array(ring)
    d_tw = gpu.zeros(M * 8)
    d_out = gpu.zeros(8)
    st = lib().rv_pfb_channelize_noalloc(gpu.stream, C.byref(g), C.byref(bp), C.byref(fp), d_taps.ptr, taps.size,
                                         d_ring.ptr, ring.shape[0], d_tw.ptr, M, d_out.ptr, 1)
    assert st == abi.RV_ERR_INVALID
    assert b"scratch" in lib().rv_last_error()
    assert abi_max * M > (1 << 20)
