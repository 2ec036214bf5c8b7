"""C4: an M = 4096 polyphase channelizer (D = 2048, T = 16) over a seeded
multitone (64 tones, amplitudes log-uniform over 90 dB, on and off bin
centres) in noise. M = 4096 is past the reference's channel cap
(kMaxChannels = 2048, core/dsp/pfb_design.cpp:67), so there is no twin: the
wide entry points run the reference's channelizer arithmetic (prototype,
branch FIR, radix-2 DIT FFT with the phase correction) at the wider grid, and
are checked

  * bit for bit against the FP32 oracle restated for wide grids, and
  * against an FP64 restatement (direct DFT, oracle/oracle.c or_pfb_f64):
    REL_RMS = 2e-6 relative RMS of the channel outputs over all channels, and
    SPUR_DBC = -110 dB for the worst single output error against the
    strongest output (the spur floor the FP32 arithmetic leaves).

The split-precision DFT on the tensor cores (rv_pfb_dft_tc: the four-step
64 x 64 factorisation as two tcgen05 GEMM stages, operands split hi + lo in
FP16 or in BF16, FP32 accumulators in tensor memory) is checked against the
same FP64 restatement, to its own stated tolerances:

  * FP16 split: TC_FP16 = (relative RMS 2e-6, spur floor -115 dBc)
  * BF16 split: TC_BF16 = (relative RMS 2e-5, spur floor -105 dBc)

(measured on a GB300: 4.8e-7 / -125.8 dBc and 4.6e-6 / -116.9 dBc, against
1.6e-7 / -139 dBc for the FP32 FFT).
"""
import ctypes as C

import numpy as np
import pytest

from bindings import cf32, oracle, same_bits
from revenant_gb300 import abi
from revenant_gb300.library import lib

M, T, D = 4096, 16, 2048
REL_RMS = 2e-6
SPUR_DBC = -110.0
TC_FP16 = (2e-6, -115.0)
TC_BF16 = (2e-5, -105.0)


def prototype():
    g = abi.GridParams(M, T, D)
    taps = np.zeros(M * T, np.float32)
    stop = C.c_double()
    assert lib().rv_design_prototype_wide(C.byref(g), 120.0, taps.ctypes.data, taps.size, C.byref(stop), None) == 0, \
        lib().rv_last_error()
    return g, taps, stop.value


def twiddles():
    tw = cf32(M)
    assert lib().rv_build_fft_twiddles(M, tw.ctypes.data, M) == 0
    return tw


def multitone(n, seed=4):
    rng = np.random.default_rng(seed)
    t = np.arange(n)
    z = 10 ** (-5) * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    for k in range(64):
        amp = 10 ** (-rng.uniform(0, 90) / 20)
        centre = rng.integers(-M // 2, M // 2) / M
        f = centre + (0.0 if k % 2 else rng.uniform(-0.4, 0.4) / M)
        z += 0.3 * amp * np.exp(2j * np.pi * (f * t + rng.uniform()))
    ring = np.zeros((n, 2), np.float32)
    ring[:, 0], ring[:, 1] = z.real, z.imag
    return ring


def oracle_fp32(g, taps, tw, ring, base_block, blocks, ring_blocks):
    o = oracle()
    branch = cf32(blocks * M)
    bp = abi.PfbBranchParams(ring.shape[0] - 1, base_block * D, blocks)
    assert o.lib.or_pfb_branch_wide(C.byref(g), C.byref(bp), taps.ctypes.data, taps.size, ring.ctypes.data,
                                    ring.shape[0], branch.ctypes.data, branch.shape[0]) == 0, o.error()
    chan = cf32(M * ring_blocks)
    fp = abi.PfbFftParams(M, D, 12, base_block, blocks, ring_blocks, ring_blocks - 1)
    assert o.pfb_fft(fp, branch, tw, chan) == 0, o.error()
    return chan


def fp64(g, taps, ring, base_block, blocks):
    re = np.zeros(M * blocks)
    im = np.zeros(M * blocks)
    assert oracle().lib.or_pfb_f64(C.byref(g), taps.ctypes.data, ring.ctypes.data, ring.shape[0] - 1, base_block * D,
                                   blocks, base_block, re.ctypes.data, im.ctypes.data) == 0
    return (re + 1j * im).reshape(M, blocks)


def check_tolerance(chan32, want, blocks, ring_blocks, first_slot):
    got = chan32.reshape(M, ring_blocks, 2)[:, first_slot:first_slot + blocks]
    got = got[..., 0].astype(np.float64) + 1j * got[..., 1]
    err = got - want
    rel = np.sqrt(np.mean(np.abs(err) ** 2) / np.mean(np.abs(want) ** 2))
    spur = 20 * np.log10(np.max(np.abs(err)) / np.max(np.abs(want)))
    return rel, spur


def test_wide_prototype_matches_the_capped_design(rv):
    """At M <= 2048 the wide designer is the reference's design_prototype."""
    g = abi.GridParams(1024, 16, 512)
    a, b = np.zeros(1024 * 16, np.float32), np.zeros(1024 * 16, np.float32)
    assert rv.rv_design_prototype(C.byref(g), 120.0, a.ctypes.data, a.size, None, None) == 0
    assert rv.rv_design_prototype_wide(C.byref(g), 120.0, b.ctypes.data, b.size, None, None) == 0
    assert same_bits(a, b)
    g4, taps, stop = prototype()
    assert abs(float(taps.astype(np.float64).sum()) - 1.0) < 1e-5 and stop < -100.0
    # the capped entry points still refuse M = 4096, as the reference does
    assert rv.rv_design_prototype(C.byref(g4), 120.0, taps.ctypes.data, taps.size, None, None) == abi.RV_ERR_INVALID


def test_oracle_fp32_within_tolerance_of_fp64():
    g, taps, _ = prototype()
    tw = twiddles()
    ring = multitone(1 << 17)
    base, blocks = M * T // D, 3
    chan = oracle_fp32(g, taps, tw, ring, base, blocks, 4)
    rel, spur = check_tolerance(chan, fp64(g, taps, ring, base, blocks), blocks, 4, base & 3)
    print("C4 oracle FP32 vs FP64: relative RMS %.2e, spur floor %.1f dBc" % (rel, spur))
    assert rel <= REL_RMS and spur <= SPUR_DBC


@pytest.mark.gpu
def test_gpu_c4_channelizer(gpu):
    g, taps, _ = prototype()
    tw = twiddles()
    n = 1 << 20
    ring = multitone(n)
    base, blocks, ring_blocks = M * T // D, 256, 512
    bp = abi.PfbBranchParams(n - 1, base * D, blocks)
    d_ring, d_taps, d_tw = gpu.array(ring), gpu.array(taps), gpu.array(tw)
    d_branch = gpu.zeros(blocks * M * 8)
    d_chan = gpu.zeros(M * ring_blocks * 8)
    assert lib().rv_pfb_branch_wide(gpu.stream, C.byref(g), C.byref(bp), d_taps.ptr, taps.size, d_ring.ptr, n,
                                    d_branch.ptr, blocks * M) == 0, lib().rv_last_error()
    fp = abi.PfbFftParams(M, D, 12, base, blocks, ring_blocks, ring_blocks - 1)
    assert lib().rv_pfb_fft(gpu.stream, C.byref(fp), d_branch.ptr, blocks * M, d_tw.ptr, M, d_chan.ptr,
                            M * ring_blocks) == 0, lib().rv_last_error()
    gpu.synchronize()
    got = d_chan.download(np.float32, (M * ring_blocks, 2))
    # bit for bit against the FP32 oracle on a slice of blocks
    want = oracle_fp32(g, taps, tw, ring, base, 8, ring_blocks)
    sl = got.reshape(M, ring_blocks, 2)[:, base:base + 8]
    assert same_bits(sl, want.reshape(M, ring_blocks, 2)[:, base:base + 8])
    # and to the stated tolerance against FP64
    rel, spur = check_tolerance(got, fp64(g, taps, ring, base, 3), 3, ring_blocks, base)
    print("C4 GPU vs FP64: relative RMS %.2e, spur floor %.1f dBc" % (rel, spur))
    assert rel <= REL_RMS and spur <= SPUR_DBC


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_gpu_c4_tensor_core_dft(gpu, precision):
    """rv_pfb_dft_tc against FP64 at its stated tolerance."""
    prec, (rel_max, spur_max) = (abi.DFT_FP16, TC_FP16) if precision == "fp16" else (abi.DFT_BF16, TC_BF16)
    g, taps, _ = prototype()
    tw = twiddles()
    n = 1 << 20
    ring = multitone(n, seed=7)
    d_ring, d_taps, d_tw = gpu.array(ring), gpu.array(taps), gpu.array(tw)
    # 256 blocks (128 tiles over the SMs), then an odd count (a half tile)
    # whose checked blocks wrap an 8-block ring (slots 6, 7, 0)
    for base, blocks, ring_blocks in ((M * T // D, 256, 512), (38, 5, 8)):
        checked = 3
        bp = abi.PfbBranchParams(n - 1, base * D, blocks)
        d_branch = gpu.zeros(blocks * M * 8)
        d_chan = gpu.zeros(M * ring_blocks * 8)
        assert lib().rv_pfb_branch_wide(gpu.stream, C.byref(g), C.byref(bp), d_taps.ptr, taps.size, d_ring.ptr, n,
                                        d_branch.ptr, blocks * M) == 0, lib().rv_last_error()
        fp = abi.PfbFftParams(M, D, 12, base, blocks, ring_blocks, ring_blocks - 1)
        assert lib().rv_pfb_dft_tc(gpu.stream, C.byref(fp), d_branch.ptr, blocks * M, d_tw.ptr, M, d_chan.ptr,
                                   M * ring_blocks, prec) == 0, lib().rv_last_error()
        timeouts = C.c_uint32(7)
        assert lib().rv_pfb_dft_tc_status(gpu.stream, C.byref(timeouts)) == 0 and timeouts.value == 0
        got = d_chan.download(np.float32, (M * ring_blocks, 2)).reshape(M, ring_blocks, 2)
        slots = [(base + b) & (ring_blocks - 1) for b in range(checked)]
        rel, spur = check_tolerance(got[:, slots].reshape(-1, 2), fp64(g, taps, ring, base, checked), checked,
                                    checked, 0)
        print("C4 tensor-core DFT (%s split) vs FP64, %d blocks: relative RMS %.2e, spur floor %.1f dBc"
              % (precision, blocks, rel, spur))
        assert rel <= rel_max and spur <= spur_max


@pytest.mark.gpu
def test_gpu_c4_tensor_core_dft_stop_path(gpu):
    """The stop path of rv_pfb_dft_tc's bounded waits, without making one run
    out: the test hook stops every CTA before it issues a copy or an MMA, the
    status call then reports RV_ERR_TIMEOUT with one count per CTA and clears
    it, the ring is left untouched, and the next call is bit-identical to one
    made before the stop."""
    g, taps, _ = prototype()
    tw = twiddles()
    n = 1 << 18
    ring = multitone(n, seed=9)
    d_ring, d_taps, d_tw = gpu.array(ring), gpu.array(taps), gpu.array(tw)
    blocks, ring_blocks, base = 64, 64, M * T // D
    bp = abi.PfbBranchParams(n - 1, base * D, blocks)
    d_branch = gpu.zeros(blocks * M * 8)
    assert lib().rv_pfb_branch_wide(gpu.stream, C.byref(g), C.byref(bp), d_taps.ptr, taps.size, d_ring.ptr, n,
                                    d_branch.ptr, blocks * M) == 0, lib().rv_last_error()
    fp = abi.PfbFftParams(M, D, 12, base, blocks, ring_blocks, ring_blocks - 1)
    d_before, d_stopped, d_after = (gpu.zeros(M * ring_blocks * 8) for _ in range(3))

    def call(d_chan):
        assert lib().rv_pfb_dft_tc(gpu.stream, C.byref(fp), d_branch.ptr, blocks * M, d_tw.ptr, M, d_chan.ptr,
                                   M * ring_blocks, abi.DFT_BF16) == 0, lib().rv_last_error()

    timeouts = C.c_uint32(0)
    call(d_before)
    assert lib().rv_pfb_dft_tc_status(gpu.stream, C.byref(timeouts)) == 0 and timeouts.value == 0
    assert lib().rv_pfb_dft_tc_stop_for_test(gpu.stream, 1) == 0
    try:
        call(d_stopped)
        assert lib().rv_pfb_dft_tc_status(gpu.stream, C.byref(timeouts)) == abi.RV_ERR_TIMEOUT
        ctas = min(blocks // 2, gpu.info.sm_count)
        assert timeouts.value == ctas, (timeouts.value, ctas)
    finally:
        assert lib().rv_pfb_dft_tc_stop_for_test(gpu.stream, 0) == 0
    assert lib().rv_pfb_dft_tc_status(gpu.stream, C.byref(timeouts)) == 0 and timeouts.value == 0
    assert not np.any(d_stopped.download(np.uint32, (M * ring_blocks * 2,)))
    call(d_after)
    assert lib().rv_pfb_dft_tc_status(gpu.stream, C.byref(timeouts)) == 0
    before = d_before.download(np.uint32, (M * ring_blocks * 2,))
    after = d_after.download(np.uint32, (M * ring_blocks * 2,))
    assert np.array_equal(before, after)


def test_tensor_core_dft_rejects_other_grids(rv):
    fp = abi.PfbFftParams(2048, 1024, 11, 0, 4, 4, 3)
    assert rv.rv_pfb_dft_tc(None, C.byref(fp), None, 0, None, 0, None, 0, abi.DFT_FP16) == abi.RV_ERR_INVALID
    one = np.zeros(2, np.float32)
    p = one.ctypes.data
    assert rv.rv_pfb_dft_tc(None, C.byref(fp), p, 1 << 30, p, 2048, p, 1 << 30, abi.DFT_FP16) == abi.RV_ERR_UNSUPPORTED
    fp = abi.PfbFftParams(M, D, 12, 0, 4, 4, 3)
    assert rv.rv_pfb_dft_tc(None, C.byref(fp), p, 1 << 30, p, M, p, 1 << 30, 7) == abi.RV_ERR_INVALID
    assert rv.rv_pfb_dft_tc(None, C.byref(fp), p, 1 << 30, p, 100, p, 1 << 30, abi.DFT_FP16) == abi.RV_ERR_INVALID
