"""Pins the oracle (oracle/oracle.c) to the reference's own CPU twins.

Every case runs the same bytes through the reference twin compiled from the
reference sources (oracle/_ref/libreftwins.so) and through the restatement,
and demands bit-identical output: the reference's conformance bar
(tests/reference/reference_diff.h:98-152, 0 ulp). Skips where the reference
sources are absent (the committed fixtures in tests/golden pin the oracle
there instead).
"""
import numpy as np
import pytest

from bindings import cf32, same_bits
import cases
from revenant_gb300 import abi


def test_det_functions_bitwise(ora, ref):
    r = np.random.default_rng(11)
    vals = np.concatenate([
        r.uniform(1e-6, 10, 20000), r.uniform(1e-30, 1e-20, 2000), r.uniform(1, 1e30, 2000),
        np.array([1.0, 2.0, 0.5, 1.41421356, 3.0, 1e-20, 65504.0])]).astype(np.float32)
    for name in ("det_rsqrt", "det_sqrt", "det_recip", "det_log2"):
        a = np.array([ora.det(name, float(v)) for v in vals], np.float32)
        b = np.array([ref.det(name, float(v)) for v in vals], np.float32)
        assert same_bits(a, b), name
    ys = r.standard_normal(20000).astype(np.float32)
    xs = r.standard_normal(20000).astype(np.float32)
    ys[:4] = [0, 0, 1, -1]
    xs[:4] = [0, -1, 0, 0]
    a = np.array([ora.det("det_atan2", float(y), float(x)) for y, x in zip(ys, xs)], np.float32)
    b = np.array([ref.det("det_atan2", float(y), float(x)) for y, x in zip(ys, xs)], np.float32)
    assert same_bits(a, b)


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
@pytest.mark.parametrize("seed", [1, 2])
def test_convert_bitwise(ora, ref, fmt, seed):
    p, packed = cases.convert_case(seed, fmt, 3001, ring_log2=12)
    a, b = cf32(4096), cf32(4096)
    assert ora.convert(fmt, p, packed, a) == 0, ora.error()
    assert ref.convert(fmt, p, packed, b) == 0, ref.error()
    assert same_bits(a, b)


def test_convert_exhaustive_codes(ora, ref):
    # every cu8/cs8 code pair position and every cs16 code (test_convert.cpp:122-240)
    for fmt, n in ((0, 65536), (1, 65536), (2, 65536)):
        if fmt == 2:
            codes = np.arange(65536, dtype=np.uint32)
            packed = (codes | (((codes * 7919) & 0xFFFF) << 16)).astype(np.uint32).view(np.uint8)
        else:
            codes = np.arange(65536, dtype=np.uint32)
            packed = codes.astype(np.uint16).view(np.uint8)
            packed = np.concatenate([packed, np.zeros(4, np.uint8)])
        p = abi.ConvertParams()
        p.ring_mask, p.dst_offset, p.src_offset, p.count = 65535, 12345, 0, n
        a, b = cf32(65536), cf32(65536)
        assert ora.convert(fmt, p, packed, a) == 0
        assert ref.convert(fmt, p, packed, b) == 0
        assert same_bits(a, b)


def test_convert_rejects_like_reference(ora, ref):
    p, packed = cases.convert_case(3, 2, 100, ring_log2=6)  # 100 samples into 64 slots
    a = cf32(64)
    assert ora.convert(2, p, packed, a) != 0
    assert ref.convert(2, p, packed, a) != 0
    p, packed = cases.convert_case(3, 0, 100, ring_log2=8)
    assert ora.convert(0, p, packed[:-8], cf32(256)) != 0
    assert ref.convert(0, p, packed[:-8], cf32(256)) != 0


@pytest.mark.parametrize("M,T,D", cases.GRIDS)
@pytest.mark.parametrize("wrap", [True, False])
def test_pfb_branch_bitwise(ora, ref, M, T, D, wrap):
    g, p, taps, ring = cases.branch_case(M * 7 + T, M, T, D, blocks=9, wrap=wrap)
    a, b = cf32(9 * M), cf32(9 * M)
    assert ora.pfb_branch(g, p, taps, ring, a) == 0, ora.error()
    assert ref.pfb_branch(g, p, taps, ring, b) == 0, ref.error()
    assert same_bits(a, b)


@pytest.mark.parametrize("M,T,D", cases.GRIDS)
def test_pfb_fft_bitwise(ora, ref, M, T, D):
    tw = np.zeros((M, 2), np.float32)
    assert ref.lib.ref_build_twiddles(M, tw.ctypes.data, M) == 0
    for base in (0, 0xFFFFFFFD, 12345):
        p, branch = cases.fft_case(M + base % 97, M, D, blocks=6, ring_blocks=8, block_base=base)
        a, b = cf32(M * 8), cf32(M * 8)
        assert ora.pfb_fft(p, branch, tw, a) == 0, ora.error()
        assert ref.pfb_fft(p, branch, tw, b) == 0, ref.error()
        assert same_bits(a, b)


def test_pfb_fft_rejects_overrun(ora, ref):
    p, branch = cases.fft_case(5, 64, 32, blocks=9, ring_blocks=8)
    tw = cases.twiddles64(64)
    assert ora.pfb_fft(p, branch, tw, cf32(64 * 8)) != 0
    assert ref.pfb_fft(p, branch, tw, cf32(64 * 8)) != 0


@pytest.mark.parametrize("M,N", [(8, 64), (64, 256), (4, 2048)])
def test_spectrum_bitwise(ora, ref, M, N):
    tw = np.zeros((N, 2), np.float32)
    assert ref.lib.ref_build_twiddles(N, tw.ctypes.data, N) == 0
    win = np.zeros(N + N // 2, np.float32)
    assert ref.lib.ref_build_spectrum_window(N, 17, 120.0, win.ctypes.data, win.size) == 0
    p, ring = cases.spectrum_case(N + M, M, N)
    a = np.zeros(M * N // 2, np.float32)
    b = np.zeros(M * N // 2, np.float32)
    assert ora.spectrum(p, ring, tw, win, a) == 0, ora.error()
    assert ref.spectrum(p, ring, tw, win, b) == 0, ref.error()
    assert same_bits(a, b)


def test_spectrum_levels_bitwise(ora, ref):
    r = np.random.default_rng(4)
    for bins in (1, 999, 1000, 65536):
        frame = r.uniform(-220, 60, bins).astype(np.float32)
        p = abi.SpectrumLevelsParams()
        p.bins, p.low_permille, p.high_permille = bins, 50, 990
        a, b = np.zeros(2, np.float32), np.zeros(2, np.float32)
        assert ora.spectrum_levels(p, frame, a) == 0
        assert ref.spectrum_levels(p, frame, b) == 0
        assert same_bits(a, b)


def _nco(ref_or_none, log2=16):
    t = np.zeros((1 << log2, 2), np.float32)
    ref_or_none.lib.ref_build_nco_table(log2, t.ctypes.data, 1 << log2)
    return t


@pytest.mark.parametrize("T,P,in_rate,out_rate", [(32, 256, 300000, 240000), (256, 256, 625000, 48000),
                                                  (33, 256, 625000, 336000), (8, 1, 1000, 1000)])
def test_vrx_fine_bitwise(ora, ref, T, P, in_rate, out_rate):
    r = np.random.default_rng(T + P)
    cfg = abi.VrxFineConfig()
    cfg.taps, cfg.phases, cfg.nco_log2 = T, P, 16
    taps = (r.standard_normal((P * T + 1, 2)) * 0.05).astype(np.float32)
    nco = _nco(ref)
    for first in (0, 10 ** 12 + 7):
        p, chan = cases.fine_case(T * 31 + first % 7, cfg, taps, nco, out_rate, in_rate, 700, first)
        a, b = cf32(p.out_mask + 1), cf32(p.out_mask + 1)
        assert ora.vrx_fine(cfg, p, chan, taps, nco, a) == 0, ora.error()
        assert ref.vrx_fine(cfg, p, chan, taps, nco, b) == 0, ref.error()
        assert same_bits(a, b)


DEMOD_CASES = [
    dict(mode="nfm", decimation=1, audio_taps=31),
    dict(mode="wfm", decimation=7, audio_taps=87),
    dict(mode="wfm", decimation=7, audio_taps=87, channels=2, pilot_taps=49),
    dict(mode="am", decimation=3, audio_taps=41, dc_taps=64),
    dict(mode="sam", decimation=3, audio_taps=41, dc_taps=64),
    dict(mode="usb", decimation=2, audio_taps=21),
    dict(mode="lsb", decimation=2, audio_taps=21),
    dict(mode="cw", decimation=1, audio_taps=15),
    dict(mode="dsb", decimation=1, audio_taps=15),
    dict(mode="raw", decimation=1, audio_taps=1, channels=2),
    dict(mode="p25p1", decimation=1, audio_taps=1, channels=2),
]


@pytest.mark.parametrize("kw", DEMOD_CASES, ids=lambda kw: "%s-%d" % (kw["mode"], kw.get("channels", 1)))
def test_vrx_demod_bitwise(ora, ref, kw):
    r = np.random.default_rng(hash(kw["mode"]) & 0xFFFF)
    cfg = cases.demod_config(**kw)
    w = cases.demod_weights(r, cfg)
    fine = cases.fm_fine_ring(r, 4096, pilot=0.1) if kw["mode"] in ("nfm", "wfm") else cases.am_fine_ring(r, 4096)
    p = abi.VrxDemodParams()
    p.in_mask, p.count, p.gain = 4095, 200, 1.7
    p.in_offset = 4000  # wraps
    a = np.zeros(200 * cfg.channels, np.float32)
    b = np.zeros(200 * cfg.channels, np.float32)
    assert ora.vrx_demod(cfg, p, fine, w, a) == 0, ora.error()
    assert ref.vrx_demod(cfg, p, fine, w, b) == 0, ref.error()
    assert same_bits(a, b)


@pytest.mark.parametrize("power", [1, 2])
def test_vrx_carrier_bitwise(ora, ref, power):
    r = np.random.default_rng(power)
    nco = _nco(ref)
    fine = cases.am_fine_ring(r, 4096)
    # offset carrier so the loop has something to pull in
    t = np.arange(4096)
    z = (fine[:, 0] + 1j * fine[:, 1]) * np.exp(1j * 0.01 * t)
    fine = np.stack([z.real, z.imag], 1).astype(np.float32)
    cfg, p = cases.carrier_params(power=power, count=3000, in_offset=3000)
    sa = np.zeros(8, np.uint32)
    sb = np.zeros(8, np.uint32)
    a, b = fine.copy(), fine.copy()
    for step in range(3):
        p.flags = 1 if step == 0 else 0
        p.shift = 0.0 if step != 2 else 0.001
        p.in_offset = (3000 + step * 3000) & 4095
        assert ora.vrx_carrier(cfg, p, nco, a, sa) == 0, ora.error()
        assert ref.vrx_carrier(cfg, p, nco, b, sb) == 0, ref.error()
        assert same_bits(a, b)
        assert np.array_equal(sa, sb)
