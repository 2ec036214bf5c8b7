"""GPU plain kernels vs the oracle, bit for bit (the reference's 0-ulp bar).

Each case builds seeded inputs, runs the kernel through the C ABI on the
device, runs the oracle on the host, and compares every output word. Cases
cover every grid the chain uses, ring wrap offsets, block counts that do not
divide launch shapes, long-stream indices and every demodulator mode.
"""
import ctypes as C

import numpy as np
import pytest

import cases
from bindings import cf32, same_bits
from revenant_gb300 import abi
from revenant_gb300.library import lib

pytestmark = pytest.mark.gpu


def run(status):
    assert status == 0, lib().rv_last_error().decode()


def test_device_info(gpu):
    assert gpu.info.cc_major >= 10
    assert gpu.info.sm_count > 0


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
@pytest.mark.parametrize("count,ring_log2", [(1, 4), (3001, 12), (4096, 12), (100003, 17)])
def test_convert(gpu, ora, fmt, count, ring_log2):
    p, packed = cases.convert_case(count + fmt, fmt, count, ring_log2=ring_log2)
    n = 1 << ring_log2
    want = cf32(n)
    assert ora.convert(fmt, p, packed, want) == 0
    src = gpu.array(packed)
    ring = gpu.zeros(n * 8)
    run(lib().rv_convert(gpu.stream, fmt, C.byref(p), src.ptr, packed.nbytes, ring.ptr, n))
    gpu.synchronize()
    assert same_bits(ring.download(np.float32, (n, 2)), want)


def test_convert_rejects_short_source(gpu):
    p, packed = cases.convert_case(1, 2, 100, ring_log2=8)
    src = gpu.array(packed)
    ring = gpu.zeros(256 * 8)
    assert lib().rv_convert(gpu.stream, 2, C.byref(p), src.ptr, packed.nbytes - 4, ring.ptr, 256) == abi.RV_ERR_INVALID


@pytest.mark.parametrize("M,T,D", cases.GRIDS)
@pytest.mark.parametrize("blocks", [1, 9, 257])
def test_pfb_branch(gpu, ora, M, T, D, blocks):
    g, p, taps, ring = cases.branch_case(M + T + blocks, M, T, D, blocks=blocks)
    want = cf32(blocks * M)
    assert ora.pfb_branch(g, p, taps, ring, want) == 0
    dt, dr, out = gpu.array(taps), gpu.array(ring), gpu.zeros(blocks * M * 8)
    run(lib().rv_pfb_branch(gpu.stream, C.byref(g), C.byref(p), dt.ptr, taps.size, dr.ptr, ring.shape[0],
                            out.ptr, blocks * M))
    gpu.synchronize()
    assert same_bits(out.download(np.float32, (blocks * M, 2)), want)


def _twiddles(M):
    tw = np.zeros((M, 2), np.float32)
    run(lib().rv_build_twiddles(M, tw.ctypes.data, M))
    return tw


@pytest.mark.parametrize("M,T,D", cases.GRIDS + [(2, 1, 1), (2048, 4, 1024)])
@pytest.mark.parametrize("blocks,base", [(1, 0), (13, 0xFFFFFFF0), (300, 777)])
def test_pfb_fft(gpu, ora, M, T, D, blocks, base):
    tw = _twiddles(M)
    ring_blocks = 1 << int(np.ceil(np.log2(blocks)))
    p, branch = cases.fft_case(M + blocks, M, D, blocks, ring_blocks=ring_blocks, block_base=base)
    want = cf32(M * ring_blocks)
    assert ora.pfb_fft(p, branch, tw, want) == 0
    db, dtw, ring = gpu.array(branch), gpu.array(tw), gpu.zeros(M * ring_blocks * 8)
    run(lib().rv_pfb_fft(gpu.stream, C.byref(p), db.ptr, branch.shape[0], dtw.ptr, M, ring.ptr, M * ring_blocks))
    gpu.synchronize()
    assert same_bits(ring.download(np.float32, (M * ring_blocks, 2)), want)


@pytest.mark.parametrize("M,N", [(8, 64), (64, 256), (64, 2048), (1024, 8)])
def test_spectrum(gpu, ora, M, N):
    tw = _twiddles(N)
    win = np.zeros(N + N // 2, np.float32)
    run(lib().rv_build_spectrum_window(N, 17, 120.0, win.ctypes.data, win.size))
    p, ring = cases.spectrum_case(M * N, M, N)
    want = np.zeros(M * N // 2, np.float32)
    assert ora.spectrum(p, ring, tw, win, want) == 0
    dr, dtw, dw, fr = gpu.array(ring), gpu.array(tw), gpu.array(win), gpu.zeros(want.nbytes)
    run(lib().rv_spectrum(gpu.stream, C.byref(p), dr.ptr, ring.shape[0], dtw.ptr, N, dw.ptr, win.size, fr.ptr,
                          want.size))
    gpu.synchronize()
    assert same_bits(fr.download(np.float32, want.shape), want)


@pytest.mark.parametrize("bins", [1, 999, 65536])
def test_spectrum_levels(gpu, ora, bins):
    frame = np.random.default_rng(bins).uniform(-230, 60, bins).astype(np.float32)
    p = abi.SpectrumLevelsParams(bins, 50, 990)
    want = np.zeros(2, np.float32)
    assert ora.spectrum_levels(p, frame, want) == 0
    df, lv = gpu.array(frame), gpu.zeros(8)
    run(lib().rv_spectrum_levels(gpu.stream, C.byref(p), df.ptr, bins, lv.ptr))
    gpu.synchronize()
    assert same_bits(lv.download(np.float32, 2), want)


def _nco():
    t = np.zeros((1 << 16, 2), np.float32)
    run(lib().rv_build_nco_table(16, t.ctypes.data, 1 << 16))
    return t


@pytest.mark.parametrize("T,P,in_rate,out_rate", [(32, 256, 300000, 240000), (256, 256, 625000, 48000),
                                                  (33, 256, 625000, 336000), (33, 256, 625000, 432000),
                                                  (8, 1, 1000, 1000)])
@pytest.mark.parametrize("first", [0, 3 * 3600 * 48000 + 11])
def test_vrx_fine(gpu, ora, T, P, in_rate, out_rate, first):
    r = np.random.default_rng(T + P + first % 101)
    cfg = abi.VrxFineConfig(T, P, 16)
    taps = (r.standard_normal((P * T + 1, 2)) * 0.05).astype(np.float32)
    nco = _nco()
    p, chan = cases.fine_case(T + first % 7, cfg, taps, nco, out_rate, in_rate, 3000, first)
    want = cf32(p.out_mask + 1)
    assert ora.vrx_fine(cfg, p, chan, taps, nco, want) == 0
    dc, dt, dn, out = gpu.array(chan), gpu.array(taps), gpu.array(nco), gpu.zeros((p.out_mask + 1) * 8)
    run(lib().rv_vrx_fine(gpu.stream, C.byref(cfg), C.byref(p), dc.ptr, chan.shape[0], dt.ptr, taps.shape[0],
                          dn.ptr, nco.shape[0], out.ptr, p.out_mask + 1))
    gpu.synchronize()
    assert same_bits(out.download(np.float32, want.shape), want)


DEMODS = [
    dict(mode="nfm", decimation=1, audio_taps=31),
    dict(mode="wfm", decimation=7, audio_taps=878),
    dict(mode="wfm", decimation=7, audio_taps=878, channels=2, pilot_taps=485),
    dict(mode="am", decimation=9, audio_taps=453, dc_taps=2160),
    dict(mode="sam", decimation=3, audio_taps=41, dc_taps=240),
    dict(mode="usb", decimation=1, audio_taps=1),
    dict(mode="lsb", decimation=2, audio_taps=21),
    dict(mode="cw", decimation=1, audio_taps=15),
    dict(mode="dsb", decimation=1, audio_taps=15),
    dict(mode="raw", decimation=1, audio_taps=1, channels=2),
    dict(mode="tetra", decimation=1, audio_taps=1, channels=2),
]


@pytest.mark.parametrize("kw", DEMODS, ids=lambda kw: "%s-%d-%d" % (kw["mode"], kw["audio_taps"], kw.get("channels", 1)))
def test_vrx_demod(gpu, ora, kw):
    r = np.random.default_rng(kw["audio_taps"])
    cfg = cases.demod_config(**kw)
    w = cases.demod_weights(r, cfg)
    n = 1 << 13
    fine = cases.fm_fine_ring(r, n, pilot=0.1) if kw["mode"] in ("nfm", "wfm") else cases.am_fine_ring(r, n)
    count = 400 if cfg.channels == 1 else 300
    count = min(count, (n - 1 - int(lib().rv_demod_fine_history(C.byref(cfg)))) // cfg.decimation)
    p = abi.VrxDemodParams(n - 1, n - 500, count, 1.3)
    want = np.zeros(count * cfg.channels, np.float32)
    assert ora.vrx_demod(cfg, p, fine, w, want) == 0, ora.error()
    df, dw, out = gpu.array(fine), gpu.array(w), gpu.zeros(want.nbytes)
    run(lib().rv_vrx_demod(gpu.stream, C.byref(cfg), C.byref(p), df.ptr, n, dw.ptr, w.size, out.ptr, want.size))
    gpu.synchronize()
    assert same_bits(out.download(np.float32, want.shape), want)


@pytest.mark.parametrize("power", [1, 2])
def test_vrx_carrier(gpu, ora, power):
    r = np.random.default_rng(power + 10)
    nco = _nco()
    fine = cases.am_fine_ring(r, 8192)
    t = np.arange(8192)
    z = (fine[:, 0] + 1j * fine[:, 1]) * np.exp(1j * 0.02 * t)
    fine = np.stack([z.real, z.imag], 1).astype(np.float32)
    cfg, p = cases.carrier_params(power=power, in_mask=8191, count=3000)
    want_ring, want_state = fine.copy(), np.zeros(8, np.uint32)
    dn, df, ds = gpu.array(nco), gpu.array(fine), gpu.zeros(32)
    for step in range(3):
        p.flags = 1 if step == 0 else 0
        p.shift = 0.0005 * step
        p.in_offset = (7000 + 3000 * step) & 8191
        assert ora.vrx_carrier(cfg, p, nco, want_ring, want_state) == 0
        run(lib().rv_vrx_carrier(gpu.stream, C.byref(cfg), C.byref(p), dn.ptr, nco.shape[0], df.ptr, 8192, ds.ptr))
    gpu.synchronize()
    assert same_bits(df.download(np.float32, fine.shape), want_ring)
    assert np.array_equal(ds.download(np.uint32, 8), want_state)
