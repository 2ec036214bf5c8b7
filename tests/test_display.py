"""The display tap (plan_vrx_display / display_block, core/dsp/vrx_reference.cpp
:2938-3080) against the reference's twins: the ladder, the decimation rule,
the whole plan with its 257-entry tap table bit for bit, and display_block's
parameters; the designed branch is flat across the pane and down by the
planned attenuation past the first frequency that folds into it; on the GPU,
rv_vrx_fine run with the display plan equals the oracle's fine stage on the
same channel.
"""
import ctypes as C

import numpy as np
import pytest

from bindings import cf32, same_bits
from revenant_gb300 import abi
from revenant_gb300.library import lib

GRIDS = [((64, 17, 32), 20_000_000), ((8, 17, 4), 2_400_000)]
REQUESTS = [dict(center=1_000_000, bandwidth=12_500, demod="nfm"), dict(center=-2_345_000, bandwidth=10_000, demod="am"),
            dict(center=3_000_000, bandwidth=3_000, demod="usb"), dict(center=-500_000, bandwidth=2_700, demod="lsb"),
            dict(center=4_000_000, bandwidth=200_000, demod="wfm"),
            dict(center=700_000, bandwidth=500, demod="cw", cw_pitch=700)]


def plan_of(grid, rate, req):
    g = abi.GridParams(*grid)
    pl = abi.VrxPlacement()
    assert lib().rv_place(C.byref(g), rate, C.byref(req), C.byref(pl)) == 0
    info = abi.VrxPlanInfo()
    assert lib().rv_plan_vrx(C.byref(g), rate, C.byref(req), C.byref(pl), C.byref(info), None, 0, None, 0) == 0
    return g, info


def display_of(info):
    d = abi.VrxDisplayPlan()
    assert lib().rv_plan_vrx_display(C.byref(info), C.byref(d), None, 0) == 0, lib().rv_last_error()
    taps = cf32(d.tap_count)
    assert lib().rv_plan_vrx_display(C.byref(info), C.byref(d), taps.ctypes.data, d.tap_count) == 0
    return d, taps


def test_ladder_and_max_decimation(ref, rv):
    assert rv.rv_display_max_decimation() == ref.lib.ref_display_max_decimation() == 25
    for rate in (625_000, 75_000, 600_000, 1_200_000, 3 * 7 * 11 * 13 * 17, 2, 0):
        a, b = (C.c_uint32 * 64)(), (C.c_uint32 * 64)()
        na, nb = C.c_uint32(), C.c_uint32()
        assert ref.lib.ref_display_ladder(rate, a, 64, C.byref(na)) == 0
        assert rv.rv_display_ladder(rate, b, 64, C.byref(nb)) == 0
        assert list(a)[:na.value] == list(b)[:nb.value]
        for reach in (1, 100, 1500, 6250, 100_000):
            assert rv.rv_display_decimation(rate, reach) == ref.lib.ref_display_decimation(rate, reach)
    n = C.c_uint32()
    rungs = (C.c_uint32 * 8)()
    rv.rv_display_ladder(625_000, rungs, 8, C.byref(n))
    assert list(rungs)[:n.value] == [1, 2, 4, 8, 20]


@pytest.mark.parametrize("grid,rate", GRIDS)
@pytest.mark.parametrize("req", REQUESTS, ids=[r["demod"] for r in REQUESTS])
def test_display_plan_and_block_match_reference(ref, rv, grid, rate, req):
    req = dict(req)
    if rate < 10_000_000:  # keep every centre inside a 2.4 MS/s span
        req["center"] = req["center"] // 10
    r = abi.request(**req)
    g, info = plan_of(grid, rate, r)
    d, taps = display_of(info)
    want = abi.VrxDisplayPlan()
    want_taps = cf32(d.tap_count)
    blk = abi.VrxFineBlock()
    assert ref.lib.ref_plan_vrx_display(C.byref(g), rate, C.byref(r), C.byref(want), want_taps.ctypes.data,
                                        d.tap_count, 3 << 14, (1 << 14) - 1, 4095, 123_456_789, 1000,
                                        C.byref(blk)) == 0, ref.error()
    assert bytes(d) == bytes(want)
    assert same_bits(taps, want_taps)
    got = abi.VrxFineBlock()
    assert rv.rv_display_block(C.byref(d), 3 << 14, (1 << 14) - 1, 4095, 123_456_789, 1000, C.byref(got)) == 0
    assert bytes(got) == bytes(blk)
    assert d.display_rate * d.decimation == d.channel_rate and d.fine.phases == 1 and d.fine.taps == 256


@pytest.mark.gpu
def test_gpu_display_tap_matches_oracle(gpu, ora):
    grid, rate = (64, 17, 32), 20_000_000
    r = abi.request(center=1_000_000, bandwidth=12_500, demod="nfm")
    g, info = plan_of(grid, rate, r)
    d, taps = display_of(info)
    # a channel of white noise, channel-major ring of 2^14 blocks
    blocks = 1 << 14
    rng = np.random.default_rng(4)
    ring = (0.05 * rng.standard_normal((grid[0] * blocks, 2))).astype(np.float32)
    nco = cf32(1 << info.fine.nco_log2)
    assert lib().rv_build_nco_table(info.fine.nco_log2, nco.ctypes.data, nco.shape[0]) == 0
    ch = info.placement.channel
    first_output = 400
    count = (blocks - 600) // d.decimation
    blk = abi.VrxFineBlock()
    assert lib().rv_display_block(C.byref(d), ch * blocks, blocks - 1, 8191, first_output, count, C.byref(blk)) == 0
    want = cf32(8192)
    assert ora.vrx_fine(d.fine, blk.params, ring, taps, nco, want) == 0, ora.error()
    d_ring, d_taps, d_nco, d_out = gpu.array(ring), gpu.array(taps), gpu.array(nco), gpu.zeros(8192 * 8)
    assert lib().rv_vrx_fine(gpu.stream, C.byref(d.fine), C.byref(blk.params), d_ring.ptr, ring.shape[0], d_taps.ptr,
                             taps.shape[0], d_nco.ptr, nco.shape[0], d_out.ptr, 8192) == 0, lib().rv_last_error()
    gpu.synchronize()
    got = d_out.download(np.float32, (8192, 2))
    assert same_bits(got, want)


@pytest.mark.parametrize("req", REQUESTS[:5], ids=[r["demod"] for r in REQUESTS[:5]])
def test_display_filter_is_flat_over_the_pane(req):
    """The designed branch, centred on the receiver's mix: within 0.1 dB of
    its centre up to pass_hz, and at least the 80 dB the display asks for
    (kDisplayAttenuationDb) beyond stop_hz, over the channel's whole band;
    the taps' float rounding bounds a deeper design near 90-100 dB."""
    g, info = plan_of((64, 17, 32), 20_000_000, abi.request(**req))
    d, taps = display_of(info)
    h = taps[:256, 0] + 1j * taps[:256, 1]
    nfft = 1 << 16
    resp = np.fft.fftshift(np.abs(np.fft.fft(h, nfft)))
    f = (np.arange(nfft) - nfft // 2) / nfft * d.channel_rate
    mix = info.mix_numerator / info.mix_denominator
    off = (f - mix + d.channel_rate / 2) % d.channel_rate - d.channel_rate / 2
    db = 20 * np.log10(np.maximum(resp, 1e-300) / resp[np.argmin(np.abs(off))])
    assert np.all(np.abs(db[np.abs(off) <= 0.9 * d.pass_hz]) < 0.1)
    stop = np.abs(off) >= d.stop_hz
    if stop.any():  # at R = 1 the stopband edge is the channel's own Nyquist
        assert db[stop].max() < -80.0
