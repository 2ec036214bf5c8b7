"""The library's host planner against the reference's own planner.

Tables (prototype, twiddles, NCO circle, spectrum window, fine taps, demod
weights) must be bit-identical, and every integer of placement and plan
(rates, rationals, tap counts, NCO delta, block parameters) equal. Runs on
CPU; skips where the reference sources are absent.
"""
import ctypes as C

import numpy as np
import pytest

from bindings import same_bits
from revenant_gb300 import abi

GRIDS = [(64, 17, 32), (8, 17, 4), (1024, 16, 512), (16, 4, 16), (2048, 9, 1024), (128, 33, 64)]


@pytest.mark.parametrize("M,T,D", GRIDS)
def test_prototype_bitwise(rv, ref, M, T, D):
    g = abi.GridParams(M, T, D)
    a = np.zeros(M * T, np.float32)
    b = np.zeros(M * T, np.float32)
    sa, sb = C.c_double(), C.c_double()
    ga, gb = C.c_uint64(), C.c_uint64()
    assert rv.rv_design_prototype(C.byref(g), 120.0, a.ctypes.data, a.size, C.byref(sa), C.byref(ga)) == 0
    assert ref.lib.ref_design_prototype(C.byref(g), 120.0, b.ctypes.data, b.size, C.byref(sb), C.byref(gb)) == 0
    assert same_bits(a, b)
    assert sa.value == sb.value and ga.value == gb.value


def test_prototype_properties(rv):
    # test_pfb.cpp:155: unit DC gain, odd design length, stopband near target
    g = abi.GridParams(64, 17, 32)
    h = np.zeros(64 * 17, np.float32)
    sb = C.c_double()
    gd = C.c_uint64()
    assert rv.rv_design_prototype(C.byref(g), 120.0, h.ctypes.data, h.size, C.byref(sb), C.byref(gd)) == 0
    assert abs(h.astype(np.float64).sum() - 1.0) < 1e-6
    assert gd.value == 64 * 16 // 2
    assert sb.value < -110.0


@pytest.mark.parametrize("M", [2, 4, 8, 64, 1024, 2048])
def test_twiddles_bitwise(rv, ref, M):
    a = np.zeros((M, 2), np.float32)
    b = np.zeros((M, 2), np.float32)
    assert rv.rv_build_twiddles(M, a.ctypes.data, M) == 0
    assert ref.lib.ref_build_twiddles(M, b.ctypes.data, M) == 0
    assert same_bits(a, b)
    if M >= 4:  # exact quadrature (test_pfb.cpp:189)
        assert tuple(a[M // 4]) == (0.0, -1.0) and tuple(a[M // 2]) == (-1.0, 0.0)


@pytest.mark.parametrize("log2", [0, 3, 10, 16])
def test_nco_table_bitwise(rv, ref, log2):
    n = 1 << log2
    a = np.zeros((n, 2), np.float32)
    b = np.zeros((n, 2), np.float32)
    assert rv.rv_build_nco_table(log2, a.ctypes.data, n) == 0
    assert ref.lib.ref_build_nco_table(log2, b.ctypes.data, n) == 0
    assert same_bits(a, b)


@pytest.mark.parametrize("N,T", [(2048, 17), (256, 17), (64, 9), (8, 17)])
def test_spectrum_window_bitwise(rv, ref, N, T):
    a = np.zeros(N + N // 2, np.float32)
    b = np.zeros(N + N // 2, np.float32)
    assert rv.rv_build_spectrum_window(N, T, 120.0, a.ctypes.data, a.size) == 0
    assert ref.lib.ref_build_spectrum_window(N, T, 120.0, b.ctypes.data, b.size) == 0
    assert same_bits(a, b)


def _requests(rate):
    out = []
    r = np.random.default_rng(7)
    modes = ["nfm", "am", "usb", "lsb", "wfm", "cw", "dsb", "sam", "raw", "p25p1", "tetra", "dmr", "dstar"]
    for i in range(120):
        mode = modes[i % len(modes)]
        bw = int(r.choice([0, 3000, 6000, 10000, 12500, 25000, 50000, 100000, 200000]))
        out.append(dict(center=int(r.integers(-int(0.45 * rate), int(0.45 * rate))), bandwidth=bw, demod=mode,
                        stereo=bool(r.integers(0, 2)), audio_rate=int(r.choice([0, 0, 24000, 48000, 192000])),
                        deemphasis=int(r.integers(0, 4))))
    out.append(dict(center=200_000, bandwidth=200_000, demod="wfm"))
    out.append(dict(center=0, passband_low=300, passband_high=2700, demod="usb"))
    return out


SCENARIOS = [((64, 17, 32), 20_000_000), ((8, 17, 4), 2_400_000), ((1024, 16, 512), 61_440_000)]


@pytest.mark.parametrize("grid,rate", SCENARIOS)
def test_place_and_plan_match_reference(rv, ref, grid, rate):
    g = abi.GridParams(*grid)
    compared = 0
    for kw in _requests(rate):
        req = abi.request(**kw)
        pa, pb = abi.VrxPlacement(), abi.VrxPlacement()
        sa = rv.rv_place(C.byref(g), rate, C.byref(req), C.byref(pa))
        sb = ref.lib.ref_place(C.byref(g), rate, C.byref(req), C.byref(pb))
        assert (sa == 0) == (sb == 0), (kw, rv.rv_last_error(), ref.error())
        if sa != 0:
            continue
        assert pa.as_dict() == pb.as_dict(), kw
        ia, ib = abi.VrxPlanInfo(), abi.VrxPlanInfo()
        sa = rv.rv_plan_vrx(C.byref(g), rate, C.byref(req), C.byref(pa), C.byref(ia), None, 0, None, 0)
        sb = ref.lib.ref_plan_vrx(C.byref(g), rate, C.byref(req), C.byref(pb), C.byref(ib), None, 0, None, 0)
        assert (sa == 0) == (sb == 0), (kw, rv.rv_last_error(), ref.error())
        if sa != 0:
            continue
        da, db = ia.as_dict(), ib.as_dict()
        assert da == db, (kw, {k: (da[k], db[k]) for k in da if da[k] != db[k]})
        ta = np.zeros((ia.fine_tap_count, 2), np.float32)
        tb = np.zeros_like(ta)
        wa = np.zeros(ia.demod_weight_count, np.float32)
        wb = np.zeros_like(wa)
        assert rv.rv_plan_vrx(C.byref(g), rate, C.byref(req), C.byref(pa), C.byref(ia), ta.ctypes.data,
                              ta.shape[0], wa.ctypes.data, wa.size) == 0
        assert ref.lib.ref_plan_vrx(C.byref(g), rate, C.byref(req), C.byref(pb), C.byref(ib), tb.ctypes.data,
                                    tb.shape[0], wb.ctypes.data, wb.size) == 0
        assert same_bits(ta, tb), kw
        assert same_bits(wa, wb), kw
        # block parameters, at a stream start and three hours in
        for first in (0, 3 * 3600 * ia.demod_rate + 17):
            fa, fb = abi.VrxFineBlock(), abi.VrxFineBlock()
            sa = rv.rv_fine_block(C.byref(ia), 4096, 65535, 8191, first, 1000, C.byref(fa))
            sb = ref.lib.ref_fine_block(C.byref(g), rate, C.byref(req), 4096, 65535, 8191, first, 1000, C.byref(fb))
            assert (sa == 0) == (sb == 0)
            if sa == 0:
                assert bytes(fa) == bytes(fb), kw
        da_, db_ = abi.VrxDemodBlock(), abi.VrxDemodBlock()
        sa = rv.rv_demod_block(C.byref(ia), (1 << 16) - 1, 12345, 100, C.byref(da_))
        sb = ref.lib.ref_demod_block(C.byref(g), rate, C.byref(req), (1 << 16) - 1, 12345, 100, C.byref(db_))
        assert (sa == 0) == (sb == 0)
        if sa == 0:
            assert bytes(da_) == bytes(db_)
        compared += 1
    assert compared > 20


def test_channel_count_for(rv, ref):
    for rate in (2_400_000, 20_000_000, 61_440_000, 1):
        for w in (0, 1, 12_500, 200_000, 10_000_000):
            assert rv.rv_channel_count_for(rate, w) == ref.lib.ref_channel_count_for(rate, w)


def test_place_refuses_truncated_wfm(rv):
    # a 200 kHz WFM receiver does not fit one channel of a 64-channel grid at
    # 2.4 MS/s (vrx_place.cpp:402-418): refused, not narrowed
    g = abi.GridParams(64, 17, 32)
    req = abi.request(center=200_000, bandwidth=200_000, demod="wfm")
    pl = abi.VrxPlacement()
    assert rv.rv_place(C.byref(g), 2_400_000, C.byref(req), C.byref(pl)) == abi.RV_ERR_INVALID
    assert b"refused" in rv.rv_last_error()
    assert rv.rv_channel_count_for(2_400_000, 200_000) == 8
