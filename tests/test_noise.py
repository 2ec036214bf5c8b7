"""Per-receiver noise stages against the reference's twins
(core/dsp/noise_reference.cpp, compiled from the reference sources into
oracle/_ref/libreftwins.so) and the oracle restatement (oracle/oracle.c).

Bit for bit everywhere: the designers (blanker window, thresholds, notch
coefficients in double, spectral frame, tables and parameters), the
blanker's flags and blanked samples, and for the line kernel and the
spectral noise reduction the audio and the whole state after every call of a
sequence of calls whose lengths do not line up with anything.
"""
import ctypes as C

import numpy as np
import pytest

from bindings import same_bits
from revenant_gb300 import abi
from revenant_gb300.library import lib

RATES = [48_000, 144_000, 625_000, 10_000, 1_000_000, 8_000]


def _p(a):
    return a.ctypes.data


# -- designers -----------------------------------------------------------------

@pytest.mark.parametrize("rate", RATES)
def test_blanker_design_oracle_library_reference(ora, ref, rv, rate):
    out = []
    for fn in (ref.fn("design_blanker"), ora.fn("design_blanker"), rv.rv_design_blanker):
        c = abi.BlankerConfig()
        assert fn(rate, C.byref(c)) == 0
        out.append((c.pass_, c.window, c.guard, c.hang, c.lead))
    assert out[0] == out[1] == out[2]
    for db in (12.0, 6.0, 20.5):
        want = np.float32(ref.fn("blanker_threshold")(db)).view(np.uint32)
        assert np.float32(ora.fn("blanker_threshold")(db)).view(np.uint32) == want
        assert np.float32(rv.rv_blanker_threshold(db)).view(np.uint32) == want


@pytest.mark.parametrize("hz,depth,width,rate", [(1000.0, 40.0, 50.0, 48_000), (15_000.0, 60.0, 200.0, 48_000),
                                                 (700.0, 30.0, 20.0, 8_000), (3_999.0, 40.0, 100.0, 8_000),
                                                 (0.0, 40.0, 50.0, 48_000), (1000.0, 40.0, 20_000.0, 48_000)])
def test_notch_design_oracle_library_reference(ora, ref, rv, hz, depth, width, rate):
    res = []
    for fn in (ref.fn("design_notch"), ora.fn("design_notch"), rv.rv_design_notch):
        d = abi.NotchDesign()
        st = fn(hz, depth, width, rate, C.byref(d))
        res.append((st == 0,) + ((d.b0, d.b1, d.b2, d.a1, d.a2) if st == 0 else ()))
    assert res[0] == res[1] == res[2]


@pytest.mark.parametrize("rate", RATES + [0, 46_080])
def test_spectral_designers_oracle_library_reference(ora, ref, rv, rate):
    cfgs = []
    for fn in (ref.fn("spectral_config_for"), ora.fn("spectral_config_for"), rv.rv_spectral_config_for):
        c = abi.SpectralConfig()
        assert fn(rate, C.byref(c)) == 0
        cfgs.append(c.frame)
    assert cfgs[0] == cfgs[1] == cfgs[2]
    c = abi.SpectralConfig(cfgs[0])
    tabs = [np.zeros(4 * c.frame, np.float32) for _ in range(3)]
    for fn, t in zip((ref.fn("design_spectral_tables"), ora.fn("design_spectral_tables"),
                      rv.rv_design_spectral_tables), tabs):
        assert fn(C.byref(c), _p(t), t.size) == 0
    assert same_bits(tabs[0], tabs[1]) and same_bits(tabs[0], tabs[2])
    for strength in (0.0, 0.5, 1.0, 2.0):
        ps = []
        for fn in (ref.fn("design_spectral_params"), ora.fn("design_spectral_params"), rv.rv_design_spectral_params):
            p = abi.SpectralParams()
            assert fn(strength, C.byref(p)) == 0
            ps.append(bytes(p))
        assert ps[0] == ps[1] == ps[2]


# -- the blanker ------------------------------------------------------------------

M, RING_BLOCKS = 8, 1 << 14


def channel_ring(seed):
    """A channel-major ring, channel 3 carrying noise, a tone and impulses."""
    rng = np.random.default_rng(seed)
    ring = (0.01 * rng.standard_normal((M * RING_BLOCKS, 2))).astype(np.float32)
    t = np.arange(RING_BLOCKS)
    ch = ring[3 * RING_BLOCKS:4 * RING_BLOCKS]
    ch[:, 0] += 0.2 * np.cos(0.05 * t)
    ch[:, 1] += 0.2 * np.sin(0.05 * t)
    for pos in range(100, RING_BLOCKS - 10, 577):
        w = 1 + pos % 4
        ch[pos:pos + w] += rng.uniform(2, 6, (w, 2))
    return ring


def blanker_calls():
    c = abi.BlankerConfig()
    assert lib().rv_design_blanker(144_000, C.byref(c)) == 0
    thr = lib().rv_blanker_threshold(12.0)
    calls, first, out_first = [], RING_BLOCKS - 1500, 7  # the first call wraps the channel ring
    for n in (900, 1, 2500, 1024, 333):
        calls.append(abi.BlankerParams(3 * RING_BLOCKS, RING_BLOCKS - 1, first & (RING_BLOCKS - 1), 4095,
                                       out_first & 4095, n, thr))
        first += n
        out_first += n
    return c, calls


def run_blanker_cpu(kind, c, calls, ring):
    flags = np.zeros(4096, np.float32)
    blanked = np.zeros((4096, 2), np.float32)
    outs = []
    for p in calls:
        assert kind.fn("blank_detect")(C.byref(c), C.byref(p), _p(ring), ring.shape[0], _p(flags), flags.size) == 0
        assert kind.fn("blank_apply")(C.byref(c), C.byref(p), _p(ring), ring.shape[0], _p(flags), flags.size,
                                      _p(blanked), blanked.shape[0]) == 0
        outs.append((flags.copy(), blanked.copy()))
    return outs


def test_blanker_oracle_vs_reference(ora, ref):
    ring = channel_ring(1)
    c, calls = blanker_calls()
    a, b = run_blanker_cpu(ref, c, calls, ring), run_blanker_cpu(ora, c, calls, ring)
    for (fa, ba), (fb, bb) in zip(a, b):
        assert same_bits(fa, fb) and same_bits(ba, bb)
    assert a[-1][0].sum() > 5  # impulses flagged


@pytest.mark.parametrize("field,value", [("window", 15), ("window", 257), ("out_mask", 1000), ("count", 4050),
                                         ("threshold", 0.0)])
def test_blanker_rejects_alike(ora, ref, rv, field, value):
    ring = channel_ring(2)
    c, calls = blanker_calls()
    p = calls[1]
    if field == "window":
        c.window = value
    else:
        setattr(p, field, value)
    flags = np.zeros(4096, np.float32)
    for kind in (ref, ora):
        assert kind.fn("blank_detect")(C.byref(c), C.byref(p), _p(ring), ring.shape[0], _p(flags), flags.size) != 0
    assert rv.rv_blank_detect(None, C.byref(c), C.byref(p), _p(ring), ring.shape[0], _p(flags),
                              flags.size) == abi.RV_ERR_INVALID


# -- the line kernel ---------------------------------------------------------------

LINE_CFG = (32, 128, 2048)


def notch_section(hz, depth, width, rate=48_000):
    d = abi.NotchDesign()
    assert lib().rv_design_notch(hz, depth, width, rate, C.byref(d)) == 0
    return [np.float32(x) for x in (d.b0, d.b1, d.b2, d.a1, d.a2)]


def line_params(kind):
    p = abi.LineParams()
    p.stride, p.delay = 1, 240
    p.mu, p.leak, p.eps = np.float32(1.0e-4), np.float32(1.0 - 3.0e-6), np.float32(1.0e-10)
    p.b0, p.b1, p.b2, p.a1, p.a2 = notch_section(1500.0, 40.0, 60.0)
    p.gb0, p.gb1, p.gb2, p.ga1, p.ga2 = 1.0, 0.0, 0.0, 0.0, 0.0
    for k in range(3):
        p.more[k].b0 = 1.0
    if kind == "notch":
        p.flags = abi.LINE_NOTCH
    elif kind == "ale":
        p.flags = abi.LINE_ALE
    elif kind == "both":
        p.flags = abi.LINE_NOTCH | abi.LINE_ALE
        p.stride = 7
    elif kind == "guard":
        p.flags = abi.LINE_ALE | abi.LINE_GUARD
        p.gb0, p.gb1, p.gb2, p.ga1, p.ga2 = notch_section(700.0, 40.0, 100.0)
    elif kind == "cascade":
        p.flags = abi.LINE_NOTCH | abi.LINE_ALE | abi.LINE_GUARD | (3 << abi.LINE_NOTCH_COUNT_SHIFT)
        p.gb0, p.gb1, p.gb2, p.ga1, p.ga2 = notch_section(700.0, 40.0, 100.0)
        for k, hz in enumerate((2500.0, 3300.0, 400.0)):
            sec = notch_section(hz, 30.0, 40.0)
            p.more[k].b0, p.more[k].b1, p.more[k].b2, p.more[k].a1, p.more[k].a2 = sec
        p.stride = 3
    return p


def line_audio(n, seed):
    rng = np.random.default_rng(seed)
    t = np.arange(n) / 48_000.0
    x = 0.3 * np.sin(2 * np.pi * 1500.0 * t) + 0.2 * np.sin(2 * np.pi * 700.0 * t)
    x += 0.1 * np.sin(2 * np.pi * 220.0 * t) * (1 + np.sin(2 * np.pi * 3 * t)) + 0.05 * rng.standard_normal(n)
    return x.astype(np.float32)


CALLS = [1000, 1, 4097, 333, 2048, 5000]


def run_line_cpu(kind, cfg, p, audio):
    state = np.zeros(24 + cfg.taps + cfg.history, np.float32)
    out, at = [], 0
    for n in CALLS:
        chunk = audio[at:at + n].copy()
        p.count = n
        assert kind.fn("noise_line")(C.byref(cfg), C.byref(p), _p(chunk), chunk.size, _p(state), state.size) == 0, \
            kind.error()
        out.append((chunk, state.copy()))
        at += n
    return out


@pytest.mark.parametrize("mode", ["notch", "ale", "both", "guard", "cascade"])
def test_line_oracle_vs_reference(ora, ref, mode):
    cfg = abi.LineConfig(*LINE_CFG)
    audio = line_audio(sum(CALLS), 3)
    a = run_line_cpu(ref, cfg, line_params(mode), audio)
    b = run_line_cpu(ora, cfg, line_params(mode), audio)
    for k, ((xa, sa), (xb, sb)) in enumerate(zip(a, b)):
        assert same_bits(xa, xb), "call %d audio" % k
        assert same_bits(sa, sb), "call %d state" % k
    if mode != "notch":
        out = np.concatenate([x for x, _ in a])
        # the predictor is learning the 1500 Hz whistle: the tail carries less
        # of it than the input did
        t = np.arange(4000)
        w = np.exp(-2j * np.pi * 1500.0 / 48_000.0 * (sum(CALLS) - 4000 + t))
        assert abs(np.dot(out[-4000:], w)) < 0.9 * abs(np.dot(audio[-4000:], w))


@pytest.mark.parametrize("field,value", [("stride", 0), ("stride", 9), ("delay", 0), ("eps", 0.0), ("flags", 64),
                                         ("delay", 2000)])
def test_line_rejects_alike(ora, ref, rv, field, value):
    cfg = abi.LineConfig(*LINE_CFG)
    p = line_params("both")
    setattr(p, field, value)
    p.count = 10
    audio = np.zeros(10, np.float32)
    state = np.zeros(24 + cfg.taps + cfg.history, np.float32)
    for kind in (ref, ora):
        assert kind.fn("noise_line")(C.byref(cfg), C.byref(p), _p(audio), 10, _p(state), state.size) != 0
    assert rv.rv_noise_line(None, C.byref(cfg), C.byref(p), _p(audio), 10, _p(state), state.size) == abi.RV_ERR_INVALID


# -- spectral noise reduction -------------------------------------------------------

def spectral_setup(frame, strength):
    c = abi.SpectralConfig(frame)
    tables = np.zeros(4 * frame, np.float32)
    assert lib().rv_design_spectral_tables(C.byref(c), _p(tables), tables.size) == 0
    p = abi.SpectralParams()
    assert lib().rv_design_spectral_params(strength, C.byref(p)) == 0
    return c, p, tables


SPEC_CALLS = [100, 1, 700, 256, 1500, 3000, 77]


def run_spectral_cpu(kind, c, p, tables, audio):
    n = c.frame
    state = np.zeros(2 + n + n + 2 * (n // 2 + 1), np.float32)
    out, at = [], 0
    for k in SPEC_CALLS:
        chunk = audio[at:at + k].copy()
        p.count = k
        assert kind.fn("noise_spectral")(C.byref(c), C.byref(p), _p(tables), tables.size, _p(chunk), chunk.size,
                                         _p(state), state.size) == 0, kind.error()
        out.append((chunk, state.copy()))
        at += k
    return out


@pytest.mark.parametrize("frame,strength", [(512, 0.5), (64, 0.0), (256, 1.0)])
def test_spectral_oracle_vs_reference(ora, ref, frame, strength):
    c, p, tables = spectral_setup(frame, strength)
    audio = line_audio(sum(SPEC_CALLS), 7)
    a = run_spectral_cpu(ref, c, p, tables, audio)
    b = run_spectral_cpu(ora, c, p, tables, audio)
    for k, ((xa, sa), (xb, sb)) in enumerate(zip(a, b)):
        assert same_bits(xa, xb), "call %d audio" % k
        assert same_bits(sa, sb), "call %d state" % k


def test_spectral_rejects_alike(ora, ref, rv):
    c, p, tables = spectral_setup(512, 0.5)
    audio = np.zeros(16, np.float32)
    state = np.zeros(2000, np.float32)
    for frame, eps in ((500, 1e-12), (1024, 1e-12), (32, 1e-12), (512, 0.0)):
        c.frame, p.eps, p.count = frame, eps, 16
        for kind in (ref, ora):
            assert kind.fn("noise_spectral")(C.byref(c), C.byref(p), _p(tables), tables.size, _p(audio), 16, _p(state),
                                             state.size) != 0
        assert rv.rv_noise_spectral(None, C.byref(c), C.byref(p), _p(tables), tables.size, _p(audio), 16, _p(state),
                                    state.size) == abi.RV_ERR_INVALID


# -- GPU ------------------------------------------------------------------------------

@pytest.mark.gpu
def test_gpu_blanker_matches_oracle(gpu, ora):
    ring = channel_ring(1)
    c, calls = blanker_calls()
    want = run_blanker_cpu(ora, c, calls, ring)
    d_ring = gpu.array(ring)
    d_flags = gpu.zeros(4096 * 4)
    d_blanked = gpu.zeros(4096 * 8)
    for k, p in enumerate(calls):
        assert lib().rv_blank_detect(gpu.stream, C.byref(c), C.byref(p), d_ring.ptr, ring.shape[0], d_flags.ptr,
                                     4096) == 0
        assert lib().rv_blank_apply(gpu.stream, C.byref(c), C.byref(p), d_ring.ptr, ring.shape[0], d_flags.ptr, 4096,
                                    d_blanked.ptr, 4096) == 0
        gpu.synchronize()
        assert same_bits(d_flags.download(np.float32, (4096,)), want[k][0]), "call %d flags" % k
        assert same_bits(d_blanked.download(np.float32, (4096, 2)), want[k][1]), "call %d blanked" % k


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["notch", "ale", "both", "guard", "cascade"])
def test_gpu_line_matches_oracle(gpu, ora, mode):
    cfg = abi.LineConfig(*LINE_CFG)
    audio = line_audio(sum(CALLS), 3)
    want = run_line_cpu(ora, cfg, line_params(mode), audio)
    p = line_params(mode)
    d_state = gpu.zeros((24 + cfg.taps + cfg.history) * 4)
    at = 0
    for k, n in enumerate(CALLS):
        d_audio = gpu.array(audio[at:at + n])
        p.count = n
        assert lib().rv_noise_line(gpu.stream, C.byref(cfg), C.byref(p), d_audio.ptr, n, d_state.ptr,
                                   24 + cfg.taps + cfg.history) == 0, lib().rv_last_error()
        gpu.synchronize()
        assert same_bits(d_audio.download(np.float32, (n,)), want[k][0]), "call %d audio" % k
        assert same_bits(d_state.download(np.float32, (24 + cfg.taps + cfg.history,)), want[k][1]), "call %d state" % k
        at += n


@pytest.mark.gpu
@pytest.mark.parametrize("frame,strength", [(512, 0.5), (64, 0.0), (256, 1.0)])
def test_gpu_spectral_matches_oracle(gpu, ora, frame, strength):
    c, p, tables = spectral_setup(frame, strength)
    audio = line_audio(sum(SPEC_CALLS), 7)
    want = run_spectral_cpu(ora, c, p, tables, audio)
    n = c.frame
    size = 2 + n + n + 2 * (n // 2 + 1)
    d_tables = gpu.array(tables)
    d_state = gpu.zeros(size * 4)
    at = 0
    for k, cnt in enumerate(SPEC_CALLS):
        d_audio = gpu.array(audio[at:at + cnt])
        p.count = cnt
        assert lib().rv_noise_spectral(gpu.stream, C.byref(c), C.byref(p), d_tables.ptr, tables.size, d_audio.ptr, cnt,
                                       d_state.ptr, size) == 0, lib().rv_last_error()
        gpu.synchronize()
        assert same_bits(d_audio.download(np.float32, (cnt,)), want[k][0]), "call %d audio" % k
        assert same_bits(d_state.download(np.float32, (size,)), want[k][1]), "call %d state" % k
        at += cnt
