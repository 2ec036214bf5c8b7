"""a16, the scene synthesiser (core/dsp/synth/wideband.cpp, modulators.cpp)
on the GPU: its noise field (Scene::fill_noise), its eight modulations
(Modulator::accumulate for CW, tone AM, NFM, USB, LSB, FSK2, BPSK, QPSK) and
its random population (Scene::create's layout, rv_scene_plan).

The oracle (oracle/oracle.c: or_scene_noise, or_emitter_accumulate) restates
them in C with the C library's transcendentals and is pinned against the
reference's own Scene and Modulator (oracle/_ref/libsynref.so) bit for bit on
this machine, the noise draws against libstdc++'s std::mt19937_64, and the
noise against tests/golden/scene_noise.npz (made by
tests/golden/make_scene_noise.py) everywhere. The layout is pinned against
the reference's truth table field for field.

On the GPU:
  * the noise draws equal the oracle's bit for bit (integers);
  * AM, SSB, FSK2 and PSK, whose anchors and tables come from the host, equal
    the oracle bit for bit; the noise, NFM and CW, which take CUDA's FP64
    log, sine or cosine per sample, equal it except where that rounding
    moves the FP32 result: at most MAX_MISMATCH_FRACTION of the samples, each
    within ULP_TOLERANCE FP32 ulp;
  * the noise field is a function of the absolute range: a render in pieces
    equals the render in one piece, bit for bit, at 2^24 samples.
"""
import ctypes as C
import os

import numpy as np
import pytest

from bindings import cf32, oracle
from revenant_gb300.library import lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SYNREF = os.path.join(ROOT, "oracle", "_ref", "libsynref.so")
GOLDEN = os.path.join(ROOT, "tests", "golden", "scene_noise.npz")
NOISE_DOMAIN = 0x1A59017E55CE0D02
MAX_MISMATCH_FRACTION = 1e-4
ULP_TOLERANCE = 1


def derive_stream_seed(master, domain):
    """wideband.cpp:46-53, restated for the draw pin."""
    m = (1 << 64) - 1
    z = (master + domain * 0x9E3779B97F4A7C15) & m
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    return z ^ (z >> 31)


def ora_lib():
    o = oracle().lib
    o.or_scene_noise_sigma.restype = C.c_double
    o.or_scene_noise_sigma.argtypes = [C.c_double]
    o.or_scene_noise.argtypes = [C.c_uint64, C.c_double, C.c_uint64, C.c_uint64, C.c_void_p]
    o.or_scene_noise_draws.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p]
    return o


def ora_noise(seed, sigma, start, count):
    out = cf32(count)
    assert ora_lib().or_scene_noise(seed, sigma, start, count, out.ctypes.data) == 0
    return out


def ora_draws(seed, start, count):
    out = np.zeros(2 * count, np.uint64)
    assert ora_lib().or_scene_noise_draws(seed, start, count, out.ctypes.data) == 0
    return out


@pytest.fixture(scope="module")
def synref():
    if not os.path.exists(SYNREF):
        pytest.skip("reference synthesiser not built (reference sources absent on this machine)")
    s = C.CDLL(SYNREF, mode=os.RTLD_LAZY)  # its emitter code paths are never called
    s.refsyn_noise.argtypes = [C.c_uint64, C.c_int64, C.c_double, C.c_uint64, C.c_uint64, C.c_void_p]
    s.refsyn_mt64.argtypes = [C.c_uint64, C.c_uint64, C.c_void_p]
    return s


def golden_cases():
    g = np.load(GOLDEN)
    for i in range(len([k for k in g.files if k.startswith("case")])):
        seed, rate, start, count = (int(x) for x in g["params%d" % i])
        yield seed, rate, float(g["dbfs%d" % i][0]), start, count, g["case%d" % i]


@pytest.mark.parametrize("seed,dbfs,start,count", [(1, -60.0, 0, 5000), (0xDEADBEEF, -40.0, 4095, 9000),
                                                   (5, -75.5, (1 << 31) + 17, 4096), (2, 10.0, 8192, 1)])
def test_oracle_matches_reference_scene(synref, seed, dbfs, start, count):
    want = np.zeros((count, 2), np.float32)
    assert synref.refsyn_noise(seed, 20_000_000, dbfs, start, count, want.ctypes.data) == 0
    sigma = ora_lib().or_scene_noise_sigma(dbfs)
    assert lib().rv_scene_noise_sigma(dbfs) == sigma
    got = ora_noise(seed, sigma, start, count)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_oracle_draws_are_the_standard_mt19937_64(synref):
    for seed, block in ((7, 0), (7, 3), (2**63 + 5, 1 << 20)):
        want = np.zeros(8192, np.uint64)
        synref.refsyn_mt64(derive_stream_seed(seed ^ block, NOISE_DOMAIN), 8192, want.ctypes.data)
        assert np.array_equal(ora_draws(seed, block * 4096, 4096), want)


def test_oracle_matches_golden_fixture():
    for seed, rate, dbfs, start, count, want in golden_cases():
        got = ora_noise(seed, ora_lib().or_scene_noise_sigma(dbfs), start, count)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (seed, start)


def ulp_distance(a, b):
    """FP32 ulps between a and b, elementwise (ordered integer view)."""
    def key(x):
        i = x.view(np.int32).astype(np.int64)
        return np.where(i < 0, -(i & 0x7FFFFFFF), i)
    return np.abs(key(a) - key(b))


def check_close(got, want):
    d = ulp_distance(got.reshape(-1), want.reshape(-1))
    mismatched = np.count_nonzero(d)
    assert d.max() <= ULP_TOLERANCE, d.max()
    assert mismatched <= max(1, MAX_MISMATCH_FRACTION * d.size), mismatched
    return mismatched


@pytest.mark.gpu
def test_gpu_draws_match_oracle(gpu):
    for seed, start, count in ((9, 0, 4096), (9, 4000, 10_000), (2**64 - 1, (1 << 33) + 123, 5000)):
        d = gpu.zeros(2 * count * 8)
        assert lib().rv_scene_noise_draws(gpu.stream, seed, start, count, d.ptr, 2 * count) == 0, lib().rv_last_error()
        gpu.synchronize()
        assert np.array_equal(d.download(np.uint64, (2 * count,)), ora_draws(seed, start, count))


@pytest.mark.gpu
def test_gpu_noise_matches_oracle_and_golden(gpu):
    cases = [(seed, dbfs, start, count, None) for seed, _, dbfs, start, count, _ in golden_cases()]
    cases += [(g[0], g[2], g[3], g[4], g[5]) for g in golden_cases()]
    cases += [(77, -60.0, 123_456, 200_000, None)]
    for seed, dbfs, start, count, want in cases:
        sigma = lib().rv_scene_noise_sigma(dbfs)
        d = gpu.zeros(count * 8)
        assert lib().rv_scene_noise(gpu.stream, seed, sigma, start, count, d.ptr, count) == 0, lib().rv_last_error()
        gpu.synchronize()
        got = d.download(np.float32, (count, 2))
        n = check_close(got, ora_noise(seed, sigma, start, count) if want is None else want)
        print("scene noise seed %d, %d samples from %d: %d of %d components off by one FP32 ulp"
              % (seed, count, start, n, 2 * count))


@pytest.mark.gpu
def test_gpu_noise_is_a_function_of_the_range(gpu):
    n, seed, sigma = 1 << 24, 11, lib().rv_scene_noise_sigma(-50.0)
    whole = gpu.zeros(n * 8)
    assert lib().rv_scene_noise(gpu.stream, seed, sigma, 0, n, whole.ptr, n) == 0
    parts = gpu.zeros(n * 8)
    cuts = [0, 1, 4095, 4097, 1_000_001, n // 2, n - 3, n]
    for a, b in zip(cuts[:-1], cuts[1:]):
        assert lib().rv_scene_noise(gpu.stream, seed, sigma, a, b - a, parts.address + 8 * a, b - a) == 0
    gpu.synchronize()
    x = whole.download(np.float32, (n, 2))
    assert np.array_equal(x.view(np.uint32), parts.download(np.float32, (n, 2)).view(np.uint32))
    # and it is the noise it claims to be: zero mean, sigma per component
    assert abs(float(x.mean())) < 5 * sigma / np.sqrt(2 * n)
    assert abs(float(x.std()) / sigma - 1.0) < 1e-3


def test_entry_points_reject_bad_arguments(rv):
    one = np.zeros(4, np.float32)
    assert rv.rv_scene_noise(None, 1, -1.0, 0, 1, one.ctypes.data, 1) == -1
    assert rv.rv_scene_noise(None, 1, 1.0, 0, 2, one.ctypes.data, 1) == -1
    assert rv.rv_scene_noise_draws(None, 1, 0, 2, one.ctypes.data, 3) == -1
    assert rv.rv_scene_noise(None, 1, 1.0, 2**64 - 2, 5, one.ctypes.data, 5) == -1


# ---- tone emitters (Modulator::accumulate_am / _nfm) and scenes of them ----

TONES = [dict(modulation=1, rate=2_400_000, carrier_offset=100_000, tone_hz=1000, deviation=0, amplitude=0.5,
              initial_phase=0.3, modulation_index=0.8),
         dict(modulation=2, rate=20_000_000, carrier_offset=-3_000_000, tone_hz=1234, deviation=5000, amplitude=0.25,
              initial_phase=2.0, modulation_index=0.0),
         dict(modulation=1, rate=61_440_000, carrier_offset=-30_720_000, tone_hz=30_000, deviation=0, amplitude=1.0,
              initial_phase=-1.0, modulation_index=1.0),
         dict(modulation=2, rate=2_400_000, carrier_offset=1_200_000, tone_hz=3000, deviation=75_000, amplitude=1.0,
              initial_phase=0.0, modulation_index=0.0),
         dict(modulation=3, rate=20_000_000, carrier_offset=7_500_000, tone_hz=1000, deviation=0, amplitude=0.5,
              initial_phase=0.7, modulation_index=0.0, tone2_hz=0, audio_low_hz=300, audio_high_hz=3000),
         dict(modulation=4, rate=2_400_000, carrier_offset=-100_000, tone_hz=700, deviation=0, amplitude=1.0,
              initial_phase=-2.5, modulation_index=0.0, tone2_hz=1900, audio_low_hz=300, audio_high_hz=3000)]
TONES += [dict(modulation=0, rate=48_000, carrier_offset=3_000, tone_hz=0, deviation=0, amplitude=0.8,
               initial_phase=0.1, modulation_index=0.0, words_per_minute=30.0, rise_fall_ms=5.0,
               message_gap_dots=7.0, text=b"CQ DE GB300, K?"),
          dict(modulation=0, rate=2_400_000, carrier_offset=-250_000, tone_hz=0, deviation=0, amplitude=1.0,
               initial_phase=0.0, modulation_index=0.0, words_per_minute=45.0, rise_fall_ms=0.0,
               message_gap_dots=10.5, text=b"test 73")]
TONES += [dict(modulation=5, rate=48_000, carrier_offset=-5_000, tone_hz=0, deviation=1200, amplitude=0.6,
               initial_phase=1.3, modulation_index=0.0, seed=12345, symbol_rate=2400.0, symbol_count=64),
          dict(modulation=5, rate=2_400_000, carrier_offset=300_000, tone_hz=0, deviation=9600, amplitude=1.0,
               initial_phase=0.0, modulation_index=0.0, seed=2**64 - 3, symbol_rate=9600.0, symbol_count=256)]
TONES += [dict(modulation=6, rate=48_000, carrier_offset=4_000, tone_hz=0, deviation=0, amplitude=0.7,
               initial_phase=0.4, modulation_index=0.0, seed=99, symbol_rate=2400.0, symbol_count=64, rolloff=0.35,
               span_symbols=8),
          dict(modulation=7, rate=20_000_000, carrier_offset=-2_000_000, tone_hz=0, deviation=0, amplitude=1.0,
               initial_phase=2.2, modulation_index=0.0, seed=7, symbol_rate=1200.0, symbol_count=256, rolloff=0.2,
               span_symbols=8),
          dict(modulation=7, rate=2_400_000, carrier_offset=50_000, tone_hz=0, deviation=0, amplitude=0.5,
               initial_phase=0.0, modulation_index=0.0, seed=31, symbol_rate=19200.0, symbol_count=256, rolloff=0.5,
               span_symbols=8)]
TONE_IDS = ["am", "nfm", "am-edge", "wide-nfm", "usb", "lsb-two-tone", "cw", "cw-hard", "fsk", "fsk-fast", "bpsk",
            "qpsk-strided", "qpsk"]


def tone(d):
    from revenant_gb300 import abi
    e = abi.ToneEmitter()
    for k, v in d.items():
        setattr(e, k, v)
    return e


def ora_tone(d, first, count, gain, io):
    from revenant_gb300 import abi
    o = oracle().lib
    o.or_emitter_accumulate.argtypes = [C.POINTER(abi.ToneEmitter), C.c_uint64, C.c_uint64, C.c_double, C.c_void_p]
    out = io.copy()
    assert o.or_emitter_accumulate(C.byref(tone(d)), first, count, gain, out.ctypes.data) == 0
    return out


def ora_scene(seed, dbfs, d, on, off, start, count):
    """Scene::render_range for noise plus one emitter burst over [on, off)."""
    out = ora_noise(seed, ora_lib().or_scene_noise_sigma(dbfs), start, count)
    lo, hi = max(on, start), min(off, start + count)
    if lo < hi:
        out[lo - start:hi - start] = ora_tone(d, lo - on, hi - lo, 1.0, out[lo - start:hi - start])
    return out


def ref_args(synref, d=None):
    synref.refsyn_set_ssb.argtypes = [C.c_int64, C.c_int64, C.c_int64]
    synref.refsyn_set_cw.argtypes = [C.c_double, C.c_double, C.c_double, C.c_char_p]
    synref.refsyn_set_fsk.argtypes = [C.c_uint64, C.c_double, C.c_uint64]
    synref.refsyn_set_psk.argtypes = [C.c_double, C.c_uint64]
    if d is not None:
        synref.refsyn_set_ssb(d.get("tone2_hz", 0), d.get("audio_low_hz", 300), d.get("audio_high_hz", 3000))
        synref.refsyn_set_cw(d.get("words_per_minute", 20.0), d.get("rise_fall_ms", 5.0),
                             d.get("message_gap_dots", 7.0), d.get("text", b"CQ DE REVENANT"))
        synref.refsyn_set_fsk(d.get("seed", 0), d.get("symbol_rate", 1200.0), d.get("symbol_count", 256))
        synref.refsyn_set_psk(d.get("rolloff", 0.35), d.get("span_symbols", 8))
    synref.refsyn_tone.argtypes = [C.c_int, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_double,
                                   C.c_double, C.c_uint64, C.c_uint64, C.c_double, C.c_void_p]
    synref.refsyn_scene_tone.argtypes = [C.c_uint64, C.c_int64, C.c_double, C.c_int, C.c_int64, C.c_int64, C.c_int64,
                                         C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_uint64, C.c_uint64,
                                         C.c_uint64, C.c_void_p]
    return synref


def tone_args(d):
    return (d["modulation"], d["rate"], d["carrier_offset"], d["tone_hz"], d["deviation"], d["amplitude"],
            d["initial_phase"], d["modulation_index"])


@pytest.mark.parametrize("d", TONES, ids=TONE_IDS)
def test_oracle_tone_emitter_matches_reference(synref, d):
    s = ref_args(synref, d)
    rng = np.random.default_rng(3)
    for first, count, gain in ((0, 5000, 1.0), (1023, 3000, 0.37), ((1 << 32) + 77, 2500, 2.5)):
        io = (1e-3 * rng.standard_normal((count, 2))).astype(np.float32)
        want = io.copy()
        assert s.refsyn_tone(*tone_args(d), first, count, gain, want.ctypes.data) == 0
        got = ora_tone(d, first, count, gain, io)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (first, gain)


@pytest.mark.parametrize("d", [TONES[0], TONES[1], TONES[5], TONES[6], TONES[8], TONES[11]],
                         ids=["am", "nfm", "lsb-two-tone", "cw", "fsk", "qpsk"])
def test_oracle_scene_with_emitter_matches_reference(synref, d):
    s = ref_args(synref, d)
    seed, dbfs, on, off, start, count = 21, -50.0, 5000, 20_000, 3000, 20_000
    want = np.zeros((count, 2), np.float32)
    assert s.refsyn_scene_tone(seed, d["rate"], dbfs, *tone_args(d)[:1], *tone_args(d)[2:], on, off, start, count,
                               want.ctypes.data) == 0
    assert np.array_equal(ora_scene(seed, dbfs, d, on, off, start, count).view(np.uint32), want.view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("d", TONES, ids=TONE_IDS)
def test_gpu_tone_emitter_matches_oracle(gpu, d):
    rng = np.random.default_rng(4)
    for first, count, gain in ((0, 100_000, 1.0), (1023, 30_000, 0.37), ((1 << 32) + 77, 25_000, 2.5)):
        io = (1e-3 * rng.standard_normal((count, 2))).astype(np.float32)
        buf = gpu.array(io)
        assert lib().rv_emitter_accumulate(gpu.stream, C.byref(tone(d)), first, count, gain, buf.ptr, count) == 0, \
            lib().rv_last_error()
        got = buf.download(np.float32, (count, 2))
        want = ora_tone(d, first, count, gain, io)
        if d["modulation"] in (1, 3, 4, 5, 6, 7):  # anchors and tables from the C library, the rest + and *
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), first
        else:  # NFM, CW: CUDA's FP64 cos/sin of the deviation, or of the keying edges
            n = check_close(got, want)
            print("%s emitter, %d samples from %d: %d of %d components off by one FP32 ulp"
                  % ("NFM" if d["modulation"] == 2 else "CW", count, first, n, 2 * count))


@pytest.mark.gpu
def test_gpu_scene_with_emitter_matches_oracle(gpu):
    """Scene::render of noise plus an AM burst, composed as the scene does:
    the noise field, then the burst's emitter indices added over its window."""
    d = TONES[0]
    seed, dbfs, on, off, start, count = 21, -50.0, 5000, 200_000, 3000, 300_000
    sigma = lib().rv_scene_noise_sigma(dbfs)
    buf = gpu.zeros(count * 8)
    assert lib().rv_scene_noise(gpu.stream, seed, sigma, start, count, buf.ptr, count) == 0
    lo, hi = max(on, start), min(off, start + count)
    assert lib().rv_emitter_accumulate(gpu.stream, C.byref(tone(d)), lo - on, hi - lo, 1.0,
                                       buf.address + 8 * (lo - start), hi - lo) == 0, lib().rv_last_error()
    got = buf.download(np.float32, (count, 2))
    check_close(got, ora_scene(seed, dbfs, d, on, off, start, count))


def test_emitter_rejects_bad_specs(rv):
    one = np.zeros(4, np.float32)
    for bad in (dict(modulation=-1), dict(modulation=8), dict(modulation=6, symbol_rate=1200.0, symbol_count=4,
                                                               rolloff=0.35, span_symbols=8), dict(modulation=0, words_per_minute=20.0, rise_fall_ms=5.0, text=b"#"),
                dict(modulation=0, words_per_minute=20.0, rise_fall_ms=5.0, text=b"   "),
                dict(modulation=0, words_per_minute=2e6, rise_fall_ms=5.0, text=b"E"), dict(tone_hz=0), dict(tone_hz=1_200_000), dict(carrier_offset=1_300_000),
                dict(amplitude=-1.0), dict(modulation=2, deviation=0), dict(rate=0), dict(modulation=5),
                dict(modulation=3, audio_low_hz=300, audio_high_hz=3000, tone_hz=200),
                dict(modulation=4, audio_low_hz=3000, audio_high_hz=300),
                dict(modulation=3, audio_low_hz=300, audio_high_hz=3000, tone2_hz=5000)):
        d = dict(TONES[0])
        d.update(bad)
        assert rv.rv_emitter_accumulate(None, C.byref(tone(d)), 0, 1, 1.0, one.ctypes.data, 1) < 0, bad


# ---- random populations (Scene::create's layout) and whole scenes ----------

POPULATIONS = [dict(seed=5, rate=2_400_000, duration=0, noise_dbfs=-60.0, emitters=12, bursts=1,
                    span=(-1_000_000, 1_000_000), snr=(5.0, 35.0), burst_seconds=(0.05, 2.0), palette=(0, 1, 2, 3, 4)),
               dict(seed=77, rate=20_000_000, duration=4_000_000, noise_dbfs=-70.0, emitters=20, bursts=3,
                    span=(-9_000_000, 9_000_000), snr=(-5.0, 30.0), burst_seconds=(0.001, 0.05),
                    palette=()),
               dict(seed=2, rate=48_000, duration=200_000, noise_dbfs=-50.0, emitters=4, bursts=2,
                    span=(-20_000, 20_000), snr=(10.0, 20.0), burst_seconds=(0.5, 2.0), palette=(0,))]


def ref_random(s, d, start=0, count=0):
    s.refsyn_random_scene.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_double, C.c_uint32, C.c_uint32,
                                      C.c_int64, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_double,
                                      C.c_uint32, C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p,
                                      C.c_uint32, C.POINTER(C.c_uint32)]
    pal = np.array(d["palette"], np.int32)
    truth = np.zeros((1024, 8))
    n = C.c_uint32()
    out = np.zeros((max(count, 1), 2), np.float32)
    assert s.refsyn_random_scene(d["seed"], d["rate"], d["duration"], d["noise_dbfs"], d["emitters"], d["bursts"],
                                 d["span"][0], d["span"][1], d["snr"][0], d["snr"][1], d["burst_seconds"][0],
                                 d["burst_seconds"][1], len(pal), pal.ctypes.data, start, count,
                                 out.ctypes.data if count else None, truth.ctypes.data, 1024, C.byref(n)) == 0
    return truth[:n.value], out[:count]


def ora_random_scene(d, start, count):
    """The scene from the library's plan, rendered by the oracle: noise, then
    each burst's emitter over its window, in burst order."""
    from revenant_gb300 import scene
    pop = scene.population(**d)
    out = ora_noise(d["seed"], ora_lib().or_scene_noise_sigma(d["noise_dbfs"]), start, count)
    for b in scene.plan(pop):
        lo, hi = max(b.start, start), min(b.end, start + count)
        if lo < hi:
            from revenant_gb300 import abi
            o = oracle().lib
            o.or_emitter_accumulate.argtypes = [C.POINTER(abi.ToneEmitter), C.c_uint64, C.c_uint64, C.c_double,
                                                C.c_void_p]
            part = np.ascontiguousarray(out[lo - start:hi - start])
            assert o.or_emitter_accumulate(C.byref(b.emitter), lo - b.start, hi - lo, b.gain, part.ctypes.data) == 0
            out[lo - start:hi - start] = part
    return out


@pytest.mark.parametrize("d", POPULATIONS, ids=["always-on", "bursty-20MSps", "cw-only"])
def test_plan_matches_reference_layout(synref, d):
    from revenant_gb300 import scene
    truth, _ = ref_random(synref, d)
    got = scene.plan(scene.population(**d))
    assert len(got) == len(truth) > 0
    for b, t in zip(got, truth):
        end = -1.0 if b.end == 2**64 - 1 else float(b.end)
        assert (float(b.start), end, float(b.emitter.carrier_offset), float(b.emitter.modulation)) == tuple(t[:4])
        assert b.mean_power == t[4] and b.snr_in_occupied_bandwidth_db == t[5]
        assert (float(b.extent_low_hz), float(b.extent_high_hz)) == tuple(t[6:8])


@pytest.mark.parametrize("d,start,count", [(POPULATIONS[0], 1000, 30_000), (POPULATIONS[1], 0, 200_000),
                                           (POPULATIONS[2], 40_000, 60_000)], ids=["always-on", "bursty", "cw"])
def test_oracle_random_scene_matches_reference_render(synref, d, start, count):
    _, want = ref_random(synref, d, start, count)
    got = ora_random_scene(d, start, count)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_plan_refuses_bad_populations(rv):
    from revenant_gb300 import abi, scene
    n = C.c_uint32()
    for bad in (dict(palette=(1, 9)), dict(span=(5, 5)), dict(bursts=0), dict(snr=(10.0, 5.0))):
        pop = scene.population(**dict(POPULATIONS[0], **bad))
        assert rv.rv_scene_plan(C.byref(pop), None, 0, C.byref(n)) == abi.RV_ERR_INVALID, bad


@pytest.mark.gpu
@pytest.mark.parametrize("d,start,count", [(POPULATIONS[0], 1000, 300_000), (POPULATIONS[1], 0, 4_000_000),
                                           (POPULATIONS[2], 0, 200_000)], ids=["always-on", "bursty", "cw"])
def test_gpu_random_scene_matches_oracle(gpu, d, start, count):
    from revenant_gb300 import scene
    buf = scene.render(gpu, scene.population(**d), start, count)
    got = buf.download(np.float32, (count, 2))
    n = check_close(got, ora_random_scene(d, start, count))
    print("random scene seed %d, %d samples: %d of %d components off by one FP32 ulp" % (d["seed"], count, n, 2 * count))


# ---- supplied audio (AM, NFM, SSB through the Hilbert phasing network) -----

AUDIO_CASES = [dict(modulation=1, rate=48_000, carrier_offset=6_000, deviation=0, amplitude=0.5, initial_phase=0.2,
                    modulation_index=0.7),
               dict(modulation=2, rate=48_000, carrier_offset=-9_000, deviation=3_000, amplitude=1.0,
                    initial_phase=1.0, modulation_index=0.0),
               dict(modulation=3, rate=48_000, carrier_offset=2_000, deviation=0, amplitude=0.8, initial_phase=0.0,
                    modulation_index=0.0, audio_low_hz=300, audio_high_hz=3000),
               dict(modulation=4, rate=48_000, carrier_offset=-12_000, deviation=0, amplitude=1.0, initial_phase=2.5,
                    modulation_index=0.0, audio_low_hz=300, audio_high_hz=3000)]
AUDIO_IDS = ["am", "nfm", "usb", "lsb"]
HILBERT_TAPS = 301


def speech_like(n, seed=6):
    rng = np.random.default_rng(seed)
    t = np.arange(n) / 48_000
    a = sum(np.sin(2 * np.pi * f * t + rng.uniform(0, 6)) / k for k, f in enumerate((420, 910, 1700, 2600), 1))
    return (0.3 * a * (1 + 0.5 * np.sin(2 * np.pi * 3 * t))).astype(np.float32)


def ora_audio(d, audio, first, count, gain, io):
    from revenant_gb300 import abi
    o = oracle().lib
    o.or_emitter_accumulate_audio.argtypes = [C.POINTER(abi.ToneEmitter), C.c_void_p, C.c_uint64, C.c_uint32,
                                              C.c_uint64, C.c_uint64, C.c_double, C.c_void_p]
    out = io.copy()
    assert o.or_emitter_accumulate_audio(C.byref(tone(d)), audio.ctypes.data, audio.size, HILBERT_TAPS, first, count,
                                         gain, out.ctypes.data) == 0
    return out


@pytest.mark.parametrize("d", AUDIO_CASES, ids=AUDIO_IDS)
def test_oracle_audio_emitter_matches_reference(synref, d):
    synref.refsyn_audio_emitter.argtypes = [C.c_int, C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_double,
                                            C.c_double, C.c_void_p, C.c_uint64, C.c_uint32, C.c_int64, C.c_int64,
                                            C.c_uint64, C.c_uint64, C.c_double, C.c_void_p]
    audio = speech_like(30_000)
    rng = np.random.default_rng(8)
    for first, count in ((0, 32_000), (1000, 5000), (29_500, 2000)):  # past the audio's end too
        io = (1e-3 * rng.standard_normal((count, 2))).astype(np.float32)
        want = io.copy()
        assert synref.refsyn_audio_emitter(d["modulation"], d["rate"], d["carrier_offset"], d["deviation"],
                                           d["amplitude"], d["initial_phase"], d["modulation_index"],
                                           audio.ctypes.data, audio.size, HILBERT_TAPS, d.get("audio_low_hz", 300),
                                           d.get("audio_high_hz", 3000), first, count, 0.8, want.ctypes.data) == 0
        got = ora_audio(d, audio, first, count, 0.8, io)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), first


@pytest.mark.gpu
@pytest.mark.parametrize("d", AUDIO_CASES, ids=AUDIO_IDS)
def test_gpu_audio_emitter_matches_oracle(gpu, d):
    audio = speech_like(100_000)
    rng = np.random.default_rng(9)
    for first, count in ((0, 120_000), (4097, 50_000)):
        io = (1e-3 * rng.standard_normal((count, 2))).astype(np.float32)
        buf = gpu.array(io)
        assert lib().rv_emitter_accumulate_audio(gpu.stream, C.byref(tone(d)), audio.ctypes.data, audio.size,
                                                 HILBERT_TAPS, first, count, 0.8, buf.ptr, count) == 0, \
            lib().rv_last_error()
        got = buf.download(np.float32, (count, 2))
        want = ora_audio(d, audio, first, count, 0.8, io)
        if d["modulation"] == 2:  # NFM: CUDA's FP64 cos/sin of the phase per sample
            n = check_close(got, want)
            print("NFM audio emitter, %d samples from %d: %d of %d components off by one FP32 ulp"
                  % (count, first, n, 2 * count))
        else:
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), first
