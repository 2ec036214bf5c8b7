"""Averaged power spectrum (lw-radio-dsp Spectrum::compute) against the FP64 oracle.

The reference computes this spectrum in float32 with pocketfft and the GPU
with its own radix-2 transform, so agreement is to a tolerance, stated here:

  REL_RMS  relative RMS error of the linear power over all bins, against the
           FP64 oracle: <= 1e-5 (the reference itself sits near 1.3e-7);
  DB_TOL   absolute dB error on every bin within 80 dB of the spectrum's peak:
           <= 0.01 dB.

Windows are exact: the reference's make_window, the oracle's and the
library's host builder agree bit for bit. The known answer is lwdsp's own
(tests/test_radio.cpp:277): a full-scale complex tone reads 0 dBFS in its bin.
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

import spectrum_average as sa  # noqa: E402  oracle/spectrum_average.py
from revenant_gb300 import abi  # noqa: E402
from revenant_gb300.library import lib  # noqa: E402

REL_RMS = 1e-5
DB_TOL = 0.01
GOLDEN = os.path.join(HERE, "golden", "lwdsp_spectrum.npz")


def golden():
    return np.load(GOLDEN)


def within(db, want_db):
    """Both tolerances; db and want_db are one or more dB rows."""
    db, want_db = np.atleast_2d(db).astype(np.float64), np.atleast_2d(want_db).astype(np.float64)
    p, q = 10.0 ** (db / 10.0), 10.0 ** (want_db / 10.0)
    rel = np.sqrt(np.mean((p - q) ** 2, axis=1)) / np.sqrt(np.mean(q * q, axis=1))
    near = want_db > want_db.max(axis=1, keepdims=True) - 80.0
    worst_db = np.abs(db - want_db)[near].max()
    assert rel.max() <= REL_RMS, "relative RMS %.3g > %.1g" % (rel.max(), REL_RMS)
    assert worst_db <= DB_TOL, "dB error %.4g > %.2g" % (worst_db, DB_TOL)


def seeded_iq(n, frames, seed):
    rng = np.random.default_rng(seed)
    t = np.arange(n * frames, dtype=np.float64)
    f = rng.uniform(-0.5, 0.5, 3)
    a = 10.0 ** (-rng.uniform(0, 4, 3))
    z = sum(a[i] * np.exp(2j * np.pi * f[i] * t) for i in range(3))
    z = z + 1e-3 * (rng.standard_normal(n * frames) + 1j * rng.standard_normal(n * frames))
    return z.astype(np.complex64)


# -- CPU: the oracle and the host window against the reference -----------------

@pytest.mark.parametrize("kind,n", [(0, 16), (1, 1024), (1, 1000), (2, 4096), (2, 8192)])
def test_window_bits_oracle_vs_library(rv, kind, n):
    w = np.zeros(n, np.float32)
    norm = C.c_double()
    assert lib().rv_build_lwdsp_window(kind, n, w.ctypes.data, C.byref(norm)) == 0
    assert np.array_equal(w.view(np.uint32), sa.window(kind, n).view(np.uint32))
    assert norm.value == sa.norm(w)


def test_window_bits_oracle_vs_reference_golden():
    g = golden()
    assert np.array_equal(g["window_hann1024"].view(np.uint32), sa.window(sa.HANN, 1024).view(np.uint32))
    assert np.array_equal(g["window_bh4096"].view(np.uint32), sa.window(sa.BLACKMAN_HARRIS, 4096).view(np.uint32))


def test_oracle_vs_reference_golden_exponential():
    g = golden()
    w = sa.window(sa.HANN, 1024)
    iq = g["hann_iq"].reshape(16, 1024)
    avg = None
    for f in range(16):  # one reference call per frame; the average carries across
        db, avg = sa.exponential_db(iq[f], w, 0.75, previous=avg)
        within(g["hann1024_exp"][f], db)


def test_oracle_vs_reference_golden_mean():
    g = golden()
    w = sa.window(sa.HANN, 1024)
    per_frame = 10.0 ** (g["hann1024_raw"].astype(np.float64) / 10.0)  # the reference's 16 spectra
    db, _ = sa.mean_db(g["hann_iq"], w, 16)
    within(10.0 * np.log10(per_frame.mean(axis=0)), db)


def test_oracle_known_answer_tone():
    """lwdsp: a full-scale 3 kHz tone at 48 kHz reads 0 dBFS at 3 kHz (4096-pt BH)."""
    g = golden()
    db, _ = sa.exponential_db(g["tone_iq"], sa.window(sa.BLACKMAN_HARRIS, 4096), 0.0)
    k = int(np.argmax(db))
    assert abs((k - 2048) * 48000.0 / 4096 - 3000.0) <= 0.005 * 3000.0
    assert abs(db[k]) < 0.5
    within(g["bh4096_tone"], db)


@pytest.mark.parametrize("kind,n,frames,alpha", [(1, 16, 8, 0.9), (2, 2048, 5, 0.5), (1, 1000, 3, 0.3)])
def test_oracle_vs_reference_live(ref, kind, n, frames, alpha):
    iq = seeded_iq(n, frames, n + frames)
    rows = np.zeros((frames, n), np.float32)
    assert ref.fn("lwdsp_spectrum")(n, kind, alpha, iq.ctypes.data, frames, rows.ctypes.data) == 0
    db, _ = sa.exponential_db(iq, sa.window(kind, n), alpha)
    within(rows[-1], db)


# -- GPU: rv_spectrum_average against the oracle -------------------------------

def _twiddles(n):
    tw = np.zeros((n, 2), np.float32)
    assert lib().rv_build_fft_twiddles(n, tw.ctypes.data, n) == 0
    return tw


@pytest.mark.parametrize("n", [16, 256, 2048])
def test_fft_twiddles_equal_the_grid_twiddles(rv, n):
    a, b = np.zeros((n, 2), np.float32), np.zeros((n, 2), np.float32)
    assert lib().rv_build_twiddles(n, a.ctypes.data, n) == 0
    assert lib().rv_build_fft_twiddles(n, b.ctypes.data, n) == 0
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def gpu_spectrum(gpu, iq, n, kind, mode, average=1, alpha=0.0, avg_in=None, resume=False):
    frames = iq.size // n
    w = np.zeros(n, np.float32)
    norm = C.c_double()
    assert lib().rv_build_lwdsp_window(kind, n, w.ctypes.data, C.byref(norm)) == 0
    p = abi.SpectrumAverageParams(size=n, frames=frames, average=average, mode=mode, alpha=alpha,
                                  norm=norm.value, resume=int(resume))
    spectra = frames // average if mode == abi.AVERAGE_MEAN else 1
    d_iq = gpu.array(iq.view(np.float32))
    d_w, d_tw = gpu.array(w), gpu.array(_twiddles(n))
    out = gpu.zeros(spectra * n * 4)
    avg = gpu.array(avg_in.astype(np.float32)) if avg_in is not None else gpu.zeros(spectra * n * 4)
    st = lib().rv_spectrum_average(gpu.stream, C.byref(p), d_iq.ptr, iq.size, d_w.ptr, n, d_tw.ptr, n,
                                   out.ptr, spectra * n, avg.ptr, spectra * n)
    assert st == 0, lib().rv_last_error().decode()
    gpu.synchronize()
    return out.download(np.float32, (spectra, n)), avg.download(np.float32, (spectra, n))


@pytest.mark.gpu
@pytest.mark.parametrize("n,frames,average,kind", [(1024, 16, 16, 1), (1024, 64, 16, 1), (16, 6, 3, 0),
                                                   (4096, 8, 4, 2), (8192, 4, 2, 1)])
def test_gpu_mean(gpu, n, frames, average, kind):
    iq = seeded_iq(n, frames, n * 7 + frames)
    db, avg = gpu_spectrum(gpu, iq, n, kind, abi.AVERAGE_MEAN, average=average)
    want, want_p = sa.mean_db(iq, sa.window(kind, n), average)
    within(db, want)
    rel = np.sqrt(np.mean((avg - want_p) ** 2, axis=1)) / np.sqrt(np.mean(want_p ** 2, axis=1))
    assert rel.max() <= REL_RMS  # the linear average handed back in avg_dev


@pytest.mark.gpu
@pytest.mark.parametrize("n,frames,alpha,kind", [(1024, 16, 0.75, 1), (2048, 9, 0.999, 2), (256, 4, 0.0, 1)])
def test_gpu_exponential(gpu, n, frames, alpha, kind):
    iq = seeded_iq(n, frames, n + 11 * frames)
    db, _ = gpu_spectrum(gpu, iq, n, kind, abi.AVERAGE_EXPONENTIAL, alpha=alpha)
    want, _ = sa.exponential_db(iq, sa.window(kind, n), alpha)
    within(db, want)


@pytest.mark.gpu
def test_gpu_vs_reference_golden(gpu):
    g = golden()
    db, _ = gpu_spectrum(gpu, g["hann_iq"], 1024, sa.HANN, abi.AVERAGE_EXPONENTIAL, alpha=0.75)
    within(db, g["hann1024_exp"][-1])
    per_frame = 10.0 ** (g["hann1024_raw"].astype(np.float64) / 10.0)
    db, _ = gpu_spectrum(gpu, g["hann_iq"], 1024, sa.HANN, abi.AVERAGE_MEAN, average=16)
    within(db, 10.0 * np.log10(per_frame.mean(axis=0)))


@pytest.mark.gpu
def test_gpu_known_answer_tone(gpu):
    g = golden()
    db, _ = gpu_spectrum(gpu, g["tone_iq"], 4096, sa.BLACKMAN_HARRIS, abi.AVERAGE_EXPONENTIAL)
    k = int(np.argmax(db[0]))
    assert abs((k - 2048) * 48000.0 / 4096 - 3000.0) <= 0.005 * 3000.0
    assert abs(db[0, k]) < 0.5
    within(db, g["bh4096_tone"])


@pytest.mark.gpu
def test_gpu_resume_matches_one_call(gpu):
    """Two calls with the average carried on equal one call, bit for bit."""
    n = 1024
    iq = seeded_iq(n, 16, 99)
    whole, whole_avg = gpu_spectrum(gpu, iq, n, sa.HANN, abi.AVERAGE_EXPONENTIAL, alpha=0.8)
    _, first_avg = gpu_spectrum(gpu, iq[:8 * n], n, sa.HANN, abi.AVERAGE_EXPONENTIAL, alpha=0.8)
    second, second_avg = gpu_spectrum(gpu, iq[8 * n:], n, sa.HANN, abi.AVERAGE_EXPONENTIAL, alpha=0.8,
                                      avg_in=first_avg, resume=True)
    assert np.array_equal(second.view(np.uint32), whole.view(np.uint32))
    assert np.array_equal(second_avg.view(np.uint32), whole_avg.view(np.uint32))


@pytest.mark.gpu
def test_gpu_rejects_bad_arguments(gpu):
    n = 1024
    d_iq, d_w, d_tw, out = gpu.zeros(n * 16 * 8), gpu.zeros(n * 4), gpu.zeros(n * 8), gpu.zeros(n * 16 * 4)
    bad = [dict(size=1000, frames=16, average=16, mode=0), dict(size=n, frames=16, average=5, mode=0),
           dict(size=n, frames=16, average=0, mode=0), dict(size=n, frames=16, mode=1, alpha=1.0),
           dict(size=n, frames=16, mode=1, alpha=0.5, resume=1), dict(size=n, frames=16, average=16, mode=2),
           dict(size=16384, frames=1, average=1, mode=0)]
    for kw in bad:
        p = abi.SpectrumAverageParams(norm=1.0, **kw)
        avg = None if kw.get("resume") else out.ptr
        st = lib().rv_spectrum_average(gpu.stream, C.byref(p), d_iq.ptr, n * 16, d_w.ptr, kw["size"], d_tw.ptr,
                                       kw["size"], out.ptr, n * 16, avg, 0 if avg is None else n * 16)
        assert st == abi.RV_ERR_INVALID, kw
