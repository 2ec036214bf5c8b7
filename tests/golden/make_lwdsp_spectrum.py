"""Writes tests/golden/lwdsp_spectrum.npz from the reference's own lw-radio-dsp.

Runs lwdsp::make_window and lwdsp::Spectrum::compute (compiled from the
reference sources into oracle/_ref/libreftwins.so by oracle/ref/Makefile) on
seeded inputs and stores inputs and outputs, so that machines without the
reference sources can still check the oracle and the GPU against it.

    python tests/golden/make_lwdsp_spectrum.py

Cases:
  hann1024_exp  1024-point Hann, averaging 0.75, 16 frames of tone + noise;
                the dB row after every call (the average carries across calls)
  hann1024_raw  the same input with averaging 0: every frame's own spectrum,
                from which the 16-frame boxcar mean is formed in FP64
  bh4096_tone   lwdsp's own known-answer case (tests/test_radio.cpp:277): a
                full-scale 3 kHz complex tone at 48 kHz, 4096-point
                Blackman-Harris, one frame
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from bindings import reference  # noqa: E402

HANN, BLACKMAN_HARRIS = 1, 2


def inputs():
    rng = np.random.default_rng(13)
    n, frames = 1024, 16
    t = np.arange(n * frames, dtype=np.float64)
    noise = rng.standard_normal(n * frames) + 1j * rng.standard_normal(n * frames)
    hann_iq = (0.7 * np.exp(2j * np.pi * (137.3 / n) * t) + 0.05 * np.exp(-2j * np.pi * (401.0 / n) * t)
               + 1e-3 * noise).astype(np.complex64)
    t = np.arange(4096, dtype=np.float64)
    tone_iq = np.exp(2j * np.pi * 3000.0 / 48000.0 * t).astype(np.complex64)
    return hann_iq, tone_iq


def main():
    ref = reference()
    if ref is None:
        raise SystemExit("the reference twins are not built; run oracle/ref/Makefile first")
    hann_iq, tone_iq = inputs()
    out = {"hann_iq": hann_iq, "tone_iq": tone_iq}
    for kind, n, name in [(HANN, 1024, "window_hann1024"), (BLACKMAN_HARRIS, 4096, "window_bh4096")]:
        w = np.zeros(n, np.float32)
        assert ref.fn("lwdsp_window")(kind, n, w.ctypes.data) == 0
        out[name] = w
    for name, alpha in [("hann1024_exp", 0.75), ("hann1024_raw", 0.0)]:
        rows = np.zeros((16, 1024), np.float32)
        assert ref.fn("lwdsp_spectrum")(1024, HANN, alpha, hann_iq.ctypes.data, 16, rows.ctypes.data) == 0
        out[name] = rows
    row = np.zeros((1, 4096), np.float32)
    assert ref.fn("lwdsp_spectrum")(4096, BLACKMAN_HARRIS, 0.0, tone_iq.ctypes.data, 1, row.ctypes.data) == 0
    out["bh4096_tone"] = row
    np.savez_compressed(os.path.join(HERE, "lwdsp_spectrum.npz"), **out)
    print("wrote", os.path.join(HERE, "lwdsp_spectrum.npz"))


if __name__ == "__main__":
    main()
