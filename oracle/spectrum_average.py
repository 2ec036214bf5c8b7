"""FP64 restatement of lw-radio-dsp's averaged power spectrum.

TEST INFRASTRUCTURE (the oracle): only the tests, the smoke check and the
benchmark's CPU baseline use this module, and only as the checker.

Follows third_party/lw-radio-dsp:
  make_window           src/primitives.cpp:124-148 (symmetric, double, rounded to float)
  power_spectrum        src/fft.cpp:31-50 (window, C2C forward FFT, |X|^2 / wsum^2,
                        fftshift: bin k reads (k + n - n/2) % n)
  Spectrum::compute     src/spectrum.cpp:32-44 (avg = a*avg + (1-a)*p, the first
                        frame seeding avg with itself; a clamped to [0, 0.999])
  power_to_db           include/lwdsp/types.h:38 (10 log10(max(p, 1e-30)))
with every step in float64 (numpy's double FFT) except the window values,
which the reference stores as floats. The boxcar MEAN over `average` frames is
not in lwdsp: it is the "averaged over 16 frames" spectrum of the plain
single-receiver configuration (1024-point Hann), restated here in FP64.
The reference transforms in float32 with pocketfft, so neither it nor the GPU
matches this to the bit; the tests state their tolerances.
"""
import numpy as np

RECTANGULAR, HANN, BLACKMAN_HARRIS = 0, 1, 2


def window(kind, n):
    """make_window: n float32 values of the symmetric window."""
    x = np.arange(n, dtype=np.float64) / float(n - 1)
    if kind == RECTANGULAR:
        v = np.ones(n)
    elif kind == HANN:
        v = 0.5 - 0.5 * np.cos(2.0 * np.pi * x)
    elif kind == BLACKMAN_HARRIS:
        v = (0.35875 - 0.48829 * np.cos(2.0 * np.pi * x) + 0.14128 * np.cos(4.0 * np.pi * x)
             - 0.01168 * np.cos(6.0 * np.pi * x))
    else:
        raise ValueError("window kind %r" % kind)
    return v.astype(np.float32)


def norm(w):
    """power_spectrum's 1 / wsum^2, wsum summed in double over the floats."""
    s = float(np.sum(w.astype(np.float64)))
    return 1.0 / (s * s)


def frame_power(iq, w):
    """Linear power per fftshifted bin of each frame; iq is (frames, n) complex."""
    n = w.size
    x = np.asarray(iq, np.complex128).reshape(-1, n) * w.astype(np.float64)
    X = np.fft.fft(x, axis=1)
    p = (X.real * X.real + X.imag * X.imag) * norm(w)
    return np.roll(p, n // 2, axis=1)  # out[k] = p[(k + n - n/2) % n]


def to_db(p):
    return 10.0 * np.log10(np.maximum(p, 1e-30))


def mean_db(iq, w, average):
    """One dB spectrum per `average` consecutive frames: the boxcar mean."""
    p = frame_power(iq, w)
    p = p.reshape(-1, average, w.size).mean(axis=1)
    return to_db(p), p


def exponential_db(iq, w, alpha, previous=None):
    """lwdsp's exponential average over every frame; returns dB and the average."""
    a = min(max(float(alpha), 0.0), 0.999)
    avg = None if previous is None else np.asarray(previous, np.float64)
    for p in frame_power(iq, w):
        if avg is None:
            avg = p
        avg = a * avg + (1.0 - a) * p
    return to_db(avg), avg
