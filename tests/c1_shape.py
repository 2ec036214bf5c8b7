"""C1's receiver in the shape the benchmark names (a 240 kS/s fine stage with
a 64-tap Kaiser resampler, then the FM discriminator and a decimation by 5 to
48 kHz mono audio), as a plan for the reference's per-dispatch kernels: the
planner's own WFM plan at C1's grid (M = 8, D = 4, T = 17) has the channel,
placement and NCO rules; its fine stage (T = 32, 336 kS/s) and audio stage are
replaced here by tables designed the planner's way (Kaiser-windowed sinc,
per-phase normalised, rotated to the filter centre) for the new rates. Both
the oracle and the GPU run exactly this plan, so the comparison is of the
kernels' arithmetic on a shape the planner never chooses."""
from fractions import Fraction
import ctypes as C

import numpy as np

FINE_TAPS, PHASES, DEMOD_RATE, AUDIO_RATE = 64, 256, 240_000, 48_000
AUDIO_TAPS = 121


def kaiser_beta(att):
    if att > 50:
        return 0.1102 * (att - 8.7)
    if att >= 21:
        return 0.5842 * (att - 21) ** 0.4 + 0.07886 * (att - 21)
    return 0.0


def fine_table(channel_rate, half_width, centre_hz, att=80.0):
    """(PHASES * FINE_TAPS + 1, 2) float32: phase p, tap k at p + k * PHASES."""
    length = PHASES * FINE_TAPS
    i = np.arange(length, dtype=np.float64)
    centre = (length - 1) / 2.0
    cutoff = half_width / channel_rate
    proto = 2 * cutoff * np.sinc(2 * cutoff * (i - centre) / PHASES) * np.kaiser(length, kaiser_beta(att))
    proto = proto.reshape(FINE_TAPS, PHASES)
    proto /= proto.sum(axis=0, keepdims=True)
    proto = proto.reshape(-1)
    angle = 2 * np.pi * float(centre_hz) * (i - centre) / (PHASES * channel_rate)
    table = np.zeros((length + 1, 2), np.float32)
    table[:length, 0] = proto * np.cos(angle)
    table[:length, 1] = proto * np.sin(angle)
    return table


def audio_taps(att=80.0, cutoff_hz=15_000):
    i = np.arange(AUDIO_TAPS, dtype=np.float64) - (AUDIO_TAPS - 1) / 2.0
    c = cutoff_hz / DEMOD_RATE
    d = 2 * c * np.sinc(2 * c * i) * np.kaiser(AUDIO_TAPS, kaiser_beta(att))
    return (d / d.sum()).astype(np.float32)


def apply(rx, history_of):
    """Turns an oracle-chain receiver (planned as stereo-off WFM at C1's grid)
    into the 240 kS/s / 64-tap shape: plan fields, fine taps, demod weights."""
    info = rx["info"]
    fc = info.channel_rate
    # the NCO's turn per output at the new output rate: the planner's own
    # delta (a signed 0.64 turn per sample at its rate) rescaled
    old = info.fine_nco_delta - (1 << 64) if info.fine_nco_delta >= 1 << 63 else info.fine_nco_delta
    info.fine_nco_delta = int(round(Fraction(old) * info.demod_rate / DEMOD_RATE)) % (1 << 64)
    info.fine.taps, info.fine.phases = FINE_TAPS, PHASES
    info.demod_rate = DEMOD_RATE
    info.output_rate = AUDIO_RATE
    info.stereo = 0
    d = info.demod
    d.decimation, d.audio_taps, d.pilot_taps, d.channels = DEMOD_RATE // AUDIO_RATE, AUDIO_TAPS, 0, 1
    centre = Fraction(info.filter_numerator, info.filter_denominator)
    rx["taps"] = fine_table(fc, info.bandwidth // 2, centre)
    rx["w"] = np.concatenate([audio_taps(), np.zeros(d.dc_taps, np.float32)])
    rx["history"] = history_of(C.byref(d))
    return info
