"""Seeded synthetic IQ captures for the chain tests and the benchmark.

Scenes are sums of modulated carriers (FM with a stereo multiplex, AM, SSB
tones, plain tones) plus white noise at a stated SNR, quantised to cu8 or
cs16 exactly as a receiver front end would deliver them. These stand in for
the reference's siggen scenes (core/dsp/synth/wideband.h); only their shape
matters to the chain, which is checked bit for bit against the oracle.
"""
import numpy as np


def quantise(z, fmt, scale=0.9):
    """complex -> interleaved codes (cs16: int16 pairs, cu8: uint8 pairs)."""
    peak = np.max(np.abs(np.concatenate([z.real, z.imag]))) or 1.0
    x = z * (scale / peak)
    if fmt == "cs16":
        out = np.empty(2 * z.size, np.int16)
        out[0::2] = np.clip(np.round(x.real * 32767), -32768, 32767)
        out[1::2] = np.clip(np.round(x.imag * 32767), -32768, 32767)
        return out
    out = np.empty(2 * z.size, np.uint8)
    out[0::2] = np.clip(np.round(x.real * 127.5 + 127.5), 0, 255)
    out[1::2] = np.clip(np.round(x.imag * 127.5 + 127.5), 0, 255)
    return out


def wfm(n, rate, offset, deviation=75_000, tone=1000.0, stereo=True, amp=1.0, t0=0):
    t = (np.arange(n) + t0) / rate
    left = np.sin(2 * np.pi * tone * t)
    right = 0.5 * np.sin(2 * np.pi * 2.5 * tone * t)
    mpx = 0.45 * (left + right)
    if stereo:
        mpx = mpx + 0.1 * np.cos(2 * np.pi * 19_000 * t) + 0.45 * (left - right) * np.cos(2 * np.pi * 38_000 * t)
    phase = 2 * np.pi * deviation * np.cumsum(mpx) / rate
    return amp * np.exp(1j * (2 * np.pi * offset * t + phase))


def nfm(n, rate, offset, deviation=2_500, tone=1000.0, amp=1.0, t0=0):
    t = (np.arange(n) + t0) / rate
    phase = 2 * np.pi * deviation * np.cumsum(np.sin(2 * np.pi * tone * t)) / rate
    return amp * np.exp(1j * (2 * np.pi * offset * t + phase))


def am(n, rate, offset, depth=0.6, tone=1000.0, amp=1.0, t0=0):
    t = (np.arange(n) + t0) / rate
    return amp * (1 + depth * np.sin(2 * np.pi * tone * t)) * np.exp(2j * np.pi * offset * t)


def ssb(n, rate, offset, tone=1000.0, amp=1.0, upper=True, t0=0):
    t = (np.arange(n) + t0) / rate
    f = offset + (tone if upper else -tone)
    return amp * np.exp(2j * np.pi * f * t)


def noise(n, rng, power):
    return np.sqrt(power / 2) * (rng.standard_normal(n) + 1j * rng.standard_normal(n))


def scene(n, rate, emitters, snr_db=30.0, seed=0):
    """Sum of (kind, offset, amp) emitters plus noise snr_db below the
    strongest one."""
    rng = np.random.default_rng(seed)
    z = np.zeros(n, np.complex128)
    for kind, offset, amp in emitters:
        z += {"wfm": wfm, "nfm": nfm, "am": am, "usb": ssb,
              "lsb": lambda n, r, o, amp: ssb(n, r, o, amp=amp, upper=False)}[kind](n, rate, offset, amp=amp)
    peak = max(a for _, _, a in emitters) if emitters else 1.0
    return z + noise(n, rng, peak ** 2 * 10 ** (-snr_db / 10))


def random_receivers(count, rate, seed, modes=("nfm", "am", "usb", "lsb", "wfm"), bw=(12_500, 200_000),
                     grid=(64, 17, 32)):
    """Seeded receiver population: offsets uniform over the span, bandwidth
    uniform in bw, modes uniform; a request the planner refuses is redrawn.
    The planner is the oracle's restatement (pinned to the reference's and
    to the GPU library's), so drawing needs no GPU library."""
    import ctypes as C

    from bindings import oracle
    from revenant_gb300 import abi

    o = oracle().lib
    rng = np.random.default_rng(seed)
    g = abi.GridParams(*grid)
    out = []
    while len(out) < count:
        mode = modes[int(rng.integers(0, len(modes)))]
        b = int(rng.uniform(*bw))
        c = int(rng.uniform(-0.45 * rate, 0.45 * rate))
        req = abi.request(center=c, bandwidth=b, demod=mode, stereo=True)
        pl = abi.VrxPlacement()
        if o.or_place(C.byref(g), rate, C.byref(req), C.byref(pl)) != 0:
            continue
        info = abi.VrxPlanInfo()
        if o.or_plan_vrx(C.byref(g), rate, C.byref(req), C.byref(pl), C.byref(info), None, 0, None, 0) != 0:
            continue
        out.append(req)
    return out
