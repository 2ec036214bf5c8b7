"""Seeded inputs for every stage of the receive chain.

Each builder returns plain numpy arrays plus the ctypes parameter structs, so
the same case can be run through the reference twins, the oracle and the GPU
library and compared byte for byte. Seeds are explicit; a failing test prints
its seed (the reference's conformance suite does the same,
tests/reference/reference_diff.h:185-210).
"""
import ctypes as C

import numpy as np

from revenant_gb300 import abi

# grids exercised everywhere: the shipped 64-channel grid, the 8-channel WFM
# grid, a 1024-channel wideband grid, and a critically-sampled one.
GRIDS = [(64, 17, 32), (8, 17, 4), (1024, 16, 512), (16, 4, 16), (128, 9, 64)]


def rng(seed):
    return np.random.default_rng(seed)


def noise_cf32(r, n, scale=0.5):
    x = r.standard_normal((n, 2)).astype(np.float32) * np.float32(scale)
    return x


def tone_cf32(n, freq, amp=0.5, phase=0.0, start=0):
    t = np.arange(start, start + n, dtype=np.float64)
    ph = 2 * np.pi * freq * t + phase
    return np.stack([amp * np.cos(ph), amp * np.sin(ph)], axis=1).astype(np.float32)


def grid(M, T, D):
    g = abi.GridParams()
    g.channels, g.taps_per_branch, g.decimation = M, T, D
    return g


def random_taps(r, n):
    """A taps table with the dynamic range of a designed prototype."""
    h = (r.standard_normal(n) * np.exp(-np.linspace(-3, 3, n) ** 2)).astype(np.float32)
    return h / np.float32(np.abs(h).sum())


def twiddles64(M):
    """The exact-quadrature twiddle circle, built like build_twiddles: this
    helper is only used where the table is an input and both sides read it."""
    j = np.arange(M)
    ang = 2 * np.pi * j / M
    w = np.stack([np.cos(ang), -np.sin(ang)], axis=1).astype(np.float32)
    q = M // 4
    if M >= 4:
        w[0] = (1, 0)
        w[q] = (0, -1)
        w[2 * q] = (-1, 0)
        w[3 * q] = (0, 1)
    return w


def convert_case(seed, fmt, count, ring_log2=12, dst_offset=None, src_offset=None):
    r = rng(seed)
    bps = abi.BYTES_PER_SAMPLE[fmt]
    if src_offset is None:
        src_offset = int(r.integers(0, 7))
    total = src_offset + count
    nbytes = ((total * bps + 3) // 4) * 4
    packed = r.integers(0, 256, nbytes, dtype=np.uint8)
    p = abi.ConvertParams()
    p.ring_mask = (1 << ring_log2) - 1
    p.dst_offset = int(r.integers(0, 1 << 32)) if dst_offset is None else dst_offset
    p.src_offset = src_offset
    p.count = count
    return p, packed


def branch_case(seed, M, T, D, blocks, ring_log2=None, wrap=True):
    r = rng(seed)
    need = M * T + (blocks - 1) * D
    if ring_log2 is None:
        ring_log2 = max(int(np.ceil(np.log2(need))), 4)
    n = 1 << ring_log2
    ring = noise_cf32(r, n)
    taps = random_taps(r, M * T)
    p = abi.PfbBranchParams()
    p.ring_mask = n - 1
    # wrap: block 0 sits just past the ring's end so the history straddles it
    p.base_offset = (n - 40) if wrap else int(r.integers(0, 1 << 32))
    p.block_count = blocks
    return grid(M, T, D), p, taps, ring


def fft_case(seed, M, D, blocks, ring_blocks=None, block_base=None):
    r = rng(seed)
    branch = noise_cf32(r, blocks * M, scale=1.0)
    if ring_blocks is None:
        ring_blocks = 1 << int(np.ceil(np.log2(max(blocks, 1))))
    p = abi.PfbFftParams()
    p.channels, p.decimation = M, D
    p.stages = int(np.log2(M))
    p.block_base = int(r.integers(0, 1 << 32)) if block_base is None else block_base
    p.block_count = blocks
    p.out_ring_blocks = ring_blocks
    p.out_ring_mask = ring_blocks - 1
    return p, branch


def spectrum_case(seed, M, N, chan_blocks=None, in_offset=None):
    r = rng(seed)
    if chan_blocks is None:
        chan_blocks = 2 * N
    ring = noise_cf32(r, M * chan_blocks, scale=0.1)
    # a few strong tones so the frame spans a wide dB range
    for k in range(min(M, 4)):
        ring[k * chan_blocks:(k + 1) * chan_blocks] += tone_cf32(chan_blocks, 0.01 * (k + 1), amp=0.8)
    p = abi.SpectrumParams()
    p.channels, p.transform = M, N
    p.stages = int(np.log2(N))
    p.chan_blocks, p.chan_mask = chan_blocks, chan_blocks - 1
    p.in_offset = int(r.integers(0, 1 << 32)) if in_offset is None else in_offset
    return p, ring


def plan_tables(lib_fn, g, rate, req):
    """Run a plan_vrx entry point (product rv_plan_vrx or ref_plan_vrx) and
    return (info, fine_taps (n,2) f32, demod_weights f32)."""
    info = abi.VrxPlanInfo()
    return info


def fine_case(seed, cfg, taps, nco, out_rate, in_rate, count, first_output=0, chan_log2=14,
              delta=None):
    """A fine-stage case with a synthetic resampler ratio; params follow
    resample_block (core/dsp/vrx_reference.cpp:2786-2850)."""
    r = rng(seed)
    M = 4
    chan_len = 1 << chan_log2
    chan = noise_cf32(r, M * chan_len, scale=0.3)
    p = abi.VrxFineParams()
    p.chan_base = 2 * chan_len
    p.chan_mask = chan_len - 1
    step_whole, step_rem = in_rate // out_rate, in_rate % out_rate
    whole, part = divmod(first_output, out_rate)
    carry_product = part * step_rem
    first_input = first_output * step_whole + whole * step_rem + carry_product // out_rate
    p.in_offset = first_input & p.chan_mask
    p.out_mask = (1 << int(np.ceil(np.log2(max(count, 2))))) - 1
    p.out_offset = first_output & p.out_mask
    p.count = count
    p.step_whole, p.step_rem = step_whole, step_rem
    p.out_rate = out_rate
    p.frac0 = carry_product % out_rate
    p.inv_out_rate = np.float32(1.0) / np.float32(out_rate)
    if delta is None:
        delta = int(r.integers(0, 1 << 63)) * 2 + 1
    phase = (delta * first_output) & ((1 << 64) - 1)
    p.nco_phase_high, p.nco_phase_low = phase >> 32, phase & 0xFFFFFFFF
    p.nco_delta_high, p.nco_delta_low = delta >> 32, delta & 0xFFFFFFFF
    return p, chan


def demod_weights(r, cfg):
    n = cfg.audio_taps + cfg.dc_taps + (0 if cfg.pilot_taps == 0 else 2 * cfg.pilot_taps + 2 * cfg.audio_taps)
    w = (r.standard_normal(n) * 0.05).astype(np.float32)
    return w


def demod_config(mode, decimation=1, audio_taps=1, dc_taps=1, channels=1, pilot_taps=0):
    c = abi.VrxDemodConfig()
    c.mode = abi.DEMOD[mode] if isinstance(mode, str) else mode
    c.decimation, c.audio_taps, c.dc_taps = decimation, audio_taps, dc_taps
    c.channels, c.pilot_taps = channels, pilot_taps
    return c


def fm_fine_ring(r, n, deviation=0.3, pilot=0.0, amp=0.7):
    """Complex baseband of an FM signal (+ optional 19/38 kHz-like stereo
    components) so the discriminator sees realistic phase steps."""
    t = np.arange(n)
    msg = 0.6 * np.sin(2 * np.pi * 0.013 * t) + pilot * np.sin(2 * np.pi * 0.0565 * t)
    if pilot:
        msg = msg + 0.3 * np.sin(2 * np.pi * 0.113 * t) * np.sin(2 * np.pi * 0.004 * t)
    phase = np.cumsum(deviation * msg)
    z = amp * np.exp(1j * phase) + 0.01 * (r.standard_normal(n) + 1j * r.standard_normal(n))
    return np.stack([z.real, z.imag], axis=1).astype(np.float32)


def am_fine_ring(r, n, amp=0.5, depth=0.6):
    t = np.arange(n)
    env = amp * (1 + depth * np.sin(2 * np.pi * 0.007 * t))
    z = env * np.exp(1j * (0.002 * t)) + 0.01 * (r.standard_normal(n) + 1j * r.standard_normal(n))
    return np.stack([z.real, z.imag], axis=1).astype(np.float32)


def carrier_params(power=1, in_mask=4095, in_offset=0, count=1000, flags=1, shift=0.0,
                   demod_rate=48000):
    # design_carrier_loop constants (core/dsp/vrx_reference.cpp:990-1030),
    # here as plain numbers so the case stands alone
    fs = float(demod_rate)

    def gains(bn, zeta=0.70710678118654752440):
        theta = bn / fs / (zeta + 1.0 / (4.0 * zeta))
        d = 1.0 + 2.0 * zeta * theta + theta * theta
        return 4.0 * zeta * theta / d, 4.0 * theta * theta / d

    k1a, k2a = gains(400.0)
    k1t, k2t = gains(30.0)
    p = abi.VrxCarrierParams()
    p.in_mask, p.in_offset, p.count, p.flags, p.shift = in_mask, in_offset, count, flags, shift
    p.k1_acquire, p.k2_acquire, p.k1_track, p.k2_track = k1a, k2a, k1t, k2t
    p.level_alpha = 1.0 - np.exp(-1.0 / (0.005 * fs))
    p.lock_alpha = 1.0 - np.exp(-1.0 / (0.020 * fs))
    p.clamp_radians = min(2 * np.pi * 5000.0 / fs, 0.5 * np.pi)
    p.hold_in = max(1, round(0.010 * fs))
    p.hold_out = max(1, round(0.200 * fs))
    c = abi.VrxCarrierConfig()
    c.power, c.nco_log2 = power, 16
    return c, p
