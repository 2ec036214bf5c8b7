"""Comb / spur cancellation kernels (core/dsp/comb_kernels_reference.cpp)
against the reference's twins and the oracle restatement, bit for bit: the
step and table, the projections of every line onto every sub-block, and the
cleaned and removed rings; the GPU against the oracle the same way. A comb
of harmonics is put into a noisy ring, projected, and the projections (as
the tracker would) handed back as amplitudes: the subtraction then takes the
comb out.
"""
import ctypes as C

import numpy as np
import pytest

from bindings import cf32, same_bits
from revenant_gb300 import abi
from revenant_gb300.library import lib

RATE = 20_000_000
RING_LOG2 = 18


def table():
    t = cf32(abi.COMB_TABLE_SIZE)
    assert lib().rv_comb_table(t.ctypes.data, abi.COMB_TABLE_SIZE) == 0
    return t


def comb_scene(n, seed, spacing=15_625.0, first=101_300.0, lines=24):
    rng = np.random.default_rng(seed)
    t = np.arange(n) / RATE
    z = 0.02 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    freqs = first + spacing * np.arange(lines)
    for k, f in enumerate(freqs):
        z += (0.05 / (1 + 0.1 * k)) * np.exp(1j * (2 * np.pi * f * t + 0.3 * k))
    out = np.zeros((n, 2), np.float32)
    out[:, 0], out[:, 1] = z.real, z.imag
    return out, freqs


def make_lines(freqs, start, amps=None):
    arr = (abi.CombLine * len(freqs))()
    for k, f in enumerate(freqs):
        step = lib().rv_comb_step(float(f), RATE)
        arr[k].step = step
        arr[k].phase0 = (start * step) & 0xFFFFFFFF
        if amps is not None:
            arr[k].amp_re, arr[k].amp_im = float(amps[k].real), float(amps[k].imag)
    return arr


def test_step_and_table_oracle_library_reference(ora, ref, rv):
    for hz in (0.0, 15_625.0, -3e6, 9_999_999.5, 1e12, float("nan"), 123.456):
        want = ref.fn("comb_step")(hz, RATE)
        assert ora.fn("comb_step")(hz, RATE) == want and rv.rv_comb_step(hz, RATE) == want
    tabs = [cf32(abi.COMB_TABLE_SIZE) for _ in range(3)]
    for fn, t in zip((ref.fn("comb_table"), ora.fn("comb_table"), rv.rv_comb_table), tabs):
        assert fn(t.ctypes.data, abi.COMB_TABLE_SIZE) == 0
    assert same_bits(tabs[0], tabs[1]) and same_bits(tabs[0], tabs[2])


def run_cpu(kind, ring, params, lines, tab):
    n = ring.shape[0]
    proj = cf32(max(params.lines * params.sub_blocks, 1))
    assert kind.fn("comb_project")(C.byref(params), ring.ctypes.data, n, lines, params.lines, tab.ctypes.data,
                                   tab.shape[0], proj.ctypes.data, proj.shape[0]) == 0, kind.error()
    cleaned = ring.copy()
    removed = cf32(params.removed_mask + 1)
    assert kind.fn("comb_subtract")(C.byref(params), ring.ctypes.data, n, lines, params.lines, tab.ctypes.data,
                                    tab.shape[0], cleaned.ctypes.data, n, removed.ctypes.data,
                                    removed.shape[0]) == 0, kind.error()
    return proj, cleaned, removed


@pytest.mark.parametrize("count,sub,first", [(65536, 16, 1000), (65536, 1, (1 << RING_LOG2) - 5000), (6000, 3, 7),
                                             (100, 4, 0)])
def test_project_subtract_oracle_vs_reference(ora, ref, count, sub, first):
    n = 1 << RING_LOG2
    ring, freqs = comb_scene(n, count + sub)
    tab = table()
    amps = np.exp(1j * np.arange(len(freqs))) * 0.03
    lines = make_lines(freqs, first, amps)
    params = abi.CombParams(n - 1, first, count, len(freqs), sub, (1 << 17) - 1, 0, 0)
    a = run_cpu(ref, ring, params, lines, tab)
    b = run_cpu(ora, ring, params, lines, tab)
    for x, y in zip(a, b):
        assert same_bits(x, y)


def test_projections_cancel_the_comb(ora):
    """Projections / length are the lines' amplitudes; subtracting them
    leaves the noise."""
    n = 1 << RING_LOG2
    ring, freqs = comb_scene(n, 3)
    tab = table()
    count = 1 << 16
    lines = make_lines(freqs, 0)
    params = abi.CombParams(n - 1, 0, count, len(freqs), 1, (1 << 17) - 1, 0, 0)
    proj, _, _ = run_cpu(ora, ring, params, lines, tab)
    amps = (proj[:, 0] + 1j * proj[:, 1]) / count
    lines = make_lines(freqs, 0, amps)
    _, cleaned, _ = run_cpu(ora, ring, params, lines, tab)
    before = np.mean(np.sum(ring[:count] ** 2, axis=1))
    after = np.mean(np.sum(cleaned[:count] ** 2, axis=1))
    noise = 2 * 0.02 ** 2
    assert after < 1.3 * noise < before


@pytest.mark.parametrize("change", ["lines", "sub", "count", "removed"])
def test_invalid_params_refused_alike(ora, ref, rv, change):
    n = 1 << 12
    ring = cf32(n)
    tab = table()
    lines = make_lines([1000.0], 0)
    p = abi.CombParams(n - 1, 0, 64, 1, 1, n - 1, 0, 0)
    if change == "lines":
        p.lines = 1025
    elif change == "sub":
        p.sub_blocks = 17
    elif change == "count":
        p.count = 65
        p.sub_blocks = 2
    elif change == "removed":
        p.removed_mask = 2 * n - 1
    proj = cf32(4096)
    for fn in (ref.fn("comb_project"), ora.fn("comb_project")):
        assert fn(C.byref(p), ring.ctypes.data, n, lines, 1, tab.ctypes.data, tab.shape[0], proj.ctypes.data,
                  proj.shape[0]) != 0
    assert rv.rv_comb_project(None, C.byref(p), ring.ctypes.data, n, lines, 1, tab.ctypes.data, tab.shape[0],
                              proj.ctypes.data, proj.shape[0]) == abi.RV_ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("count,sub,first", [(65536, 16, 1000), (65536, 1, (1 << RING_LOG2) - 5000), (6000, 3, 7)])
def test_gpu_comb_matches_oracle(gpu, ora, count, sub, first):
    n = 1 << RING_LOG2
    ring, freqs = comb_scene(n, count + sub)
    tab = table()
    amps = np.exp(1j * np.arange(len(freqs))) * 0.03
    lines = make_lines(freqs, first, amps)
    params = abi.CombParams(n - 1, first, count, len(freqs), sub, (1 << 17) - 1, 0, 0)
    proj, cleaned, removed = run_cpu(ora, ring, params, lines, tab)
    d_ring = gpu.array(ring)
    d_lines = gpu.array(np.frombuffer(bytes(lines), np.uint8))
    d_tab = gpu.array(tab)
    d_proj = gpu.zeros(proj.nbytes)
    d_removed = gpu.zeros(removed.nbytes)
    L = lib()
    assert L.rv_comb_project(gpu.stream, C.byref(params), d_ring.ptr, n, d_lines.ptr, len(freqs), d_tab.ptr,
                             tab.shape[0], d_proj.ptr, proj.shape[0]) == 0, L.rv_last_error()
    assert L.rv_comb_subtract(gpu.stream, C.byref(params), d_ring.ptr, n, d_lines.ptr, len(freqs), d_tab.ptr,
                              tab.shape[0], d_ring.ptr, n, d_removed.ptr, removed.shape[0]) == 0  # in place
    gpu.synchronize()
    assert same_bits(d_proj.download(np.float32, proj.shape), proj)
    assert same_bits(d_ring.download(np.float32, ring.shape), cleaned)
    assert same_bits(d_removed.download(np.float32, removed.shape), removed)
