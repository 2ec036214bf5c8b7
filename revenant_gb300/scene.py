"""Host mirror of the scene synthesiser (siggen::Scene, core/dsp/synth/
wideband.h): its noise field, its eight modulations and its random population.

``plan(population)`` lays out a random population's bursts as the reference
does (rv_scene_plan); ``render(device, population, start, count)`` fills a
device buffer with samples [start, start + count) of that scene: the noise
field (rv_scene_noise), then each burst's emitter over its window at its gain
(rv_emitter_accumulate), in burst order, as Scene::render_range adds them.
All the work happens in librevenant_gb300.so.
"""
import ctypes as C

from . import abi
from .library import check, lib


def population(seed, rate, duration, noise_dbfs=-60.0, emitters=8, bursts=1, span=(-1_000_000, 1_000_000),
               snr=(5.0, 35.0), burst_seconds=(0.05, 2.0), palette=()):
    p = abi.ScenePopulation()
    p.seed, p.rate, p.duration_samples, p.noise_dbfs = seed, rate, duration, noise_dbfs
    p.emitter_count, p.bursts_per_emitter = emitters, bursts
    p.span_low_hz, p.span_high_hz = span
    p.snr_min_db, p.snr_max_db = snr
    p.min_burst_seconds, p.max_burst_seconds = burst_seconds
    p.palette_count = len(palette)
    for i, m in enumerate(palette):
        p.palette[i] = m
    return p


def plan(pop):
    """The scene's bursts, sorted by start (list of abi.SceneBurst)."""
    n = C.c_uint32()
    check(lib().rv_scene_plan(C.byref(pop), None, 0, C.byref(n)))
    buf = (abi.SceneBurst * max(n.value, 1))()
    check(lib().rv_scene_plan(C.byref(pop), buf, n.value, C.byref(n)))
    return list(buf[:n.value])


def render(device, pop, start, count, out=None):
    """Samples [start, start + count) of the scene into a device buffer (cf32)."""
    out = out or device.zeros(count * 8)
    check(lib().rv_scene_noise(device.stream, pop.seed, lib().rv_scene_noise_sigma(pop.noise_dbfs), start, count,
                               out.address, count))
    end = start + count
    for b in plan(pop):
        lo, hi = max(b.start, start), min(b.end, end)
        if lo < hi:
            check(lib().rv_emitter_accumulate(device.stream, C.byref(b.emitter), lo - b.start, hi - lo, b.gain,
                                              out.address + 8 * (lo - start), hi - lo))
    return out
