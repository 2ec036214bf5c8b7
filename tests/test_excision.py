"""Span-wide impulse excision against the reference's twins
(core/dsp/impulse_excision_reference.cpp, compiled from the reference sources
into oracle/_ref/libreftwins.so) and the oracle restatement (oracle/oracle.c).

Everything here is bit for bit: the designed configuration, the ring sizes,
every block's plan from the cursor, and after every block the segment powers,
the median levels, the flags, the cleaned ring, the removed ring and the
counters. The scenes put impulses of every width from one sample to past
max_width, bursts long enough to be spared, a strong carrier, a gap that
restarts the stage, and blocks that are not whole segments.
"""
import ctypes as C

import numpy as np
import pytest

from bindings import oracle, reference, same_bits
from revenant_gb300 import abi
from revenant_gb300.library import lib

RATES = [2_400_000, 20_000_000, 61_440_000, 100_000, 4_000_000_000]
WIDTHS = [20e-6, 1e-6, 1e-3, 0.0]


def design(kind_fn, rate, width):
    c = abi.ExcisionConfig()
    assert kind_fn(rate, width, C.byref(c)) == 0
    return c


def cfg_tuple(c):
    return (c.pass_, c.seg_log2, c.segments, c.max_width, c.hang, c.lead)


# -- host bookkeeping ------------------------------------------------------------

@pytest.mark.parametrize("rate", RATES)
@pytest.mark.parametrize("width", WIDTHS)
def test_design_oracle_library_reference(ora, ref, rv, rate, width):
    a = design(ref.fn("design_excision"), rate, width)
    assert cfg_tuple(design(ora.fn("design_excision"), rate, width)) == cfg_tuple(a)
    assert cfg_tuple(design(rv.rv_design_excision, rate, width)) == cfg_tuple(a)


@pytest.mark.parametrize("db", [15.0, 12.0, 0.0, -3.0, 40.5])
def test_threshold_bits(ora, ref, rv, db):
    want = np.float32(ref.fn("excision_threshold")(db))
    assert np.float32(ora.fn("excision_threshold")(db)).view(np.uint32) == want.view(np.uint32)
    assert np.float32(rv.rv_excision_threshold(db)).view(np.uint32) == want.view(np.uint32)


@pytest.mark.parametrize("rate,block,frames,log2", [(20_000_000, 65536, 2, 20), (2_400_000, 16384, 3, 18),
                                                     (61_440_000, 1 << 20, 1, 22), (20_000_000, 1 << 20, 4, 20)])
def test_rings_oracle_library_reference(ora, ref, rv, rate, block, frames, log2):
    c = design(ref.fn("design_excision"), rate, 20e-6)
    out = []
    for fn in (ref.fn("size_excision_rings"), ora.fn("size_excision_rings"), rv.rv_size_excision_rings):
        r = abi.ExcisionRings()
        st = fn(C.byref(c), block, frames, (1 << log2) - 1, C.byref(r))
        out.append((st == 0, r.seg_mask, r.flag_mask, r.removed_mask) if st == 0 else (False,))
    assert out[0] == out[1] == out[2]


def plans(kind, c, ring_mask, rings, threshold, starts, counts):
    """Every block's plan: kind is 'ref', 'ora' or 'rv'."""
    n = len(starts)
    out = (abi.ExcisionPlan * n)()
    if kind == "ref":
        st = np.array(starts, np.uint64)
        ct = np.array(counts, np.uint32)
        assert reference().fn("excision_plans")(C.byref(c), ring_mask, C.byref(rings), threshold, st.ctypes.data,
                                                ct.ctypes.data, n, out) == 0
        return out
    init, plan = ((oracle().lib.or_excision_cursor_init, oracle().lib.or_excision_plan_block) if kind == "ora" else
                  (lib().rv_excision_cursor_init, lib().rv_excision_plan_block))
    cur = abi.ExcisionCursor()
    assert init(C.byref(cur), C.byref(c), ring_mask, C.byref(rings), threshold) == 0
    for b in range(n):
        assert plan(C.byref(cur), starts[b], counts[b], C.byref(out[b])) == 0
    return out


def block_sequence(block, nblocks, seed):
    """Contiguous blocks with odd lengths, one empty block and one gap."""
    rng = np.random.default_rng(seed)
    starts, counts, at = [], [], 1000
    for b in range(nblocks):
        n = block if b % 3 else int(rng.integers(1, block))
        if b == nblocks // 2:
            at += 77_777  # a gap: the stage restarts
        if b == 2:
            n = 0
        starts.append(at)
        counts.append(n)
        at += n
    return starts, counts


def test_cursor_plans_oracle_library_reference(ref, ora, rv):
    c = design(ref.fn("design_excision"), 20_000_000, 20e-6)
    ring_mask = (1 << 20) - 1
    rings = abi.ExcisionRings()
    assert ref.fn("size_excision_rings")(C.byref(c), 65536, 2, ring_mask, C.byref(rings)) == 0
    thr = ref.fn("excision_threshold")(15.0)
    starts, counts = block_sequence(65536, 24, 3)
    want = plans("ref", c, ring_mask, rings, thr, starts, counts)
    for kind in ("ora", "rv"):
        got = plans(kind, c, ring_mask, rings, thr, starts, counts)
        assert bytes(got) == bytes(want), kind
    assert sum(p.restarted for p in want) == 2
    assert want[-1].cleaned_end > starts[-1]


# -- the passes -------------------------------------------------------------------

def scene(n, seed, rate=20_000_000, max_width=400):
    """Noise, a carrier, impulses of widths 1..max_width + 60 and long bursts."""
    rng = np.random.default_rng(seed)
    z = 0.05 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    t = np.arange(n)
    z += 0.3 * np.exp(2j * np.pi * 0.01234 * t)
    pos = 40_000
    widths = list(range(1, 12)) + [30, 100, max_width - 5, max_width, max_width + 1, max_width + 60, 2, 1]
    for w in widths:
        if pos + w >= n:
            break
        amp = rng.uniform(3, 30)
        z[pos:pos + w] += amp * np.exp(2j * np.pi * rng.uniform(0, 1, w))
        pos += int(rng.integers(2_000, 9_000))
    if n > 400_000:
        z[300_000:306_000] += 2.0 * np.exp(2j * np.pi * 0.2 * np.arange(6000))  # a burst: spared
    out = np.zeros((n, 2), np.float32)
    out[:, 0], out[:, 1] = z.real, z.imag
    return out


class Rings:
    def __init__(self, ring_mask, rings):
        self.ring = np.zeros((ring_mask + 1, 2), np.float32)
        self.seg_power = np.zeros(rings.seg_mask + 1, np.float32)
        self.seg_level = np.zeros(rings.seg_mask + 1, np.float32)
        self.flags = np.zeros(rings.flag_mask + 1, np.uint32)
        self.removed = np.zeros((rings.removed_mask + 1, 2), np.float32)
        self.counters = np.zeros(4, np.uint32)

    def arrays(self):
        return (self.ring, self.seg_power, self.seg_level, self.flags, self.removed, self.counters)


def run_block_cpu(kind, c, plan, r):
    f = kind.fn
    d = lambda a: a.ctypes.data  # noqa: E731
    n = r.ring.shape[0]
    if plan.segment.count:
        assert f("excise_segment")(C.byref(c), C.byref(plan.segment), d(r.ring), n, d(r.seg_power),
                                   r.seg_power.size) == 0, kind.error()
    if plan.reference.count:
        assert f("excise_reference")(C.byref(c), C.byref(plan.reference), d(r.seg_power), d(r.seg_level),
                                     r.seg_power.size) == 0, kind.error()
    if plan.flag.count:
        assert f("excise_flag")(C.byref(c), C.byref(plan.flag), d(r.ring), n, d(r.seg_level), r.seg_level.size,
                                d(r.flags), r.flags.size) == 0, kind.error()
    if plan.apply.count:
        assert f("excise_apply")(C.byref(c), C.byref(plan.apply), d(r.ring), n, d(r.flags), r.flags.size, d(r.ring),
                                 d(r.removed), r.removed.shape[0], d(r.counters)) == 0, kind.error()


def setup(rate, block, log2, frames=2):
    c = abi.ExcisionConfig()
    assert lib().rv_design_excision(rate, 20e-6, C.byref(c)) == 0
    ring_mask = (1 << log2) - 1
    rings = abi.ExcisionRings()
    assert lib().rv_size_excision_rings(C.byref(c), block, frames, ring_mask, C.byref(rings)) == 0
    return c, ring_mask, rings, lib().rv_excision_threshold(15.0)


def write_block(ring, signal, start, count, origin):
    mask = ring.shape[0] - 1
    idx = (np.arange(start, start + count) & mask)
    ring[idx] = signal[start - origin:start - origin + count]


@pytest.mark.parametrize("rate,block,log2", [(20_000_000, 65536, 19), (2_400_000, 8192, 16)])
def test_passes_oracle_vs_reference(ora, ref, rate, block, log2):
    c, ring_mask, rings, thr = setup(rate, block, log2)
    starts, counts = block_sequence(block, 16, rate)
    origin = starts[0]
    signal = scene(starts[-1] + counts[-1] - origin, 5, rate, c.max_width)
    ps = plans("ref", c, ring_mask, rings, thr, starts, counts)
    a, b = Rings(ring_mask, rings), Rings(ring_mask, rings)
    for k in range(len(starts)):
        for r in (a, b):
            write_block(r.ring, signal, starts[k], counts[k], origin)
        run_block_cpu(ref, c, ps[k], a)
        run_block_cpu(ora, c, ps[k], b)
        for x, y in zip(a.arrays(), b.arrays()):
            assert same_bits(x, y), "block %d" % k
    assert a.counters[abi.EXCISE_COUNTER_EVENTS] > 3 and a.counters[abi.EXCISE_COUNTER_SPARED] >= 1


def test_cleaned_plus_removed_is_raw(ora):
    """The audit property: cleaned + removed == raw, bit for bit, over every
    sample an apply pass covered (the removed ring is sized to one block)."""
    rate, block, log2 = 20_000_000, 65536, 19
    c, ring_mask, rings, thr = setup(rate, block, log2)
    starts = [k * block for k in range(6)]
    counts = [block] * 6
    signal = scene(6 * block, 9, rate, c.max_width)
    ps = plans("ora", c, ring_mask, rings, thr, starts, counts)
    r = Rings(ring_mask, rings)
    for k in range(6):
        write_block(r.ring, signal, starts[k], counts[k], 0)
        run_block_cpu(ora, c, ps[k], r)
        p = ps[k].apply
        if p.count == 0:
            continue
        start = ps[k].cleaned_end - p.count
        idx = np.arange(start, ps[k].cleaned_end)
        cleaned = r.ring[idx & ring_mask]
        removed = r.removed[idx & rings.removed_mask]
        assert same_bits(cleaned + removed, signal[idx])
        # excised samples are -0 in the ring and whole runs no longer than max_width
        cut = np.all(cleaned.view(np.uint32) == 0x80000000, axis=1)
        edges = np.flatnonzero(np.diff(np.concatenate([[0], cut.astype(np.int8), [0]])))
        assert np.all(edges[1::2] - edges[::2] <= c.max_width)


@pytest.mark.parametrize("field,value", [("seg_log2", 1), ("seg_log2", 13), ("segments", 1), ("segments", 65),
                                         ("max_width", 0), ("max_width", 4097), ("hang", 17), ("lead", 17)])
def test_invalid_configs_refused_alike(ora, ref, rv, field, value):
    c, ring_mask, rings, thr = setup(20_000_000, 65536, 19)
    setattr(c, field, value)
    p = abi.ExcisionParams(ring_mask, 0, 16, rings.seg_mask, rings.flag_mask, rings.removed_mask, 0, thr)
    ring = np.zeros((ring_mask + 1, 2), np.float32)
    seg = np.zeros(rings.seg_mask + 1, np.float32)
    assert ref.fn("excise_segment")(C.byref(c), C.byref(p), ring.ctypes.data, ring_mask + 1, seg.ctypes.data,
                                    seg.size) != 0
    assert ora.fn("excise_segment")(C.byref(c), C.byref(p), ring.ctypes.data, ring_mask + 1, seg.ctypes.data,
                                    seg.size) != 0
    # the library refuses before it touches a device
    assert rv.rv_excise_segment(None, C.byref(c), C.byref(p), ring.ctypes.data, ring_mask + 1, seg.ctypes.data,
                                seg.size) == abi.RV_ERR_INVALID


@pytest.mark.parametrize("change", ["mask", "unaligned", "threshold", "flag_ring", "short_ring"])
def test_invalid_params_refused_alike(ora, ref, rv, change):
    c, ring_mask, rings, thr = setup(20_000_000, 65536, 19)
    p = abi.ExcisionParams(ring_mask, 128, 16, rings.seg_mask, rings.flag_mask, rings.removed_mask, 0, thr)
    n = ring_mask + 1
    if change == "mask":
        p.seg_mask = 1000
    elif change == "unaligned":
        p.first = 5
    elif change == "threshold":
        p.threshold = 0.0
    elif change == "flag_ring":
        p.count = rings.flag_mask
    elif change == "short_ring":
        n = ring_mask
    ring = np.zeros((ring_mask + 1, 2), np.float32)
    level = np.zeros(rings.seg_mask + 1, np.float32)
    flags = np.zeros(rings.flag_mask + 1, np.uint32)
    pass_ = "excise_flag" if change == "flag_ring" else "excise_reference" if change == "unaligned" else "excise_flag"
    for kind in (ref, ora):
        if pass_ == "excise_flag":
            st = kind.fn(pass_)(C.byref(c), C.byref(p), ring.ctypes.data, n, level.ctypes.data, level.size,
                                flags.ctypes.data, flags.size)
        else:
            st = kind.fn(pass_)(C.byref(c), C.byref(p), level.ctypes.data, level.ctypes.data, level.size)
        assert st != 0, (kind, change)
    if pass_ == "excise_flag":
        st = rv.rv_excise_flag(None, C.byref(c), C.byref(p), ring.ctypes.data, n, level.ctypes.data, level.size,
                               flags.ctypes.data, flags.size)
    else:
        st = rv.rv_excise_reference(None, C.byref(c), C.byref(p), level.ctypes.data, level.ctypes.data, level.size)
    assert st == abi.RV_ERR_INVALID


# -- GPU --------------------------------------------------------------------------

def run_gpu(gpu, c, ps, starts, counts, signal, origin, ring_mask, rings, check_every=None, ora=None):
    """Blocks through rv_excise_block on device rings; returns the host copies."""
    n = ring_mask + 1
    d_ring = gpu.zeros(n * 8)
    d_seg_p = gpu.zeros((rings.seg_mask + 1) * 4)
    d_seg_l = gpu.zeros((rings.seg_mask + 1) * 4)
    d_flags = gpu.zeros((rings.flag_mask + 1) * 4)
    d_removed = gpu.zeros((rings.removed_mask + 1) * 8)
    d_counters = gpu.zeros(16)
    ref_rings = Rings(ring_mask, rings) if ora is not None else None
    for k in range(len(starts)):
        if counts[k]:
            idx = np.arange(starts[k], starts[k] + counts[k]) & ring_mask
            block = np.ascontiguousarray(signal[starts[k] - origin:starts[k] - origin + counts[k]])
            # the block lands in the ring in at most two pieces
            split = int(np.argmax(np.diff(idx) < 0)) + 1 if np.any(np.diff(idx) < 0) else counts[k]
            for lo, hi in ((0, split), (split, counts[k])):
                if hi > lo:
                    d_ring.upload(block[lo:hi], int(idx[lo]) * 8)
        st = lib().rv_excise_block(gpu.stream, C.byref(c), C.byref(ps[k]), d_ring.ptr, n, d_seg_p.ptr, d_seg_l.ptr,
                                   rings.seg_mask + 1, d_flags.ptr, rings.flag_mask + 1, d_removed.ptr,
                                   rings.removed_mask + 1, d_counters.ptr)
        assert st == 0, lib().rv_last_error().decode()
        if ref_rings is not None:
            write_block(ref_rings.ring, signal, starts[k], counts[k], origin)
            run_block_cpu(ora, c, ps[k], ref_rings)
            if check_every and (k % check_every == 0 or k == len(starts) - 1):
                gpu.synchronize()
                got = (d_ring.download(np.float32, (n, 2)), d_seg_p.download(np.float32, (rings.seg_mask + 1,)),
                       d_seg_l.download(np.float32, (rings.seg_mask + 1,)),
                       d_flags.download(np.uint32, (rings.flag_mask + 1,)),
                       d_removed.download(np.float32, (rings.removed_mask + 1, 2)), d_counters.download(np.uint32, (4,)))
                for name, x, y in zip(("ring", "seg_power", "seg_level", "flags", "removed", "counters"), got,
                                      ref_rings.arrays()):
                    assert same_bits(x, y), "block %d: %s" % (k, name)
    gpu.synchronize()
    return ref_rings


@pytest.mark.gpu
@pytest.mark.parametrize("rate,block,log2,nblocks", [(20_000_000, 65536, 19, 16), (2_400_000, 8192, 16, 16),
                                                      (20_000_000, 1 << 20, 22, 6)])
def test_gpu_excision_matches_oracle(gpu, ora, rate, block, log2, nblocks):
    c, ring_mask, rings, thr = setup(rate, block, log2)
    starts, counts = block_sequence(block, nblocks, rate + 1)
    origin = starts[0]
    signal = scene(starts[-1] + counts[-1] - origin, 11, rate, c.max_width)
    ps = plans("rv", c, ring_mask, rings, thr, starts, counts)
    r = run_gpu(gpu, c, ps, starts, counts, signal, origin, ring_mask, rings, check_every=1, ora=ora)
    assert r.counters[abi.EXCISE_COUNTER_EVENTS] > 2


@pytest.mark.gpu
def test_gpu_single_passes_match_oracle(gpu, ora):
    """Each entry point on its own, with distinct raw and cleaned rings."""
    c, ring_mask, rings, thr = setup(20_000_000, 65536, 18)
    n = ring_mask + 1
    sig = scene(n, 21)
    r = Rings(ring_mask, rings)
    r.ring[:] = sig
    seg_count = (n >> c.seg_log2) - c.segments - 4
    seg = abi.ExcisionParams(ring_mask, 0, min(seg_count, rings.seg_mask - c.segments - 2), rings.seg_mask,
                             rings.flag_mask, rings.removed_mask, 0, thr)
    samples = (seg.count << c.seg_log2)
    flag = abi.ExcisionParams(ring_mask, 0, min(samples, rings.flag_mask - 2 * c.max_width - 40), rings.seg_mask,
                              rings.flag_mask, rings.removed_mask, 0, thr)
    apply = abi.ExcisionParams(ring_mask, 0, min(flag.count - c.max_width - c.lead, rings.removed_mask + 1),
                               rings.seg_mask, rings.flag_mask, rings.removed_mask, 0, thr)
    plan = abi.ExcisionPlan(seg, seg, flag, apply, 0, 0, 0)
    run_block_cpu(ora, c, plan, r)
    d_raw = gpu.array(sig)
    d_seg_p = gpu.zeros(r.seg_power.nbytes)
    d_seg_l = gpu.zeros(r.seg_level.nbytes)
    d_flags = gpu.zeros(r.flags.nbytes)
    d_clean = gpu.array(sig)
    d_removed = gpu.zeros(r.removed.nbytes)
    d_counters = gpu.zeros(16)
    L = lib()
    assert L.rv_excise_segment(gpu.stream, C.byref(c), C.byref(seg), d_raw.ptr, n, d_seg_p.ptr, r.seg_power.size) == 0
    assert L.rv_excise_reference(gpu.stream, C.byref(c), C.byref(seg), d_seg_p.ptr, d_seg_l.ptr, r.seg_power.size) == 0
    assert L.rv_excise_flag(gpu.stream, C.byref(c), C.byref(flag), d_raw.ptr, n, d_seg_l.ptr, r.seg_level.size,
                            d_flags.ptr, r.flags.size) == 0
    assert L.rv_excise_apply(gpu.stream, C.byref(c), C.byref(apply), d_raw.ptr, n, d_flags.ptr, r.flags.size,
                             d_clean.ptr, d_removed.ptr, r.removed.shape[0], d_counters.ptr) == 0
    gpu.synchronize()
    assert same_bits(d_seg_p.download(np.float32, r.seg_power.shape), r.seg_power)
    assert same_bits(d_seg_l.download(np.float32, r.seg_level.shape), r.seg_level)
    assert same_bits(d_flags.download(np.uint32, r.flags.shape), r.flags)
    assert same_bits(d_clean.download(np.float32, r.ring.shape), r.ring)
    assert same_bits(d_removed.download(np.float32, r.removed.shape), r.removed)
    assert same_bits(d_counters.download(np.uint32, (4,)), r.counters)
    assert same_bits(d_raw.download(np.float32, sig.shape), sig)  # raw untouched
