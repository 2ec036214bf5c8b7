"""The whole receive chain on the GPU against the oracle chain.

Audio from the plain chain (one launch per stage per receiver, the
reference's recording) must equal the oracle-driven chain bit for bit, and
the batched chain (fused coarse kernel + batched receivers) must equal the
plain chain bit for bit, for every mode, across runs of uneven sizes
(blocking invariance, tests/reference/test_vrx.cpp:1241).
"""
import ctypes as C

import numpy as np
import pytest

import signals
from oracle_chain import OracleChain
from revenant_gb300 import abi
from revenant_gb300.chain import Chain

pytestmark = pytest.mark.gpu

WFM_SCENE = [("wfm", 200_000, 1.0), ("nfm", -300_000, 0.3), ("am", 500_000, 0.3), ("usb", 100_000, 0.2),
             ("am", -500_000, 0.3)]


def c1_requests():
    return [
        abi.request(center=200_000, bandwidth=200_000, demod="wfm", stereo=True),
        abi.request(center=200_000, bandwidth=200_000, demod="wfm", stereo=False),
        abi.request(center=-300_000, bandwidth=12_500, demod="nfm"),
        abi.request(center=500_000, bandwidth=10_000, demod="am"),
        abi.request(center=100_000, bandwidth=3_000, demod="usb"),
        abi.request(center=-100_000, bandwidth=3_000, demod="lsb"),
        abi.request(center=-500_000, bandwidth=10_000, demod="sam"),
        abi.request(center=-500_000, bandwidth=6_000, demod="dsb"),
        abi.request(center=100_000, bandwidth=1_200, demod="cw"),
        abi.request(center=-300_000, bandwidth=12_500, demod="raw"),
    ]


RUNS_A = [4096, 30000, 65536, 1000, 20000, 10000]
RUNS_B = [8192] * 15 + [7752]  # same total as RUNS_A, different blocking


def feed(chain, codes, runs, bps_values):
    at = 0
    for n in runs:
        chain.run(codes[at * bps_values:(at + n) * bps_values])
        at += n
    return at


@pytest.fixture(scope="module")
def c1_capture():
    n = sum(RUNS_A)
    z = signals.scene(n, 2_400_000, WFM_SCENE, snr_db=25.0, seed=1)
    return signals.quantise(z, "cu8")


def test_plain_chain_matches_oracle_chain(gpu, c1_capture):
    reqs = c1_requests()
    ch = Chain(gpu, grid=(8, 17, 4), rate=2_400_000, fmt=abi.FORMAT_CU8, mode=abi.CHAIN_PLAIN, max_run_samples=1 << 17)
    oc = OracleChain((8, 17, 4), 2_400_000, abi.FORMAT_CU8, reqs)
    ids = [ch.add_receiver(r) for r in reqs]
    at = 0
    for n in RUNS_A:
        part = c1_capture[2 * at:2 * (at + n)]
        ch.run(part)
        oc.run(part, n)
        at += n
    for i, rid in enumerate(ids):
        got, want = ch.audio(rid), oc.audio(i)
        assert got.size == want.size and got.size > 0, (i, got.size, want.size)
        bad = np.nonzero(got.view(np.uint32) != want.view(np.uint32))[0]
        assert bad.size == 0, "receiver %d (mode %d): %d of %d values differ, first at %s" % (
            i, reqs[i].demod, bad.size, got.size, bad[:5])


def test_batched_chain_matches_plain_chain_and_is_blocking_invariant(gpu, c1_capture):
    reqs = c1_requests()
    out, rings = {}, {}
    for mode, runs in ((abi.CHAIN_PLAIN, RUNS_A), (abi.CHAIN_BATCHED, RUNS_A), (abi.CHAIN_BATCHED, RUNS_B),
                       (abi.CHAIN_HOISTED, RUNS_A)):
        ch = Chain(gpu, grid=(8, 17, 4), rate=2_400_000, fmt=abi.FORMAT_CU8, mode=mode, max_run_samples=1 << 17)
        ids = [ch.add_receiver(r) for r in reqs]
        at = 0
        for n in runs:
            ch.run(c1_capture[2 * at:2 * (at + n)])
            at += n
        out[(mode, tuple(runs))] = [ch.audio(i) for i in ids]
        rings[(mode, tuple(runs))] = [ch.rings(i)[0] for i in ids]
        ch.close()
    plain = out[(abi.CHAIN_PLAIN, tuple(RUNS_A))]
    plain_rings = rings[(abi.CHAIN_PLAIN, tuple(RUNS_A))]
    problems = []
    for key in ((abi.CHAIN_BATCHED, tuple(RUNS_A)), (abi.CHAIN_BATCHED, tuple(RUNS_B)), (abi.CHAIN_HOISTED, tuple(RUNS_A))):
        for i, (a, b) in enumerate(zip(plain, out[key])):
            fine_same = np.array_equal(plain_rings[i].view(np.uint32), rings[key][i].view(np.uint32))
            if a.size != b.size or not np.array_equal(a.view(np.uint32), b.view(np.uint32)):
                bad = np.nonzero(a.view(np.uint32) != b.view(np.uint32))[0] if a.size == b.size else []
                problems.append("receiver %d mode %d runs %d: sizes %d/%d, %d values differ (first %s), fine rings equal: %s"
                                % (i, reqs[i].demod, len(key[1]), a.size, b.size, len(bad), list(bad[:4]), fine_same))
            elif not fine_same:
                problems.append("receiver %d: audio equal but fine rings differ" % i)
    assert not problems, "\n".join(problems)


def test_batched_wideband_receivers_match_plain(gpu):
    rate, n = 20_000_000, 1 << 19
    reqs = signals.random_receivers(24, rate, seed=3)
    emitters = [("am", r.center, 0.2) for r in reqs[:6]]
    z = signals.scene(n, rate, emitters + [("wfm", reqs[0].center, 1.0)], snr_db=30.0, seed=3)
    codes = signals.quantise(z, "cs16")
    res = []
    for mode in (abi.CHAIN_PLAIN, abi.CHAIN_BATCHED, abi.CHAIN_HOISTED):
        ch = Chain(gpu, grid=(64, 17, 32), rate=rate, fmt=abi.FORMAT_CS16, mode=mode, max_run_samples=1 << 17)
        ids = [ch.add_receiver(r) for r in reqs]
        for k in range(n // (1 << 17)):
            ch.run(codes[2 * k * (1 << 17):2 * (k + 1) * (1 << 17)])
        res.append([ch.audio(i) for i in ids])
        ch.close()
    for other in res[1:]:
        for i, (a, b) in enumerate(zip(res[0], other)):
            assert a.size == b.size and a.size > 0
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), "receiver %d mode %d differs" % (i, reqs[i].demod)


def test_wfm_stereo_recovers_the_tone(gpu, c1_capture):
    """Known answer: the 1 kHz left tone comes out of the stereo WFM receiver
    (test_vrx.cpp:2156 asks for amplitude 1 +- 0.02 of the modulating tone and
    purity above 0.95 on a clean channel; here the check is the tone's
    dominance in L and its weaker presence in R)."""
    ch = Chain(gpu, grid=(8, 17, 4), rate=2_400_000, fmt=abi.FORMAT_CU8, mode=abi.CHAIN_BATCHED, max_run_samples=1 << 17)
    rid = ch.add_receiver(abi.request(center=200_000, bandwidth=200_000, demod="wfm", stereo=True))
    at = 0
    for n in RUNS_A:
        ch.run(c1_capture[2 * at:2 * (at + n)])
        at += n
    a = ch.audio(rid).reshape(-1, 2)[2000:]
    spec_l = np.abs(np.fft.rfft(a[:, 0] * np.hanning(a.shape[0])))
    f = np.fft.rfftfreq(a.shape[0], 1 / 48000)
    k1 = np.argmin(np.abs(f - 1000))
    assert spec_l[k1 - 2:k1 + 3].max() > 20 * np.median(spec_l)


def _run_pair(gpu, grid, rate, fmt, reqs, codes, runs, bps_values, late=None, late_at=None,
              variants=((False, False), (True, False))):
    """The same feed through batched chains: (captured, pipelined) per variant."""
    out = []
    for captured, pipelined in variants:
        ch = Chain(gpu, grid=grid, rate=rate, fmt=fmt, mode=abi.CHAIN_BATCHED, max_run_samples=max(runs),
                   pipelined=pipelined)
        if captured:
            ch.capture_graph()
        ids = [ch.add_receiver(r) for r in reqs]
        at = 0
        for k, n in enumerate(runs):
            if late is not None and k == late_at:
                ids.append(ch.add_receiver(late))
            ch.run(codes[at * bps_values:(at + n) * bps_values])
            at += n
        ch.drain()
        out.append(([ch.audio(i) for i in ids], ch.stats()))
        ch.close()
    return out


def test_captured_chain_matches_direct_batched(gpu, c1_capture):
    """One CUDA graph per chain, replayed every run: the same bits as direct launches."""
    (direct, _), (graph, st) = _run_pair(gpu, (8, 17, 4), 2_400_000, abi.FORMAT_CU8, c1_requests(), c1_capture,
                                         RUNS_A, 2)
    for i, (a, b) in enumerate(zip(direct, graph)):
        assert a.size == b.size and a.size > 0, "receiver %d" % i
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), "receiver %d differs when captured" % i
    assert st.graph_launches == len(RUNS_A)
    assert 1 <= st.graph_captures < len(RUNS_A)


def test_captured_chain_replays_without_recapture(gpu, c1_capture):
    (direct, _), (graph, st) = _run_pair(gpu, (8, 17, 4), 2_400_000, abi.FORMAT_CU8, c1_requests()[:4], c1_capture,
                                         RUNS_B, 2)
    for a, b in zip(direct, graph):
        assert a.size > 0 and np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert st.graph_launches == len(RUNS_B)
    assert st.graph_captures <= 2  # equal runs: the first capture's capacities hold


def test_captured_chain_with_a_receiver_added_mid_stream(gpu, c1_capture):
    reqs = c1_requests()
    (direct, _), (graph, st) = _run_pair(gpu, (8, 17, 4), 2_400_000, abi.FORMAT_CU8, reqs[:3], c1_capture, RUNS_B, 2,
                                         late=reqs[6], late_at=5)
    assert len(graph) == 4
    for i, (a, b) in enumerate(zip(direct, graph)):
        assert a.size > 0 and np.array_equal(a.view(np.uint32), b.view(np.uint32)), "receiver %d" % i


def test_captured_wideband_chain_matches_direct(gpu):
    rate, n = 20_000_000, 1 << 19
    reqs = signals.random_receivers(24, rate, seed=4)
    z = signals.scene(n, rate, [("am", r.center, 0.2) for r in reqs[:6]], snr_db=30.0, seed=4)
    codes = signals.quantise(z, "cs16")
    runs = [1 << 17, 100_000, 1 << 17, (1 << 19) - 2 * (1 << 17) - 100_000]
    (direct, _), (graph, _) = _run_pair(gpu, (64, 17, 32), rate, abi.FORMAT_CS16, reqs, codes, runs, 2)
    for i, (a, b) in enumerate(zip(direct, graph)):
        assert a.size > 0 and np.array_equal(a.view(np.uint32), b.view(np.uint32)), "receiver %d" % i


@pytest.mark.parametrize("mode", [abi.CHAIN_PLAIN, abi.CHAIN_HOISTED])
def test_plain_chain_refuses_capture(gpu, mode):
    from revenant_gb300.library import lib
    ch = Chain(gpu, grid=(8, 17, 4), rate=2_400_000, fmt=abi.FORMAT_CU8, mode=mode, max_run_samples=4096)
    assert lib().rv_chain_capture_graph(ch.handle) == abi.RV_ERR_UNSUPPORTED
    ch.close()


@pytest.mark.parametrize("captured", [False, True])
def test_pipelined_chain_matches_synchronous(gpu, c1_capture, captured):
    """Runs queued while the previous one executes (two slots, input copies on
    a second stream): the audio is the synchronous chain's, bit for bit."""
    (sync, _), (piped, st) = _run_pair(gpu, (8, 17, 4), 2_400_000, abi.FORMAT_CU8, c1_requests(), c1_capture, RUNS_A,
                                       2, variants=((False, False), (captured, True)))
    for i, (a, b) in enumerate(zip(sync, piped)):
        assert a.size == b.size and a.size > 0, "receiver %d" % i
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), "receiver %d differs when pipelined" % i
    assert st.runs == len(RUNS_A)


def test_pipelined_chain_with_a_receiver_added_mid_stream(gpu, c1_capture):
    reqs = c1_requests()
    (sync, _), (piped, _) = _run_pair(gpu, (8, 17, 4), 2_400_000, abi.FORMAT_CU8, reqs[:3], c1_capture, RUNS_B, 2,
                                      late=reqs[6], late_at=5, variants=((False, False), (True, True)))
    for i, (a, b) in enumerate(zip(sync, piped)):
        assert a.size > 0 and np.array_equal(a.view(np.uint32), b.view(np.uint32)), "receiver %d" % i


def test_pipelined_wideband_chain_from_device_memory(gpu):
    from revenant_gb300.chain import Chain as _Chain
    rate, n, run = 20_000_000, 1 << 19, 1 << 17
    reqs = signals.random_receivers(16, rate, seed=6)
    z = signals.scene(n, rate, [("am", r.center, 0.2) for r in reqs[:4]], snr_db=30.0, seed=6)
    codes = signals.quantise(z, "cs16")
    dev = gpu.array(codes)
    out = []
    for pipelined in (False, True):
        ch = _Chain(gpu, grid=(64, 17, 32), rate=rate, fmt=abi.FORMAT_CS16, mode=abi.CHAIN_BATCHED,
                    max_run_samples=run, pipelined=pipelined)
        ids = [ch.add_receiver(r) for r in reqs]
        for k in range(n // run):
            ch.run(_At(dev, k * run * 4), run)
        ch.drain()
        out.append([ch.audio(i) for i in ids])
        ch.close()
    for i, (a, b) in enumerate(zip(*out)):
        assert a.size > 0 and np.array_equal(a.view(np.uint32), b.view(np.uint32)), "receiver %d" % i


def test_plain_chain_refuses_pipelining(gpu):
    with pytest.raises(Exception):
        Chain(gpu, grid=(8, 17, 4), rate=2_400_000, fmt=abi.FORMAT_CU8, mode=abi.CHAIN_PLAIN, max_run_samples=4096,
              pipelined=True)


class _At:
    """A device buffer address plus a byte offset, for Chain.run."""

    def __init__(self, buf, offset):
        self.address = buf.address + offset


def test_autotuned_chain_matches_the_rule(gpu):
    """rv_chain_autotune times fine-tile shapes per receiver class and keeps
    the fastest: the audio must not change (a shape moves work between
    threads, never an output's arithmetic), and tuning after the first run is
    refused."""
    rate, n, run = 20_000_000, 1 << 19, 1 << 17
    reqs = signals.random_receivers(24, rate, seed=5)
    z = signals.scene(n, rate, [("am", r.center, 0.2) for r in reqs[:6]], snr_db=30.0, seed=5)
    codes = signals.quantise(z, "cs16")
    res = []
    for tune in (False, True):
        ch = Chain(gpu, grid=(64, 17, 32), rate=rate, fmt=abi.FORMAT_CS16, mode=abi.CHAIN_BATCHED, max_run_samples=run)
        ids = [ch.add_receiver(r) for r in reqs]
        if tune:
            rep = ch.autotune(run)
            assert rep["classes"] > 0 and rep["shapes_timed"] >= rep["classes"]
            assert rep["tiles_per_sm"] in (2, 4, 8) and rep["default_ms"] > 0 and rep["tuned_ms"] > 0
        for k in range(n // run):
            ch.run(codes[2 * k * run:2 * (k + 1) * run])
        res.append([ch.audio(i) for i in ids])
        if tune:
            from revenant_gb300.library import lib
            assert lib().rv_chain_autotune(ch.handle, run, C.byref(abi.ChainTuneReport())) == abi.RV_ERR_INVALID
        ch.close()
    for i, (a, b) in enumerate(zip(*res)):
        assert a.size == b.size and a.size > 0
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), "receiver %d differs after tuning" % i
