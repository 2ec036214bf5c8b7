"""Fast mode (rv_chain_create with RV_CHAIN_FAST): the batched chain with the
fine stage as split-precision BF16 GEMMs on the tensor cores (hi*hi + hi*lo +
lo*hi products accumulated in FP32) and the DC-removal and mono audio FIRs as
fused multiply-adds. It is a tolerance mode, not a bit-exact one, so it is
checked against the bit-exact batched chain (itself pinned to the oracle
chain bit for bit in test_gpu_chain_c3.py) on the benchmark's own receiver
mix, to the tolerances stated here:

* every receiver's fine ring within FINE_REL_MAX relative RMS;
* per demodulation mode, the median receiver's audio within AUDIO_REL_MEDIAN
  relative RMS, and every receiver within AUDIO_REL_MAX (the FM
  discriminators and the carrier loops turn a difference near a decision
  threshold into a larger one on a few samples).

The fast chain launched directly and replayed from its captured CUDA graph
must agree bit for bit (the GEMM tiles accumulate in a fixed order)."""
import numpy as np
import pytest

import bench
from revenant_gb300 import abi
from revenant_gb300.chain import Chain

pytestmark = pytest.mark.gpu

RUN = 1 << 19
SAMPLES = 1 << 21
FINE_REL_MAX = 1e-3
AUDIO_REL_MEDIAN = 1e-4
AUDIO_REL_MAX = 0.1


def rel_rms(got, want):
    got, want = got.astype(np.float64), want.astype(np.float64)
    return float(np.sqrt(np.mean((got - want) ** 2)) / max(np.sqrt(np.mean(want ** 2)), 1e-30))


def run_chain(gpu, mode, reqs, codes, graph=False):
    ch = Chain(gpu, grid=bench.GRID, rate=bench.RATE, fmt=abi.FORMAT_CS16, mode=mode, max_run_samples=RUN,
               pipelined=graph)
    ids = [ch.add_receiver(r) for r in reqs]
    if graph:
        ch.capture_graph()
    for at in range(0, SAMPLES, RUN):
        ch.run(codes[2 * at:2 * (at + RUN)])
    ch.drain()
    audio = [ch.audio(i) for i in ids]
    fine = [ch.rings(i)[0].copy() for i in ids]
    ch.close()
    return audio, fine


@pytest.fixture(scope="module")
def workload():
    return bench.receivers(bench.RECEIVERS), bench.capture(SAMPLES, seed=bench.SEED)


def test_fast_chain_within_tolerance_of_exact(gpu, workload):
    reqs, codes = workload
    exact_audio, exact_fine = run_chain(gpu, abi.CHAIN_BATCHED, reqs, codes)
    fast_audio, fast_fine = run_chain(gpu, abi.CHAIN_FAST, reqs, codes)
    problems = []
    audio_rel = {}
    for i, r in enumerate(reqs):
        f = rel_rms(fast_fine[i], exact_fine[i])
        if not f <= FINE_REL_MAX:
            problems.append("receiver %d (mode %d): fine relative RMS %.3g" % (i, r.demod, f))
        if fast_audio[i].size != exact_audio[i].size or exact_audio[i].size == 0:
            problems.append("receiver %d: %d vs %d audio values" % (i, fast_audio[i].size, exact_audio[i].size))
            continue
        a = rel_rms(fast_audio[i], exact_audio[i])
        audio_rel.setdefault(r.demod, []).append(a)
        if not a <= AUDIO_REL_MAX:
            problems.append("receiver %d (mode %d): audio relative RMS %.3g" % (i, r.demod, a))
    for mode, rels in audio_rel.items():
        med = float(np.median(rels))
        if not med <= AUDIO_REL_MEDIAN:
            problems.append("mode %d: median audio relative RMS %.3g over %d receivers" % (mode, med, len(rels)))
    assert not problems, "\n".join(problems[:20])


def test_fast_chain_graph_replay_is_bit_identical(gpu, workload):
    reqs, codes = workload
    reqs = reqs[:64]
    direct_audio, direct_fine = run_chain(gpu, abi.CHAIN_FAST, reqs, codes)
    graph_audio, graph_fine = run_chain(gpu, abi.CHAIN_FAST, reqs, codes, graph=True)
    for i in range(len(reqs)):
        assert np.array_equal(direct_fine[i].view(np.uint32), graph_fine[i].view(np.uint32)), i
        assert np.array_equal(direct_audio[i].view(np.uint32), graph_audio[i].view(np.uint32)), i
