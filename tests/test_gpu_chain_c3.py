"""The benchmark's own workload, in small: its 256 receivers (seeded
offsets, 12.5-200 kHz, NFM/AM/USB/LSB/WFM with stereo) on the M = 64,
T = 17, D = 32 grid at 20 MS/s, over the first 2^18 samples of its capture,
through the batched chain as the benchmark runs it (one captured CUDA graph
per run, runs pipelined) and through the oracle chain (the reference's twins
restated in C, receivers spread over host threads). Every receiver's audio
must be equal bit for bit."""
from concurrent.futures import ThreadPoolExecutor
import os

import numpy as np
import pytest

import bench
from oracle_chain import OracleChain
from revenant_gb300 import abi
from revenant_gb300.chain import Chain

pytestmark = pytest.mark.gpu

RUN = 1 << 16
SAMPLES = 1 << 18


def test_bench_receiver_mix_matches_oracle_chain(gpu):
    reqs = bench.receivers(bench.RECEIVERS)
    codes = bench.capture(SAMPLES, seed=bench.SEED)
    ch = Chain(gpu, grid=bench.GRID, rate=bench.RATE, fmt=abi.FORMAT_CS16, mode=abi.CHAIN_BATCHED, max_run_samples=RUN,
               pipelined=True)
    ids = [ch.add_receiver(r) for r in reqs]
    ch.capture_graph()
    threads = max(2, min(32, os.cpu_count() or 2))
    master = OracleChain(bench.GRID, bench.RATE, abi.FORMAT_CS16, [], ring_log2=20, chan_log2=17)
    groups = [OracleChain(bench.GRID, bench.RATE, abi.FORMAT_CS16, reqs[i::threads], ring_log2=4, chan_log2=17)
              for i in range(threads)]
    for g in groups:
        g.chan = master.chan
    with ThreadPoolExecutor(max_workers=threads) as pool:
        for at in range(0, SAMPLES, RUN):
            part = codes[2 * at:2 * (at + RUN)]
            ch.run(part)
            before = master.next_block
            master.run(part, RUN)
            after = master.next_block
            if after > before:
                list(pool.map(lambda g: g.receivers(before, after - 1), groups))
    ch.drain()
    problems = []
    for i, rid in enumerate(ids):
        want = groups[i % threads].audio(i // threads)
        got = ch.audio(rid)
        if got.size == 0 or got.size != want.size or not np.array_equal(got.view(np.uint32), want.view(np.uint32)):
            problems.append("receiver %d (mode %d, %d Hz): %d vs %d values" % (i, reqs[i].demod, reqs[i].bandwidth,
                                                                              got.size, want.size))
    ch.close()
    assert not problems, "\n".join(problems[:20])
