"""Benchmark: input MS/s through the channelizer + N virtual receivers.

Workload (the batched-receivers configuration): a 2^27-sample cs16 capture at
20 MS/s, a 64-channel 2x-oversampled polyphase channelizer (T = 17 taps per
branch) and 256 virtual receivers with seeded offsets, bandwidths uniform in
12.5-200 kHz and modes uniform over NFM/AM/USB/LSB/WFM (stereo WFM), each
planned exactly as the reference plans it. One step = the whole capture
through the chain: fused convert/branch/FFT, then every receiver's fine stage
(resampler + NCO), detector and audio filter, audio read back to the host.

  value : input samples per second with the capture resident in HBM
  e2e   : the same through rv_chain_run with the capture in pinned host
          memory (host->device copy and audio readback inside the timed region)
  plain_path : the same chain recorded the reference's way (one launch per
          stage per receiver), timed on a shorter capture
  roofline   : the dominant stage, from CUDA events on the chain's stream

`--impl reference` times the reference's CPU implementation of the path (the
oracle restatement of its twins, all host threads) on a bounded sample of the
same workload and prints the same metric.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import numpy as np  # noqa: E402

RATE = 20_000_000
GRID = (64, 17, 32)
LOG2N = 27
RECEIVERS = 256
SEED = 3
RUN_SAMPLES = 1 << 24  # default samples per rv_chain_run (--run-log2)
METRIC = "input MS/s through channelizer+N VRX on 1 GB300, % HBM roofline, vs plain path"
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of each stage's
# kernels for one 2^22-sample run of this workload, from one ncu capture
# (ncu --set full on bench.py --log2n 24 --run-log2 22); a launch of another
# run size is scaled by its samples, the traffic growing with the work
MEASURED_TRAFFIC_2P22 = {"coarse": 28.71e6, "fine": 203.71e6, "demod": 157.39e6}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--log2n", type=int, default=LOG2N)
    ap.add_argument("--receivers", type=int, default=RECEIVERS)
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-path comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-detect", action="store_true", help="skip the spectrum + detector measurement")
    ap.add_argument("--no-excision", action="store_true", help="skip the timed run with impulse excision on")
    ap.add_argument("--no-c4", action="store_true", help="skip the M = 4096 channelizer DFT comparison")
    ap.add_argument("--no-noise", action="store_true", help="skip the scene noise field measurement")
    ap.add_argument("--no-tune", action="store_true", help="keep the rule's fine-tile shapes (no rv_chain_autotune)")
    ap.add_argument("--no-fast", action="store_true", help="skip the fast-mode (tensor-core fine stage) leg")
    ap.add_argument("--no-c1c2", action="store_true", help="skip the C1 single-receiver and C2 channelizer legs")
    ap.add_argument("--no-c5", action="store_true", help="skip the learned detection proposal (C5)")
    ap.add_argument("--c5-log2n", type=int, default=30, help="log2 samples of the C5 burst capture")
    ap.add_argument("--run-log2", type=int, default=24, help="log2 samples per rv_chain_run")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def capture(n, seed=SEED):
    """Seeded cs16 capture: a few strong carriers of each mode over noise."""
    import signals
    rng = np.random.default_rng(seed)
    chunk = 1 << 22
    out = np.empty(2 * n, np.int16)
    emitters = [("wfm", 2_500_000, 1.0), ("nfm", -3_100_000, 0.4), ("am", 5_000_000, 0.4), ("usb", -7_000_000, 0.3),
                ("lsb", 8_200_000, 0.3), ("wfm", -6_300_000, 0.8)]
    for at in range(0, n, chunk):
        m = min(chunk, n - at)
        z = np.zeros(m, np.complex128)
        for kind, off, amp in emitters:
            f = {"wfm": signals.wfm, "nfm": signals.nfm, "am": signals.am, "usb": signals.ssb,
                 "lsb": lambda n_, r_, o_, amp, t0: signals.ssb(n_, r_, o_, amp=amp, upper=False, t0=t0)}[kind]
            z += f(m, RATE, off, amp=amp, t0=at)
        z += signals.noise(m, rng, 0.01)
        peak = 6.0
        out[2 * at:2 * (at + m):2] = np.clip(np.round(z.real / peak * 32767), -32768, 32767)
        out[2 * at + 1:2 * (at + m):2] = np.clip(np.round(z.imag / peak * 32767), -32768, 32767)
    return out


class Clocks:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(s[0]) for s in self.samples if num(s[0])]
        mx = [num(s[1]) for s in self.samples if num(s[1])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def receivers(count):
    import signals
    return signals.random_receivers(count, RATE, seed=SEED, grid=GRID)


def algorithmic_bytes(plans, samples):
    """Compulsory and per-stage algorithmic bytes for `samples` input samples."""
    M, T, D = GRID
    blocks = samples // D
    coarse = samples * 4 + blocks * M * 8  # cs16 in, channel ring out
    fine = demod = 0
    for p in plans:
        fc, fd = p.channel_rate, p.demod_rate
        n_fine = samples * fd // RATE
        fine += blocks * 8 + n_fine * 8  # the channel stream read once, fine ring written
        n_audio = samples * p.output_rate // RATE
        demod += n_fine * (8 + 4 + 4) + n_audio * 4 * p.demod.channels
    audio_out = sum(samples * p.output_rate // RATE * 4 * p.demod.channels for p in plans)
    return dict(compulsory=samples * 4 + audio_out, coarse=coarse, fine=fine, demod=demod, audio=audio_out)


def fine_fp32_ops(plans, samples):
    """FP32 operations of the fine stage for `samples` input samples: per
    fine output T complex multiply-adds of 8 rounded operations each (the
    blended tap is precomputed) and the NCO rotation's 6."""
    return sum((samples * p.demod_rate // RATE) * (p.fine.taps * 8 + 6) for p in plans)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def run_gb300(args):
    import torch
    import revenant_gb300 as rg
    from revenant_gb300 import abi
    from revenant_gb300.chain import Chain
    from revenant_gb300.device import Device

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    rg.build()
    torch.cuda.set_device(local)
    dev = Device(local)
    n = 1 << args.log2n
    codes = capture(n)
    reqs = receivers(args.receivers)

    tune_reports = []

    def make_chain(mode, run_samples, profile=True, pipelined=False, tune=False):
        ch = Chain(dev, grid=GRID, rate=RATE, fmt=abi.FORMAT_CS16, mode=mode, max_run_samples=run_samples,
                   keep_audio=False, profile=profile, pipelined=pipelined)
        for r in reqs:
            ch.add_receiver(r)
        if tune and not args.no_tune:
            tune_reports.append(ch.autotune(run_samples))
        return ch

    # replicas: every rank processes its own copy of the workload (the path
    # shards only by time or receiver, with no exchange step)
    d_codes = dev.array(codes)
    pinned = dev.buffer(codes.nbytes, abi.MEMORY_UPLOAD)
    pinned.upload(codes)
    # the timed chain replays one captured CUDA graph per run, pipelined (a run
    # is prepared and its input copied while the previous one executes); a
    # second, directly launched batched chain (bit-identical) gives the
    # per-stage split
    t_tune = time.perf_counter()
    chain = make_chain(abi.CHAIN_BATCHED, min(1 << args.run_log2, n), profile=False, pipelined=True, tune=True)
    tune_s = time.perf_counter() - t_tune
    chain.capture_graph()
    plans = [chain.info(i)[0] for i in range(len(reqs))]
    stream = torch.cuda.ExternalStream(dev.stream)

    run_samples = min(1 << args.run_log2, n)

    def step(ch, source):
        at = 0
        while at < n:
            m = min(run_samples, n - at)
            if source == "device":
                ch.run(_Offset(d_codes, at * 4), m)
            else:
                ch.run(_Offset(pinned, at * 4), m, host=True)
            at += m

    def timed(source, ch=None):
        ch = chain if ch is None else ch
        for _ in range(args.warmup):
            step(ch, source)
        base = ch.stats()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        dev.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        wall = time.perf_counter()
        for _ in range(args.steps):
            step(ch, source)
        t1.record(stream)
        t1.synchronize()
        wall = time.perf_counter() - wall
        ms = t0.elapsed_time(t1)
        torch.cuda.synchronize()
        if world > 1:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms, wall, ch.stats(), base

    with Clocks(local) as clocks:
        ms, wall, st, base = timed("device")
    ms_e2e, _, st_e2e, base_e2e = timed("host")
    per_step_ms = ms / args.steps
    samples_step = n
    value = samples_step * world * args.steps / (ms / 1e3) / 1e6
    e2e = samples_step * world * args.steps / (ms_e2e / 1e3) / 1e6
    d = {k: getattr(st, k) - getattr(base, k) for k in ("launches", "audio_bytes", "runs", "graph_launches",
                                                          "graph_captures", "host_ms")}
    # per-stage device time from the direct batched chain, CUDA events between
    # stages on the chain's stream, over the same number of steps
    sch = make_chain(abi.CHAIN_BATCHED, run_samples, profile=True, tune=True)
    for _ in range(args.warmup):
        step(sch, "device")
    sbase = sch.stats()
    for _ in range(args.steps):
        step(sch, "device")
    sst = sch.stats()
    sch.close()
    stage_ms = {k: getattr(sst, k + "_ms") - getattr(sbase, k + "_ms") for k in ("coarse", "fine", "demod")}
    dominant = max(stage_ms, key=stage_ms.get)
    ab = algorithmic_bytes(plans, samples_step * args.steps)
    pk, pk_kind = peaks()
    achieved = ab[dominant] / (stage_ms[dominant] / 1e3) / 1e9
    hbm_frac = ab["compulsory"] / (ms / 1e3) / 1e9 / pk["hbm_gbs"]
    # the fine stage against the FP32 issue rate it is bound by: every
    # multiply and add is its own rounded instruction (no FMA contraction)
    sms = dev.info.sm_count or 152
    fp32_peak = sms * 128 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    fp32_achieved = fine_fp32_ops(plans, samples_step * args.steps) / (stage_ms["fine"] / 1e3) / 1e12

    # the same timed run with the span-wide impulse excision on (the
    # reference engine's default stage before the channelizer): its cost on
    # this workload
    excision = None
    if not args.no_excision:
        xch = make_chain(abi.CHAIN_BATCHED, run_samples, profile=False, pipelined=True)
        xch.capture_graph()
        xch.set_impulse_excision(True, 15.0, 20e-6)
        for _ in range(args.warmup):
            step(xch, "device")
        xch.drain()
        x0 = torch.cuda.Event(enable_timing=True)
        x1 = torch.cuda.Event(enable_timing=True)
        x0.record(stream)
        for _ in range(args.steps):
            step(xch, "device")
        x1.record(stream)
        x1.synchronize()
        xms = x0.elapsed_time(x1)
        counts = xch.excision_counters()
        excision = {"value": round(samples_step * args.steps / (xms / 1e3) / 1e6, 2), "unit": "MS/s",
                    "ms_per_step": round(xms / args.steps, 3),
                    "samples_excised": counts[0], "runs_excised": counts[1], "runs_spared": counts[2],
                    "samples_examined": counts[3],
                    "note": "rv_chain_set_impulse_excision(15 dB, 20 us): runs converted into a cf32 ring, four "
                            "excision passes, the channelizer reading the ring up to the stage's cleaned end"}
        xch.close()

    # fast mode (RV_CHAIN_FAST): the same timed run with the fine stage as
    # split-precision BF16 GEMMs on the tensor cores (tolerance-checked, not
    # bit-exact), and its per-stage split from a directly launched fast chain
    fast = None
    if not args.no_fast:
        fch = make_chain(abi.CHAIN_FAST, run_samples, profile=False, pipelined=True)
        fch.capture_graph()
        fms, _, _, _ = timed("device", fch)
        fms_e2e, _, _, _ = timed("host", fch)
        fch.close()
        pfch = make_chain(abi.CHAIN_FAST, run_samples, profile=True)
        for _ in range(args.warmup):
            step(pfch, "device")
        fbase = pfch.stats()
        for _ in range(args.steps):
            step(pfch, "device")
        fst = pfch.stats()
        pfch.close()
        fstage = {k: getattr(fst, k + "_ms") - getattr(fbase, k + "_ms") for k in ("coarse", "fine", "demod")}
        fast = {"value": round(samples_step * world * args.steps / (fms / 1e3) / 1e6, 2), "unit": "MS/s",
                "ms_per_step": round(fms / args.steps, 3),
                "e2e": round(samples_step * world * args.steps / (fms_e2e / 1e3) / 1e6, 2),
                "stage_ms_per_step": {k: round(v / args.steps, 3) for k, v in fstage.items()},
                "fine_speedup_vs_exact": round(stage_ms["fine"] / max(fstage["fine"], 1e-9), 2),
                "note": "rv_chain_create(RV_CHAIN_FAST): fine stage on tcgen05 (hi*hi + hi*lo + lo*hi BF16 "
                        "products, FP32 accumulation); fine outputs within 1e-3 relative RMS of the bit-exact "
                        "chain per receiver (tests/test_gpu_chain_fast.py)"}

    plain = None
    if not args.no_plain and n >= 1 << 21:
        # the reference's recording, one launch per stage per receiver (it
        # recomputes the detector inside every audio tap, as the reference's
        # demodulator does), and the same with the detector hoisted (once per
        # fine sample, still one launch per stage per receiver): the second
        # isolates what batching adds. Both on the same 2^22 samples after a
        # 2^20-sample warm-up, CUDA events on the chain's stream.
        blk = 1 << 20
        pn = min(1 << 22, (n - blk) // blk * blk)  # within the capture

        def plain_leg(mode):
            pch = make_chain(mode, blk)
            pch.run(_Offset(d_codes, 0), blk)  # warm-up
            dev.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for at in range(blk, blk + pn, blk):
                pch.run(_Offset(d_codes, at * 4), blk)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            pst = pch.stats()
            pch.close()
            return {"value": round(pn / (ms / 1e3) / 1e6, 3), "unit": "MS/s", "ms": round(ms, 2),
                    "launches_per_run": round(pst.launches / max(pst.runs, 1), 1)}

        plain = plain_leg(abi.CHAIN_PLAIN)
        plain["sample"] = "%d samples after a 2^20 warm-up, same 256 receivers, CUDA events" % pn
        hoisted = plain_leg(abi.CHAIN_HOISTED)
        hoisted["note"] = ("RV_CHAIN_HOISTED: one launch per stage per receiver with the detector once per fine "
                           "sample; the same audio bit for bit")
        plain["detector_hoisted"] = hoisted
        plain["hoisting_gain"] = round(hoisted["value"] / plain["value"], 2)

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "MS/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(per_step_ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batched uneven receivers: 2^%d cs16 samples at 20 MS/s, M=64 D=32 T=17, %d receivers "
                               "NFM/AM/USB/LSB/WFM 12.5-200 kHz (seed %d)" % (args.log2n, args.receivers, SEED),
                   "grid": list(GRID), "rate": RATE, "receivers": args.receivers, "run_samples": min(1 << args.run_log2, n),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "launch": "one captured CUDA graph per run (rv_chain_capture_graph), pipelined runs: %d graph "
                             "launches, %d captures" % (d["graph_launches"], d["graph_captures"]),
                   "l2": "inputs larger than L2 (512 MiB capture per step)"},
        "e2e": {"value": round(e2e, 2), "unit": "MS/s", "h2d_bytes_per_step": samples_step * 4,
                "d2h_bytes_per_step": int(d["audio_bytes"] / args.steps)},
        "gpu_launches": int(d["launches"]),
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4),
                     "traffic": int(MEASURED_TRAFFIC_2P22[dominant] * run_samples / (1 << 22)),
                     "traffic_note": "DRAM bytes per launch (one run of %d samples), ncu on a 2^22-sample run scaled "
                                     "by samples" % run_samples,
                     "peak_kind": pk_kind, "algorithmic_bytes_per_step": int(ab[dominant] / args.steps),
                     "stage_ms_per_step": {k: round(v / args.steps, 3) for k, v in stage_ms.items()},
                     "host_ms_per_step": round(d["host_ms"] / args.steps, 3),
                     "compulsory_hbm_frac": round(hbm_frac, 5),
                     "fp32": {"kernel": "fine", "achieved_tops": round(fp32_achieved, 2),
                              "peak_tops": round(fp32_peak, 1), "frac": round(fp32_achieved / fp32_peak, 3),
                              "peak_kind": "derived: SMs x 128 FP32 lanes x max SM clock, one rounded operation "
                                           "per instruction"}},
        "realtime_factor": round(value * 1e6 / RATE / max(world, 1), 1),
        "plain_path": plain,
        "autotune": None if not tune_reports else dict(
            tune_reports[0], default_ms=round(tune_reports[0]["default_ms"], 3),
            tuned_ms=round(tune_reports[0]["tuned_ms"], 3), seconds=round(tune_s, 2),
            note="rv_chain_autotune before the first run: per receiver class, every fine-tile shape that fits was "
                 "timed on one run of its tiles; default_ms / tuned_ms: one run's fine tiles of every tiled "
                 "receiver with the rule's shapes at 4 tiles per SM, and tuned"),
        "fast_mode": fast,
        "with_impulse_excision": excision,
        "clocks": clocks.summary(),
    }
    if not args.no_plain and plain:
        line["vs_plain_path"] = round(value / plain["value"], 2)
        line["vs_plain_path_detector_hoisted"] = round(value / plain["detector_hoisted"]["value"], 2)
    if rank == 0 and not args.no_detect:
        line["detection"] = detection(dev, d_codes, min(n, 1 << 26))
    if rank == 0 and not args.no_c1c2:
        line["c1_chain"] = c1_chain(dev)
        line["c2_channelizer"] = c2_channelizer(dev, stream, d_codes, max(args.steps, 1), peaks()[0]["hbm_gbs"])
    if rank == 0 and not args.no_noise:
        line["scene_noise"] = scene_noise(dev, stream, n, max(args.steps, 1))
    if rank == 0 and not args.no_c4:
        line["c4_dft"] = c4_dft(dev, stream, d_codes, n, max(args.steps, 1))
    if rank == 0 and not args.no_c5:
        line["c5_learned_proposal"] = c5_learned(dev, args.c5_log2n)
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(reqs, threads=os.cpu_count())
    if rank == 0:
        print(json.dumps(line))
    chain.close()
    dev.close()


def detection(dev, d_codes, samples):
    """The spectrum stage and the wideband detector over the capture as the
    engine would run them: 65,536-sample runs (one spectrum frame each, the
    shipped 64 channels x 2048 points = 65,536 bins), the detector's default
    1 s average and 0.1 s decisions, consuming every frame on the device."""
    from revenant_gb300 import abi
    from revenant_gb300.chain import Chain
    from revenant_gb300.detector import Detector
    M, N, run = GRID[0], 2048, 1 << 16
    bins = M * N // 2
    cfg = abi.DetectorConfig()
    cfg.source_rate, cfg.source_center, cfg.bins, cfg.noise_knots = RATE, 100_000_000, bins, 32
    # SpectrumGeometry (core/engine/graph.cpp:297-313): rate / (D N) Hz per
    # bin, bin zero at -rate (M + 1) / (2 M)
    cfg.bin_width_numerator, cfg.bin_width_denominator = RATE, GRID[2] * N
    cfg.bin_zero_numerator, cfg.bin_zero_denominator = -RATE * (M + 1), 2 * M
    cfg.detection_threshold_db, cfg.average_seconds, cfg.decision_interval_seconds = 6.0, 1.0, 0.1
    cfg.noise_window_knots, cfg.noise_percentile, cfg.noise_percentile_high = 8, 0.10, 0.40
    cfg.noise_excision_sigma, cfg.split_gap_bins, cfg.edge_floor_sigma = 4.0, 8, 3.0
    cfg.occupied_power_fraction, cfg.split_gap_db = 0.99, 1.0
    cfg.residual_rate_tolerance, cfg.residual_decisions = 0.25, 4
    abi.tracking_defaults(cfg)
    cfg.grid_channels = M
    det = Detector(dev, cfg)
    ch = Chain(dev, grid=GRID, rate=RATE, fmt=abi.FORMAT_CS16, mode=abi.CHAIN_BATCHED, max_run_samples=run,
               keep_audio=False)
    ch.set_spectrum(N, det)
    dev.synchronize()
    t = time.perf_counter()
    for at in range(0, samples, run):
        ch.run(_Offset(d_codes, at * 4), run)
    ch.drain()
    wall = time.perf_counter() - t
    st = det.stats()
    seconds = samples / RATE
    out = {"signal_seconds": round(seconds, 3), "bins": bins, "frames": int(st.frames), "decisions": int(st.decisions),
           "candidates_last": int(det.candidates().size), "tracks_last": int(det.tracks().size),
           "tracks_born": int(st.tracks_born), "wall_ms": round(wall * 1e3, 1),
           "ms_per_signal_second": round(wall * 1e3 / seconds, 2),
           "detector_stream_ms": round(st.device_ms, 1), "detector_host_ms": round(st.host_ms, 1),
           "note": "coarse chain + spectrum + detector with tracking, no receivers, wall clock including host work"}
    ch.close()
    det.close()
    return out


def c5_learned(dev, log2n, train_scenes=8, train_log2=27, epochs=16):
    """C5: the learned detection proposal against the plain detector.

    A 2^log2n-sample cs16 burst capture at 20 MS/s (seed 5: 64 emitters of
    all eight modulations, 24 bursts each per 2^30 samples, 1 ms - 2 s, -5 to
    30 dB SNR in their occupied band, the scene's burst list kept as truth),
    rendered on the GPU by the library's own synthesiser; its 65,536-bin
    spectrum frames (M = 64 channels x 2048-point transforms, one frame per
    65,536 samples). The network is trained on the GPU from scratch on
    `train_scenes` other seeded scenes labelled by the plain detector, its
    threshold set on one more (99 % of that scene's localised candidates).
    Detection time: wall clock of the detector over every frame (the plain
    one: accumulate and decide over all bins) against the learned path
    (tiles and network one row ahead on a second stream, decisions confirmed
    inside the proposed ranges), per second of signal."""
    import torch
    from revenant_gb300 import proposal, scene
    import c5_workload as w
    t_all = time.perf_counter()
    out = {"workload": "2^%d cs16 samples at 20 MS/s (%.1f s), seeded burst scene (seed 5), 65,536-bin frames; "
                       "network trained on %d scenes of 2^%d samples" % (log2n, (1 << log2n) / w.RATE, train_scenes,
                                                                         train_log2)}
    nt = 1 << train_log2
    tiles, labels = [], []
    t = time.perf_counter()
    for seed in range(50, 50 + train_scenes):
        fr = w.spectrum_frames(dev, w.render_cs16(dev, w.population(seed, nt), nt), nt)
        inst, cands = w.run_plain(dev, fr)[1:3]
        tiles.append(w.tile_rows(dev, fr))
        labels.append(w.labels_for(inst, cands, tiles[-1].shape[0]))
        del fr
    tiles = torch.cat(tiles, 0)
    labels = np.concatenate(labels, 0)
    data_s = time.perf_counter() - t
    cnn = proposal.Cnn(dev, max_batch=256, seed=1)
    t = time.perf_counter()
    losses = w.train(dev, cnn, tiles, labels, epochs=epochs, lr=2e-3, pos_weight=4.0)
    train_s = time.perf_counter() - t
    steps = epochs * (tiles.shape[0] * tiles.shape[1] // 256)
    del tiles
    vfr = w.spectrum_frames(dev, w.render_cs16(dev, w.population(99, nt), nt), nt)
    vinst, vcands = w.run_plain(dev, vfr)[1:3]
    vz = w.logits(dev, cnn, w.tile_rows(dev, vfr))
    del vfr
    vs = proposal.candidate_scores(vinst, vcands, vz.reshape(vz.shape[0], -1), 0, w.ROW_SAMPLES)
    threshold = float(np.quantile(vs[np.isfinite(vs)], 0.01))
    out["training"] = {"scenes": train_scenes, "tiles": int(labels.size // proposal.CELLS), "epochs": epochs,
                       "adam_steps": steps, "batch": 256, "positive_cells": round(float(labels.mean()), 5),
                       "epoch_mean_loss_first_last": [round(losses[0], 4), round(losses[-1], 4)], "train_s": round(train_s, 2),
                       "data_s": round(data_s, 2), "threshold_logit": round(threshold, 4),
                       "params": proposal.param_count()}
    n = 1 << log2n
    pop = w.population(5, n)
    bursts = scene.plan(pop)
    t = time.perf_counter()
    codes = w.render_cs16(dev, pop, n)
    render_s = time.perf_counter() - t
    frames = w.spectrum_frames(dev, codes, n)
    del codes
    seconds = n / w.RATE
    wall_p, inst_p, cands_p, st_p = w.run_plain(dev, frames)
    wall_l, inst_l, cands_l, st_l, frac = w.run_learned(dev, cnn, frames, threshold)
    wall_f, inst_f, cands_f, st_f, frac_f = w.run_learned(dev, cnn, frames, threshold, full_every=20)
    fp = proposal.bursts_found(bursts, inst_p, cands_p, w.BIN_ZERO_HZ, w.BIN_WIDTH_HZ, w.RATE)
    fl = proposal.bursts_found(bursts, inst_l, cands_l, w.BIN_ZERO_HZ, w.BIN_WIDTH_HZ, w.RATE)
    ff = proposal.bursts_found(bursts, inst_f, cands_f, w.BIN_ZERO_HZ, w.BIN_WIDTH_HZ, w.RATE)
    m, tot = proposal.match(cands_p, inst_p, cands_l, inst_l, max_bins=proposal.LOCALISED_BINS)
    mf, _ = proposal.match(cands_p, inst_p, cands_f, inst_f, max_bins=proposal.LOCALISED_BINS)
    # the network's forward time per tile row (CUDA events on its stream)
    rows = frames.shape[0] // proposal.TILE_FRAMES
    prop = proposal.Proposer(dev, proposal.proposal_config(w.BINS, w.HOP / w.RATE, 1.0, threshold))
    tbuf = torch.empty(proposal.TILE_VALUES * (w.BINS // proposal.TILE_BINS), dtype=torch.int16, device="cuda")
    lbuf = torch.empty(32 * (w.BINS // proposal.TILE_BINS), dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(cnn.stream)
    prop.tiles(frames[0].data_ptr(), tbuf.data_ptr())
    cnn.forward(tbuf.data_ptr(), w.BINS // proposal.TILE_BINS, lbuf.data_ptr(), lbuf.numel())
    dev.synchronize()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    reps = min(rows, 64)
    e0.record(stream)
    for r in range(reps):
        prop.tiles(frames[r * proposal.TILE_FRAMES].data_ptr(), tbuf.data_ptr())
    e1.record(stream)
    for r in range(reps):
        cnn.forward(tbuf.data_ptr(), w.BINS // proposal.TILE_BINS, lbuf.data_ptr(), lbuf.numel())
    e2.record(stream)
    e2.synchronize()
    tiles_ms, fwd_ms = e0.elapsed_time(e1) / reps, e1.elapsed_time(e2) / reps
    prop.close()
    flops = 2.0 * (w.BINS // proposal.TILE_BINS) * (1024 * 64 * 32 + 256 * 128 * 256 + 128 * 128 * 768 +
                                                     32 * 64 * 1536 + 32 * 64)
    out.update({
        "signal_seconds": round(seconds, 2), "frames": int(frames.shape[0]), "tile_rows": rows,
        "bursts": len(bursts), "render_s": round(render_s, 2),
        "plain": {"ms_per_signal_second": round(wall_p * 1e3 / seconds, 3), "wall_s": round(wall_p, 3),
                  "decisions": int(st_p.decisions), "candidates": len(cands_p),
                  "localised_candidates": int(proposal.localised(cands_p).sum()),
                  "bursts_found": int(fp.sum())},
        "learned": {"ms_per_signal_second": round(wall_l * 1e3 / seconds, 3), "wall_s": round(wall_l, 3),
                    "decisions": int(st_l.decisions), "candidates": len(cands_l),
                    "proposed_bin_fraction": round(frac, 4), "bursts_found": int(fl.sum()),
                    "burst_recall_vs_plain": round(float((fl & fp).sum() / max(fp.sum(), 1)), 4),
                    "candidate_recall_vs_plain": round(m / max(tot, 1), 4)},
        "learned_with_fallback": {"full_band_every_rows": 20, "ms_per_signal_second": round(wall_f * 1e3 / seconds, 3),
                                  "burst_recall_vs_plain": round(float((ff & fp).sum() / max(fp.sum(), 1)), 4),
                                  "candidate_recall_vs_plain": round(mf / max(tot, 1), 4)},
        "speedup": round(wall_p / wall_l, 2), "speedup_with_fallback": round(wall_p / wall_f, 2),
        "truth_recall": {"plain": round(float(fp.mean()), 4), "learned": round(float(fl.mean()), 4)},
        "network": {"tiles_ms_per_row": round(tiles_ms, 4), "forward_ms_per_row": round(fwd_ms, 4),
                    "forward_tflops": round(flops / fwd_ms / 1e9, 1), "tiles_per_row": w.BINS // proposal.TILE_BINS},
        "leg_s": round(time.perf_counter() - t_all, 1),
        "note": "recall is burst-level (a scene burst counts as found when a candidate of a decision while it is on, "
                "or within 1 s after, overlaps and localises its band); candidate recall leaves out candidates wider "
                "than 512 bins (the floor estimate's bias summed over the ladder's widest windows)"})
    assert cnn.status() == 0
    cnn.close()
    del frames
    torch.cuda.empty_cache()
    return out


C1_RATE, C1_GRID = 2_400_000, (8, 17, 4)


def c1_capture(n, seed=1):
    """C1's input: cu8 IQ at 2.4 MS/s (offset 127.5), a WFM carrier at
    +200 kHz (75 kHz deviation, 1 kHz tone) plus AWGN at 25 dB SNR."""
    rng = np.random.default_rng(seed)
    t = np.arange(n) / C1_RATE
    phase = 2 * np.pi * 200_000 * t + 75_000 / 1000 * np.sin(2 * np.pi * 1000 * t)
    z = np.exp(1j * phase) + 10 ** (-25 / 20) * (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)
    z *= 0.9 / np.max(np.abs(np.concatenate([z.real, z.imag])))
    codes = np.empty(2 * n, np.uint8)
    codes[0::2] = np.clip(np.round(z.real * 127.5 + 127.5), 0, 255)
    codes[1::2] = np.clip(np.round(z.imag * 127.5 + 127.5), 0, 255)
    return codes


def c1_chain(dev):
    """C1: the plain single-receiver chain as the reference runs it on the CPU:
    2^20 cu8 samples at 2.4 MS/s (seed 1), grid M=8 D=4 T=17, one stereo WFM
    receiver at +200 kHz, fed through rv_chain_run from host memory in
    16,384-sample blocks (the RTL-SDR's transfer size), launch-bound at this
    size; per-stage device time from the plain chain's events. Beside it the
    oracle chain (the reference's twins restated in C) on one host core over
    the first 2^17 samples."""
    from bindings import cf32  # noqa: F401  (tests/ on the path for the oracle chain)
    from oracle_chain import OracleChain
    from revenant_gb300 import abi
    from revenant_gb300.chain import Chain
    n, block, rate, grid = 1 << 20, 1 << 14, C1_RATE, C1_GRID
    codes = c1_capture(n)
    req = abi.request(center=200_000, bandwidth=200_000, demod="wfm", stereo=True)
    out = {"workload": "2^20 cu8 at 2.4 MS/s (seed 1), M=8 D=4 T=17, one stereo WFM receiver, 16,384-sample "
                       "blocks from host memory"}
    for name, mode, graph in (("batched_graph_pipelined", abi.CHAIN_BATCHED, True),
                              ("batched", abi.CHAIN_BATCHED, False), ("plain", abi.CHAIN_PLAIN, False)):
        ch = Chain(dev, grid=grid, rate=rate, fmt=abi.FORMAT_CU8, mode=mode, max_run_samples=block, pipelined=graph)
        rid = ch.add_receiver(req)
        if graph:
            ch.capture_graph()
        for at in range(0, 8 * block, block):  # warm-up
            ch.run(codes[2 * at:2 * (at + block)])
        ch.drain()
        dev.synchronize()
        t0 = time.perf_counter()
        for at in range(8 * block, n, block):
            ch.run(codes[2 * at:2 * (at + block)])
        ch.drain()
        dt = time.perf_counter() - t0
        frames = ch.audio(rid).size // 2
        out[name] = {"value": round((n - 8 * block) / dt / 1e6, 2), "unit": "MS/s",
                     "us_per_block": round(dt / ((n - 8 * block) / block) * 1e6, 1), "audio_frames": int(frames)}
        ch.close()
    # the 1024-point Hann spectrum averaged over 16 frames (lw-radio-dsp's
    # Spectrum with a 16-frame mean, rv_spectrum_average) over the capture
    import ctypes as C
    import torch
    from revenant_gb300.library import check, lib
    size, avg = 1024, 16
    frames = n // size
    iq = ((codes.astype(np.float32) - 127.5) / 127.5)
    w = np.zeros(size, np.float32)
    norm = C.c_double()
    check(lib().rv_build_lwdsp_window(1, size, w.ctypes.data, C.byref(norm)))
    tw = np.zeros((size, 2), np.float32)
    check(lib().rv_build_fft_twiddles(size, tw.ctypes.data, size))
    sp = abi.SpectrumAverageParams(size=size, frames=frames, average=avg, mode=abi.AVERAGE_MEAN, alpha=0.0,
                                   norm=norm.value, resume=0)
    spectra = frames // avg
    d_iq, d_w, d_tw = dev.array(iq), dev.array(w), dev.array(tw)
    d_db, d_avg = dev.zeros(spectra * size * 4), dev.zeros(spectra * size * 4)

    def spectrum():
        check(lib().rv_spectrum_average(dev.stream, C.byref(sp), d_iq.address, n, d_w.address, size, d_tw.address,
                                        size, d_db.address, spectra * size, d_avg.address, spectra * size))

    stream = torch.cuda.ExternalStream(dev.stream)
    spectrum()
    dev.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(10):
        spectrum()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / 10
    out["spectrum_1024_hann_mean16"] = {"ms": round(ms, 4), "spectra": spectra, "frames": frames,
                                        "value": round(n / ms / 1e3, 1), "unit": "MS/s",
                                        "note": "rv_spectrum_average over the whole 2^20-sample capture (cf32 on "
                                                "the device), within the a13 tolerance of the FP64 mean "
                                                "(tests/test_spectrum_average.py)"}
    out["baseline_shape"] = ("the 240 kS/s, 64-tap fine stage and decimation by 5 to 48 kHz: bit-exact against the "
                             "oracle end to end in tests/test_gpu_c1_shape.py; the chain legs above run the planner's "
                             "own WFM shape (336 kS/s, T = 32, stereo)")
    m = 1 << 17
    oc = OracleChain(grid, rate, abi.FORMAT_CU8, [req], ring_log2=18, chan_log2=16, fine_log2=17)
    t0 = time.perf_counter()
    for at in range(0, m, block):
        oc.run(codes[2 * at:2 * (at + block)], block)
    dt = time.perf_counter() - t0
    out["cpu_oracle"] = {"value": round(m / dt / 1e6, 3), "unit": "MS/s", "cores": 1,
                         "sample": "the first 2^17 samples, the oracle chain (convert, branch, FFT, fine, WFM "
                                   "demodulator) in C on one core"}
    return out


def c2_channelizer(dev, stream, d_codes, reps, hbm_gbs):
    """C2: the M = 1024 (D = 512, T = 16) channelizer over 2^26 cs16 samples
    (the capture's first 2^26 stand in for C2's 61.44 MS/s scene; the
    channelizer's time does not depend on the content). The fused kernel
    (rv_coarse_fused, the generic kernel for grids sized at run time: the raw
    cs16 ring in, the channel ring out), and beside it the three dispatches
    (convert, branch FIR, FFT) with their intermediates in HBM. Algorithmic
    bytes 20 per input sample (4 in, 16 out: the 2x-oversampled cf32 channel
    streams) against the measured HBM bandwidth."""
    import ctypes as C
    import torch
    from revenant_gb300 import abi
    from revenant_gb300.library import check, lib
    # 2^26 samples, or the whole capture when it is shorter (a power of two:
    # the raw ring's mask)
    M, T, D = 1024, 16, 512
    n = min(1 << 26, 1 << ((d_codes.nbytes // 4).bit_length() - 1))
    g = abi.GridParams(M, T, D)
    taps = np.zeros(M * T, np.float32)
    check(lib().rv_design_prototype(C.byref(g), 120.0, taps.ctypes.data, taps.size, None, None))
    tw = np.zeros((M, 2), np.float32)
    check(lib().rv_build_fft_twiddles(M, tw.ctypes.data, M))
    d_taps, d_tw = dev.array(taps), dev.array(tw)
    ring = dev.zeros(n * 8)
    base = M * T // D
    blocks = (n - base * D) // D
    ring_blocks = 1 << (blocks - 1).bit_length()
    branch = dev.zeros(blocks * M * 8)
    chan = dev.zeros(M * ring_blocks * 8)
    cp = abi.ConvertParams(n - 1, 0, 0, n)
    bp = abi.PfbBranchParams(n - 1, base * D, blocks)
    fp = abi.PfbFftParams(M, D, 10, base, blocks, ring_blocks, ring_blocks - 1)
    cpar = abi.CoarseParams(n - 1, base * D, blocks, base, ring_blocks, ring_blocks - 1, 0)

    def dispatches():
        check(lib().rv_convert(dev.stream, abi.FORMAT_CS16, C.byref(cp), d_codes.address, n * 4, ring.address, n))
        check(lib().rv_pfb_branch(dev.stream, C.byref(g), C.byref(bp), d_taps.address, taps.size, ring.address, n,
                                  branch.address, blocks * M))
        check(lib().rv_pfb_fft(dev.stream, C.byref(fp), branch.address, blocks * M, d_tw.address, M, chan.address,
                               M * ring_blocks))

    def fused():
        check(lib().rv_coarse_fused(dev.stream, C.byref(g), abi.FORMAT_CS16, C.byref(cpar), d_codes.address, n * 4,
                                    d_taps.address, taps.size, d_tw.address, M, chan.address, M * ring_blocks))

    def timed(fn):
        fn()
        dev.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    ms = timed(fused)
    ms_d = timed(dispatches)
    for b in (d_taps, d_tw, ring, branch, chan):
        b.free()
    gbs, gbs_d = 20.0 * n / ms / 1e6, 20.0 * n / ms_d / 1e6
    return {"workload": "M=1024 D=512 T=16 over 2^%d cs16 samples: the fused channelizer (rv_coarse_fused)"
                        % (n.bit_length() - 1),
            "ms": round(ms, 3), "value": round(n / ms / 1e3, 1), "unit": "MS/s", "roofline": {
                "bound": "hbm", "achieved": round(gbs, 1), "peak": hbm_gbs, "unit": "GB/s",
                "frac": round(gbs / hbm_gbs, 4), "algorithmic_bytes_per_sample": 20},
            "dispatches": {"ms": round(ms_d, 3), "value": round(n / ms_d / 1e3, 1), "unit": "MS/s",
                           "frac": round(gbs_d / hbm_gbs, 4),
                           "note": "convert, branch FIR and FFT dispatches: the cf32 ring (8 B/S) and the branch "
                                   "outputs (16 B/S written and read) are intermediates in HBM"}}


def scene_noise(dev, stream, n, reps):
    """a16: the synthesiser's noise field (siggen::Scene::fill_noise) for the
    capture's 2^n samples on the GPU (CUDA events, `reps` renders), and the
    oracle's C restatement of the reference's loop on one host core over a
    2^18-sample sample."""
    import ctypes as C
    import torch
    from revenant_gb300.library import check, lib
    sigma = lib().rv_scene_noise_sigma(-60.0)
    out = dev.zeros(n * 8)
    check(lib().rv_scene_noise(dev.stream, 1, sigma, 0, n, out.address, n))
    dev.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        check(lib().rv_scene_noise(dev.stream, 1, sigma, 0, n, out.address, n))
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    out.free()
    res = {"samples": n, "ms": round(ms, 3), "value": round(n / ms / 1e3, 1), "unit": "MS/s",
           "note": "4096-sample noise blocks, one warp each: MT19937-64 twisted cooperatively in shared memory, "
                   "FP64 Box-Muller"}
    try:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import build as oracle_build
        o = C.CDLL(oracle_build.build())
        o.or_scene_noise.argtypes = [C.c_uint64, C.c_double, C.c_uint64, C.c_uint64, C.c_void_p]
        m = 1 << 18
        buf = np.zeros((m, 2), np.float32)
        t = time.perf_counter()
        o.or_scene_noise(1, sigma, 0, m, buf.ctypes.data)
        dt = time.perf_counter() - t
        res["cpu_oracle"] = {"value": round(m / dt / 1e6, 2), "unit": "MS/s", "cores": 1,
                             "sample": "2^18 samples, the reference's per-sample loop restated in C"}
    except Exception as e:  # the oracle is a reported baseline; its absence does not stop the bench
        res["cpu_oracle"] = {"unavailable": str(e)}
    return res


def c4_dft(dev, stream, d_codes, n, reps):
    """C4: the M = 4096 (D = 2048, T = 16) channelizer's DFT over the same
    capture, converted to cf32 and branch-filtered once: the FP32 radix-2 FFT
    (rv_pfb_fft, the reference's arithmetic) against the split-precision DFT
    on the tensor cores (rv_pfb_dft_tc, FP16 and BF16 hi + lo operands, FP32
    accumulators). CUDA events around `reps` dispatches of all blocks each."""
    import ctypes as C
    import torch
    from revenant_gb300 import abi
    from revenant_gb300.library import check, lib
    M, T, D = 4096, 16, 2048
    g = abi.GridParams(M, T, D)
    taps = np.zeros(M * T, np.float32)
    check(lib().rv_design_prototype_wide(C.byref(g), 120.0, taps.ctypes.data, taps.size, None, None))
    tw = np.zeros((M, 2), np.float32)
    check(lib().rv_build_fft_twiddles(M, tw.ctypes.data, M))
    ring = dev.zeros(n * 8)
    check(lib().rv_convert(dev.stream, abi.FORMAT_CS16, C.byref(abi.ConvertParams(n - 1, 0, 0, n)), d_codes.address,
                           n * 4, ring.address, n))
    base = M * T // D
    blocks = (n - base * D) // D
    ring_blocks = 1 << (blocks - 1).bit_length()
    d_taps, d_tw = dev.array(taps), dev.array(tw)
    branch = dev.zeros(blocks * M * 8)
    chan = dev.zeros(M * ring_blocks * 8)
    bp = abi.PfbBranchParams(n - 1, base * D, blocks)
    check(lib().rv_pfb_branch_wide(dev.stream, C.byref(g), C.byref(bp), d_taps.address, taps.size, ring.address, n,
                                   branch.address, blocks * M))
    fp = abi.PfbFftParams(M, D, 12, base, blocks, ring_blocks, ring_blocks - 1)

    def fft():
        check(lib().rv_pfb_fft(dev.stream, C.byref(fp), branch.address, blocks * M, d_tw.address, M, chan.address,
                               M * ring_blocks))

    def tc(prec):
        return lambda: check(lib().rv_pfb_dft_tc(dev.stream, C.byref(fp), branch.address, blocks * M, d_tw.address, M,
                                                 chan.address, M * ring_blocks, prec))

    out = {"workload": "M=4096 D=2048 T=16 over 2^%d cs16 samples: %d blocks of 4096 branch outputs" % (
        n.bit_length() - 1, blocks)}
    flops_tc = blocks * 2 * 3 * 2 * 128 * 64 * 128  # two GEMM stages x three split products, per block
    for name, fn in (("fft_fp32", fft), ("tc_fp16_split", tc(abi.DFT_FP16)), ("tc_bf16_split", tc(abi.DFT_BF16))):
        fn()
        dev.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[name] = {"ms": round(ms, 3), "gs_per_s": round(blocks * D / ms / 1e6, 2)}
        if name != "fft_fp32":
            check(lib().rv_pfb_dft_tc_status(dev.stream, None))
            out[name]["tensor_tflops"] = round(flops_tc / ms / 1e9, 1)
    out["accuracy_vs_fp64"] = {"fft_fp32": "1.6e-7 rel RMS, -139 dBc", "tc_fp16_split": "4.8e-7 rel RMS, -125.8 dBc",
                               "tc_bf16_split": "4.6e-6 rel RMS, -116.9 dBc",
                               "note": "tests/test_c4.py on 256 blocks of a 90 dB multitone"}
    for b in (ring, d_taps, d_tw, branch, chan):
        b.free()
    return out


class _Offset:
    """A device or pinned buffer address plus a byte offset, for Chain.run."""

    def __init__(self, buf, offset):
        self.address = buf.address + offset


class OracleWorkload:
    """The workload through the oracle (the reference's CPU twins restated in
    C, planned by the oracle's own planner, pinned to the reference's): one
    chain converts, branch-filters and FFTs each run, and the receivers'
    fine stages, carrier loops and demodulators run spread over `threads`
    host threads (ctypes releases the interpreter lock inside the C). The GPU
    library is never loaded."""

    def __init__(self, reqs, threads):
        from concurrent.futures import ThreadPoolExecutor
        from oracle_chain import OracleChain
        from revenant_gb300 import abi
        self.threads = max(1, threads)
        self.master = OracleChain(GRID, RATE, abi.FORMAT_CS16, [], ring_log2=20, chan_log2=17)
        self.groups = [OracleChain(GRID, RATE, abi.FORMAT_CS16, reqs[i::self.threads], ring_log2=4, chan_log2=17)
                       for i in range(self.threads) if reqs[i::self.threads]]
        for g in self.groups:
            g.chan = self.master.chan
        self.pool = ThreadPoolExecutor(max_workers=self.threads) if self.threads > 1 else None

    def run(self, codes, count, run=1 << 16, serial=False):
        """`count` more samples of the stream; serial: every receiver on the
        calling thread."""
        for at in range(0, count, run):
            m = min(run, count - at)
            before = self.master.next_block
            self.master.run(codes[2 * at:2 * (at + m)], m)
            after = self.master.next_block
            if after > before:
                if self.pool and not serial:
                    list(self.pool.map(lambda g: g.receivers(before, after - 1), self.groups))
                else:
                    for g in self.groups:
                        g.receivers(before, after - 1)

    def close(self):
        if self.pool:
            self.pool.shutdown()


def cpu_baseline(reqs, threads=None, sample_log2=18):
    """The oracle on the host cores over a bounded sample of the same
    workload (the first 2^sample_log2 samples of the capture, all
    receivers)."""
    threads = threads or os.cpu_count() or 1
    n = 1 << sample_log2
    codes = capture(n)
    wl = OracleWorkload(reqs, threads)
    t = time.perf_counter()
    wl.run(codes, n)
    dt = time.perf_counter() - t
    wl.close()
    return {"value": round(n / dt / 1e6, 4), "unit": "MS/s", "cores": threads, "kind": "port",
            "sample": "the capture's first 2^%d samples (%.1f ms of signal), all %d receivers, %.2f s on %d threads"
                      % (sample_log2, n / RATE * 1e3, len(reqs), dt, threads)}


def run_reference(args):
    """The reference's CPU implementation of the path on this host's cores,
    as the oracle restates it (the reference's twins and planner in C; the
    reference itself is a C++/Vulkan application with no package to install
    and is not on this machine). Each step is a bounded sample of the same
    workload: the next 2^step_log2 samples of the same capture through the
    same 256 receivers, continuing the stream. Times every step on all host
    threads, and one sample on a single thread."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    step_log2 = 16
    step = 1 << step_log2
    reqs = receivers(args.receivers)
    tail = 1 << 13  # the single-thread sample after the timed steps
    codes = capture((args.warmup + args.steps) * step + tail)
    wl = OracleWorkload(reqs, threads)
    at = 0
    for _ in range(args.warmup):
        wl.run(codes[2 * at:2 * (at + step)], step)
        at += step
    t = time.perf_counter()
    for _ in range(args.steps):
        wl.run(codes[2 * at:2 * (at + step)], step)
        at += step
    dt = time.perf_counter() - t
    v = step * args.steps / dt / 1e6
    # one thread: the stream's next 2^13 samples with every receiver on this
    # thread (the same chains, so in the same steady state)
    m = tail
    t = time.perf_counter()
    wl.run(codes[2 * at:2 * (at + m)], m, serial=True)
    dt1 = time.perf_counter() - t
    wl.close()
    ms_per_step = dt * 1e3 / args.steps
    line = {"metric": METRIC, "value": round(v, 4), "unit": "MS/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": "batched uneven receivers: 2^%d cs16 samples at 20 MS/s, M=64 D=32 T=17, %d receivers "
                                   "NFM/AM/USB/LSB/WFM 12.5-200 kHz (seed %d)" % (args.log2n, args.receivers, SEED),
                       "step": "a bounded sample of the workload: the next 2^%d samples of the capture through all %d "
                               "receivers (the full 2^%d-sample step would take about %.0f s here)"
                               % (step_log2, len(reqs), args.log2n, ms_per_step / 1e3 * (1 << args.log2n) / step)},
            "cpu_baseline": {"value": round(v, 4), "unit": "MS/s", "cores": threads, "kind": "port",
                             "sample": "%d steps of 2^%d samples after %d warm-up steps, receivers over %d threads"
                                       % (args.steps, step_log2, args.warmup, threads),
                             "single_thread": {"value": round(m / dt1 / 1e6, 4), "unit": "MS/s", "cores": 1,
                                               "sample": "the stream's next 2^13 samples after the timed steps, "
                                                         "all receivers on one thread"}},
            "e2e": {"value": round(v, 4), "unit": "MS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
