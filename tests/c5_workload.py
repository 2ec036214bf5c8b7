"""The learned-proposal workload: seeded burst scenes rendered on the GPU by
the library's own scene synthesiser (rv_scene_plan, rv_scene_noise,
rv_emitter_accumulate), quantised to cs16, their spectrum frames, the plain
detector's decisions over them, training tiles labelled by those decisions,
and the training loop. Shared by the tests and bench.py; PyTorch only holds
device memory and gathers training batches.

Scene: 20 MS/s, bursts of 1 ms to 2 s from random modulations (all eight the
synthesiser renders) at -5 to 30 dB SNR in their occupied bandwidth, over
+-9 MHz, noise at -60 dBFS over the full band; the scene's own burst list is
the truth.
"""
import ctypes as C

import numpy as np
import torch

from revenant_gb300 import abi, proposal, scene
from revenant_gb300.detector import Detector
from revenant_gb300.library import check, lib

RATE = 20_000_000
GRID = (64, 17, 32)
BIN_WIDTH_HZ = RATE / (32 * 2048)
BIN_ZERO_HZ = -RATE * 65 / 128
TRANSFORM = 2048
BINS = GRID[0] * TRANSFORM // 2
HOP = TRANSFORM * GRID[2]            # source samples per frame
ROW_SAMPLES = HOP * proposal.TILE_FRAMES


class _Addr:
    def __init__(self, address):
        self.address = address


def population(seed, n, emitters=64, bursts=None):
    """64 emitters; by default 24 bursts each per 2^30 samples (53.7 s)."""
    bursts = bursts if bursts is not None else max(1, round(24 * n / (1 << 30)))
    return scene.population(seed, RATE, n, noise_dbfs=-60.0, emitters=emitters, bursts=bursts,
                            span=(-9_000_000, 9_000_000), snr=(-5.0, 30.0), burst_seconds=(0.001, 2.0))


def render_cs16(dev, pop, n, chunk=1 << 24):
    """The scene's first n samples as cs16 words on the device (torch int32)."""
    codes = torch.empty(n, dtype=torch.int32, device="cuda")
    buf = torch.empty(2 * min(chunk, n), dtype=torch.float32, device="cuda")
    for start in range(0, n, chunk):
        m = min(chunk, n - start)
        scene.render(dev, pop, start, m, _Addr(buf.data_ptr()))
        dev.synchronize()
        z = buf[:2 * m].view(m, 2)
        q = torch.clamp(torch.round(z * 32768.0), -32768, 32767).to(torch.int32)
        codes[start:start + m] = (q[:, 0] & 0xFFFF) | (q[:, 1] << 16)
    torch.cuda.synchronize()
    return codes


def spectrum_frames(dev, codes, n):
    """[frames][BINS] float32 dB on the device; frame k covers samples [k HOP, (k + 1) HOP)."""
    frames = n // HOP
    out = torch.empty((frames, BINS), dtype=torch.float32, device="cuda")
    sg = proposal.Spectrogram(dev, grid=GRID, rate=RATE, transform=TRANSFORM, run_samples=min(1 << 24, n))
    made = sg.frames(codes.data_ptr(), n, out.data_ptr(), frames)
    sg.close()
    assert made == frames, (made, frames)
    return out


def detector_config():
    M, N = GRID[0], TRANSFORM
    cfg = abi.DetectorConfig()
    cfg.source_rate, cfg.source_center, cfg.bins, cfg.noise_knots = RATE, 100_000_000, BINS, 32
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
    return cfg


def run_plain(dev, frames, rows=None):
    """The plain detector over whole tile rows of frames; returns (wall
    seconds, instants, candidates, stats)."""
    import time
    det = Detector(dev, detector_config())
    det.log_candidates(True)
    rows = rows if rows is not None else frames.shape[0] // proposal.TILE_FRAMES
    torch.cuda.synchronize()
    t = time.perf_counter()
    for r in range(rows):
        f0 = r * proposal.TILE_FRAMES
        det.consume_frames((frames[f0].data_ptr(), proposal.TILE_FRAMES), f0 * HOP, HOP, HOP, device=True)
    dev.synchronize()
    wall = time.perf_counter() - t
    inst, cands = det.read_log()
    st = det.stats()
    det.close()
    return wall, inst, cands, st


def run_learned(dev, cnn, frames, threshold, rows=None, full_every=0, pad_bins=64, hold_rows=1):
    """The learned proposal plus confirmation over whole tile rows; returns
    (wall seconds, instants, candidates, stats, proposed-bin fraction)."""
    import time
    det = Detector(dev, detector_config())
    det.log_candidates(True)
    prop = proposal.Proposer(dev, proposal.proposal_config(BINS, HOP / RATE, 1.0, threshold, hold_rows, pad_bins))
    ld = proposal.LearnedDetector(dev, cnn, det, prop, full_every=full_every)
    rows = rows if rows is not None else frames.shape[0] // proposal.TILE_FRAMES
    torch.cuda.synchronize()
    t = time.perf_counter()
    ld.consume_rows(frames.data_ptr(), rows, 0, HOP, HOP, BINS * 4)
    dev.synchronize()
    wall = time.perf_counter() - t
    inst, cands = det.read_log()
    st = det.stats()
    frac = ld.region_bins / max(1, rows * BINS)
    ld.close()
    prop.close()
    det.close()
    return wall, inst, cands, st, frac


def tile_rows(dev, frames, rows=None):
    """Every tile row of the frames: torch uint16 [rows][tiles][TILE_VALUES] (BF16 bits)."""
    rows = rows if rows is not None else frames.shape[0] // proposal.TILE_FRAMES
    tiles = BINS // proposal.TILE_BINS
    out = torch.empty((rows, tiles, proposal.TILE_VALUES), dtype=torch.int16, device="cuda")
    prop = proposal.Proposer(dev, proposal.proposal_config(BINS, HOP / RATE, 1.0))
    for r in range(rows):
        prop.tiles(frames[r * proposal.TILE_FRAMES].data_ptr(), out[r].data_ptr())
    dev.synchronize()
    prop.close()
    return out


def labels_for(instants, candidates, rows, pad_bins=64):
    """[rows][tiles][CELLS] float32 labels from the plain detector's decisions."""
    lab = proposal.row_labels(instants, candidates, 0, ROW_SAMPLES, rows, BINS, pad_bins)
    return lab.reshape(rows, BINS // proposal.TILE_BINS, proposal.CELLS)


def threshold_for(instants, candidates, logits_rows, recall=0.997, pad_bins=64):
    """The logit threshold that proposes `recall` of the candidates (by their
    core cells' best logit); logits_rows [rows][tiles][CELLS]."""
    z = logits_rows.reshape(logits_rows.shape[0], -1)
    s = proposal.candidate_scores(instants, candidates, z, 0, ROW_SAMPLES, pad_bins)
    s = s[np.isfinite(s)]
    return float(np.quantile(s, 1.0 - recall)) if s.size else 0.0


def train(dev, cnn, tiles, labels, epochs=8, batch=256, lr=1e-3, pos_weight=8.0, seed=0, flip=True):
    """Adam over shuffled tiles; tiles [rows][tiles][values], labels numpy
    [rows][tiles][cells]. With `flip`, every other epoch sees each tile and
    its labels mirrored in frequency. Returns each epoch's mean loss over
    every eighth batch."""
    flat = tiles.reshape(-1, proposal.TILE_VALUES)
    lab = torch.from_numpy(np.ascontiguousarray(labels.reshape(-1, proposal.CELLS))).cuda()
    n = flat.shape[0]
    rng = np.random.default_rng(seed)
    cfg = proposal.train_config(learning_rate=lr, pos_weight=pos_weight)
    steps = epochs * (n // batch)
    step = 0
    xb = torch.empty((batch, proposal.TILE_VALUES), dtype=torch.int16, device="cuda")
    yb = torch.empty((batch, proposal.CELLS), dtype=torch.float32, device="cuda")
    losses = []
    torch.cuda.synchronize()
    # the gathers run on the network's stream, ahead of each step that reads them
    with torch.cuda.stream(torch.cuda.ExternalStream(cnn.stream)):
        for _ in range(epochs):
            order = torch.from_numpy(rng.permutation(n)).cuda()
            seen = []
            for at in range(0, n - batch + 1, batch):
                idx = order[at:at + batch]
                torch.index_select(flat, 0, idx, out=xb)
                torch.index_select(lab, 0, idx, out=yb)
                if flip and len(losses) % 2 == 1:
                    xb.copy_(xb.view(batch, proposal.TILE_FRAMES, proposal.TILE_BINS, proposal.TILE_CHANNELS)
                             .flip(2).reshape(batch, proposal.TILE_VALUES))
                    yb.copy_(yb.flip(1))
                sample = (at // batch) % 8 == 0
                cfg.learning_rate = lr * (0.05 + 0.95 * 0.5 * (1.0 + np.cos(np.pi * step / max(steps, 1))))
                step += 1
                got = cnn.train_step(xb.data_ptr(), yb.data_ptr(), batch, cfg, want_loss=sample)
                if sample:
                    seen.append(got)
            losses.append(float(np.mean(seen)))
    dev.synchronize()
    return losses


def logits(dev, cnn, tiles):
    """Logits [rows][tiles][CELLS] (numpy) of every tile row."""
    rows, per = tiles.shape[0], tiles.shape[1]
    out = torch.empty((rows, per, proposal.CELLS), dtype=torch.float32, device="cuda")
    for r in range(rows):
        cnn.forward(tiles[r].data_ptr(), per, out[r].data_ptr(), per * proposal.CELLS)
    dev.synchronize()
    return out.cpu().numpy()
