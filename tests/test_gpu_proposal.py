"""The learned proposal's tile builder, its proposed ranges and the
detector's confirmation over ranges, on the GPU through the C ABI.

- tiles against the FP64 restatement (oracle/proposal.py): every value within
  one BF16 rounding plus 2e-3 (the GPU averages in FP32);
- ranges: exactly the restatement's;
- the confirmation over the whole band: the plain detector's candidates,
  every integer field equal (the region path's prefix sums and knot means
  round differently, which moves no decision here);
- end to end on seeded scenes from the library's synthesiser: trained on the
  GPU, thresholded on a validation scene, the learned proposal keeps >= 97 %
  of the bursts the plain detector finds on a held-out scene (burst-level
  recall, the bench reports the C5 figure) while the detector looks at no
  more than 35 % of the bins, and proposes no more than 1.25 times the bins of
  a threshold on the averaged power alone tuned to the same validation recall
  (on eight small training scenes the two come out close, and training on
  the GPU is not bit-reproducible: the backward pass accumulates with
  atomics; the bench's C5 leg measures the network on its 2^30-sample scene).
"""
import os
import sys

import numpy as np
import pytest
import torch

from revenant_gb300 import proposal, scene
from revenant_gb300.detector import Detector
from revenant_gb300.library import lib

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import proposal as oracle_proposal  # noqa: E402

import c5_workload as w  # noqa: E402

pytestmark = pytest.mark.gpu


def bf16_to_f64(bits):
    return (np.asarray(bits).view(np.uint16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def test_tiles_match_restatement(gpu):
    bins = 4 * 256
    rng = np.random.default_rng(7)
    frames = (-110.0 + 5.6 * rng.standard_normal((2 * 64, bins))).astype(np.float32)
    frames[:, 300:340] += 20.0  # a carrier
    frames[70:90, 700:720] += 30.0  # a burst in the second row
    cfg = proposal.proposal_config(bins, 65536 / 20e6, 1.0)
    prop = proposal.Proposer(gpu, cfg)
    d_frames = gpu.array(frames)
    d_tiles = gpu.zeros(4 * proposal.TILE_VALUES * 2)
    a, q = oracle_proposal.alphas(65536 / 20e6, 1.0)
    state = {}
    for r in range(2):
        prop.tiles(d_frames.address + r * 64 * bins * 4, d_tiles.address)
        gpu.synchronize()
        got = bf16_to_f64(d_tiles.download(np.uint16, (4 * proposal.TILE_VALUES,))).reshape(4, 64, 256, 2)
        want = oracle_proposal.tile_row(frames[64 * r:64 * (r + 1)], state, a, q)
        assert np.all(np.abs(got - want) <= 2.0 ** -8 * np.abs(want) + 2e-3), r
    prop.close()


@pytest.mark.parametrize("hold,pad", [(0, 16), (1, 16), (2, 64), (0, 0)])
def test_regions_match_restatement(gpu, hold, pad):
    bins = 8 * 256
    cells = bins // 8
    rng = np.random.default_rng(hold * 10 + pad)
    prop = proposal.Proposer(gpu, proposal.proposal_config(bins, 0.003, 1.0, threshold=0.5, hold_rows=hold,
                                                           pad_bins=pad))
    history = []
    for row in range(5):
        z = rng.standard_normal(cells).astype(np.float32) - 2.0
        z[0] = 3.0 if row == 1 else -3.0        # the first cell, padding clipped at 0
        z[cells - 1] = 3.0 if row == 2 else -3.0  # the last cell, clipped at bins
        d = gpu.array(z)
        got = prop.regions(d.address)
        history.append(z > 0.5)
        want = oracle_proposal.regions(history[-(hold + 1):], bins, pad)
        assert np.array_equal(got, want), (row, got, want)
    prop.close()


@pytest.fixture(scope="module")
def small_scene(gpu):
    n = 1 << 26
    pop = w.population(5, n)
    codes = w.render_cs16(gpu, pop, n)
    frames = w.spectrum_frames(gpu, codes, n)
    return pop, frames


def test_full_band_confirmation_equals_plain_detector(gpu, small_scene):
    pop, frames = small_scene
    _, inst_p, cands_p, st_p = w.run_plain(gpu, frames)
    det = Detector(gpu, w.detector_config())
    det.log_candidates(True)
    det.set_regions(np.array([[0, w.BINS]], np.uint32))
    rows = frames.shape[0] // 64
    for r in range(rows):
        f0 = r * 64
        det.consume_frames((frames[f0].data_ptr(), 64), f0 * w.HOP, w.HOP, w.HOP, device=True)
    inst, cands = det.read_log()
    det.close()
    assert st_p.decisions > 10 and len(cands_p) > 50
    assert np.array_equal(inst, inst_p)
    for field in ("first_bin", "last_bin", "center", "bandwidth"):
        assert np.array_equal(cands[field], cands_p[field]), field


def test_regions_reject_bad_ranges(gpu):
    det = Detector(gpu, w.detector_config())
    bad = [np.array([[10, 5]], np.uint32), np.array([[0, w.BINS + 1]], np.uint32),
           np.array([[0, 100], [50, 200]], np.uint32)]
    for r in bad:
        assert lib().rv_detector_set_regions(det.handle, r.ctypes.data, r.shape[0]) != 0
    det.close()


def _scene_frames(gpu, seed, n):
    codes = w.render_cs16(gpu, w.population(seed, n), n)
    return w.spectrum_frames(gpu, codes, n)


def test_learned_proposal_keeps_the_plain_detectors_bursts(gpu):
    n = 1 << 27
    tiles, labels = [], []
    for seed in range(60, 68):
        fr = _scene_frames(gpu, seed, n)
        inst, cands = w.run_plain(gpu, fr)[1:3]
        tiles.append(w.tile_rows(gpu, fr))
        labels.append(w.labels_for(inst, cands, tiles[-1].shape[0]))
        del fr
    cnn = proposal.Cnn(gpu, max_batch=256, seed=3)
    losses = w.train(gpu, cnn, torch.cat(tiles, 0), np.concatenate(labels, 0), epochs=16, lr=2e-3, pos_weight=4.0)
    del tiles
    assert losses[-1] < losses[0]
    # threshold: 99 % of the validation scene's localised candidates
    vfr = _scene_frames(gpu, 69, n)
    vinst, vcands = w.run_plain(gpu, vfr)[1:3]
    vtiles = w.tile_rows(gpu, vfr)
    vz = w.logits(gpu, cnn, vtiles)
    vs = proposal.candidate_scores(vinst, vcands, vz.reshape(vz.shape[0], -1), 0, w.ROW_SAMPLES)
    vs = vs[np.isfinite(vs)]
    threshold = float(np.quantile(vs, 0.01))
    # the same recall from the averaged power alone: the best channel-1 value
    # over a cell's bins in the row's last frame
    raw = vtiles.view(torch.int16).cpu().numpy().view(np.uint16)
    pw = bf16_to_f64(raw).reshape(vtiles.shape[0], vtiles.shape[1], 64, 256, 2)[:, :, -1, :, 1]
    pw = pw.reshape(vtiles.shape[0], vtiles.shape[1], 32, 8).max(axis=3)
    ps = proposal.candidate_scores(vinst, vcands, pw.reshape(pw.shape[0], -1), 0, w.ROW_SAMPLES)
    ps = ps[np.isfinite(ps)]
    power_threshold = float(np.quantile(ps, 0.01))
    cnn_frac = float((vz > threshold).mean())
    power_frac = float((pw > power_threshold).mean())
    assert cnn_frac < 1.25 * power_frac, (cnn_frac, power_frac)
    # held-out scene
    pop = w.population(5, n)
    fr = w.spectrum_frames(gpu, w.render_cs16(gpu, pop, n), n)
    _, inst_p, cands_p, _ = w.run_plain(gpu, fr)
    _, inst_l, cands_l, _, frac = w.run_learned(gpu, cnn, fr, threshold)
    bursts = scene.plan(pop)
    fp = proposal.bursts_found(bursts, inst_p, cands_p, w.BIN_ZERO_HZ, w.BIN_WIDTH_HZ, w.RATE)
    fl = proposal.bursts_found(bursts, inst_l, cands_l, w.BIN_ZERO_HZ, w.BIN_WIDTH_HZ, w.RATE)
    assert fp.sum() >= 20
    recall = (fl & fp).sum() / fp.sum()
    assert recall >= 0.97, (recall, fp.sum())
    assert frac <= 0.35, frac
    assert cnn.status() == 0
    cnn.close()
