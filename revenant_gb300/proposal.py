"""Host mirror of the learned detection proposal (rv_cnn_*, rv_proposer_*).

``Cnn(device, max_batch, seed)`` wraps the spectrogram network whose forward
and backward passes run on the tensor cores in librevenant_gb300.so;
``Proposer(device, config)`` builds tile rows from spectrum frames and turns
the network's logits into bin ranges for the detector to confirm
(``Detector.set_regions``). The helpers below it label tile rows from the
plain detector's candidates and score one detector's candidates against
another's; they are host bookkeeping, not part of the signal path.
"""
import ctypes as C

import numpy as np

from . import abi
from .library import check, lib

TILE_FRAMES, TILE_BINS, TILE_CHANNELS = abi.TILE_FRAMES, abi.TILE_BINS, abi.TILE_CHANNELS
CELLS, CELL_BINS = abi.CNN_CELLS, abi.CNN_CELL_BINS
TILE_VALUES = TILE_FRAMES * TILE_BINS * TILE_CHANNELS  # BF16 values per tile


def param_count():
    return int(lib().rv_cnn_param_count())


def train_config(learning_rate=1e-3, beta1=0.9, beta2=0.999, epsilon=1e-8, weight_decay=0.0, pos_weight=4.0):
    c = abi.CnnTrainConfig()
    c.learning_rate, c.beta1, c.beta2, c.epsilon = learning_rate, beta1, beta2, epsilon
    c.weight_decay, c.pos_weight = weight_decay, pos_weight
    return c


class Cnn:
    def __init__(self, device, max_batch=256, seed=1):
        self.device = device
        self.max_batch = max_batch
        h = C.c_void_p()
        check(lib().rv_cnn_create(device.handle, max_batch, seed, C.byref(h)))
        self.handle = h
        self.params_count = param_count()

    @property
    def stream(self):
        return lib().rv_cnn_stream(self.handle)

    def params(self):
        out = np.zeros(self.params_count, np.float32)
        check(lib().rv_cnn_get_params(self.handle, out.ctypes.data, out.size))
        return out

    def set_params(self, values):
        v = np.ascontiguousarray(values, np.float32)
        check(lib().rv_cnn_set_params(self.handle, v.ctypes.data, v.size))

    def grads(self):
        out = np.zeros(self.params_count, np.float32)
        check(lib().rv_cnn_get_grads(self.handle, out.ctypes.data, out.size))
        return out

    def forward(self, tiles_address, batch, logits_address=None, logits_len=0):
        check(lib().rv_cnn_forward(self.handle, C.c_void_p(tiles_address), batch,
                                   C.c_void_p(logits_address) if logits_address else None, logits_len))

    def backward(self, dlogits_address, n):
        check(lib().rv_cnn_backward(self.handle, C.c_void_p(dlogits_address), n))

    def train_step(self, tiles_address, labels_address, batch, config, want_loss=True):
        loss = C.c_float()
        check(lib().rv_cnn_train_step(self.handle, C.c_void_p(tiles_address), C.c_void_p(labels_address), batch,
                                      C.byref(config), C.byref(loss) if want_loss else None))
        return float(loss.value) if want_loss else None

    def status(self):
        t = C.c_uint32()
        check(lib().rv_cnn_status(self.handle, C.byref(t)))
        return t.value

    def close(self):
        if self.handle:
            lib().rv_cnn_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def proposal_config(bins, frame_seconds, average_seconds=1.0, threshold=0.0, hold_rows=1, pad_bins=64):
    c = abi.ProposalConfig()
    c.bins, c.hold_rows, c.frame_seconds, c.average_seconds = bins, hold_rows, frame_seconds, average_seconds
    c.threshold, c.pad_bins = threshold, pad_bins
    return c


class Proposer:
    def __init__(self, device, config):
        self.device = device
        self.config = config
        self.tiles_per_row = config.bins // TILE_BINS
        h = C.c_void_p()
        check(lib().rv_proposer_create(device.handle, C.byref(config), C.byref(h)))
        self.handle = h
        self._ranges = np.zeros((self.tiles_per_row * CELLS, 2), np.uint32)

    def tiles(self, frames_address, tiles_address):
        """One tile row from TILE_FRAMES frames at a device address."""
        check(lib().rv_proposer_tiles(self.handle, C.c_void_p(frames_address), TILE_FRAMES * self.config.bins,
                                      C.c_void_p(tiles_address), self.tiles_per_row * TILE_VALUES))

    def regions(self, logits_address):
        n = C.c_uint32()
        check(lib().rv_proposer_regions(self.handle, C.c_void_p(logits_address), self.tiles_per_row * CELLS,
                                        self._ranges.ctypes.data, self._ranges.shape[0], C.byref(n)))
        return self._ranges[:n.value]

    def reset(self):
        check(lib().rv_proposer_reset(self.handle))

    def close(self):
        if self.handle:
            lib().rv_proposer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def core_cells(first_bin, last_bin, pad_bins):
    """The cells a candidate's core covers: its bins less min(width / 4,
    pad_bins / 2) at either edge, so that padding the core's cells by
    pad_bins covers the whole candidate again. Returns [lo, hi) in cells."""
    width = last_bin - first_bin + 1
    margin = min(width // 4, pad_bins // 2)
    return (first_bin + margin) // CELL_BINS, (last_bin - margin) // CELL_BINS + 1


def row_of(instant, row_first_sample, row_samples):
    """The tile row whose frames complete a decision at `instant` (the end
    of the frame that made it)."""
    return (int(instant) - 1 - row_first_sample) // row_samples


# Candidates wider than this are not bursts or carriers but the floor
# estimate's own bias summed over the ladder's widest windows (they come in
# near 1024, 2048, 4096 and 8192 bins at a few dB over the threshold); they
# label no cells and the recall figures leave them out.
LOCALISED_BINS = 512


def localised(candidates, max_bins=LOCALISED_BINS):
    """Mask of the candidates no wider than max_bins."""
    return np.asarray([int(c["last_bin"]) - int(c["first_bin"]) + 1 <= max_bins for c in candidates], bool)


def row_labels(instants, candidates, row_first_sample, row_samples, rows, bins, pad_bins=64,
               max_bins=LOCALISED_BINS):
    """Labels [rows][bins / 8] (float32 0/1): a cell of tile row r is 1 when
    the core (core_cells) of a localised candidate of a decision made by one
    of the row's frames covers it."""
    labels = np.zeros((rows, bins // CELL_BINS), np.float32)
    for t, c in zip(instants, candidates):
        if int(c["last_bin"]) - int(c["first_bin"]) + 1 > max_bins:
            continue
        r = row_of(t, row_first_sample, row_samples)
        if 0 <= r < rows:
            lo, hi = core_cells(int(c["first_bin"]), int(c["last_bin"]), pad_bins)
            labels[r, lo:hi] = 1.0
    return labels


def candidate_scores(instants, candidates, logits, row_first_sample, row_samples, pad_bins=64,
                     max_bins=LOCALISED_BINS):
    """Per localised candidate, the highest logit over its core cells in its
    row (logits [rows][bins / 8]): the threshold below which it is proposed
    (-inf for the others)."""
    out = np.full(len(candidates), -np.inf)
    for i, (t, c) in enumerate(zip(instants, candidates)):
        if int(c["last_bin"]) - int(c["first_bin"]) + 1 > max_bins:
            continue
        r = row_of(t, row_first_sample, row_samples)
        if 0 <= r < logits.shape[0]:
            lo, hi = core_cells(int(c["first_bin"]), int(c["last_bin"]), pad_bins)
            out[i] = logits[r, lo:hi].max()
    return out


def match(reference, reference_instants, other, other_instants, min_overlap=0.5, max_bins=None):
    """Of the reference candidates (those no wider than max_bins, if given),
    how many have a candidate of `other` at the same decision instant
    covering at least `min_overlap` of their bins. Returns (matched, total)."""
    if max_bins is not None:
        keep = localised(reference, max_bins)
        reference = [c for c, k in zip(reference, keep) if k]
        reference_instants = [t for t, k in zip(reference_instants, keep) if k]
    by_instant = {}
    for t, c in zip(other_instants, other):
        by_instant.setdefault(int(t), []).append((int(c["first_bin"]), int(c["last_bin"])))
    matched = 0
    for t, c in zip(reference_instants, reference):
        lo, hi = int(c["first_bin"]), int(c["last_bin"])
        width = hi - lo + 1
        for a, b in by_instant.get(int(t), ()):
            if min(hi, b) - max(lo, a) + 1 >= min_overlap * width:
                matched += 1
                break
    return matched, len(reference)


def bursts_found(bursts, instants, candidates, bin_zero_hz, bin_width_hz, rate, tail_seconds=1.0, slack_bins=2):
    """Per scene burst (rv_scene_burst truth), whether a candidate of a
    decision made while it was on, or within tail_seconds after (the
    detector's average remembers it that long), overlaps its occupied band
    (extent_low_hz .. extent_high_hz, widened by slack_bins either side) and
    localises it: no wider than max(4 x the band, the band + 64 bins)."""
    inst = np.asarray(instants, np.int64)
    first = np.asarray([int(c["first_bin"]) for c in candidates], np.int64)
    last = np.asarray([int(c["last_bin"]) for c in candidates], np.int64)
    order = np.argsort(inst, kind="stable")
    inst, first, last = inst[order], first[order], last[order]
    tail = int(tail_seconds * rate)
    found = np.zeros(len(bursts), bool)
    for i, b in enumerate(bursts):
        lo_bin = int(np.floor((b.extent_low_hz - bin_zero_hz) / bin_width_hz)) - slack_bins
        hi_bin = int(np.ceil((b.extent_high_hz - bin_zero_hz) / bin_width_hz)) + slack_bins
        end = b.end if b.end < (1 << 62) else (1 << 62)
        a, z = np.searchsorted(inst, b.start, "left"), np.searchsorted(inst, end + tail, "right")
        if a < z:
            span = hi_bin - lo_bin + 1
            widest = max(4 * span, span + 64)
            found[i] = bool(np.any((first[a:z] <= hi_bin) & (last[a:z] >= lo_bin) &
                                   (last[a:z] - first[a:z] + 1 <= widest)))
    return found


class Spectrogram:
    """The detector's spectrum frames for a whole capture: the channelizer
    (rv_chain with no receivers) and one rv_spectrum (the engine's
    per-channel transform, M x N/2 bins in dB) per N channel blocks. Frame k
    is blocks [k N, (k + 1) N): source samples [k N D, (k + 1) N D)."""

    def __init__(self, device, grid=(64, 17, 32), rate=20_000_000, transform=2048, run_samples=1 << 24,
                 fmt=abi.FORMAT_CS16):
        from .chain import Chain
        self.device = device
        self.grid, self.rate, self.transform = grid, rate, transform
        self.run_samples = run_samples
        self.bins = grid[0] * transform // 2
        self.hop = transform * grid[2]
        self.chain = Chain(device, grid=grid, rate=rate, fmt=fmt, mode=abi.CHAIN_BATCHED, max_run_samples=run_samples,
                           keep_audio=False)
        ring, blocks = C.c_void_p(), C.c_uint32()
        check(lib().rv_chain_channel_ring(self.chain.handle, C.byref(ring), C.byref(blocks)))
        self.ring, self.ring_blocks = ring.value, blocks.value
        if self.ring_blocks < run_samples // grid[2] + transform:
            raise ValueError("channel ring of %d blocks too short for %d-sample runs" % (self.ring_blocks, run_samples))
        window = np.zeros(transform + transform // 2, np.float32)
        check(lib().rv_build_spectrum_window(transform, grid[1], 120.0, window.ctypes.data, window.size))
        tw = np.zeros((transform, 2), np.float32)
        check(lib().rv_build_twiddles(transform, tw.ctypes.data, transform))
        self.window, self.twiddles = device.array(window), device.array(tw)
        self.frames_done = 0
        self.samples_in = 0

    def frames(self, codes_address, count, out_address, capacity, bytes_per_sample=4):
        """Feeds `count` samples (device address) and writes every frame they
        complete to out_address (float32 [capacity][bins]); returns how many."""
        M, T, D = self.grid
        N = self.transform
        made = 0
        at = 0
        while at < count:
            m = min(self.run_samples, count - at)

            class _A:
                address = codes_address + at * bytes_per_sample
            self.chain.run(_A, m)
            self.chain.drain()
            at += m
            self.samples_in += m
            blocks = (self.samples_in - 1) // D + 1
            while (self.frames_done + 1) * N <= blocks:
                if made >= capacity:
                    raise ValueError("frame buffer of %d frames is full" % capacity)
                k = self.frames_done
                sp = abi.SpectrumParams(M, N, N.bit_length() - 1, self.ring_blocks, self.ring_blocks - 1,
                                        (k * N) & (self.ring_blocks - 1))
                check(lib().rv_spectrum(self.device.stream, C.byref(sp), C.c_void_p(self.ring), M * self.ring_blocks,
                                        self.twiddles.ptr, N, self.window.ptr, N + N // 2,
                                        C.c_void_p(out_address + made * self.bins * 4), self.bins))
                self.frames_done += 1
                made += 1
            self.device.synchronize()
        return made

    def close(self):
        self.chain.close()


class LearnedDetector:
    """The learned proposal in front of the wideband detector, one tile row
    (RV_TILE_FRAMES frames) at a time: tiles, the network's logits, the
    proposed bin ranges, then the detector consumes the row's frames with its
    decisions confirmed inside those ranges only. Every `full_every`-th tile
    row (0: never) the detector decides over the full band instead: the
    fallback that catches what the network missed.

    The tiles and the network run on a stream of their own, one row ahead:
    while the detector confirms row r on the context's stream (host work
    between small launches), the GPU already builds and classifies row r + 1."""

    def __init__(self, device, cnn, detector, proposer, full_every=0):
        self.device, self.cnn, self.detector, self.proposer = device, cnn, detector, proposer
        self.full_every = full_every
        self.rows = 0
        tiles = proposer.tiles_per_row
        self.tiles = device.buffer(tiles * TILE_VALUES * 2)
        self.logits = device.buffer(tiles * CELLS * 4)
        self.region_bins = 0
        s = C.c_void_p()
        check(lib().rv_stream_create(device.handle, C.byref(s)))
        self.stream = s.value
        check(lib().rv_cnn_set_stream(cnn.handle, C.c_void_p(self.stream)))
        check(lib().rv_proposer_set_stream(proposer.handle, C.c_void_p(self.stream)))

    def _classify(self, frames_address):
        p = self.proposer
        p.tiles(frames_address, self.tiles.address)
        self.cnn.forward(self.tiles.address, p.tiles_per_row, self.logits.address, p.tiles_per_row * CELLS)

    def _confirm(self, frames_address, start, hop, count, ranges):
        if self.full_every and self.rows % self.full_every == 0:
            self.detector.set_regions(None)
        else:
            self.detector.set_regions(ranges)
            self.region_bins += int((ranges[:, 1] - ranges[:, 0]).sum()) if len(ranges) else 0
        self.rows += 1
        return self.detector.consume_frames((frames_address, TILE_FRAMES), start, hop, count, device=True)

    def consume_row(self, frames_address, start, hop, count):
        """The row's frames at a device address, frame f covering source
        samples [start + f hop, + count). Returns the detector's decisions."""
        self._classify(frames_address)
        ranges = self.proposer.regions(self.logits.address)
        return self._confirm(frames_address, start, hop, count, ranges)

    def consume_rows(self, frames_address, rows, start, hop, count, frame_stride):
        """`rows` consecutive tile rows of frames (frame f at frames_address +
        f frame_stride bytes), the network one row ahead of the detector.
        Returns the detector's decisions."""
        made = 0
        row_bytes = TILE_FRAMES * frame_stride
        if rows:
            self._classify(frames_address)
        for r in range(rows):
            at = frames_address + r * row_bytes
            ranges = self.proposer.regions(self.logits.address).copy()  # waits for row r's logits
            if r + 1 < rows:
                self._classify(at + row_bytes)
            made += self._confirm(at, start + r * TILE_FRAMES * hop, hop, count, ranges)
        return made

    def close(self):
        check(lib().rv_cnn_set_stream(self.cnn.handle, None))
        check(lib().rv_proposer_set_stream(self.proposer.handle, None))
        check(lib().rv_stream_destroy(C.c_void_p(self.stream)))
        self.tiles.free()
        self.logits.free()
