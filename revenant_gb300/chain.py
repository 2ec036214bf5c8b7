"""Host mirror of the chain API (rv_chain_*): the engine-level entry point.

A ``Chain`` owns one rv_chain on a ``Device``: add receivers with
``add_receiver(center=..., bandwidth=..., demod=...)``, feed raw IQ with
``run(samples)`` (numpy uint8 / int16 on the host, or a device ``Buffer``),
and read each receiver's audio with ``audio(id)``. All the work happens in
librevenant_gb300.so.
"""
import ctypes as C

import numpy as np

from . import abi
from .library import check, lib


class Chain:
    def __init__(self, device, grid=(64, 17, 32), rate=20_000_000, fmt=abi.FORMAT_CS16, mode=abi.CHAIN_BATCHED,
                 max_run_samples=1 << 20, keep_audio=True, attenuation_db=120.0, profile=False, pipelined=False):
        self.device = device
        cfg = abi.ChainConfig()
        cfg.grid = abi.GridParams(*grid)
        cfg.rate = rate
        cfg.format = fmt
        cfg.mode = mode
        cfg.max_run_samples = max_run_samples
        cfg.keep_audio = 1 if keep_audio else 0
        cfg.attenuation_db = attenuation_db
        cfg.profile = 1 if profile else 0
        cfg.pipelined = 1 if pipelined else 0
        self.config = cfg
        self.bytes_per_sample = 4 if fmt == abi.FORMAT_CS16 else 2
        handle = C.c_void_p()
        check(lib().rv_chain_create(device.handle, C.byref(cfg), C.byref(handle)))
        self.handle = handle
        self.ids = []

    def add_receiver(self, request=None, **kw):
        req = request if request is not None else abi.request(**kw)
        rid = C.c_uint32()
        check(lib().rv_chain_add_receiver(self.handle, C.byref(req), C.byref(rid)))
        self.ids.append(rid.value)
        return rid.value

    def run(self, samples, count=None, host=False):
        """Feed samples: a host numpy array of raw bytes / int16 codes, or any
        object with an ``address`` (a Buffer): device memory, or host memory
        (pinned) when ``host`` is true; then ``count`` samples from there."""
        if hasattr(samples, "address"):
            check(lib().rv_chain_run(self.handle, C.c_void_p(samples.address), count, 0 if host else 1))
            return
        a = np.ascontiguousarray(samples)
        n = a.nbytes // self.bytes_per_sample
        check(lib().rv_chain_run(self.handle, a.ctypes.data_as(C.c_void_p), n, 0))

    def info(self, rid):
        info = abi.VrxPlanInfo()
        frames, first = C.c_uint64(), C.c_uint64()
        check(lib().rv_chain_receiver_info(self.handle, rid, C.byref(info), C.byref(frames), C.byref(first)))
        return info, frames.value, first.value

    def audio(self, rid):
        info, frames, _ = self.info(rid)
        cap = max(frames * info.demod.channels, 1)
        out = np.empty(cap, np.float32)
        n = C.c_uint64()
        check(lib().rv_chain_read_audio(self.handle, rid, out.ctypes.data_as(C.c_void_p), cap, C.byref(n)))
        return out[:n.value]

    def rings(self, rid):
        """(fine ring (n, 2) float32, detector ring float32 or None) copied
        from the device."""
        fine, det, mask = C.c_void_p(), C.c_void_p(), C.c_uint32()
        check(lib().rv_chain_receiver_rings(self.handle, rid, C.byref(fine), C.byref(det), C.byref(mask)))
        n = mask.value + 1
        f = np.empty((n, 2), np.float32)
        self.device.copy_to_host(f, fine.value)
        d = None
        if det.value:
            d = np.empty(n, np.float32)
            self.device.copy_to_host(d, det.value)
        return f, d

    def capture_graph(self):
        """Run the batched kernels from one captured CUDA graph from now on."""
        check(lib().rv_chain_capture_graph(self.handle))

    def autotune(self, run_samples):
        """Time the fine-tile shapes per receiver class on runs of
        `run_samples` and keep the fastest (before the first run); returns
        the report as a dict."""
        rep = abi.ChainTuneReport()
        check(lib().rv_chain_autotune(self.handle, int(run_samples), C.byref(rep)))
        return {k: getattr(rep, k) for k, _ in rep._fields_ if k != "reserved"}

    def set_front_end(self, dc=True, iq=True, lag=1):
        """Front-end DC / IQ-imbalance correction from the next run on."""
        check(lib().rv_chain_set_front_end(self.handle, 1 if dc else 0, 1 if iq else 0, lag))

    def set_impulse_excision(self, on=True, threshold_db=15.0, max_width_seconds=20e-6):
        """Span-wide impulse excision from the next run on (off by default)."""
        check(lib().rv_chain_set_impulse_excision(self.handle, 1 if on else 0, threshold_db, max_width_seconds))

    def excision_counters(self):
        """(samples excised, runs excised, runs spared, samples examined)."""
        out = (C.c_uint64 * 4)()
        check(lib().rv_chain_excision_counters(self.handle, out))
        return tuple(int(x) for x in out)

    def front_end_estimate(self):
        st = abi.FrontEnd()
        check(lib().rv_chain_front_end_estimate(self.handle, C.byref(st)))
        return st

    def set_spectrum(self, transform, detector=None):
        """One spectrum frame per run over the last `transform` channel blocks;
        an attached Detector consumes each frame on the device."""
        check(lib().rv_chain_set_spectrum(self.handle, transform, detector.handle if detector else None))

    def spectrum(self):
        """(frame dB float32 or None, start, count, sequence) of the latest frame."""
        bins, start, count, seq = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(lib().rv_chain_read_spectrum(self.handle, None, 0, C.byref(bins), C.byref(start), C.byref(count),
                                           C.byref(seq)))
        if bins.value == 0:
            return None, start.value, count.value, seq.value
        out = np.zeros(bins.value, np.float32)
        check(lib().rv_chain_read_spectrum(self.handle, out.ctypes.data, out.size, C.byref(bins), C.byref(start),
                                           C.byref(count), C.byref(seq)))
        return out, start.value, count.value, seq.value

    def drain(self):
        check(lib().rv_chain_drain(self.handle))

    def stats(self):
        s = abi.ChainStats()
        check(lib().rv_chain_get_stats(self.handle, C.byref(s)))
        return s

    def close(self):
        if self.handle:
            lib().rv_chain_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
