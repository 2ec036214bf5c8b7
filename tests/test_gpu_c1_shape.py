"""C1 end to end in the benchmark's named shape (tests/c1_shape.py): the
2^18-sample cu8 capture at 2.4 MS/s through convert, the M = 8 channelizer,
the 64-tap resampler to 240 kS/s with its NCO, the FM discriminator and the
decimation by 5 to 48 kHz, once with the oracle's kernels and once with the
GPU's plain kernels (rv_convert, rv_pfb_branch, rv_pfb_fft, rv_vrx_fine,
rv_vrx_demod) driven the same way (the oracle chain's DemodStage cursor
arithmetic). The channel ring, the fine ring and the audio must be equal bit
for bit, and the audio must carry the 1 kHz tone."""
import ctypes as C

import numpy as np
import pytest

import bench
import c1_shape
from oracle_chain import OracleChain
from revenant_gb300 import abi
from revenant_gb300.library import lib

pytestmark = pytest.mark.gpu

SAMPLES, BLOCK = 1 << 18, 1 << 14


class GpuKernels:
    """The oracle wrapper's kernel calls (numpy in, numpy out) made through
    the library's plain GPU kernels; planner calls go to the oracle."""

    def __init__(self, gpu, ora):
        self.gpu, self.ora = gpu, ora
        self.lib = ora.lib

    def error(self):
        return lib().rv_last_error()

    def fn(self, name):
        return self.ora.fn(name)

    def _call(self, status, outs):
        assert status == 0, lib().rv_last_error()
        self.gpu.synchronize()
        for host, dev in outs:
            host[...] = dev.download(host.dtype, host.shape)
        return 0

    def convert(self, fmt, params, packed, ring):
        d_in, d_ring = self.gpu.array(packed), self.gpu.array(ring)
        return self._call(lib().rv_convert(self.gpu.stream, fmt, C.byref(params), d_in.ptr, packed.nbytes, d_ring.ptr,
                                           ring.shape[0]), [(ring, d_ring)])

    def pfb_branch(self, grid, params, taps, ring, out):
        d_t, d_r, d_o = self.gpu.array(taps), self.gpu.array(ring), self.gpu.array(out)
        return self._call(lib().rv_pfb_branch(self.gpu.stream, C.byref(grid), C.byref(params), d_t.ptr, taps.size, d_r.ptr,
                                              ring.shape[0], d_o.ptr, out.shape[0]), [(out, d_o)])

    def pfb_fft(self, params, branch, tw, ring):
        d_b, d_t, d_r = self.gpu.array(branch), self.gpu.array(tw), self.gpu.array(ring)
        return self._call(lib().rv_pfb_fft(self.gpu.stream, C.byref(params), d_b.ptr, branch.shape[0], d_t.ptr,
                                           tw.shape[0], d_r.ptr, ring.shape[0]), [(ring, d_r)])

    def vrx_fine(self, config, params, chan, taps, nco, fine):
        d_c, d_t, d_n, d_f = (self.gpu.array(a) for a in (chan, taps, nco, fine))
        return self._call(lib().rv_vrx_fine(self.gpu.stream, C.byref(config), C.byref(params), d_c.ptr, chan.shape[0],
                                            d_t.ptr, taps.shape[0], d_n.ptr, nco.shape[0], d_f.ptr, fine.shape[0]),
                          [(fine, d_f)])

    def vrx_demod(self, config, params, fine, weights, audio):
        d_f, d_w, d_a = self.gpu.array(fine), self.gpu.array(weights), self.gpu.array(audio)
        return self._call(lib().rv_vrx_demod(self.gpu.stream, C.byref(config), C.byref(params), d_f.ptr, fine.shape[0],
                                             d_w.ptr, weights.size, d_a.ptr, audio.size), [(audio, d_a)])


def chain(kernels=None, gpu=None):
    req = abi.request(center=200_000, bandwidth=200_000, demod="wfm", stereo=False)
    ch = OracleChain(bench.C1_GRID, bench.C1_RATE, abi.FORMAT_CU8, [req], ring_log2=18, chan_log2=16, fine_log2=16)
    info = c1_shape.apply(ch.rx[0], ch.ora.lib.or_demod_fine_history)
    if kernels is not None:
        ch.ora = kernels(gpu, ch.ora)
    return ch, info


def test_c1_baseline_shape_matches_oracle(gpu):
    codes = bench.c1_capture(SAMPLES)
    want, info = chain()
    got, _ = chain(GpuKernels, gpu)
    assert info.demod_rate == 240_000 and info.fine.taps == 64 and info.demod.decimation == 5
    for at in range(0, SAMPLES, BLOCK):
        part = codes[2 * at:2 * (at + BLOCK)]
        want.run(part, BLOCK)
        got.run(part, BLOCK)
    assert np.array_equal(got.chan.view(np.uint32), want.chan.view(np.uint32))
    assert np.array_equal(got.rx[0]["fine"].view(np.uint32), want.rx[0]["fine"].view(np.uint32))
    a, b = got.audio(0), want.audio(0)
    assert a.size > 4000 and a.size == b.size
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    # the demodulated 1 kHz tone stands well above the rest of the audio band
    x = a[len(a) // 4:] - np.mean(a[len(a) // 4:])
    spec = np.abs(np.fft.rfft(x * np.hanning(x.size))) ** 2
    freqs = np.fft.rfftfreq(x.size, 1 / 48_000)
    tone = spec[np.abs(freqs - 1000) < 50].sum()
    rest = spec[(freqs > 100) & (np.abs(freqs - 1000) > 200) & (freqs < 15_000)].sum()
    assert tone > 100 * rest, (tone, rest)
