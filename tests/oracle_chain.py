"""The receive chain driven through the oracle, run by run.

Mirrors what the reference's Graph::on_block and DemodStage::record do per
source block (core/engine/graph.cpp:5118-5330, core/engine/vrx_stage.cpp:
1119-1430): convert the new samples into the ring, branch-filter and FFT the
new channel blocks, then for every receiver run the fine stage over the
outputs whose inputs now exist, the carrier loop if the mode has one, and the
demodulator over the audio frames whose fine history is complete. Tables
and block parameters come from the oracle's own planner restatement
(oracle/planner.c: or_place, or_plan_vrx, or_fine_block, ...), which
tests/test_oracle_planner.py pins to the reference's planner, so a chain
without front-end correction never calls the GPU library. Test
infrastructure only.
"""
import ctypes as C

import numpy as np

from bindings import cf32, oracle
from revenant_gb300 import abi
from revenant_gb300.library import lib


def _check(st):
    assert st == 0, lib().rv_last_error().decode()


def _ok(o, st):
    assert st == 0, o.error()


def highest_output_for(newest, fc, fd):
    bound = newest + 1
    whole, part = divmod(bound, fc)
    return whole * fd - 1 if part == 0 else whole * fd + (part * fd - 1) // fc


def lowest_output_for(needed, fc, fd):
    whole, part = divmod(needed, fc)
    return whole * fd + (part * fd + fc - 1) // fc


class OracleChain:
    def __init__(self, grid, rate, fmt, requests, ring_log2=20, chan_log2=17, fine_log2=17):
        self.ora = oracle()
        self.g = abi.GridParams(*grid)
        self.rate, self.fmt = rate, fmt
        M, T, D = grid
        o = self.ora.lib
        self.taps = np.zeros(M * T, np.float32)
        _ok(self.ora, o.or_design_prototype(C.byref(self.g), 120.0, self.taps.ctypes.data, self.taps.size))
        self.tw = np.zeros((M, 2), np.float32)
        _ok(self.ora, o.or_build_twiddles(M, self.tw.ctypes.data, M))
        self.nco = np.zeros((1 << 16, 2), np.float32)
        _ok(self.ora, o.or_build_nco_table(16, self.nco.ctypes.data, 1 << 16))
        self.ring = cf32(1 << ring_log2)
        self.ring_mask = (1 << ring_log2) - 1
        self.chan_blocks = 1 << chan_log2
        self.chan = cf32(M * self.chan_blocks)
        self.fine_mask = (1 << fine_log2) - 1
        self.samples_in = 0
        self.next_block = 0
        # front-end correction (Graph::record_front_end_correction,
        # core/engine/graph.cpp:1382-1436): off until set_front_end
        self.fe_dc = self.fe_iq = False
        self.fe_lag = 1
        self.fe_was_on = False
        self.fe = None  # the estimate, made when the correction is first turned on
        self.fe_pending = []  # (run index, count, chunk sums) not yet in the estimate
        self.run_index = 0
        self.rx = []
        for req in requests:
            pl = abi.VrxPlacement()
            _ok(self.ora, o.or_place(C.byref(self.g), rate, C.byref(req), C.byref(pl)))
            info = abi.VrxPlanInfo()
            _ok(self.ora, o.or_plan_vrx(C.byref(self.g), rate, C.byref(req), C.byref(pl), C.byref(info), None, 0, None, 0))
            taps = np.zeros((info.fine_tap_count, 2), np.float32)
            w = np.zeros(info.demod_weight_count, np.float32)
            _ok(self.ora, o.or_plan_vrx(C.byref(self.g), rate, C.byref(req), C.byref(pl), C.byref(info), taps.ctypes.data,
                                     taps.shape[0], w.ctypes.data, w.size))
            self.rx.append(dict(info=info, taps=taps, w=w, fine=cf32(self.fine_mask + 1), state=np.zeros(8, np.uint32),
                                started=False, reset=True, audio=[],
                                history=o.or_demod_fine_history(C.byref(info.demod))))

    def set_front_end(self, dc, iq, lag=1):
        self.fe_dc, self.fe_iq, self.fe_lag = bool(dc), bool(iq), lag

    def set_impulse_excision(self, on=True, threshold_db=15.0, max_width_seconds=20e-6, max_block=1 << 16):
        """The span-wide impulse excision (Graph::plan_impulse_excision and
        record_impulse_excision, core/engine/graph.cpp:1461-1525) with the
        oracle's cursor and passes, in place on the ring."""
        o = self.ora
        self.ex_on = bool(on)
        if not on:
            return
        self.ex_cfg = abi.ExcisionConfig()
        assert o.fn("design_excision")(self.rate, max_width_seconds, C.byref(self.ex_cfg)) == 0
        self.ex_rings = abi.ExcisionRings()
        assert o.fn("size_excision_rings")(C.byref(self.ex_cfg), max_block, 1, self.ring_mask,
                                           C.byref(self.ex_rings)) == 0, o.error()
        self.ex_cursor = abi.ExcisionCursor()
        thr = o.fn("excision_threshold")(threshold_db)
        assert o.lib.or_excision_cursor_init(C.byref(self.ex_cursor), C.byref(self.ex_cfg), self.ring_mask,
                                             C.byref(self.ex_rings), thr) == 0
        r = self.ex_rings
        self.ex_seg_power = np.zeros(r.seg_mask + 1, np.float32)
        self.ex_seg_level = np.zeros(r.seg_mask + 1, np.float32)
        self.ex_flags = np.zeros(r.flag_mask + 1, np.uint32)
        self.ex_removed = cf32(r.removed_mask + 1)
        self.ex_counters = np.zeros(4, np.uint32)
        self.ex_examined = 0

    def excise(self, start, count):
        """Plans this run and runs the passes; returns the channel limit."""
        o = self.ora
        plan = abi.ExcisionPlan()
        assert o.lib.or_excision_plan_block(C.byref(self.ex_cursor), start, count, C.byref(plan)) == 0
        d = lambda a: a.ctypes.data  # noqa: E731
        n = self.ring.shape[0]
        c = self.ex_cfg
        if plan.segment.count:
            assert o.fn("excise_segment")(C.byref(c), C.byref(plan.segment), d(self.ring), n, d(self.ex_seg_power),
                                          self.ex_seg_power.size) == 0, o.error()
        if plan.reference.count:
            assert o.fn("excise_reference")(C.byref(c), C.byref(plan.reference), d(self.ex_seg_power),
                                            d(self.ex_seg_level), self.ex_seg_power.size) == 0, o.error()
        if plan.flag.count:
            assert o.fn("excise_flag")(C.byref(c), C.byref(plan.flag), d(self.ring), n, d(self.ex_seg_level),
                                       self.ex_seg_level.size, d(self.ex_flags), self.ex_flags.size) == 0, o.error()
        if plan.apply.count:
            assert o.fn("excise_apply")(C.byref(c), C.byref(plan.apply), d(self.ring), n, d(self.ex_flags),
                                        self.ex_flags.size, d(self.ring), d(self.ex_removed),
                                        self.ex_removed.shape[0], d(self.ex_counters)) == 0, o.error()
        self.ex_examined += plan.apply.count
        return min(start + count, plan.cleaned_end)

    def front_end(self, destination, count):
        """Moments of this run's samples, the estimate updated with the runs
        at least `lag` before this one, then this run corrected in place."""
        o = self.ora
        on = self.fe_dc or self.fe_iq
        if on and not self.fe_was_on:
            if self.fe is None:
                self.fe = abi.FrontEnd()
                _check(lib().rv_front_end_init(C.byref(self.fe)))
            _check(lib().rv_front_end_reset(C.byref(self.fe)))
            self.fe_pending = []
        self.fe_was_on = on
        while self.fe_pending and self.fe_pending[0][0] <= self.run_index - self.fe_lag:
            _, n, sums = self.fe_pending.pop(0)
            assert o.lib.or_front_end_update(C.byref(self.fe), sums.ctypes.data, sums.size, n, self.rate) == 0
        if not on or count == 0:
            return
        chunks = (count + 63) // 64
        sums = np.zeros(chunks * 5, np.float32)
        mp = abi.IqMomentsParams(self.ring_mask, destination, count)
        assert o.fn("iq_moments")(C.byref(mp), self.ring.ctypes.data, self.ring.shape[0], sums.ctypes.data,
                                  sums.size) == 0, o.error()
        self.fe_pending.append((self.run_index, count, sums))
        if not self.fe.measured:
            return
        cp = abi.IqCorrectParams()
        assert o.lib.or_front_end_correction(C.byref(self.fe), int(self.fe_dc), int(self.fe_iq), C.byref(cp)) == 0
        cp.ring_mask, cp.offset, cp.count = self.ring_mask, destination, count
        n = self.ring.shape[0]
        assert o.fn("iq_correct")(C.byref(cp), self.ring.ctypes.data, n, self.ring.ctypes.data, n) == 0, o.error()

    def run(self, packed, count):
        M, D = self.g.channels, self.g.decimation
        o = self.ora
        cp = abi.ConvertParams(self.ring_mask, self.samples_in & 0xFFFFFFFF, 0, count)
        assert o.convert(self.fmt, cp, packed, self.ring) == 0, o.error()
        self.front_end(self.samples_in & self.ring_mask, count)
        self.run_index += 1
        first_block = self.next_block
        limit = self.samples_in + count
        if getattr(self, "ex_on", False):
            limit = self.excise(self.samples_in, count)
        self.samples_in += count
        if limit <= first_block * D:
            return
        last_block = (limit - 1) // D
        if last_block < first_block:
            return
        blocks = last_block - first_block + 1
        self.next_block = last_block + 1
        branch = cf32(blocks * M)
        bp = abi.PfbBranchParams(self.ring_mask, (first_block * D) & 0xFFFFFFFF, blocks)
        assert o.pfb_branch(self.g, bp, self.taps, self.ring, branch) == 0, o.error()
        fp = abi.PfbFftParams(M, D, int(np.log2(M)), first_block & 0xFFFFFFFF, blocks, self.chan_blocks,
                              self.chan_blocks - 1)
        assert o.pfb_fft(fp, branch, self.tw, self.chan) == 0, o.error()
        self.receivers(first_block, last_block)

    def receivers(self, first_block, last_block):
        """Advance every receiver over channel blocks [first_block, last_block]
        already in the channel ring (DemodStage::record)."""
        o = self.ora
        for r in self.rx:
            info = r["info"]
            fc, fd, dec = info.channel_rate, info.demod_rate, info.demod.decimation
            if not r["started"]:
                r["first"] = lowest_output_for(first_block + info.fine.taps - 1, fc, fd)
                r["next_out"] = r["first"]
                r["next_audio"] = (r["first"] + r["history"] + dec - 1) // dec
                r["started"] = True
            limit = highest_output_for(last_block, fc, fd)
            if limit + 1 > r["next_out"]:
                n_total = limit + 1 - r["next_out"]
                rem = fc % fd
                per = n_total if rem == 0 else max(1, (0xFFFFFFFF - fd) // rem)
                done = 0
                while done < n_total:
                    n = min(n_total - done, per)
                    fb = abi.VrxFineBlock()
                    _ok(o, o.lib.or_fine_block(C.byref(info), info.placement.channel * self.chan_blocks,
                                               self.chan_blocks - 1, self.fine_mask, r["next_out"] + done, n,
                                               C.byref(fb)))
                    assert o.vrx_fine(info.fine, fb.params, self.chan, r["taps"], self.nco, r["fine"]) == 0, o.error()
                    done += n
                if info.carrier.power:
                    cpar = abi.VrxCarrierParams()
                    _ok(o, o.lib.or_carrier_block(C.byref(info), self.fine_mask, r["next_out"], n_total,
                                                  1 if r["reset"] else 0, 0.0, C.byref(cpar)))
                    assert o.vrx_carrier(info.carrier, cpar, self.nco, r["fine"], r["state"]) == 0, o.error()
                    r["reset"] = False
                r["next_out"] += n_total
            if r["next_out"] > r["first"]:
                audio_limit = (r["next_out"] - 1) // dec
                if audio_limit + 1 > r["next_audio"]:
                    n = audio_limit + 1 - r["next_audio"]
                    db = abi.VrxDemodBlock()
                    _ok(o, o.lib.or_demod_block(C.byref(info), self.fine_mask, r["next_audio"], n, C.byref(db)))
                    out = np.zeros(n * info.demod.channels, np.float32)
                    assert o.vrx_demod(info.demod, db.params, r["fine"], r["w"], out) == 0, o.error()
                    r["audio"].append(out)
                    r["next_audio"] += n

    def audio(self, i):
        a = self.rx[i]["audio"]
        return np.concatenate(a) if a else np.zeros(0, np.float32)
