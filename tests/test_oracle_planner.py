"""The oracle's planner restatement (oracle/planner.c) against the
reference's own planner compiled from its sources, and against the GPU
library's planner: every table bit for bit, every integer of placement, plan
and block parameters equal. This is what lets the oracle chain, and the
benchmark's reference arm, plan receivers without the GPU library. CPU
only; the reference comparisons skip where the reference sources are absent.
"""
import ctypes as C

import numpy as np
import pytest

from bindings import same_bits
from revenant_gb300 import abi
from test_planner import GRIDS, SCENARIOS, _requests


def _plan(o, g, rate, req):
    pl = abi.VrxPlacement()
    if o.place(C.byref(g), rate, C.byref(req), C.byref(pl)) != 0:
        return None
    info = abi.VrxPlanInfo()
    if o.plan_vrx(C.byref(g), rate, C.byref(req), C.byref(pl), C.byref(info), None, 0, None, 0) != 0:
        return pl, None, None, None
    taps = np.zeros((info.fine_tap_count, 2), np.float32)
    w = np.zeros(info.demod_weight_count, np.float32)
    assert o.plan_vrx(C.byref(g), rate, C.byref(req), C.byref(pl), C.byref(info), taps.ctypes.data, taps.shape[0],
                      w.ctypes.data, w.size) == 0
    return pl, info, taps, w


@pytest.mark.parametrize("M,T,D", [g for g in GRIDS if g[0] <= 2048])
def test_prototype_matches(ora, rv, M, T, D):
    g = abi.GridParams(M, T, D)
    a = np.zeros(M * T, np.float32)
    b = np.zeros(M * T, np.float32)
    assert ora.lib.or_design_prototype(C.byref(g), 120.0, a.ctypes.data, a.size) == 0
    assert rv.rv_design_prototype(C.byref(g), 120.0, b.ctypes.data, b.size, None, None) == 0
    assert same_bits(a, b)


@pytest.mark.parametrize("M", [2, 8, 64, 1024, 2048])
def test_twiddles_and_nco_match(ora, rv, M):
    a = np.zeros((M, 2), np.float32)
    b = np.zeros((M, 2), np.float32)
    assert ora.lib.or_build_twiddles(M, a.ctypes.data, M) == 0
    assert rv.rv_build_twiddles(M, b.ctypes.data, M) == 0
    assert same_bits(a, b)
    n = 1 << 16
    a = np.zeros((n, 2), np.float32)
    b = np.zeros((n, 2), np.float32)
    assert ora.lib.or_build_nco_table(16, a.ctypes.data, n) == 0
    assert rv.rv_build_nco_table(16, b.ctypes.data, n) == 0
    assert same_bits(a, b)


def _compare(ora, other_plan, other_fine_block, other_demod_block, grid, rate):
    g = abi.GridParams(*grid)
    compared = 0
    for kw in _requests(rate):
        req = abi.request(**kw)
        mine = _plan(_Or(ora), g, rate, req)
        theirs = other_plan(g, rate, req)
        assert (mine is None) == (theirs is None), kw
        if mine is None:
            continue
        assert mine[0].as_dict() == theirs[0].as_dict(), kw
        assert (mine[1] is None) == (theirs[1] is None), kw
        if mine[1] is None:
            continue
        da, db = mine[1].as_dict(), theirs[1].as_dict()
        assert da == db, (kw, {k: (da[k], db[k]) for k in da if da[k] != db[k]})
        assert same_bits(mine[2], theirs[2]), kw
        assert same_bits(mine[3], theirs[3]), kw
        for first in (0, 3 * 3600 * mine[1].demod_rate + 17):
            fa = abi.VrxFineBlock()
            assert ora.lib.or_fine_block(C.byref(mine[1]), 4096, 65535, 8191, first, 1000, C.byref(fa)) == 0
            fb = other_fine_block(g, rate, req, theirs[1], first)
            assert bytes(fa) == bytes(fb), kw
        da_ = abi.VrxDemodBlock()
        assert ora.lib.or_demod_block(C.byref(mine[1]), (1 << 16) - 1, 12345, 100, C.byref(da_)) == 0
        assert bytes(da_) == bytes(other_demod_block(g, rate, req, theirs[1])), kw
        compared += 1
    assert compared > 20


class _Or:
    def __init__(self, ora):
        self.ora = ora

    def place(self, *a):
        return self.ora.lib.or_place(*a)

    def plan_vrx(self, *a):
        return self.ora.lib.or_plan_vrx(*a)


class _Named:
    def __init__(self, place, plan_vrx):
        self.place, self.plan_vrx = place, plan_vrx


@pytest.mark.parametrize("grid,rate", SCENARIOS)
def test_plans_match_the_gpu_librarys_planner(ora, rv, grid, rate):
    lib = _Named(rv.rv_place, rv.rv_plan_vrx)

    def fine_block(g, rate_, req, info, first):
        b = abi.VrxFineBlock()
        assert rv.rv_fine_block(C.byref(info), 4096, 65535, 8191, first, 1000, C.byref(b)) == 0
        return b

    def demod_block(g, rate_, req, info):
        b = abi.VrxDemodBlock()
        assert rv.rv_demod_block(C.byref(info), (1 << 16) - 1, 12345, 100, C.byref(b)) == 0
        return b

    _compare(ora, lambda g, r, q: _plan(lib, g, r, q), fine_block, demod_block, grid, rate)


@pytest.mark.parametrize("grid,rate", SCENARIOS)
def test_plans_match_the_references_planner(ora, ref, grid, rate):
    lib = _Named(ref.lib.ref_place, ref.lib.ref_plan_vrx)

    def fine_block(g, rate_, req, info, first):
        b = abi.VrxFineBlock()
        assert ref.lib.ref_fine_block(C.byref(g), rate_, C.byref(req), 4096, 65535, 8191, first, 1000, C.byref(b)) == 0
        return b

    def demod_block(g, rate_, req, info):
        b = abi.VrxDemodBlock()
        assert ref.lib.ref_demod_block(C.byref(g), rate_, C.byref(req), (1 << 16) - 1, 12345, 100, C.byref(b)) == 0
        return b

    _compare(ora, lambda g, r, q: _plan(lib, g, r, q), fine_block, demod_block, grid, rate)
