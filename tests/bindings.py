"""ctypes views of the three C libraries the tests compare.

- ``oracle()``  : oracle/_build/liboracle.so, the CPU restatement (or_*).
- ``reference()``: oracle/_ref/libreftwins.so, the reference's own twins
  compiled from its sources (ref_*); None where the sources are absent.
- the GPU library is bound in revenant_gb300 itself (rv_*).

All three share one calling convention, so a test can run the same case
through each and compare the bytes.
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from revenant_gb300 import abi  # noqa: E402  (struct definitions)

P = C.c_void_p
U32, U64, I32, I64, F32, F64 = C.c_uint32, C.c_uint64, C.c_int32, C.c_int64, C.c_float, C.c_double
ptr = C.POINTER


def _sig(lib, prefix):
    def f(name, res, *args):
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = list(args)
    f("last_error", C.c_char_p)
    for n in ("det_rsqrt", "det_sqrt", "det_recip", "det_log2"):
        f(n, F32, F32)
    f("det_atan2", F32, F32, F32)
    f("convert", I32, I32, ptr(abi.ConvertParams), P, U64, P, U64)
    f("pfb_branch", I32, ptr(abi.GridParams), ptr(abi.PfbBranchParams), P, U64, P, U64, P, U64)
    f("pfb_fft", I32, ptr(abi.PfbFftParams), P, U64, P, U64, P, U64)
    f("fft_radix2", I32, P, P, P, U32, U32)
    f("spectrum", I32, ptr(abi.SpectrumParams), P, U64, P, U64, P, U64, P, U64)
    f("spectrum_levels", I32, ptr(abi.SpectrumLevelsParams), P, U64, P)
    f("vrx_fine", I32, ptr(abi.VrxFineConfig), ptr(abi.VrxFineParams), P, U64, P, U64, P, U64, P, U64)
    f("vrx_demod", I32, ptr(abi.VrxDemodConfig), ptr(abi.VrxDemodParams), P, U64, P, U64, P, U64)
    f("vrx_carrier", I32, ptr(abi.VrxCarrierConfig), ptr(abi.VrxCarrierParams), P, U64, P, U64, P)
    f("iq_moments", I32, ptr(abi.IqMomentsParams), P, U64, P, U64)
    f("iq_correct", I32, ptr(abi.IqCorrectParams), P, U64, P, U64)
    f("comb_step", U32, F64, I64)
    f("comb_table", I32, P, U64)
    f("comb_project", I32, ptr(abi.CombParams), P, U64, P, U64, P, U64, P, U64)
    f("comb_subtract", I32, ptr(abi.CombParams), P, U64, P, U64, P, U64, P, U64, P, U64)
    f("design_blanker", I32, I64, ptr(abi.BlankerConfig))
    f("blanker_threshold", F32, F64)
    f("blank_detect", I32, ptr(abi.BlankerConfig), ptr(abi.BlankerParams), P, U64, P, U64)
    f("blank_apply", I32, ptr(abi.BlankerConfig), ptr(abi.BlankerParams), P, U64, P, U64, P, U64)
    f("noise_line", I32, ptr(abi.LineConfig), ptr(abi.LineParams), P, U64, P, U64)
    f("design_notch", I32, F64, F64, F64, I64, ptr(abi.NotchDesign))
    f("spectral_config_for", I32, I64, ptr(abi.SpectralConfig))
    f("design_spectral_tables", I32, ptr(abi.SpectralConfig), P, U64)
    f("design_spectral_params", I32, F64, ptr(abi.SpectralParams))
    f("noise_spectral", I32, ptr(abi.SpectralConfig), ptr(abi.SpectralParams), P, U64, P, U64, P, U64)
    f("design_excision", I32, I64, F64, ptr(abi.ExcisionConfig))
    f("excision_threshold", F32, F64)
    f("size_excision_rings", I32, ptr(abi.ExcisionConfig), U64, U32, U32, ptr(abi.ExcisionRings))
    f("excise_segment", I32, ptr(abi.ExcisionConfig), ptr(abi.ExcisionParams), P, U64, P, U64)
    f("excise_reference", I32, ptr(abi.ExcisionConfig), ptr(abi.ExcisionParams), P, P, U64)
    f("excise_flag", I32, ptr(abi.ExcisionConfig), ptr(abi.ExcisionParams), P, U64, P, U64, P, U64)
    f("excise_apply", I32, ptr(abi.ExcisionConfig), ptr(abi.ExcisionParams), P, U64, P, U64, P, P, U64, P)


_oracle = None
_reference = None


def oracle():
    global _oracle
    if _oracle is None:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import build as oracle_build  # oracle/build.py
        lib = C.CDLL(oracle_build.build())
        _sig(lib, "or_")
        lib.or_coarse_cs16.restype = I32
        lib.or_coarse_cs16.argtypes = [ptr(abi.GridParams), P, P, P, U64, U64, U32, U32, P, I32]
        lib.or_front_end_update.restype = I32
        lib.or_front_end_update.argtypes = [ptr(abi.FrontEnd), P, U64, U32, I64]
        lib.or_front_end_correction.restype = I32
        lib.or_front_end_correction.argtypes = [ptr(abi.FrontEnd), I32, I32, ptr(abi.IqCorrectParams)]
        lib.or_excision_cursor_init.restype = I32
        lib.or_excision_cursor_init.argtypes = [ptr(abi.ExcisionCursor), ptr(abi.ExcisionConfig), U32,
                                                ptr(abi.ExcisionRings), F32]
        lib.or_excision_plan_block.restype = I32
        lib.or_excision_plan_block.argtypes = [ptr(abi.ExcisionCursor), U64, U32, ptr(abi.ExcisionPlan)]
        lib.or_pfb_branch_wide.restype = I32
        lib.or_pfb_branch_wide.argtypes = [ptr(abi.GridParams), ptr(abi.PfbBranchParams), P, U64, P, U64, P, U64]
        lib.or_pfb_f64.restype = I32
        lib.or_pfb_f64.argtypes = [ptr(abi.GridParams), P, P, U32, U32, U32, U32, P, P]
        # the planner restatement (oracle/planner.c)
        for name, res, args in (
                ("design_prototype", I32, [ptr(abi.GridParams), F64, P, U64]),
                ("build_twiddles", I32, [U32, P, U64]),
                ("build_nco_table", I32, [U32, P, U64]),
                ("place", I32, [ptr(abi.GridParams), I64, ptr(abi.VrxRequest), ptr(abi.VrxPlacement)]),
                ("plan_vrx", I32, [ptr(abi.GridParams), I64, ptr(abi.VrxRequest), ptr(abi.VrxPlacement),
                                   ptr(abi.VrxPlanInfo), P, U64, P, U64]),
                ("fine_block", I32, [ptr(abi.VrxPlanInfo), U32, U32, U32, U64, U32, ptr(abi.VrxFineBlock)]),
                ("demod_fine_history", U32, [ptr(abi.VrxDemodConfig)]),
                ("demod_block", I32, [ptr(abi.VrxPlanInfo), U32, U64, U32, ptr(abi.VrxDemodBlock)]),
                ("carrier_block", I32, [ptr(abi.VrxPlanInfo), U32, U64, U32, I32, F32, ptr(abi.VrxCarrierParams)])):
            fn = getattr(lib, "or_" + name)
            fn.restype = res
            fn.argtypes = args
        _oracle = Lib(lib, "or_")
    return _oracle


def reference():
    """The reference's own twins, or None when they were not built here."""
    global _reference
    if _reference is None:
        path = os.path.join(ROOT, "oracle", "_ref", "libreftwins.so")
        if not os.path.exists(path):
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import build as oracle_build
            try:
                built = oracle_build.build_reference()
            except Exception:
                built = None
            if not built or not os.path.exists(path):
                return None
        lib = C.CDLL(path)
        _sig(lib, "ref_")
        lib.ref_design_prototype.restype = I32
        lib.ref_design_prototype.argtypes = [ptr(abi.GridParams), F64, P, U64, ptr(F64), ptr(U64)]
        lib.ref_build_twiddles.restype = I32
        lib.ref_build_twiddles.argtypes = [U32, P, U64]
        lib.ref_build_nco_table.restype = I32
        lib.ref_build_nco_table.argtypes = [U32, P, U64]
        lib.ref_build_spectrum_window.restype = I32
        lib.ref_build_spectrum_window.argtypes = [U32, U32, F64, P, U64]
        lib.ref_place.restype = I32
        lib.ref_place.argtypes = [ptr(abi.GridParams), I64, ptr(abi.VrxRequest), ptr(abi.VrxPlacement)]
        lib.ref_channel_count_for.restype = U32
        lib.ref_channel_count_for.argtypes = [I64, I64]
        lib.ref_plan_vrx.restype = I32
        lib.ref_plan_vrx.argtypes = [ptr(abi.GridParams), I64, ptr(abi.VrxRequest),
                                     ptr(abi.VrxPlacement), ptr(abi.VrxPlanInfo), P, U64, P, U64]
        lib.ref_fine_block.restype = I32
        lib.ref_fine_block.argtypes = [ptr(abi.GridParams), I64, ptr(abi.VrxRequest), U32, U32, U32,
                                       U64, U32, ptr(abi.VrxFineBlock)]
        lib.ref_demod_block.restype = I32
        lib.ref_demod_block.argtypes = [ptr(abi.GridParams), I64, ptr(abi.VrxRequest), U32, U64, U32,
                                        ptr(abi.VrxDemodBlock)]
        lib.ref_front_end_sequence.restype = I32
        lib.ref_front_end_sequence.argtypes = [P, U64, P, U32, I64, I32, I32, P, P]
        lib.ref_lwdsp_window.restype = I32
        lib.ref_lwdsp_window.argtypes = [U32, U32, P]
        lib.ref_display_max_decimation.restype = U32
        lib.ref_display_max_decimation.argtypes = []
        lib.ref_display_ladder.restype = I32
        lib.ref_display_ladder.argtypes = [I64, P, U32, ptr(U32)]
        lib.ref_display_decimation.restype = U32
        lib.ref_display_decimation.argtypes = [I64, I64]
        lib.ref_plan_vrx_display.restype = I32
        lib.ref_plan_vrx_display.argtypes = [ptr(abi.GridParams), I64, ptr(abi.VrxRequest), ptr(abi.VrxDisplayPlan),
                                             P, U64, U32, U32, U32, U64, U32, ptr(abi.VrxFineBlock)]
        lib.ref_excision_plans.restype = I32
        lib.ref_excision_plans.argtypes = [ptr(abi.ExcisionConfig), U32, ptr(abi.ExcisionRings), F32, P, P, U32, P]
        lib.ref_lwdsp_spectrum.restype = I32
        lib.ref_lwdsp_spectrum.argtypes = [U32, U32, F32, P, U64, P]
        _reference = Lib(lib, "ref_")
    return _reference


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Lib:
    """numpy-friendly wrappers; each returns (status, outputs...)."""

    def __init__(self, lib, prefix):
        self.lib = lib
        self.prefix = prefix

    def fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def error(self):
        return self.fn("last_error")().decode()

    def det(self, name, *args):
        return self.fn(name)(*args)

    def convert(self, fmt, params, packed, ring):
        st = self.fn("convert")(fmt, C.byref(params), _p(packed), packed.nbytes, _p(ring), ring.shape[0])
        return st

    def pfb_branch(self, grid, params, taps, ring, out):
        return self.fn("pfb_branch")(C.byref(grid), C.byref(params), _p(taps), taps.size,
                                     _p(ring), ring.shape[0], _p(out), out.shape[0])

    def pfb_fft(self, params, branch, tw, ring):
        return self.fn("pfb_fft")(C.byref(params), _p(branch), branch.shape[0], _p(tw), tw.shape[0],
                                  _p(ring), ring.shape[0])

    def fft_radix2(self, tw, x, out, size, batch):
        return self.fn("fft_radix2")(_p(tw), _p(x), _p(out), size, batch)

    def spectrum(self, params, ring, tw, window, frame):
        return self.fn("spectrum")(C.byref(params), _p(ring), ring.shape[0], _p(tw), tw.shape[0],
                                   _p(window), window.size, _p(frame), frame.size)

    def spectrum_levels(self, params, frame, levels):
        return self.fn("spectrum_levels")(C.byref(params), _p(frame), frame.size, _p(levels))

    def vrx_fine(self, config, params, chan, taps, nco, fine):
        return self.fn("vrx_fine")(C.byref(config), C.byref(params), _p(chan), chan.shape[0],
                                   _p(taps), taps.shape[0], _p(nco), nco.shape[0], _p(fine), fine.shape[0])

    def vrx_demod(self, config, params, fine, weights, audio):
        return self.fn("vrx_demod")(C.byref(config), C.byref(params), _p(fine), fine.shape[0],
                                    _p(weights), weights.size, _p(audio), audio.size)

    def vrx_carrier(self, config, params, nco, fine, state):
        return self.fn("vrx_carrier")(C.byref(config), C.byref(params), _p(nco), nco.shape[0],
                                      _p(fine), fine.shape[0], _p(state))


def cf32(n):
    """Zeroed complex-float buffer as an (n, 2) float32 array."""
    return np.zeros((n, 2), dtype=np.float32)


def same_bits(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))


_detref = None


def detector_reference():
    """The reference's own wideband detector (oracle/_ref/libdetref.so), or None."""
    global _detref
    if _detref is None:
        path = os.path.join(ROOT, "oracle", "_ref", "libdetref.so")
        if not os.path.exists(path):
            return None
        lib = C.CDLL(path)
        lib.refdet_last_error.restype = C.c_char_p
        lib.refdet_create.restype = I32
        lib.refdet_create.argtypes = [ptr(abi.DetectorConfig), ptr(P)]
        lib.refdet_destroy.restype = None
        lib.refdet_destroy.argtypes = [P]
        lib.refdet_consume.restype = I32
        lib.refdet_consume.argtypes = [P, P, U64, U64, ptr(I32)]
        lib.refdet_candidates.restype = I32
        lib.refdet_candidates.argtypes = [P, P, U32, ptr(U32)]
        lib.refdet_state.restype = I32
        lib.refdet_state.argtypes = [P, P, P, U64]
        lib.refdet_stats.restype = I32
        lib.refdet_stats.argtypes = [P, ptr(abi.DetectorStats)]
        lib.refdet_tracks.restype = I32
        lib.refdet_tracks.argtypes = [P, P, U32, ptr(U32)]
        _detref = lib
    return _detref


def _struct_array(rows, struct):
    dt = np.dtype([(name, np.int64 if t in (C.c_int64,) else np.uint64 if t is C.c_uint64 else
                    np.uint32 if t is C.c_uint32 else np.float64) for name, t in struct._fields_])
    out = np.zeros(len(rows), dt)
    for i, c in enumerate(rows):
        for name, _ in struct._fields_:
            out[i][name] = getattr(c, name)
    return out


def candidates_array(cands):
    """ctypes candidates -> numpy structured array (one row each)."""
    return _struct_array(cands, abi.DetectorCandidate)


def tracks_array(tracks):
    """ctypes tracks -> numpy structured array (one row each)."""
    return _struct_array(tracks, abi.DetectorTrack)


def candidates_from_array(arr):
    """numpy structured candidates -> list of abi.DetectorCandidate."""
    out = []
    for row in arr:
        c = abi.DetectorCandidate()
        for name, _ in abi.DetectorCandidate._fields_:
            setattr(c, name, row[name].item())
        out.append(c)
    return out
