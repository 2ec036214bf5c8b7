"""Build and load librevenant_gb300.so (CUDA for sm_103a + C++ host code).

``build()`` compiles every translation unit under csrc/ with nvcc for
sm_103a only (``-gencode arch=compute_103a,code=sm_103a``), in parallel, into
an in-tree shared library. ``lib()`` loads it once and declares the C
signatures from include/revenant_gb300.h. Nothing here implements a kernel;
if the library cannot be loaded every entry point raises.
"""
import ctypes as C
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
SO = os.path.join(OUT, "librevenant_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "--fmad=false", "-ftz=true", "-prec-div=true",
              "-prec-sqrt=true", "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
             "-I" + INCLUDE, "-I" + CSRC]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _sources():
    cu, cpp = [], []
    for name in sorted(os.listdir(CSRC)):
        path = os.path.join(CSRC, name)
        if name.endswith(".cu"):
            cu.append(path)
        elif name.endswith(".cpp"):
            cpp.append(path)
    return cu, cpp


def _headers():
    hs = [os.path.join(INCLUDE, n) for n in os.listdir(INCLUDE)]
    hs += [os.path.join(CSRC, n) for n in os.listdir(CSRC) if n.endswith((".h", ".cuh"))]
    return hs


def build(force=False, verbose=False):
    """Compile csrc/ into _build/librevenant_gb300.so (sm_103a only)."""
    cu, cpp = _sources()
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    headers_mtime = max([os.path.getmtime(h) for h in _headers()] + [os.path.getmtime(__file__)])
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(OUT, "obj", os.path.basename(src) + ".o")
        if (not force and os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
                and os.path.getmtime(obj) >= headers_mtime):
            return obj
        if src.endswith(".cu"):
            cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj + ".tmp"]
        else:
            cmd = ["g++"] + CXX_FLAGS + ["-c", src, "-o", obj + ".tmp"]
        if verbose:
            print(" ".join(cmd))
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (src, res.stdout, res.stderr))
        os.replace(obj + ".tmp", obj)
        return obj

    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as pool:
        objs = list(pool.map(compile_one, cu + cpp))
    if force or not os.path.exists(SO) or any(os.path.getmtime(o) > os.path.getmtime(SO) for o in objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", SO + ".tmp"] + objs + ["-lcudart", "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed\n%s%s" % (res.stdout, res.stderr))
        os.replace(SO + ".tmp", SO)
    return SO


_lock = threading.Lock()
_lib = None


class LibraryError(RuntimeError):
    pass


def load(path=SO):
    """Load the shared library and declare its signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise LibraryError("librevenant_gb300.so is not built (%s); run "
                               "revenant_gb300.build() first" % path)
        lib = C.CDLL(path)
        _declare(lib)
        _lib = lib
        return lib


def lib():
    return load()


P = C.c_void_p
U32, U64, I32, I64, F32, F64 = C.c_uint32, C.c_uint64, C.c_int32, C.c_int64, C.c_float, C.c_double
ptr = C.POINTER

# name -> (restype, argtypes); the single list the ABI test walks.
SIGNATURES = {
    "rv_last_error": (C.c_char_p, []),
    "rv_abi_version": (I32, []),
    "rv_context_create": (I32, [I32, ptr(P)]),
    "rv_context_destroy": (I32, [P]),
    "rv_context_device_info": (I32, [P, ptr(abi.DeviceInfo)]),
    "rv_context_stream": (P, [P]),
    "rv_context_synchronize": (I32, [P]),
    "rv_buffer_create": (I32, [P, U64, I32, ptr(P)]),
    "rv_buffer_destroy": (I32, [P]),
    "rv_buffer_address": (P, [P]),
    "rv_buffer_size": (U64, [P]),
    "rv_buffer_upload": (I32, [P, U64, P, U64]),
    "rv_buffer_download": (I32, [P, U64, P, U64]),
    "rv_buffer_clear": (I32, [P]),
    "rv_copy": (I32, [P, P, P, U64]),
    "rv_convert": (I32, [P, I32, ptr(abi.ConvertParams), P, U64, P, U64]),
    "rv_pfb_branch": (I32, [P, ptr(abi.GridParams), ptr(abi.PfbBranchParams), P, U64, P, U64, P, U64]),
    "rv_pfb_fft": (I32, [P, ptr(abi.PfbFftParams), P, U64, P, U64, P, U64]),
    "rv_spectrum": (I32, [P, ptr(abi.SpectrumParams), P, U64, P, U64, P, U64, P, U64]),
    "rv_spectrum_levels": (I32, [P, ptr(abi.SpectrumLevelsParams), P, U64, P]),
    "rv_spectrum_average": (I32, [P, ptr(abi.SpectrumAverageParams), P, U64, P, U64, P, U64, P, U64, P, U64]),
    "rv_build_lwdsp_window": (I32, [U32, U32, P, ptr(F64)]),
    "rv_vrx_fine": (I32, [P, ptr(abi.VrxFineConfig), ptr(abi.VrxFineParams), P, U64, P, U64, P, U64, P, U64]),
    "rv_vrx_demod": (I32, [P, ptr(abi.VrxDemodConfig), ptr(abi.VrxDemodParams), P, U64, P, U64, P, U64]),
    "rv_vrx_carrier": (I32, [P, ptr(abi.VrxCarrierConfig), ptr(abi.VrxCarrierParams), P, U64, P, U64, P]),
    "rv_pfb_channelize_noalloc": (I32, [P, ptr(abi.GridParams), ptr(abi.PfbBranchParams), ptr(abi.PfbFftParams),
                                        P, U64, P, U64, P, U64, P, U64]),
    "rv_coarse_fused": (I32, [P, ptr(abi.GridParams), I32, ptr(abi.CoarseParams), P, U64, P, U64, P, U64, P, U64]),
    "rv_chain_create": (I32, [P, ptr(abi.ChainConfig), ptr(P)]),
    "rv_chain_destroy": (I32, [P]),
    "rv_chain_add_receiver": (I32, [P, ptr(abi.VrxRequest), ptr(U32)]),
    "rv_chain_run": (I32, [P, P, U64, I32]),
    "rv_chain_receiver_info": (I32, [P, U32, ptr(abi.VrxPlanInfo), ptr(U64), ptr(U64)]),
    "rv_chain_read_audio": (I32, [P, U32, P, U64, ptr(U64)]),
    "rv_chain_get_stats": (I32, [P, ptr(abi.ChainStats)]),
    "rv_chain_capture_graph": (I32, [P]),
    "rv_chain_autotune": (I32, [P, U32, ptr(abi.ChainTuneReport)]),
    "rv_chain_set_front_end": (I32, [P, I32, I32, U32]),
    "rv_chain_set_impulse_excision": (I32, [P, I32, F64, F64]),
    "rv_chain_excision_counters": (I32, [P, P]),
    "rv_chain_set_spectrum": (I32, [P, U32, P]),
    "rv_chain_read_spectrum": (I32, [P, P, U64, ptr(U64), ptr(U64), ptr(U64), ptr(U64)]),
    "rv_chain_front_end_estimate": (I32, [P, ptr(abi.FrontEnd)]),
    "rv_iq_moments": (I32, [P, ptr(abi.IqMomentsParams), P, U64, P, U64]),
    "rv_iq_correct": (I32, [P, ptr(abi.IqCorrectParams), P, U64, P, U64]),
    "rv_front_end_init": (I32, [ptr(abi.FrontEnd)]),
    "rv_front_end_reset": (I32, [ptr(abi.FrontEnd)]),
    "rv_front_end_update": (I32, [ptr(abi.FrontEnd), P, U64, U32, I64]),
    "rv_front_end_correction": (I32, [ptr(abi.FrontEnd), I32, I32, ptr(abi.IqCorrectParams)]),
    "rv_detector_create": (I32, [P, ptr(abi.DetectorConfig), ptr(P)]),
    "rv_detector_destroy": (I32, [P]),
    "rv_detector_consume": (I32, [P, P, U64, U64, I32, ptr(I32)]),
    "rv_detector_consume_frames": (I32, [P, P, U32, U64, U64, U64, I32, ptr(U32)]),
    "rv_detector_candidates": (I32, [P, P, U32, ptr(U32)]),
    "rv_detector_state": (I32, [P, P, P, U64]),
    "rv_detector_get_stats": (I32, [P, ptr(abi.DetectorStats)]),
    "rv_detector_tracks": (I32, [P, I32, P, U32, ptr(U32)]),
    "rv_design_prototype_wide": (I32, [ptr(abi.GridParams), F64, P, U64, ptr(F64), ptr(U64)]),
    "rv_pfb_branch_wide": (I32, [P, ptr(abi.GridParams), ptr(abi.PfbBranchParams), P, U64, P, U64, P, U64]),
    "rv_comb_step": (U32, [F64, I64]),
    "rv_comb_table": (I32, [P, U64]),
    "rv_comb_project": (I32, [P, ptr(abi.CombParams), P, U64, P, U64, P, U64, P, U64]),
    "rv_comb_subtract": (I32, [P, ptr(abi.CombParams), P, U64, P, U64, P, U64, P, U64, P, U64]),
    "rv_scene_noise_sigma": (F64, [F64]),
    "rv_scene_noise": (I32, [P, U64, F64, U64, U64, P, U64]),
    "rv_scene_plan": (I32, [ptr(abi.ScenePopulation), P, U32, ptr(U32)]),
    "rv_emitter_accumulate_audio": (I32, [P, ptr(abi.ToneEmitter), P, U64, U32, U64, U64, F64, P, U64]),
    "rv_emitter_accumulate": (I32, [P, ptr(abi.ToneEmitter), U64, U64, F64, P, U64]),
    "rv_scene_noise_draws": (I32, [P, U64, U64, U64, P, U64]),
    "rv_pfb_dft_tc": (I32, [P, ptr(abi.PfbFftParams), P, U64, P, U64, P, U64, I32]),
    "rv_pfb_dft_tc_status": (I32, [P, ptr(U32)]),
    "rv_pfb_dft_tc_stop_for_test": (I32, [P, I32]),
    "rv_capture_writer_open": (I32, [C.c_char_p, ptr(abi.CaptureConfig), C.c_char_p, ptr(P)]),
    "rv_capture_writer_write": (I32, [P, ptr(abi.CaptureBlock), P, U64]),
    "rv_capture_writer_set_gain": (I32, [P, I32, F64]),
    "rv_capture_writer_annotate": (I32, [P, U64, ptr(abi.CaptureAnnotation)]),
    "rv_capture_writer_set_clock": (I32, [P, I64]),
    "rv_capture_writer_get_stats": (I32, [P, ptr(abi.CaptureWriterStats)]),
    "rv_capture_writer_close": (I32, [P]),
    "rv_capture_list": (I32, [C.c_char_p, P, U32, ptr(U32)]),
    "rv_capture_read": (I32, [C.c_char_p, ptr(abi.CaptureSegment), U64, U64, P]),
    "rv_capture_recover": (I32, [C.c_char_p, P]),
    "rv_display_max_decimation": (U32, []),
    "rv_display_ladder": (I32, [I64, P, U32, ptr(U32)]),
    "rv_display_decimation": (U32, [I64, I64]),
    "rv_plan_vrx_display": (I32, [ptr(abi.VrxPlanInfo), ptr(abi.VrxDisplayPlan), P, U64]),
    "rv_display_block": (I32, [ptr(abi.VrxDisplayPlan), U32, U32, U32, U64, U32, ptr(abi.VrxFineBlock)]),
    "rv_design_blanker": (I32, [I64, ptr(abi.BlankerConfig)]),
    "rv_blanker_threshold": (F32, [F64]),
    "rv_blank_detect": (I32, [P, ptr(abi.BlankerConfig), ptr(abi.BlankerParams), P, U64, P, U64]),
    "rv_blank_apply": (I32, [P, ptr(abi.BlankerConfig), ptr(abi.BlankerParams), P, U64, P, U64, P, U64]),
    "rv_design_notch": (I32, [F64, F64, F64, I64, ptr(abi.NotchDesign)]),
    "rv_line_state_size": (U64, [ptr(abi.LineConfig)]),
    "rv_noise_line": (I32, [P, ptr(abi.LineConfig), ptr(abi.LineParams), P, U64, P, U64]),
    "rv_spectral_config_for": (I32, [I64, ptr(abi.SpectralConfig)]),
    "rv_design_spectral_tables": (I32, [ptr(abi.SpectralConfig), P, U64]),
    "rv_design_spectral_params": (I32, [F64, ptr(abi.SpectralParams)]),
    "rv_spectral_state_size": (U64, [ptr(abi.SpectralConfig)]),
    "rv_noise_spectral": (I32, [P, ptr(abi.SpectralConfig), ptr(abi.SpectralParams), P, U64, P, U64, P, U64]),
    "rv_design_excision": (I32, [I64, F64, ptr(abi.ExcisionConfig)]),
    "rv_excision_threshold": (F32, [F64]),
    "rv_size_excision_rings": (I32, [ptr(abi.ExcisionConfig), U64, U32, U32, ptr(abi.ExcisionRings)]),
    "rv_excision_cursor_init": (I32, [ptr(abi.ExcisionCursor), ptr(abi.ExcisionConfig), U32,
                                      ptr(abi.ExcisionRings), F32]),
    "rv_excision_plan_block": (I32, [ptr(abi.ExcisionCursor), U64, U32, ptr(abi.ExcisionPlan)]),
    "rv_excise_segment": (I32, [P, ptr(abi.ExcisionConfig), ptr(abi.ExcisionParams), P, U64, P, U64]),
    "rv_excise_reference": (I32, [P, ptr(abi.ExcisionConfig), ptr(abi.ExcisionParams), P, P, U64]),
    "rv_excise_flag": (I32, [P, ptr(abi.ExcisionConfig), ptr(abi.ExcisionParams), P, U64, P, U64, P, U64]),
    "rv_excise_apply": (I32, [P, ptr(abi.ExcisionConfig), ptr(abi.ExcisionParams), P, U64, P, U64, P, P, U64, P]),
    "rv_excise_block": (I32, [P, ptr(abi.ExcisionConfig), ptr(abi.ExcisionPlan), P, U64, P, P, U64, P, U64, P, U64,
                              P]),
    "rv_tracker_create": (I32, [ptr(abi.DetectorConfig), ptr(P)]),
    "rv_tracker_destroy": (I32, [P]),
    "rv_tracker_update": (I32, [P, U64, F64, P, U32]),
    "rv_tracker_level_bins": (I32, [P, U32, P, U32, ptr(U32)]),
    "rv_tracker_fold_levels": (I32, [P, U32, P, U32, U32]),
    "rv_tracker_tracks": (I32, [P, I32, P, U32, ptr(U32)]),
    "rv_tracker_get_stats": (I32, [P, ptr(abi.DetectorStats)]),
    "rv_chain_drain": (I32, [P]),
    "rv_chain_channel_ring": (I32, [P, ptr(P), ptr(U32)]),
    "rv_chain_receiver_rings": (I32, [P, U32, ptr(P), ptr(P), ptr(U32)]),
    "rv_validate_grid": (I32, [ptr(abi.GridParams)]),
    "rv_design_prototype": (I32, [ptr(abi.GridParams), F64, P, U64, ptr(F64), ptr(U64)]),
    "rv_build_twiddles": (I32, [U32, P, U64]),
    "rv_build_fft_twiddles": (I32, [U32, P, U64]),
    "rv_build_nco_table": (I32, [U32, P, U64]),
    "rv_build_spectrum_window": (I32, [U32, U32, F64, P, U64]),
    "rv_place": (I32, [ptr(abi.GridParams), I64, ptr(abi.VrxRequest), ptr(abi.VrxPlacement)]),
    "rv_channel_count_for": (U32, [I64, I64]),
    "rv_plan_vrx": (I32, [ptr(abi.GridParams), I64, ptr(abi.VrxRequest), ptr(abi.VrxPlacement),
                          ptr(abi.VrxPlanInfo), P, U64, P, U64]),
    "rv_fine_block": (I32, [ptr(abi.VrxPlanInfo), U32, U32, U32, U64, U32, ptr(abi.VrxFineBlock)]),
    "rv_demod_block": (I32, [ptr(abi.VrxPlanInfo), U32, U64, U32, ptr(abi.VrxDemodBlock)]),
    "rv_carrier_block": (I32, [ptr(abi.VrxPlanInfo), U32, U64, U32, I32, F32, ptr(abi.VrxCarrierParams)]),
    "rv_demod_fine_history": (U32, [ptr(abi.VrxDemodConfig)]),
    "rv_stream_create": (I32, [P, ptr(P)]),
    "rv_stream_destroy": (I32, [P]),
    "rv_stream_synchronize": (I32, [P]),
    "rv_cnn_set_stream": (I32, [P, P]),
    "rv_proposer_set_stream": (I32, [P, P]),
    "rv_cnn_param_count": (U64, []),
    "rv_cnn_create": (I32, [P, U32, U64, ptr(P)]),
    "rv_cnn_destroy": (I32, [P]),
    "rv_cnn_set_params": (I32, [P, P, U64]),
    "rv_cnn_get_params": (I32, [P, P, U64]),
    "rv_cnn_get_grads": (I32, [P, P, U64]),
    "rv_cnn_stream": (P, [P]),
    "rv_cnn_forward": (I32, [P, P, U32, P, U64]),
    "rv_cnn_backward": (I32, [P, P, U64]),
    "rv_cnn_train_step": (I32, [P, P, P, U32, ptr(abi.CnnTrainConfig), ptr(F32)]),
    "rv_cnn_status": (I32, [P, ptr(U32)]),
    "rv_gemm_bf16": (I32, [P, P, P, U32, U32, U32, P, P]),
    "rv_proposer_create": (I32, [P, ptr(abi.ProposalConfig), ptr(P)]),
    "rv_proposer_destroy": (I32, [P]),
    "rv_proposer_tiles": (I32, [P, P, U64, P, U64]),
    "rv_proposer_regions": (I32, [P, P, U64, P, U32, ptr(U32)]),
    "rv_proposer_reset": (I32, [P]),
    "rv_detector_set_regions": (I32, [P, P, U32]),
    "rv_detector_log_candidates": (I32, [P, I32]),
    "rv_detector_read_log": (I32, [P, P, P, U32, ptr(U32)]),
}


def _declare(lib):
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def check(status):
    """Raise with rv_last_error() when a call returned a negative status."""
    if status != abi.RV_OK:
        raise LibraryError("revenant_gb300 error %d: %s" % (status, lib().rv_last_error().decode()))
    return status
