"""The C ABI: the library loads (without a GPU), exports every entry point
include/revenant_gb300.h declares, and its structs have the reference's
layouts (core/dsp/*.h static_asserts on the push-constant blocks)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from revenant_gb300 import abi
from revenant_gb300.library import INCLUDE, SIGNATURES

HEADERS = [os.path.join(INCLUDE, n) for n in sorted(os.listdir(INCLUDE)) if n.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w\*\s]+?\b(rv_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(rv):
    names = declared_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(rv, n)]
    assert not missing, missing
    # and the Python mirror declares a signature for each
    assert not [n for n in names if n not in SIGNATURES], [n for n in names if n not in SIGNATURES]


def test_abi_version(rv):
    assert rv.rv_abi_version() == 1


def test_struct_sizes_match_reference_push_constants():
    # core/dsp/convert.h:141, pfb_branch_reference.h:53, vrx_reference.h:269/584/716
    assert C.sizeof(abi.ConvertParams) == 16
    assert C.sizeof(abi.PfbBranchParams) == 12
    assert C.sizeof(abi.VrxFineParams) == 60
    assert C.sizeof(abi.VrxDemodParams) == 16
    assert C.sizeof(abi.VrxCarrierParams) == 56
    assert C.sizeof(abi.PfbFftParams) == 28
    assert C.sizeof(abi.SpectrumParams) == 24
    assert C.sizeof(abi.SpectrumLevelsParams) == 12


def test_struct_sizes_match_c_header(tmp_path):
    """Compile the header with the host C compiler and compare every sizeof."""
    structs = {name: getattr(abi, cls) for name, cls in [
        ("rv_convert_params", "ConvertParams"), ("rv_grid_params", "GridParams"),
        ("rv_pfb_branch_params", "PfbBranchParams"), ("rv_pfb_fft_params", "PfbFftParams"),
        ("rv_spectrum_params", "SpectrumParams"), ("rv_spectrum_levels_params", "SpectrumLevelsParams"),
        ("rv_vrx_fine_config", "VrxFineConfig"), ("rv_vrx_fine_params", "VrxFineParams"),
        ("rv_vrx_demod_config", "VrxDemodConfig"), ("rv_vrx_demod_params", "VrxDemodParams"),
        ("rv_vrx_carrier_config", "VrxCarrierConfig"), ("rv_vrx_carrier_params", "VrxCarrierParams"),
        ("rv_vrx_request", "VrxRequest"), ("rv_vrx_placement", "VrxPlacement"),
        ("rv_vrx_plan_info", "VrxPlanInfo"), ("rv_vrx_fine_block", "VrxFineBlock"),
        ("rv_vrx_demod_block", "VrxDemodBlock"), ("rv_device_info", "DeviceInfo")]}
    for extra in getattr(abi, "EXTRA_STRUCTS", {}).items():
        structs[extra[0]] = extra[1]
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "revenant_gb300.h"\nint main(void){\n' +
                   "".join('printf("%%s %%zu\\n", "%s", sizeof(%s));\n' % (n, n) for n in structs) + "return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.check_call(["gcc", "-I" + INCLUDE, str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)]).decode().split("\n")
    for line in out:
        if line.strip():
            name, size = line.split()
            assert C.sizeof(structs[name]) == int(size), name


def test_launch_without_gpu_reports_error_not_crash(rv):
    # a context on a machine with no device reports RV_ERR_NO_DEVICE
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert rv.rv_context_create(0, C.byref(h)) == abi.RV_ERR_NO_DEVICE
    assert rv.rv_last_error()
