"""revenant_gb300 — GB300-native receive chain behind a C ABI.

The product is the shared library revenant_gb300/_build/librevenant_gb300.so
(CUDA kernels for sm_103a plus the C++ host planner and chain runner), whose
entry points are declared in include/revenant_gb300.h. This package only
builds and loads it; there is no Python or CPU implementation of any kernel,
and every call into the chain fails loudly if the library is missing.
"""
from . import abi  # noqa: F401
from .library import build, lib, load  # noqa: F401
