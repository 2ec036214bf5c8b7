"""Writes tests/golden/scene_noise.npz from the reference's own scene
synthesiser.

Renders noise-only scenes with siggen::Scene (core/dsp/synth/wideband.cpp,
compiled from the reference sources into oracle/_ref/libsynref.so by
oracle/ref/Makefile) over ranges that start mid-block, cross noise-block
boundaries and sit far into the stream, so that machines without the
reference sources can check rv_scene_noise against it.

    python tests/golden/make_scene_noise.py
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libsynref.so")

# (seed, rate, noise dBFS, start, count)
CASES = [(1, 20_000_000, -60.0, 3000, 2000), (0xDEADBEEF, 2_400_000, -40.0, 4095, 3000),
         (5, 61_440_000, -75.5, (1 << 30) - 1000, 2000), (123456789, 20_000_000, 0.0, 77_777, 1500)]


def reference():
    lib = C.CDLL(LIB, mode=os.RTLD_LAZY)  # its emitter code paths are never called
    lib.refsyn_noise.argtypes = [C.c_uint64, C.c_int64, C.c_double, C.c_uint64, C.c_uint64, C.c_void_p]
    lib.refsyn_mt64.argtypes = [C.c_uint64, C.c_uint64, C.c_void_p]
    return lib


def main():
    lib = reference()
    out = {}
    for i, (seed, rate, dbfs, start, count) in enumerate(CASES):
        buf = np.zeros((count, 2), np.float32)
        assert lib.refsyn_noise(seed, rate, dbfs, start, count, buf.ctypes.data) == 0
        out["case%d" % i] = buf
        out["params%d" % i] = np.array([seed, rate, start, count], np.uint64)
        out["dbfs%d" % i] = np.array([dbfs])
    np.savez_compressed(os.path.join(HERE, "scene_noise.npz"), **out)


if __name__ == "__main__":
    main()
