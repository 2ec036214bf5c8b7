"""Builds the oracle (test infrastructure) into oracle/_build/liboracle.so.

The oracle is the CPU restatement in oracle.c; it is compiled with the
reference's floating-point discipline (no contraction, no fast math). When the
reference sources are present, ``build_reference`` also compiles the
reference's own twins into oracle/_ref/libreftwins.so via oracle/ref/Makefile.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libreftwins.so")


def build(force=False):
    src = os.path.join(HERE, "oracle.c")
    deps = [src, os.path.join(HERE, "oracle.h"),
            os.path.join(HERE, "..", "include", "revenant_gb300.h")]
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-Wno-unused-function", "-pthread",
           src, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


def build_reference(ref_root="/root/reference"):
    """Compile the reference's own twins when its sources are present."""
    if not os.path.isdir(os.path.join(ref_root, "core", "dsp")):
        return None
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref"),
                           "REF=" + ref_root])
    return REF_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_reference())
