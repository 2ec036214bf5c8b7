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
    srcs = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "planner.c")]
    deps = srcs + [os.path.join(HERE, "oracle.h"), os.path.join(HERE, "..", "include", "revenant_gb300.h")]
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-Wno-unused-function", "-pthread"] + srcs + ["-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


def reference_root():
    """The reference's source tree: $REVENANT_REFERENCE, else a checkout named
    `reference` beside this repository; None when neither holds it."""
    root = os.environ.get("REVENANT_REFERENCE") or os.path.join(HERE, os.pardir, os.pardir, "reference")
    root = os.path.abspath(root)
    return root if os.path.isdir(os.path.join(root, "core", "dsp")) else None


def build_reference(ref_root=None):
    """Compile the reference's own twins when its sources are present."""
    ref_root = ref_root or reference_root()
    if ref_root is None:
        return None
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref"),
                           "REF=" + ref_root])
    return REF_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_reference())
