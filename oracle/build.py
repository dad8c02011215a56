"""Build the CPU restatement (oracle/restate.c) into oracle/lib/liborc.so.

Test infrastructure: used by tests/, the smoke check and bench.py's CPU
baseline leg.  Compiled with -ffp-contract=off so no FMA contraction changes a
cell's arithmetic on either x86-64 or aarch64.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "lib", "liborc.so")


def build(force=False):
    src = os.path.join(HERE, "restate.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
                           src, "-o", LIB + ".tmp", "-lm"])
    os.replace(LIB + ".tmp", LIB)
    return LIB


def reference_source():
    """The reference's dvm_sys source tree: $DVMH_REF_SRC, else a checkout named
    reference/ beside this repository; None where neither exists (the GPU machine)."""
    env = os.environ.get("DVMH_REF_SRC")
    if env:
        return env if os.path.isdir(env) else None
    sibling = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference", "dvm_sys")
    return sibling if os.path.isdir(sibling) else None


def build_reference():
    """Build the reference runtime from its sources (only where they exist)."""
    ref = reference_source()
    if ref is None:
        return None
    root = os.path.dirname(HERE)
    subprocess.check_call(["make", "-s", "-f", "oracle/ref.mk", "-j8", "REF=" + ref], cwd=root)
    return os.path.join(HERE, "_ref", "ref_driver")


if __name__ == "__main__":
    print(build(force=True))
