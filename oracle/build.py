"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle.c into ``oracle/liboracle.so`` with floating-point contraction
disabled, so products and sums round exactly as the reference's Rust code does
on both x86_64 and aarch64.  OpenMP is used when the compiler supports it.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle.c")]
DEPS = SOURCES + [os.path.join(HERE, "oracle.h"), os.path.join(HERE, "oracle_body.inc")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in DEPS)


def build(force=False, verbose=False):
    """Compile liboracle.so if missing or older than its sources; return its path."""
    if not force and not _stale():
        return LIB
    base = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
            "-fno-fast-math", "-Wall", "-Wno-unused-function"]
    tmp = LIB + ".tmp%d" % os.getpid()
    for extra in (["-fopenmp"], []):
        cmd = base + extra + SOURCES + ["-o", tmp, "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stderr)
        if r.returncode == 0:
            os.replace(tmp, LIB)
            return LIB
    raise RuntimeError("oracle build failed:\n" + r.stderr)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
