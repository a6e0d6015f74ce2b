"""Build recipe of the engine library ``kbw_gb300/libkbwg.so``.

Compiles every translation unit under csrc/ with nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and links one
shared library exporting the C ABI of include/kbwg.h.  No torch headers are
involved; the library depends on the CUDA runtime only.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libkbwg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(ROOT, "include", "kbwg.h")]


# Device headers compiled again at run time by NVRTC (csrc/jit.cpp): embedded
# in the library as string literals so that it needs no source tree.
JIT_HEADERS = ["common.cuh", "sweep.h", "ff.cuh", "ff2.cuh", "sweep_dev.cuh", "jit_dev.cuh", "adjoint_dev.cuh"]
JIT_INC = os.path.join(OBJ, "jit_sources.inc")


def write_jit_sources():
    """Write _build/jit_sources.inc (only when its content changes)."""
    delim = "KBWGJIT"
    names, bodies = [], []
    for h in JIT_HEADERS:
        with open(os.path.join(CSRC, h)) as f:
            text = f.read()
        if ")" + delim + '"' in text:
            raise RuntimeError("%s contains the raw-string delimiter" % h)
        names.append('"%s"' % h)
        bodies.append('R"%s(%s)%s"' % (delim, text, delim))
    out = ("// Generated by kbw_gb300/build.py from csrc/: device headers for NVRTC.\n"
           "static const char *const kJitHeaderNames[] = {%s};\n"
           "static const char *const kJitHeaderSources[] = {\n%s};\n"
           "static const int kJitHeaderCount = %d;\n") % (", ".join(names), ",\n".join(bodies), len(names))
    old = None
    if os.path.exists(JIT_INC):
        with open(JIT_INC) as f:
            old = f.read()
    if old != out:
        with open(JIT_INC, "w") as f:
            f.write(out)


def _compile(src, verbose):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    newest_dep = max(os.path.getmtime(p) for p in headers() + [src, __file__, JIT_INC])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj, ""
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", OBJ] + ARCH
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"] if verbose else []
    cmd += ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(verbose=False, force=False):
    """Compile (incrementally) and link libkbwg.so; return its path."""
    os.makedirs(OBJ, exist_ok=True)
    if force:
        for f in os.listdir(OBJ):
            os.remove(os.path.join(OBJ, f))
    write_jit_sources()
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc(), "-shared"] + ARCH + objs + ["-o", tmp, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="--force" in sys.argv))
