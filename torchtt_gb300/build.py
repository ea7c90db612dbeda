"""Builds ``libttgb300.so`` (the CUDA kernels and the C ABI of include/ttgb300.h) in-tree.

Every ``csrc/*.cu`` translation unit is compiled in parallel by ``nvcc`` for sm_103a only, then
linked into ``torchtt_gb300/libttgb300.so``. Objects are cached in ``torchtt_gb300/_build`` and
rebuilt when a source or header is newer. No torch headers are involved: the library depends on
the CUDA runtime alone.

Usage: ``python -m torchtt_gb300.build``
"""
import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libttgb300.so")
ROOT = os.path.dirname(HERE)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I" + os.path.join(ROOT, "include")]


def _nvcc():
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the GB300 library needs the CUDA toolkit")


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def build(verbose=False, jobs=None):
    """Compile and link; returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdr = max(_newest_header(), os.path.getmtime(os.path.abspath(__file__)))
    srcs = sources()
    objs = []
    todo = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr):
            todo.append((s, o))

    def compile_one(so):
        s, o = so
        cmd = [nvcc] + ARCH + FLAGS + ["-cudart", "shared", "-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (s, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return o

    if todo:
        jobs = jobs or min(len(todo), os.cpu_count() or 4)
        with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
            list(ex.map(compile_one, todo))
    newest_obj = max(os.path.getmtime(o) for o in objs)
    if todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest_obj:
        tmp = LIB + ".tmp"
        # the CUDA runtime is linked dynamically so that the process holds one runtime (torch's)
        cmd = [nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    if verbose:
        print("built", LIB, "(%d objects recompiled)" % len(todo))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
