"""Build the in-tree CUDA library edlib_gb300/_lib/libedgpu.so for sm_103a.

Each translation unit is compiled by nvcc in parallel (``-gencode arch=compute_103a,code=sm_103a``)
and linked into one shared library with the CUDA runtime linked statically, so the library has no
dependency beyond the driver.  Objects are rebuilt only when a source or header is newer.
"""
import concurrent.futures
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libedgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    newest_hdr = max(os.path.getmtime(h) for h in headers)
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(OUT_DIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), newest_hdr):
            jobs.append([nvcc()] + ARCH + FLAGS + list(extra) + ["-c", s, "-o", o])
    logs = []
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            logs = list(ex.map(_run, jobs))
    if jobs or not os.path.exists(LIB):
        logs.append(_run([nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs))
    if verbose:
        print("\n".join(l for l in logs if l.strip()))
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="-f" in sys.argv, verbose=True, extra=("-Xptxas", "-v") if "-v" in sys.argv else ()))
