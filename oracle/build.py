"""Build recipes for the oracle (test infrastructure only).

* ``build_port()`` compiles the CPU restatement ``oracle/edoracle.cpp`` into
  ``oracle/_build/libedoracle.so`` (plain g++, OpenMP, no external libraries).  It builds on
  x86-64 and aarch64 alike.
* ``build_ref()`` compiles the UNMODIFIED reference headers, where they lie in the read-only
  reference checkout, against the stand-in headers in ``oracle/refshim`` into the harness
  binary ``oracle/_ref/edlib_ref``.  It links LAPACK ``dsyev`` from scipy's bundled OpenBLAS
  for the ARPACK stand-in.  Only possible where the reference tree exists.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# where the read-only reference checkout lies; EDLIB_REFERENCE_ROOT points elsewhere
REF_ROOT = os.environ.get("EDLIB_REFERENCE_ROOT", "/root/reference")


def reference_root():
    """The reference checkout's root directory (it may not exist on this machine)."""
    return REF_ROOT


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def port_lib_path():
    return os.path.join(HERE, "_build", "libedoracle.so")


def build_port(force=False):
    out = port_lib_path()
    src = os.path.join(HERE, "edoracle.cpp")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    _run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-Wall", "-Wno-unused-variable",
          src, "-o", out])
    return out


def _openblas():
    import scipy  # noqa: F401  (locate the bundled OpenBLAS next to scipy)
    libdir = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cands = glob.glob(os.path.join(libdir, "libscipy_openblas*.so"))
    if not cands:
        raise RuntimeError("scipy's bundled OpenBLAS not found in %s" % libdir)
    return libdir, os.path.basename(cands[0])


def ref_bin_path():
    return os.path.join(HERE, "_ref", "edlib_ref")


def build_ref(force=False):
    """Compile the reference harness; returns its path, or None where the reference is absent."""
    inc = os.path.join(REF_ROOT, "include")
    if not os.path.isdir(inc):
        return None
    out = ref_bin_path()
    shim = os.path.join(HERE, "refshim")
    srcs = [os.path.join(shim, "ref_harness.cpp"), os.path.join(shim, "arpack_standin.cpp")]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    libdir, lib = _openblas()
    _run(["g++", "-O2", "-std=c++14", "-fopenmp", "-w", "-I", shim, "-I", inc] + srcs +
         ["-L", libdir, "-l:" + lib, "-Wl,-rpath," + libdir, "-o", out])
    return out


if __name__ == "__main__":
    print(build_port(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
