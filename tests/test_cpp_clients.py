"""The C ABI compiles and links from plain C, and the C++ GPU storage compiles and links inside the reference's
own Hamiltonian / GreensFunction / ChiLoc templates (no GPU needed; tests/test_gpu_clients.py runs the C
client on the GPU)."""
import os
import subprocess

import pytest

from edlib_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle.build import reference_root  # noqa: E402

REF_INCLUDE = os.path.join(reference_root(), "include")


@pytest.fixture(scope="module")
def lib():
    return build.build()


def test_c_client_compiles_and_links(lib, tmp_path):
    out = str(tmp_path / "abi_c_client")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "abi_c_client.c"), "-o", out, "-L", os.path.dirname(lib),
                        "-ledgpu", "-Wl,-rpath," + os.path.dirname(lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(not os.path.isdir(REF_INCLUDE), reason="reference headers not present")
def test_gpu_storage_links_inside_reference_templates(lib, tmp_path, golden_dir):
    """The binding a maintainer adds on the reference side: the reference's own Hamiltonian, GreensFunction and
    ChiLoc instantiated on the GPU storage, linked into an executable with the ARPACK stand-in (the reference's
    Storage base calls ARPACK), LAPACK from scipy's OpenBLAS and libedgpu.so.  Run on this machine it reaches
    the library and stops at the missing device with the reference's error behaviour (an exception, exit 1)."""
    from oracle.build import _openblas
    exe = str(tmp_path / "reference_binding")
    libdir, blas = _openblas()
    r = subprocess.run(["g++", "-std=c++14", "-w", "-I", os.path.join(ROOT, "oracle", "refshim"), "-I",
                        REF_INCLUDE, "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "reference_binding.cpp"),
                        os.path.join(ROOT, "oracle", "refshim", "arpack_standin.cpp"), "-o", exe,
                        "-L", os.path.dirname(lib), "-ledgpu", "-Wl,-rpath," + os.path.dirname(lib),
                        "-L", libdir, "-l:" + blas, "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe, os.path.join(golden_dir, "gf_chi_2x2.txt")], capture_output=True, text=True, timeout=120)
    if r.returncode == 0:  # a machine with a GPU runs it through
        return
    assert r.returncode == 1 and "edgpu_ctx_create" in r.stderr, (r.returncode, r.stdout[-2000:], r.stderr[-2000:])
