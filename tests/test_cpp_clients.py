"""The C ABI compiles and links from plain C, and the C++ GPU storage compiles inside the reference's
own Hamiltonian / GreensFunction / ChiLoc templates (build checks, no GPU needed; the reference's
Storage base needs ARPACK symbols at link time, so that check stops at the object file)."""
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
def test_gpu_storage_compiles_in_reference_templates(lib, tmp_path):
    out = str(tmp_path / "reference_binding.o")
    r = subprocess.run(["g++", "-std=c++14", "-w", "-c", "-I", os.path.join(ROOT, "oracle", "refshim"), "-I",
                        REF_INCLUDE, "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "reference_binding.cpp"), "-o", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
