"""CPU-side checks of the C ABI library: it builds, loads, and exports every declared entry point."""
import ctypes
import os

import pytest

from edlib_gb300 import _abi, build


@pytest.fixture(scope="module")
def libpath():
    return build.build()


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    names = _abi.header_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(_abi.header_symbols()) == set(_abi._SIGS)


def test_loader_signatures(libpath):
    L = _abi.lib()
    assert os.path.samefile(L._name, libpath)
    assert L.edgpu_last_error(None) == b"null context"
