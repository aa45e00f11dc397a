"""edgpu_vv_noalloc -- the dot product for callers that cannot allocate device memory -- against the
allocating Storage::vv entry point (edgpu_vv) and against a correctly rounded host sum (math.fsum) of the
same products, through the C ABI on caller-owned device arrays.

Collected last on purpose, so a run that stops at the first failure has run every other test first."""
import ctypes
import math

import numpy as np
import pytest

from edlib_gb300 import models

pytestmark = pytest.mark.gpu


def test_vv_noalloc_matches_vv_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    from edlib_gb300 import _abi, build, ed
    build.build()
    L = _abi.lib()
    params, data = models.hubbard_ring8()
    ham = ed.Hamiltonian(params, data, storage="CRS")  # owner of the allocating edgpu_vv path
    stream = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    for n in (4900, 853776):
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        for call in range(2):
            v = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
            w = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
            rc = L.edgpu_vv_noalloc(v.data_ptr(), w.data_ptr(), n, out.data_ptr(), stream)
            assert rc == _abi.OK
            torch.cuda.synchronize()
            vh, wh = v.cpu().numpy(), w.cpu().numpy()
            exact = math.fsum((vh * wh).tolist())  # correctly rounded sum of the rounded FP64 products
            want = ham.storage.vv(vh, wh)
            got = float(out.item())
            scale = float(np.dot(np.abs(vh), np.abs(wh)))
            assert abs(want - exact) <= 1e-13 * scale, (n, call, want, exact)
            assert abs(got - exact) <= 1e-13 * scale, (n, call, got, exact)
            assert abs(got - want) <= 1e-13 * scale, (n, call, got, want)


def test_vv_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from edlib_gb300 import _abi, build
    build.build()
    L = _abi.lib()
    v = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = L.edgpu_vv_noalloc(v.data_ptr(), v.data_ptr(), 8388608 + 1, out.data_ptr(), None)
    assert rc == _abi.ERR_CAPACITY
    assert L.edgpu_vv_noalloc(None, None, -1, out.data_ptr(), None) == _abi.ERR_ARG
