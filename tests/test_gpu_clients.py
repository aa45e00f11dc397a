"""The C ABI driven from plain C on the GPU: tests/cpp/abi_c_client.c, compiled here against include/edgpu.h and
libedgpu.so, runs the reference's Lanczos test workflow (2x2 plaquette, CRS, FP64: Hamiltonian::diag,
GreensFunction::compute, ChiLoc for Sz and N) and its printed results are compared with the reference's own
golden vectors (gom1 / xiats / xiatd, 1e-10 / 1e-9 as the reference's test) and with the compiled reference's
output for the same input."""
import os
import subprocess

import numpy as np
import pytest

from edlib_gb300 import build

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _parse(out):
    E, G, CS, CN = {}, {}, {}, {}
    for line in out.splitlines():
        f = line.split()
        if not f:
            continue
        if f[0] == "E":
            E[int(f[1])] = float(f[2])
        elif f[0] == "G":
            G[int(f[1])] = float(f[2]) + 1j * float(f[3])
        elif f[0] == "CHISZ":
            CS[int(f[1])] = float(f[2])
        elif f[0] == "CHIN":
            CN[int(f[1])] = float(f[2])
    arr = lambda d: np.array([d[k] for k in sorted(d)])
    return arr(E), arr(G), arr(CS), arr(CN)


def test_c_client_runs_the_reference_lanczos_workflow(tmp_path, golden_dir):
    lib = build.build()
    exe = str(tmp_path / "abi_c_client")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "abi_c_client.c"), "-o", exe, "-L", os.path.dirname(lib),
                        "-ledgpu", "-Wl,-rpath," + os.path.dirname(lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, os.path.join(golden_dir, "gf_chi_2x2.txt")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "no device" not in r.stdout
    E, G, CS, CN = _parse(r.stdout)
    ref = np.load(os.path.join(golden_dir, "gf_chi_2x2.npz"))
    gold = np.load(os.path.join(golden_dir, "gf_chi_2x2_reference.npz"))
    assert E.size == ref["E"].size
    assert np.abs(E - ref["E"]).max() <= 1e-10 * np.abs(ref["E"]).max()
    g = gold["gom1"]
    assert np.abs(G[:200] - (g[:, 1] + 1j * g[:, 2])).max() < 1e-10
    assert np.abs(G - ref["G"][:, 0, 0]).max() < 1e-10
    assert np.abs(CS[:200] + 0.25 * gold["xiats"][:, 1]).max() < 1e-9
    assert np.abs(CN[:200] + gold["xiatd"][:, 1]).max() < 1e-9
    assert np.abs(CS - ref["CHISZ"][:, 0].real).max() < 1e-9
    assert np.abs(CN - ref["CHIN"][:, 0].real).max() < 1e-9
