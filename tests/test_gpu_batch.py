"""Batched solves: several impurity models in one batched eigen-solve and one batched Lanczos run.
Each result must be the same alone and in the mix (per-item partial sums are reduced in a fixed order,
so the batch composition does not enter the arithmetic)."""
import numpy as np
import pytest

from edlib_gb300 import models

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ed():
    from edlib_gb300 import build
    build.build()
    from edlib_gb300 import ed as _ed
    return _ed


def _models(n):
    out = []
    for seed in range(n):
        p, d = models.random_siam(100 + seed, 5 + (seed % 3))
        p.update({"arpack.NEV": 4, "lanc.BETA": 20.0, "lanc.NOMEGA": 64, "lanc.NLANC": 60})
        out.append((p, d))
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_each_result_same_alone_and_in_the_mix(ed, precision):
    specs = _models(4)  # 6, 7, 8 and 6 sites: uneven sectors in one batch
    alone = []
    for p, d in specs:
        h = ed.Hamiltonian(ed.Params(p), d, storage="SRS", precision=precision)
        h.diag()
        G = ed.GreensFunction(ed.Params(p), h).compute()
        chi = ed.ChiLoc(ed.Params(p), h).compute("Sz", 0.0)
        alone.append(([e.eigenvalue() for e in h.eigenpairs()], G, chi))
    hams = [ed.Hamiltonian(ed.Params(p), d, storage="SRS", precision=precision) for p, d in specs]
    ed.diag_many(hams)
    Gs, _, _ = ed.greens_function_many(ed.Params(specs[0][0]), hams)
    Cs, _, _ = ed.chiloc_many(ed.Params(specs[0][0]), hams, "Sz", [0.0] * len(hams))
    for q, h in enumerate(hams):
        E = [e.eigenvalue() for e in h.eigenpairs()]
        assert len(E) == len(alone[q][0])
        assert np.array_equal(np.array(E), np.array(alone[q][0]))
        assert np.array_equal(Gs[q], alone[q][1])
        assert np.array_equal(Cs[q], alone[q][2])


def test_batched_results_match_oracle(ed):
    from oracle.oracle import OracleED
    specs = _models(3)
    hams = [ed.Hamiltonian(ed.Params(p), d, storage="SRS", precision="fp64") for p, d in specs]
    ed.diag_many(hams)
    Gs, _, _ = ed.greens_function_many(ed.Params(specs[0][0]), hams)
    for (p, d), h, G in zip(specs, hams, Gs):
        o = OracleED(p, d, "SRS", "SIAM")
        o.diag()
        E0 = np.array([e for e, _, _ in o.eigenpairs])
        E = np.array([e.eigenvalue() for e in h.eigenpairs()])
        assert np.abs(E - E0).max() <= 1e-10 * np.abs(E0).max()
        assert np.abs(G - o.greens_function()["G"]).max() < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_plain_path_equals_batched(ed, precision):
    """max_batch = 1 (one sector, one start vector at a time: the reference's loop order) gives the same
    numbers as the all-at-once batch."""
    p, d = _models(1)[0]
    out = []
    for mb in (1, 0):
        h = ed.Hamiltonian(ed.Params(p), d, storage="SRS", precision=precision)
        h.max_batch = mb
        h.diag()
        G = ed.GreensFunction(ed.Params(p), h).compute()
        chi = ed.ChiLoc(ed.Params(p), h).compute("N", 1.0)
        out.append((np.array([e.eigenvalue() for e in h.eigenpairs()]), G, chi))
        h.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])
