"""The oracle restatement against the reference's own golden vectors and against the reference
headers compiled unmodified (fixtures produced by tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from edlib_gb300 import models
from oracle.oracle import OracleED


def _load(golden_dir, case):
    params, data = models.read_input(os.path.join(golden_dir, case + ".txt"))
    ref = np.load(os.path.join(golden_dir, case + ".npz"))
    return params, data, ref


def test_gf_chi_plaquette_matches_reference_golden_files(golden_dir):
    """The reference's Lanczos test: G within 1e-10, chi within 1e-9 of gom1/xiats/xiatd."""
    params, data, _ = _load(golden_dir, "gf_chi_2x2")
    gold = np.load(os.path.join(golden_dir, "gf_chi_2x2_reference.npz"))
    o = OracleED(params, data, "CRS", "HUBBARD")
    o.diag()
    G = o.greens_function()["G"]
    so = o.static_observables()
    chs = o.chiloc("Sz", sum(so["M"]) / (2.0 * len(so["M"])))["chi"]
    chn = o.chiloc("N", sum(so["N"]) / len(so["N"]))["chi"]
    g = gold["gom1"]
    assert np.abs(G[:200, 0, :] - (g[:, 1] + 1j * g[:, 2])[:, None]).max() < 1e-10
    assert np.abs(chs[:200, 0] + 0.25 * gold["xiats"][:, 1]).max() < 1e-9
    assert np.abs(chn[:200, 0] + gold["xiatd"][:, 1]).max() < 1e-9


def test_gf_chi_plaquette_matches_compiled_reference(golden_dir):
    params, data, ref = _load(golden_dir, "gf_chi_2x2")
    o = OracleED(params, data, "CRS", "HUBBARD")
    o.diag()
    E = np.array([e for e, _, _ in o.eigenpairs])
    assert E.size == ref["E"].size
    assert np.abs(E - ref["E"]).max() < 1e-12
    G = o.greens_function()["G"]
    assert np.abs(G - ref["G"]).max() < 1e-12


def test_ring4_known_answer(golden_dir):
    """4-site ring in a field: E0 = -11.8443 +- 1e-4 in sector (2,2) (reference Hubbard test)."""
    params, data, ref = _load(golden_dir, "ring4_field")
    o = OracleED(params, data, "SOCRS", "HUBBARD")
    o.diag()
    e0, sec, _ = o.eigenpairs[0]
    assert abs(e0 - (-11.8443)) < 1e-4 and sec == (2, 2)
    assert np.abs(np.array([e for e, _, _ in o.eigenpairs]) - ref["E"]).max() < 1e-12
    so = o.static_observables()
    assert np.abs(so["N"] - 1.0).max() < 1e-8
    assert (so["N_up"] > so["N_dn"]).all() and (so["M"] > 0).all()


@pytest.mark.parametrize("case,model,storage", [("siam6_srs", "SIAM", "SRS"), ("kanamori2_srs", "SIAM", "SRS"),
                                                ("kanamori2_srs", "SIAM", "CRS")])
def test_anderson_matches_compiled_reference(golden_dir, case, model, storage):
    params, data, ref = _load(golden_dir, case)
    o = OracleED(params, data, storage, model)
    o.diag()
    E = np.array([e for e, _, _ in o.eigenpairs])
    assert np.abs(E - ref["E"]).max() < 1e-11
    G = o.greens_function()["G"]
    assert np.abs(G - ref["G"]).max() < 1e-10
    so = o.static_observables()
    chs = o.chiloc("Sz", sum(so["M"]) / (2.0 * len(so["M"])))["chi"]
    assert np.abs(chs - ref["CHISZ"]).max() < 1e-9


@pytest.mark.parametrize("case,model,storage,sec", [
    ("hubbard6_av_crs", "HUBBARD", "CRS", (3, 2)), ("hubbard6_av_srs", "HUBBARD", "SRS", (3, 2)),
    ("hubbard6_av_socrs", "HUBBARD", "SOCRS", (3, 2)), ("kanamori3_av_crs", "SIAM", "CRS", (4, 3)),
    ("kanamori3_av_srs", "SIAM", "SRS", (4, 3))])
def test_av_matches_compiled_reference(golden_dir, case, model, storage, sec):
    params, data, ref = _load(golden_dir, case)
    o = OracleED(params, data, storage, model)
    n = o.fill(*sec)
    v = np.sin(0.37 * np.arange(n) + 0.1)
    w = o.av(v)
    assert np.abs(w - ref["W"]).max() <= 1e-13 * max(1.0, np.abs(ref["W"]).max())


def test_tables_nsymmetry_rank_equals_inverse_table():
    """SRS relies on NSymmetry's combinadic rank equalling SzSymmetry's ninv table."""
    p, d = models.random_siam(0, 9)
    o = OracleED(p, d, "SRS", "SIAM")
    for k in range(o.ns + 1):
        b = o.basis(k)
        assert b.size == o.binom(o.ns, k)
        ranks = [o.lib.eo_nsym_index(o.h, k, int(m)) for m in b]
        assert ranks == list(range(b.size))


def test_real_frequency_mesh_matches_compiled_reference(golden_dir):
    """RealFreqMeshFactory: G and chi at w + i pi / beta on a linear EMIN..EMAX grid, no zero-frequency
    correction (MeshFactory.h:27-34, Lanczos.h:146-148, ChiLoc.h:384-390)."""
    params, data, ref = _load(golden_dir, "siam6_real")
    o = OracleED(params, data, "SRS", "SIAM")
    o.diag()
    G = o.greens_function(mesh="real")["G"]
    assert np.abs(G - ref["G"]).max() < 1e-10
    so = o.static_observables()
    chs = o.chiloc("Sz", sum(so["M"]) / (2.0 * len(so["M"])), mesh="real")["chi"]
    assert np.abs(chs - ref["CHISZ"]).max() < 1e-9
    chn = o.chiloc("N", sum(so["N"]) / len(so["N"]), mesh="real")["chi"]
    assert np.abs(chn - ref["CHIN"]).max() < 1e-9


def test_self_energy_matches_compiled_reference(golden_dir):
    """GreensFunction::compute_selfenergy on the 2x2 plaquette with every orbital pair: the oracle's G_ij,
    bare G0 (HubbardModel.h:180-201) and Sigma = G0^-1 - G_ij^-1 (FermionicModel.h:83-108) against the
    reference harness."""
    params, data, ref = _load(golden_dir, "sigma_2x2")
    o = OracleED(params, data, "CRS", "HUBBARD")
    o.diag()
    Gij = o.greens_function()["G_ij"]
    assert np.abs(Gij - ref["GIJ"]).max() < 1e-12
    G0, S = o.self_energy(Gij)
    assert np.abs(G0 - ref["G0"]).max() < 1e-13
    assert np.abs(S - ref["SIGMA"]).max() < 1e-10
    # Sigma of the reference's own G_ij: the Dyson step alone
    _, S_ref_g = o.self_energy(ref["GIJ"])
    assert np.abs(S_ref_g - ref["SIGMA"]).max() < 1e-11


def test_anderson_bare_green_function_matches_compiled_reference(golden_dir):
    """One-orbital Anderson impurity: G0 = 1 / (z - H0 - sum_k V_k^2 / (z - eps_k))
    (SingleImpurityAndersonModel.h:377-391) against the reference harness."""
    params, data, ref = _load(golden_dir, "siam6_sigma")
    o = OracleED(params, data, "SRS", "SIAM")
    G0 = o.bare_greens_function()
    assert np.abs(G0 - ref["G0"]).max() < 1e-14


OBS_KEYS = {"N": "OBS_N", "N_up": "OBS_N_up", "N_dn": "OBS_N_dn", "M": "OBS_M", "D_occ": "OBS_D_occ",
            "M_i M_j": "OBS_M_i_M_j", "N_eff": "OBS_N_eff", "E": "OBS_E"}


@pytest.mark.parametrize("case,model,storage", [("gf_chi_2x2", "HUBBARD", "CRS"), ("kanamori2_srs", "SIAM", "SRS"),
                                                ("siam6_srs", "SIAM", "SRS")])
def test_static_observables_and_nonlocal_chi_match_compiled_reference(golden_dir, case, model, storage):
    """Every static observable of StaticObservables::calculate_static_observables (StaticObservables.h:
    106-158, 356-421) and the non-local susceptibilities chi_ij of ChiLoc::compute with its
    non_local_correction (ChiLoc.h:180-233, 256-276) against the compiled reference."""
    params, data, ref = _load(golden_dir, case)
    o = OracleED(params, data, storage, model)
    o.diag()
    so = o.static_observables()
    for k, rk in OBS_KEYS.items():
        assert np.abs(np.asarray(so[k]) - ref[rk]).max() < 1e-10, k
    cs = o.chiloc("Sz", sum(so["M"]) / (2.0 * len(so["M"])))
    cn = o.chiloc("N", sum(so["N"]) / len(so["N"]))
    assert np.abs(cs["chi_ij"] - ref["CHISZIJ"]).max() < 1e-9
    assert np.abs(cn["chi_ij"] - ref["CHINIJ"]).max() < 1e-9
    assert np.abs(ref["CHISZIJ"]).max() > 0 and np.abs(ref["CHINIJ"]).max() > 0
