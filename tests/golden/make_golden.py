"""Generate the golden fixtures in this directory.

Two sources, both the reference itself:
1. the reference's own golden files for its Lanczos test (test/input/GF_Chi/{gom1,xiats,xiatd}.dat,
   first 200 rows, the rows that test compares) are copied into ``gf_chi_2x2_reference.npz``;
2. the reference EDLib headers compiled unmodified against the stand-in headers
   (``oracle/_ref/edlib_ref``, built by ``oracle/build.py``) are run on the small models
   below, and their eigenvalues, G(i w_n), chi(i w_n), G0 / Sigma and raw H*v products are stored as
   ``<case>.npz`` next to the model input ``<case>.txt`` they were computed from.

Run from the repository root:  python tests/golden/make_golden.py [case ...]  (no case: all of them)
Needs the reference checkout (read-only) and therefore only runs where it is present; the
fixtures are committed so tests elsewhere do not need it.
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from edlib_gb300 import models  # noqa: E402
from oracle import build  # noqa: E402

REF_TEST_INPUT = os.path.join(build.reference_root(), "test", "input", "GF_Chi")


def run_ref(case, params, data, model, storage, mode):
    p = dict(params)
    p["harness.MODEL"] = model
    p["harness.STORAGE"] = storage
    path = os.path.join(HERE, case + ".txt")
    models.write_input(path, p, data)
    exe = build.build_ref()
    r = subprocess.run([exe, path, mode], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-3000:])
    out = {"E": [], "Esec": [], "G": {}, "GIJ": {}, "G0": {}, "SIGMA": {}, "CHISZ": {}, "CHIN": {}, "CHISZIJ": {},
           "CHINIJ": {}, "W": {}, "OBS": {}}
    for line in r.stdout.splitlines():
        t = line.split()
        if t[0] == "E":
            out["E"].append(float(t[1]))
            out["Esec"].append((int(t[2]), int(t[3])))
        elif t[0] in ("G", "GIJ", "G0", "SIGMA"):
            out[t[0]][(int(t[1]), int(t[2]), int(t[3]))] = complex(float(t[4]), float(t[5]))
        elif t[0] in ("CHISZ", "CHIN", "CHISZIJ", "CHINIJ"):
            out[t[0]][(int(t[1]), int(t[2]))] = complex(float(t[3]), float(t[4]))
        elif t[0] == "W":
            out["W"][int(t[1])] = float(t[2])
        elif t[0] == "OBS":
            out["OBS"][t[2]] = np.array([float(x) for x in t[3:]])
    return out


def dense(dct, ndim):
    if not dct:
        return np.zeros((0,) * ndim, complex)
    shape = tuple(max(k[i] for k in dct) + 1 for i in range(ndim))
    a = np.zeros(shape, complex)
    for k, v in dct.items():
        a[k] = v
    return a


def save(case, res, extra=None):
    arrs = {"E": np.array(res["E"]), "Esec": np.array(res["Esec"], dtype=np.int32).reshape(-1, 2)}
    if res["G"]:
        arrs["G"] = dense(res["G"], 3)
    for k in ("GIJ", "G0", "SIGMA"):
        if res[k]:
            arrs[k] = dense(res[k], 3)
    for k in ("CHISZ", "CHIN", "CHISZIJ", "CHINIJ"):
        if res[k]:
            arrs[k] = dense(res[k], 2)
    if res["W"]:
        arrs["W"] = np.array([res["W"][i] for i in range(len(res["W"]))])
    for k, v in res["OBS"].items():
        arrs["OBS_" + k] = v
    if extra:
        arrs.update(extra)
    np.savez_compressed(os.path.join(HERE, case + ".npz"), **arrs)


def main(only=()):
    def want(case):
        return not only or case in only

    # self-energy (GreensFunction::compute_selfenergy): the 2x2 plaquette with every orbital pair in
    # GreensFunction_orbitals, so G_ij is the full 4x4 matrix the Dyson equation inverts; and the bare
    # G0 of a one-orbital Anderson impurity (its solve_dyson is not run, the harness says why)
    if want("sigma_2x2"):
        p, d = models.plaquette_2x2_gf_chi()
        d["GreensFunction_orbitals/values"] = np.array([[i, j] for i in range(4) for j in range(4)], dtype=np.float64)
        p.update({"arpack.NEV": 20, "lanc.NOMEGA": 64, "lanc.BETA": 10.0})
        save("sigma_2x2", run_ref("sigma_2x2", p, d, "HUBBARD", "CRS", "sigma"))
    if want("siam6_sigma"):
        p, d = models.random_siam(3, 5)
        p.update({"arpack.NEV": 4, "lanc.BETA": 10.0, "lanc.NOMEGA": 64})
        save("siam6_sigma", run_ref("siam6_sigma", p, d, "SIAM", "SRS", "sigma"))
    if only and not (set(only) - {"sigma_2x2", "siam6_sigma"}):
        return

    # 1. the reference's own golden vectors (Lanczos test)
    g = np.loadtxt(os.path.join(REF_TEST_INPUT, "gom1.dat"))[:200]
    xs = np.loadtxt(os.path.join(REF_TEST_INPUT, "xiats.dat"))[:200]
    xd = np.loadtxt(os.path.join(REF_TEST_INPUT, "xiatd.dat"))[:200]
    np.savez_compressed(os.path.join(HERE, "gf_chi_2x2_reference.npz"), gom1=g, xiats=xs, xiatd=xd)

    # 2. reference harness runs
    p, d = models.plaquette_2x2_gf_chi()
    save("gf_chi_2x2", run_ref("gf_chi_2x2", p, d, "HUBBARD", "CRS", "chi"))

    # the full-size 8-site ring of the plain CPU-runnable configuration (CRS, FP64, all sectors, 10
    # eigen-pairs per sector, beta = 50, G on 200 Matsubara points): about 13 minutes of CPU
    p, d = models.hubbard_ring8()
    save("ring8_cfg1", run_ref("ring8_cfg1", p, d, "HUBBARD", "CRS", "gf"))

    p, d = models.ring4_magnetic()
    save("ring4_field", run_ref("ring4_field", p, d, "HUBBARD", "SOCRS", "eigen"))

    p, d = models.random_siam(3, 5)
    p.update({"arpack.NEV": 4, "lanc.BETA": 10.0, "lanc.NOMEGA": 64})
    save("siam6_srs", run_ref("siam6_srs", p, d, "SIAM", "SRS", "chi"))

    # the same Anderson model on the real-frequency mesh (RealFreqMeshFactory): G and chi at w + i pi / beta
    p, d = models.random_siam(3, 5)
    p.update({"arpack.NEV": 4, "lanc.BETA": 10.0, "lanc.NOMEGA": 64, "lanc.EMIN": -4.0, "lanc.EMAX": 4.0})
    save("siam6_real", run_ref("siam6_real", p, d, "SIAM", "SRS", "real"))

    p, d = models.random_kanamori_siam(7, nbath_per_orb=[2, 2], norb=2)
    p.update({"arpack.NEV": 6, "lanc.BETA": 10.0, "lanc.NOMEGA": 64, "lanc.NLANC": 60})
    save("kanamori2_srs", run_ref("kanamori2_srs", p, d, "SIAM", "SRS", "chi"))

    # raw H*v products, v[i] = sin(0.37 i + 0.1)
    h = models.hubbard(models.ring_hopping(6, 1.0) + models.square_hopping(2, 3, 0.0, 0.25), 4.0, 2.0, hmag=0.1)
    for st in ("CRS", "SRS", "SOCRS"):
        p = {"NSITES": 6, "storage.MAX_DIM": 400, "storage.MAX_SIZE": 400 * 40, "harness.NUP": 3, "harness.NDN": 2}
        save("hubbard6_av_" + st.lower(), run_ref("hubbard6_av_" + st.lower(), p, h, "HUBBARD", st, "av"))
    p, d = models.random_kanamori_siam(11, nbath_per_orb=[1, 2, 1], norb=3)
    for st in ("CRS", "SRS"):
        p2 = dict(p)
        p2.update({"storage.MAX_DIM": 5000, "storage.MAX_SIZE": 5000 * 80, "harness.NUP": 4, "harness.NDN": 3})
        save("kanamori3_av_" + st.lower(), run_ref("kanamori3_av_" + st.lower(), p2, d, "SIAM", st, "av"))


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
