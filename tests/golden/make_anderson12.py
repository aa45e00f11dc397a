"""Full-size fixture of the 12-orbital Anderson impurity (11 bath sites, seed 0): every one of its 169
sectors' 8 lowest eigenvalues, G(i w_n), chi_Sz and chi_N on 1024 Matsubara points (beta = 100, 100
Lanczos steps) and the static observables, all from the oracle's FP64 restatement (spin-resolved H*v,
scipy's ARPACK build for the sector eigen-solves, dense LAPACK below 2500 states).

The oracle itself is pinned to the reference (tests/test_oracle_golden.py); this fixture carries it to
the size of the benchmarked workload, which the compiled reference harness cannot reach here (its ARPACK
stand-in is dense).  Run from the repository root: ``python tests/golden/make_anderson12.py`` (about
half an hour on one core); writes ``tests/golden/anderson12_seed0.npz``.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from edlib_gb300 import models  # noqa: E402
from oracle.oracle import OracleED  # noqa: E402


def main():
    params, data = models.anderson_12(0)
    t0 = time.time()
    o = OracleED(params, data, "SRS", "SIAM")
    o.diag()
    t1 = time.time()
    E = np.array([e for e, _, _ in o.eigenpairs])
    Esec = np.array([s for _, s, _ in o.eigenpairs], dtype=np.int32)
    gf = o.greens_function()
    so = o.static_observables()
    cs = o.chiloc("Sz", sum(so["M"]) / (2.0 * len(so["M"])))
    cn = o.chiloc("N", sum(so["N"]) / len(so["N"]))
    t2 = time.time()
    out = {"E": E, "Esec": Esec, "G": gf["G"], "Z": np.array([gf["Z"]]), "CHISZ": cs["chi"], "CHIN": cn["chi"]}
    for k, v in so.items():
        out["OBS_" + k.replace(" ", "_")] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "anderson12_seed0.npz"), **out)
    print("pairs %d, E0 %.14f, diag %.0f s, G + chi %.0f s" % (E.size, E[0], t1 - t0, t2 - t1))


if __name__ == "__main__":
    main()
