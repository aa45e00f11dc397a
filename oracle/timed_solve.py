"""Timed CPU solves with the oracle restatement (test and baseline infrastructure only).

The reference's CPU path for one impurity model, end to end: Hamiltonian::diag over every sector
(Hamiltonian.h:54-101; ARPACK through scipy's build, dense LAPACK below 2500 states), then
GreensFunction::compute, StaticObservables and ChiLoc::compute for Sz and N
(GreensFunction.h:109-159, StaticObservables.h:106-158, ChiLoc.h:180-233), with the storage's H*v of the
restatement: SpinResolvedStorage (one thread, as the reference's has no threading) or SOCRSStorage (OpenMP
over OMP_NUM_THREADS cores, as the reference's).

Run as a script (``python -m oracle.timed_solve --seed 0 --storage SRS``) so that OMP_NUM_THREADS takes effect
in a fresh process; prints one JSON line with the wall times of each phase and of every sector's
eigen-solve.  ``--sectors 4,4`` restricts the eigen-solve to the listed sectors and runs the Green's-function
and susceptibility recurrences of the lowest pair found there (a bounded sample).
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from edlib_gb300 import models  # noqa: E402
from oracle.oracle import OracleED  # noqa: E402


def solve(seed, storage, sectors=None):
    params, data = models.anderson_12(seed)
    o = OracleED(params, data, storage, "SIAM")
    per_sector = {}
    t0 = time.perf_counter()
    pairs = []
    order = o.sector_order() if sectors is None else sectors
    for sec in order:
        ts = time.perf_counter()
        evals, evecs = o._sector_eigs(*sec)
        per_sector["%d,%d" % tuple(sec)] = time.perf_counter() - ts
        for e, v in zip(evals, evecs):
            pairs.append((float(e), tuple(sec), v))
    o.eigenpairs = [pairs[i] for i in sorted(range(len(pairs)), key=lambda i: pairs[i][0])]
    t1 = time.perf_counter()
    o.greens_function()
    t2 = time.perf_counter()
    so = o.static_observables()
    o.chiloc("Sz", sum(so["M"]) / (2.0 * len(so["M"])))
    o.chiloc("N", sum(so["N"]) / len(so["N"]))
    t3 = time.perf_counter()
    return {"seconds": t3 - t0, "diag_s": t1 - t0, "gf_s": t2 - t1, "chi_obs_s": t3 - t2, "pairs": len(pairs),
            "E0": o.eigenpairs[0][0] if pairs else None, "storage": storage,
            "threads": int(os.environ.get("OMP_NUM_THREADS", "1")), "per_sector_s": per_sector}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--storage", default="SRS", choices=["SRS", "SOCRS", "CRS"])
    ap.add_argument("--sectors", default=None, help="N_up,N_dn[;N_up,N_dn...]: a bounded sample")
    ap.add_argument("--av", action="store_true", help="only time H*v on sector (6,6)")
    a = ap.parse_args()
    if a.av:
        params, data = models.anderson_12(a.seed)
        o = OracleED(params, data, a.storage, "SIAM")
        n = o.fill(6, 6)
        v = np.random.default_rng(0).standard_normal(n)
        o.av(v)
        t0 = time.perf_counter()
        for _ in range(5):
            o.av(v)
        print(json.dumps({"av_s": (time.perf_counter() - t0) / 5, "dim": n, "storage": a.storage,
                          "threads": int(os.environ.get("OMP_NUM_THREADS", "1"))}))
        return 0
    secs = None
    if a.sectors:
        secs = [tuple(int(x) for x in s.split(",")) for s in a.sectors.split(";")]
    print(json.dumps(solve(a.seed, a.storage, secs)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
