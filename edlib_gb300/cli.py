"""Command-line driver: one exact-diagonalisation solve of a preset model, the flow of the reference's
main.cpp (diag, static observables, G(i w_n), chi_Sz, chi_N), printed as one JSON line.

    python -m edlib_gb300.cli anderson12 --precision fp32
    python -m edlib_gb300.cli ring8 --storage CRS --precision fp64
    python -m edlib_gb300.cli input.txt          # a text model input (see edlib_gb300.models)
"""
import argparse
import json
import time

import numpy as np

from . import ed, models

PRESETS = {
    "anderson12": (models.anderson_12, "SRS"),
    "ring8": (models.hubbard_ring8, "CRS"),
    "plaquette2x2": (models.plaquette_2x2_gf_chi, "CRS"),
    "hubbard4x4": (models.hubbard_4x4, "SRS"),
}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("model", help="preset (%s) or a text model input file" % ", ".join(PRESETS))
    ap.add_argument("--storage", default=None, choices=["CRS", "SRS", "SOCRS"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32", "mixed"])
    ap.add_argument("--no-gf", action="store_true", help="eigen-pairs only")
    ap.add_argument("--no-chi", action="store_true", help="no susceptibilities")
    ap.add_argument("--orbital-pairs", action="store_true",
                    help="hubbard4x4: G(k) through G_0j of every site (the reference's route) instead of the "
                         "cos / sin orbital combinations")
    ap.add_argument("--multiplicity-check", type=int, default=0,
                    help="0 full check for missed degenerate copies, 1 none, c >= 2: c - 1 restart cycles")
    ap.add_argument("--ncv", type=int, default=0, help="arpack.NCV (default: the input's, else 2 NEV + 3)")
    args = ap.parse_args(argv)
    if args.model in PRESETS:
        fn, storage = PRESETS[args.model]
        params, data = fn()
    else:
        params, data = models.read_input(args.model)
        storage = "SRS"
    if args.ncv > 0:
        params = dict(params)
        params["arpack.NCV"] = args.ncv
    storage = args.storage or storage
    p = ed.Params(params)
    t0 = time.perf_counter()
    ham = ed.Hamiltonian(p, data, storage=storage, precision=args.precision)
    ham.multiplicity_check = args.multiplicity_check
    ham.diag()
    t1 = time.perf_counter()
    out = {"model": args.model, "storage": storage, "precision": args.precision,
           "eigenvalues": [e.eigenvalue() for e in ham.eigenpairs()[:10]], "npairs": len(ham.eigenpairs()),
           "diag_s": round(t1 - t0, 4)}
    if not args.no_gf:
        gf = ed.GreensFunction(p, ham)
        so = ed.StaticObservables(p).calculate_static_observables(ham)
        out["N"] = so["N"].tolist()
        if args.model == "hubbard4x4" and not args.orbital_pairs:
            # G(k = (pi/2, pi/2)) from the orbital combinations cos(k r_j), sin(k r_j)
            Gw = gf.compute_weighted(models.lattice_k_weights(4, 4, (np.pi / 2, np.pi / 2)))
            gk = (Gw[:, 0, :] + Gw[:, 1, :]) / 16.0
            out["Gk_pi2_pi2"] = [[gk[q, 0].real, gk[q, 0].imag] for q in range(3)]
        else:
            G = gf.compute()
            out["G0"] = [G[0, 0, 0].real, G[0, 0, 0].imag]
            if args.model == "hubbard4x4":  # the reference's route: G(k) as the Fourier sum of G_0j
                gk = models.lattice_gk(gf.G_ij, 4, 4, (np.pi / 2, np.pi / 2))
                out["Gk_pi2_pi2"] = [[gk[q, 0].real, gk[q, 0].imag] for q in range(3)]
        if not args.no_chi:
            chi = ed.ChiLoc(p, ham)
            cs = chi.compute("Sz", float(np.sum(so["M"]) / (2.0 * len(so["M"]))))
            cn = chi.compute("N", float(np.sum(so["N"]) / len(so["N"])))
            out.update({"chiSz0": cs[0, 0].real, "chiN0": cn[0, 0].real})
        out["gf_s"] = round(time.perf_counter() - t1, 4)
    out["stats"] = ham.stats()
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
