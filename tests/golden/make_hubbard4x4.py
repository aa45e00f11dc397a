"""Ground-state energy of the periodic 4x4 Hubbard cluster (t = 1, t' = -0.3, U = 8, mu = U/2) in its
half-filling sector (8, 8), 165,636,900 states, from the oracle's FP64 restatement: its spin-resolved
per-spin hopping matrices (the restatement of SpinResolvedStorage::fill_spin, pinned to the reference's own
H*v) and the Hubbard diagonal, applied as Y = D o X + X H_dn^T + H_up X on the 12870 x 12870 matrix X of a
sector vector (SpinResolvedStorage::av, SpinResolvedStorage.h:58-115) with scipy's sparse products over column
blocks in threads, then a plain FP64 Lanczos recurrence (Lanczos.h:36-77) until the lowest Ritz value of its
tridiagonal matrix stops moving (1e-14 relative over 50 steps).  A few minutes per hundred steps on 8 cores;
writes ``tests/golden/hubbard4x4_e0.npz``.  Run from the repository root.
"""
import os
import sys
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.sparse as sp
from scipy.linalg import eigh_tridiagonal

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from edlib_gb300 import models  # noqa: E402
from oracle.oracle import OracleED  # noqa: E402


def main(max_steps=600, threads=8):
    params, data = models.hubbard_4x4()
    o = OracleED(params, data, "SRS", "HUBBARD")
    n = o.fill(8, 8)
    ns = 16
    up_rp, up_col, up_val = o.srs_csr(0)
    dn_rp, dn_col, dn_val = o.srs_csr(1)
    Nu, Nd = up_rp.size - 1, dn_rp.size - 1
    assert Nu * Nd == n
    Hup = sp.csr_matrix((up_val, up_col, up_rp), shape=(Nu, Nu))
    Hdn = sp.csr_matrix((dn_val, dn_col, dn_rp), shape=(Nd, Nd))
    # HubbardModel::diagonal (HubbardModel.h:116-132) with uniform U and mu[spin] = U/2, no field or exchange:
    # -mu (N_up + N_dn) + U (doubly occupied sites); checked against the restatement on sampled states
    U = float(data["interaction/values"][0])
    mu = float(data["chemical_potential/values"][0])
    bu, bd = o.basis(8).astype(np.int64), o.basis(8).astype(np.int64)
    dbl = np.zeros((Nu, Nd))
    for b in range(ns):
        dbl += np.outer((bu >> b) & 1, (bd >> b) & 1)
    D = -mu * 16.0 + U * dbl
    rng = np.random.default_rng(3)
    for i in rng.integers(0, n, size=64):
        st = o.lib.eo_state_by_index(o.h, 8, 8, int(i))
        assert abs(o.lib.eo_diagonal(o.h, st) - D.reshape(-1)[i]) < 1e-12
    # the restatement's H*v of one vector against the matrix form below
    blocks = np.array_split(np.arange(Nd), threads)
    rblocks = np.array_split(np.arange(Nu), threads)
    pool = ThreadPoolExecutor(threads)

    def hv(X):
        Y = D * X
        parts = list(pool.map(lambda c: (c, Hup @ X[:, c]), blocks))
        for c, P in parts:
            Y[:, c] += P
        parts = list(pool.map(lambda r: (r, (Hdn @ X[r, :].T).T), rblocks))
        for r, P in parts:
            Y[r, :] += P
        return Y

    x = np.sin(0.37 * np.arange(n) + 0.1)
    w_ref = o.av(x)
    w_mat = hv(x.reshape(Nu, Nd)).reshape(-1)
    assert np.abs(w_ref - w_mat).max() <= 1e-12 * np.abs(w_ref).max()
    del x, w_ref, w_mat
    v = rng.standard_normal((Nu, Nd))
    v /= np.linalg.norm(v)
    v_old = np.zeros_like(v)
    alpha, beta = [], [0.0]
    e_hist = []
    t0 = time.time()
    for it in range(max_steps):
        w = hv(v)
        if it > 0:
            w -= beta[-1] * v_old
        a = float(np.vdot(v, w))
        w -= a * v
        b = float(np.linalg.norm(w))
        alpha.append(a)
        beta.append(b)
        v_old, v = v, w / b
        if it >= 20 and it % 10 == 0:
            e0 = eigh_tridiagonal(np.array(alpha), np.array(beta[1:-1]), eigvals_only=True,
                                  select="i", select_range=(0, 0))[0]
            e_hist.append((it, e0))
            print("step %d E0 %.15f (%.0f s)" % (it, e0, time.time() - t0), flush=True)
            if len(e_hist) >= 6 and abs(e_hist[-1][1] - e_hist[-6][1]) <= 1e-14 * abs(e0):
                break
    E0 = e_hist[-1][1]
    np.savez_compressed(os.path.join(HERE, "hubbard4x4_e0.npz"), E0=np.array([E0]), steps=np.array([e_hist[-1][0]]))
    print("E0 %.15f after %d Lanczos steps" % (E0, e_hist[-1][0]))


if __name__ == "__main__":
    main()
