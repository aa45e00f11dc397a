"""FP64 CPU oracle for the EDLib hot path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use this
module, and only as the checker.  It drives the C++ restatement in ``oracle/edoracle.cpp``
(tables, models, CRS / SRS / SOCRS fill and H*v, a / a+, the Lanczos recurrence and the
continued fraction) and restates in Python the sector loop and the Green's-function /
susceptibility bookkeeping of the reference:

* ``diag``            -- include/edlib/Hamiltonian.h:54-101, include/edlib/Storage.h:43-146
* ``greens_function`` -- include/edlib/GreensFunction.h:109-159, 241-359, 389-462
* ``chiloc``          -- include/edlib/ChiLoc.h:180-411, 474-530
* ``static_observables`` -- include/edlib/StaticObservables.h:106-158, 356-421

ARPACK (an un-vendored dependency of the reference, arpack-ng ">= 3.5.0") is replaced by dense
LAPACK ``eigh`` for sectors up to ``DENSE_MAX`` states and by scipy's own ARPACK build
(``scipy.sparse.linalg.eigsh``, the same dsaupd/dseupd algorithm, which="SA", tol=1e-14,
maxiter=1000, ncv as the reference clamps it) above that.
"""
import ctypes
import math
import os

import numpy as np

from . import build as _build

DENSE_MAX = 2500
STORAGES = {"CRS": 0, "SRS": 1, "SOCRS": 2}
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_lib = None


def _load():
    global _lib
    if _lib is None:
        path = _build.build_port()
        lib = ctypes.CDLL(path)
        lib.eo_create_hubbard.restype = ctypes.c_void_p
        lib.eo_create_hubbard.argtypes = [ctypes.c_int, _D, _D, _D, _D, _D]
        lib.eo_create_siam.restype = ctypes.c_void_p
        lib.eo_create_siam.argtypes = [ctypes.c_int, ctypes.c_int, _D, _D, _D, ctypes.c_double, _D]
        lib.eo_destroy.argtypes = [ctypes.c_void_p]
        lib.eo_num_transitions.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.eo_binom.restype = ctypes.c_longlong
        lib.eo_binom.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        lib.eo_sector_order.argtypes = [ctypes.c_void_p, _I, ctypes.c_int, _I]
        lib.eo_basis.argtypes = [ctypes.c_void_p, ctypes.c_int, _I]
        lib.eo_nsym_index.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong]
        lib.eo_state_by_index.restype = ctypes.c_longlong
        lib.eo_state_by_index.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_longlong]
        lib.eo_diagonal.restype = ctypes.c_double
        lib.eo_diagonal.argtypes = [ctypes.c_void_p, ctypes.c_longlong]
        lib.eo_fill.restype = ctypes.c_longlong
        lib.eo_fill.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.eo_error.restype = ctypes.c_char_p
        lib.eo_error.argtypes = [ctypes.c_void_p]
        lib.eo_av.argtypes = [ctypes.c_void_p, _D, _D, ctypes.c_int]
        lib.eo_srs_csr.restype = ctypes.c_longlong
        lib.eo_srs_csr.argtypes = [ctypes.c_void_p, ctypes.c_int, _I, _I, _D, _I]
        lib.eo_zero_eigenpair.restype = ctypes.c_double
        lib.eo_zero_eigenpair.argtypes = [ctypes.c_void_p]
        lib.eo_a_adag.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, _D, _D, ctypes.c_int]
        lib.eo_diag_op.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, _D, _D]
        lib.eo_lanczos.argtypes = [ctypes.c_void_p, _D, ctypes.c_int, _D, _D]
        lib.eo_frac_points.argtypes = [_D, _D, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                       _D, ctypes.c_int, _D]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I)


# EDLib parameter defaults (include/edlib/EDParams.h:11-37)
DEFAULTS = {
    "NSITES": 4, "NSPINS": 2, "arpack.NEV": 2, "storage.MAX_DIM": 5000, "storage.MAX_SIZE": 70000,
    "storage.EIGENVALUES_ONLY": 0, "lanc.NOMEGA": 32, "lanc.EMIN": -3.0, "lanc.EMAX": 3.0, "lanc.NLANC": 100,
    "lanc.BETA": 10.0, "lanc.BOLTZMANN_CUTOFF": 1e-12, "siam.NORBITALS": 1,
}


def read_input(path):
    """Read the text model-input format ("param K V" and "data path ndim dims... values") into
    (params, data)."""
    params, data = {}, {}
    toks = open(path).read().split()
    i = 0
    while i < len(toks):
        t = toks[i]
        if t == "param":
            params[toks[i + 1]] = toks[i + 2]
            i += 3
        elif t == "data":
            name, nd = toks[i + 1], int(toks[i + 2])
            shape = [int(x) for x in toks[i + 3:i + 3 + nd]]
            n = int(np.prod(shape)) if nd else 1
            vals = np.array([float(x) for x in toks[i + 3 + nd:i + 3 + nd + n]])
            data[name] = vals.reshape(shape) if nd else vals[0]
            i += 3 + nd + n
        else:
            raise ValueError("bad token %r" % t)
    return params, data


class OracleED:
    """One model (Hubbard or single-impurity Anderson) with one storage kind."""

    def __init__(self, params, data, storage="CRS", model="HUBBARD"):
        self.p = dict(DEFAULTS)
        self.p.update(params)
        self.data = data
        self.lib = _load()
        self.storage = STORAGES[storage]
        self.model = model
        ns = int(self.p["NSITES"])
        self.ns = ns
        if model == "HUBBARD":
            t = np.ascontiguousarray(data["hopping/values"], dtype=np.float64).reshape(ns, ns)
            U = np.ascontiguousarray(data["interaction/values"], dtype=np.float64).reshape(ns)
            xmu = np.ascontiguousarray(data["chemical_potential/values"], dtype=np.float64).reshape(ns)
            hm = np.ascontiguousarray(data.get("magnetic_field/values", np.zeros(ns)), dtype=np.float64)
            J = np.ascontiguousarray(data.get("exchange/values", np.zeros((ns, ns))), dtype=np.float64)
            self.h = self.lib.eo_create_hubbard(ns, _dp(t), _dp(U), _dp(xmu), _dp(hm), _dp(J))
            self.nint = ns
            self.t, self.xmu = t, xmu
        else:
            ml = int(self.p["siam.NORBITALS"])
            epsk = np.ascontiguousarray(data["Bath/Epsk/values"], dtype=np.float64).reshape(ns - ml, 2)
            vk = np.ascontiguousarray(np.stack([np.asarray(data["Bath/Vk_%d/values" % m], dtype=np.float64)
                                                for m in range(ml)]).reshape(ml, ns - ml, 2))
            h0 = np.ascontiguousarray(np.stack([np.asarray(data["H0_%d/values" % m], dtype=np.float64)
                                                for m in range(ml)]).reshape(ml, ml, 2))
            U = np.ascontiguousarray(data["interaction/values"], dtype=np.float64).reshape(-1)
            self.h = self.lib.eo_create_siam(ns, ml, _dp(epsk), _dp(vk), _dp(h0), float(data["mu"]), _dp(U))
            self.nint = ml
            self.epsk, self.vk, self.h0 = epsk, vk, h0
        self.eigenpairs = []

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.eo_destroy(self.h)
            self.h = None

    # ---------------------------------------------------------------- tables / sectors
    def binom(self, n, k):
        return int(self.lib.eo_binom(self.h, n, k))

    def dim(self, nup, ndn):
        return self.binom(self.ns, nup) * self.binom(self.ns, ndn)

    def sector_order(self):
        if str(self.p.get("arpack.SECTOR", "0")) in ("1", "TRUE", "true", "True"):
            lst = np.ascontiguousarray(np.asarray(self.data["sectors/values"], dtype=np.int32).reshape(-1, 2))
            out = np.zeros_like(lst)
            n = self.lib.eo_sector_order(self.h, _ip(lst), lst.shape[0], _ip(out))
        else:
            out = np.zeros(((self.ns + 1) ** 2, 2), dtype=np.int32)
            n = self.lib.eo_sector_order(self.h, None, 0, _ip(out))
        return [tuple(int(x) for x in r) for r in out[:n]]

    def basis(self, k):
        out = np.zeros(self.binom(self.ns, k), dtype=np.int32)
        self.lib.eo_basis(self.h, k, _ip(out))
        return out

    # ---------------------------------------------------------------- storage
    def fill(self, nup, ndn):
        n = self.lib.eo_fill(self.h, self.storage, nup, ndn)
        if n < 0:
            raise RuntimeError(self.lib.eo_error(self.h).decode())
        self.cur = (nup, ndn)
        return n

    def av(self, v, w=None, clear=True):
        v = np.ascontiguousarray(v, dtype=np.float64)
        w = np.zeros_like(v) if w is None else np.ascontiguousarray(w, dtype=np.float64).copy()
        self.lib.eo_av(self.h, _dp(v), _dp(w), 1 if clear else 0)
        return w

    def srs_csr(self, which):
        nrows = ctypes.c_int(0)
        nnz = self.lib.eo_srs_csr(self.h, which, None, None, None, ctypes.byref(nrows))
        rp = np.zeros(nrows.value + 1, dtype=np.int32)
        col = np.zeros(max(nnz, 1), dtype=np.int32)
        val = np.zeros(max(nnz, 1), dtype=np.float64)
        self.lib.eo_srs_csr(self.h, which, _ip(rp), _ip(col), _dp(val), ctypes.byref(nrows))
        return rp, col[:nnz], val[:nnz]

    def dense(self):
        n = self.lib.eo_fill(self.h, self.storage, *self.cur)
        H = np.zeros((n, n))
        e = np.zeros(n)
        for j in range(n):
            e[j] = 1.0
            H[:, j] = self.av(e)
            e[j] = 0.0
        return H

    # ---------------------------------------------------------------- eigen-solve
    def _sector_eigs(self, nup, ndn):
        n = self.fill(nup, ndn)
        if n == 0:
            return [], []
        if n == 1:
            return [self.lib.eo_zero_eigenpair(self.h)], [np.ones(1)]
        nev_p = int(self.p["arpack.NEV"])
        ncv_p = int(self.p["arpack.NCV"]) if "arpack.NCV" in self.p else 2 * nev_p + 3
        ncv = min(ncv_p, n)
        nev = min(nev_p, ncv - 1)
        if n <= DENSE_MAX:
            H = self.dense()
            w, V = np.linalg.eigh(H)
            return list(w[:nev]), [V[:, i].copy() for i in range(nev)]
        from scipy.sparse.linalg import LinearOperator, eigsh
        op = LinearOperator((n, n), matvec=lambda x: self.av(np.asarray(x).reshape(-1)), dtype=np.float64)
        w, V = eigsh(op, k=nev, which="SA", ncv=ncv, tol=1e-14, maxiter=1000)
        order = np.argsort(w, kind="stable")
        return [w[i] for i in order], [V[:, i].copy() for i in order]

    def diag(self):
        """Eigen-pairs of every sector: list of (E, (nup, ndn), evec), ascending E with ties in
        insertion order (the effective ordering of std::set<EigenPair>)."""
        pairs = []
        for (nup, ndn) in self.sector_order():
            evals, evecs = self._sector_eigs(nup, ndn)
            for e, v in zip(evals, evecs):
                pairs.append((float(e), (nup, ndn), v))
        order = sorted(range(len(pairs)), key=lambda i: pairs[i][0])
        self.eigenpairs = [pairs[i] for i in order]
        return self.eigenpairs

    # ---------------------------------------------------------------- operators
    def a_adag(self, im, sec, tsec, vin, annihilate):
        out = np.zeros(self.dim(*tsec))
        vin = np.ascontiguousarray(vin, dtype=np.float64)
        self.lib.eo_a_adag(self.h, im, sec[0], sec[1], tsec[0], tsec[1], _dp(vin), _dp(out), 1 if annihilate else 0)
        return out

    def diag_op(self, op, mu, nu, sec, vin):
        vin = np.ascontiguousarray(vin, dtype=np.float64)
        out = np.zeros_like(vin)
        self.lib.eo_diag_op(self.h, 0 if op == "Sz" else 1, mu, -1 if nu is None else nu, sec[0], sec[1],
                            _dp(vin), _dp(out))
        return out

    def lanczos(self, sec, v):
        """Fill sector `sec` and run the plain Lanczos recurrence (Lanczos.h:36-77)."""
        self.fill(*sec)
        nl = int(self.p["lanc.NLANC"])
        v = np.ascontiguousarray(v, dtype=np.float64).copy()
        a = np.zeros(nl)
        b = np.zeros(nl + 1)
        n = self.lib.eo_lanczos(self.h, _dp(v), nl, _dp(a), _dp(b))
        return n, a, b

    def frac_points(self, a, b, nlanc, isign, expectation, expb, ener):
        ener = np.ascontiguousarray(np.stack([ener.real, ener.imag], axis=-1).reshape(-1))
        out = np.zeros(ener.size)
        self.lib.eo_frac_points(_dp(a), _dp(b), nlanc, isign, expectation, expb, _dp(ener), ener.size // 2, _dp(out))
        return out[0::2] + 1j * out[1::2]

    # ---------------------------------------------------------------- meshes
    def matsubara(self, fermionic):
        beta = float(self.p["lanc.BETA"])
        nw = int(self.p["lanc.NOMEGA"])
        return (2.0 * np.arange(nw) + (1 if fermionic else 0)) * math.pi / beta

    def real_mesh(self):
        """RealFreqMeshFactory (MeshFactory.h:27-34): a linear grid of NOMEGA points from EMIN to EMAX."""
        nw = int(self.p["lanc.NOMEGA"])
        emin, emax = float(self.p["lanc.EMIN"]), float(self.p["lanc.EMAX"])
        return emin + (emax - emin) * np.arange(nw) / float(nw - 1)

    def _orbitals(self, key):
        if key in self.data:
            lst = np.asarray(self.data[key], dtype=np.int64).reshape(-1, 2)
        else:
            lst = np.array([[i, i] for i in range(self.nint)])
        diag = sorted(set(int(r[0]) for r in lst if r[0] == r[1]))
        pairs = [(int(r[0]), int(r[1])) for r in lst if r[0] != r[1]]
        for pr in pairs:
            for o in pr:
                if o not in diag:
                    diag.append(o)
        return diag, pairs

    def _boltzmann(self):
        beta = float(self.p["lanc.BETA"])
        cutoff = float(self.p["lanc.BOLTZMANN_CUTOFF"])
        E0 = self.eigenpairs[0][0]
        Z = 0.0
        for e, _, _ in self.eigenpairs:
            Z += math.exp(-(e - E0) * beta)
        keep = []
        for e, s, v in self.eigenpairs:
            bf = math.exp(-(e - E0) * beta)
            if abs(cutoff - bf) > np.finfo(np.float64).eps and bf < cutoff:
                continue
            keep.append((e, s, v, bf))
        return E0, Z, keep

    def _cf(self, norm, E, E0, nlanc, a, b, isign, w, sym, real=False):
        beta = float(self.p["lanc.BETA"])
        expb = 0.0 if beta * (E - E0) > 25 else math.exp(-beta * (E - E0))
        if real:
            # Lanczos::freq_point on a real mesh: z = w + i pi / beta (Lanczos.h:146-148); every point of the
            # symmetrised fraction is evaluated, no static term (Lanczos.h:106-124, 166-169)
            z = w + 1j * math.pi / beta
            vals = self.frac_points(a, b, nlanc, isign, norm, expb, z + E * isign)
            if sym:
                vals = vals + self.frac_points(a, b, nlanc, isign, norm, expb, -z + E * isign)
            return vals, None
        if not sym:
            z = 1j * w + E * isign
            return self.frac_points(a, b, nlanc, isign, norm, expb, z), None
        z1 = 1j * w[1:] + E * isign
        z2 = -1j * w[1:] + E * isign
        return (self.frac_points(a, b, nlanc, isign, norm, expb, z1) +
                self.frac_points(a, b, nlanc, isign, norm, expb, z2)), -norm * beta * expb

    def _particles(self, orbs, spin, sec, vec, create):
        nup, ndn = sec
        if create:
            # SzSymmetry::can_create_particle (SzSymmetry.h:169-171) only excludes N > Ns + 1
            tsec = (nup + (1 - spin), ndn + spin)
        else:
            if (nup if spin == 0 else ndn) <= 0:
                return None
            tsec = (nup - (1 - spin), ndn - spin)
        if max(tsec) > self.ns:
            return None
        out = np.zeros(self.dim(*tsec))
        for orb in orbs:
            out += self.a_adag(orb + spin * self.ns, sec, tsec, vec, not create)
        norm = float(np.dot(out, out)) if out.size else 0.0
        if not abs(norm) > 1e-10:
            return None
        return tsec, out / math.sqrt(norm), norm

    def greens_function(self, mesh="matsubara"):
        """G(i w_n) (GreensFunction.h:109-159), or G(w + i pi/beta) on the real mesh.  Returns dict with G,
        G_g, G_l, G_ij, Z."""
        real = mesh == "real"
        w = self.real_mesh() if real else self.matsubara(True)
        nw = w.size
        n = self.nint
        diag, pairs = self._orbitals("GreensFunction_orbitals/values")
        Gg = np.zeros((nw, n, 2), complex)
        Gl = np.zeros((nw, n, 2), complex)
        Ggij = np.zeros((nw, n * n, 2), complex)
        Glij = np.zeros((nw, n * n, 2), complex)
        E0, Z, keep = self._boltzmann()
        for (E, sec, vec, bf) in keep:
            for orb in diag:
                for spin in range(2):
                    for create, tgt, isign in ((True, Gg, 1), (False, Gl, -1)):
                        r = self._particles([orb], spin, sec, vec, create)
                        if r is None:
                            continue
                        tsec, v0, norm = r
                        nl, a, b = self.lanczos(tsec, v0)
                        tgt[:, orb, spin] += self._cf(norm, E, E0, nl, a, b, isign, w, False, real)[0]
            for (i, j) in pairs:
                for spin in range(2):
                    for create, tgt, isign in ((True, Ggij, 1), (False, Glij, -1)):
                        r = self._particles([i, j], spin, sec, vec, create)
                        if r is None:
                            continue
                        tsec, v0, norm = r
                        nl, a, b = self.lanczos(tsec, v0)
                        tgt[:, n * i + j, spin] += self._cf(norm, E, E0, nl, a, b, isign, w, False, real)[0]
        Gg /= Z
        Gl /= Z
        Ggij /= Z
        Glij /= Z
        for (i, j) in pairs:
            for o in (i, j):
                Ggij[:, n * i + j, :] -= Gg[:, o, :]
                Glij[:, n * i + j, :] -= Gl[:, o, :]
            Ggij[:, n * i + j, :] *= 0.5
            Glij[:, n * i + j, :] *= 0.5
        for o in diag:
            Ggij[:, n * o + o, :] = Gg[:, o, :]
            Glij[:, n * o + o, :] = Gl[:, o, :]
        return {"G": Gg + Gl, "G_g": Gg, "G_l": Gl, "G_ij": Ggij + Glij, "Z": Z, "omega": w}

    def bare_greens_function(self, mesh="matsubara"):
        """G0[nw, n*n, 2] on the mesh of greens_function().  Hubbard (HubbardModel.h:180-201): the inverse of
        (z + xmu_I) delta_IJ + t_IJ per spin.  Anderson impurity (SingleImpurityAndersonModel.h:377-391):
        1 / (z - H0_mm - sum_k V_mk^2 / (z - eps_k)) on the diagonal of the impurity-orbital block."""
        real = mesh == "real"
        w = self.real_mesh() if real else self.matsubara(True)
        z = w + 1j * math.pi / float(self.p["lanc.BETA"]) if real else 1j * w
        n = self.nint
        G0 = np.zeros((w.size, n * n, 2), complex)
        for iw in range(w.size):
            for s in range(2):
                if self.model == "HUBBARD":
                    g = np.linalg.inv(np.diag(z[iw] + self.xmu).astype(complex) + self.t)
                else:
                    g = np.zeros((n, n), complex)
                    for m in range(n):
                        delta = np.sum(self.vk[m, :, s] ** 2 / (z[iw] - self.epsk[:, s]))
                        g[m, m] = 1.0 / (z[iw] - self.h0[m, m, s] - delta)
                G0[iw, :, s] = g.reshape(-1)
        return G0

    def self_energy(self, G_ij, mesh="matsubara"):
        """(G0, Sigma) with Sigma = G0^-1 - G_ij^-1 per frequency and spin (FermionicModel.h:83-108) on the
        n_int x n_int orbital block."""
        G0 = self.bare_greens_function(mesh)
        n = self.nint
        S = np.zeros_like(G0)
        for iw in range(G0.shape[0]):
            for s in range(2):
                S[iw, :, s] = (np.linalg.inv(G0[iw, :, s].reshape(n, n)) -
                               np.linalg.inv(G_ij[iw, :, s].reshape(n, n))).reshape(-1)
        return G0, S

    def static_observables(self):
        """Boltzmann-averaged N, N_up, N_dn, M, D_occ, M_i M_j, N_eff, E (StaticObservables.h:106-158)."""
        n = self.nint
        E0, _, keep = self._boltzmann()
        acc = {k: np.zeros(n) for k in ("N", "N_up", "N_dn", "M", "D_occ")}
        acc["M_i M_j"] = np.zeros(n * n)
        acc["N_eff"] = np.zeros(1)
        acc["E"] = np.zeros(1)
        tot = 0.0
        ns = self.ns
        for (E, sec, vec, bf) in keep:
            states = np.array([self.lib.eo_state_by_index(self.h, sec[0], sec[1], i) for i in range(vec.size)],
                              dtype=np.int64)
            wgt = vec * vec
            up = np.stack([(states >> (2 * ns - 1 - o)) & 1 for o in range(n)])
            dn = np.stack([(states >> (2 * ns - 1 - (o + ns))) & 1 for o in range(n)])
            dn2 = np.stack([(states >> (2 * ns - 1 - (o + n))) & 1 for o in range(n)])
            acc["N"] += bf * ((up + dn) @ wgt)
            acc["N_up"] += bf * (up @ wgt)
            acc["N_dn"] += bf * (dn @ wgt)
            acc["M"] += bf * ((up - dn) @ wgt)
            acc["D_occ"] += bf * ((up * dn) @ wgt)
            mm = np.einsum("ak,bk,k->ab", up - dn, up - dn2, wgt)
            acc["M_i M_j"] += bf * mm.reshape(-1)
            acc["N_eff"] += bf * (1.0 / float(np.dot(wgt, wgt)))
            acc["E"] += bf * E
            tot += bf
        return {k: v / tot for k, v in acc.items()}

    def chiloc(self, op="Sz", avg=None, mesh="matsubara"):
        """chi(i W_n) for op in {Sz, N} (ChiLoc.h:180-233, 358-411), or chi(w + i pi/beta) on the real mesh
        (no zero-frequency correction there, ChiLoc.h:384-390)."""
        real = mesh == "real"
        w = self.real_mesh() if real else self.matsubara(False)
        nw = w.size
        n = self.nint
        beta = float(self.p["lanc.BETA"])
        if avg is None:
            avg = 0.0 if op == "Sz" else 1.0
        diag, pairs = self._orbitals("ChiLoc_orbitals/values")
        g = np.zeros((nw, n), complex)
        gij = np.zeros((nw, n * n), complex)
        E0, Z, keep = self._boltzmann()
        for (E, sec, vec, bf) in keep:
            for orb in diag:
                out = self.diag_op(op, orb, None, sec, vec)
                norm = float(np.dot(out, out))
                out = out / math.sqrt(norm)
                if norm > 1e-9:
                    nl, a, b = self.lanczos(sec, out)
                    if real:
                        g[:, orb] += self._cf(norm, E, E0, nl, a, b, 1, w, True, True)[0]
                        continue
                    vals, st = self._cf(norm, E, E0, nl, a, b, 1, w, True)
                    g[0, orb] += st
                    g[1:, orb] += vals
            for (i, j) in pairs:
                out = self.diag_op(op, i, j, sec, vec)
                norm = float(np.dot(out, out))
                out = out / math.sqrt(norm)
                nl, a, b = self.lanczos(sec, out)
                if real:
                    gij[:, n * i + j] += self._cf(norm, E, E0, nl, a, b, 1, w, True, True)[0]
                    continue
                vals, st = self._cf(norm, E, E0, nl, a, b, 1, w, True)
                gij[0, n * i + j] += st
                gij[1:, n * i + j] += vals
        g /= Z
        gij /= Z

        def tail(G, col, f):
            om1, om2 = w[f], w[f - 1]
            om1_2, om2_2 = om1 * om1, om2 * om2
            g1, g2 = G[f, col].real, G[f - 1, col].real
            c2 = -(g2 * om2_2 * om2_2 - g1 * om1_2 * om1_2) / (om1_2 - om2_2)
            c4 = -(g1 * om1_2 * om1_2 * om2_2 - g2 * om2_2 * om2_2 * om1_2) / (om1_2 - om2_2)
            return c2, c4, c2 * beta * beta / 24.0 + c4 * beta * beta * beta * beta / 1440.0

        def zero_freq(G, col):
            c2, c4, t = tail(G, col, nw - 1)
            s = 0.0
            for k in range(1, nw):
                om = w[k]
                s = s + G[k, col].real - c2 / (om * om) - c4 / (om * om * om * om)
            G[0, col] -= 2 * s + 2 * t - avg * avg * beta

        if not real:
            for orb in diag:
                zero_freq(g, orb)
            for (i, j) in pairs:
                zero_freq(gij, n * i + j)
        for (i, j) in pairs:
            for o in (i, j):
                gij[:, n * i + j] -= g[:, o]
            gij[:, n * i + j] *= 0.5
        for o in diag:
            gij[:, n * o + o] = g[:, o]
        return {"chi": g, "chi_ij": gij, "Z": Z, "omega": w}
