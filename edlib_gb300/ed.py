"""EDLib-shaped host interface over the GB300 C ABI.

Mirrors the reference's call surface for the hot path (names, argument meaning, error behaviour):

* ``Hamiltonian(params, data, storage)``   -- EDLib::Hamiltonian<Storage> (include/edlib/Hamiltonian.h:22-117);
  ``diag()``, ``eigenpairs`` (ascending, ties in insertion order), ``storage`` (the Storage concept:
  ``fill``, ``av``, ``a_adag``, ``vv``, ``vector_size``).
* ``EigenPair``                            -- include/edlib/EigenPair.h:12-47
* ``GreensFunction(params, ham)``          -- include/edlib/GreensFunction.h:54-159 (``compute``, ``G``, ``G_ij``, ``Z``)
* ``ChiLoc(params, ham)``                  -- include/edlib/ChiLoc.h:123-233 (``compute(op, avg)``, ``G``, ``G_ij``)
* ``StaticObservables(params)``            -- include/edlib/StaticObservables.h:44-158
* ``define_parameters`` / ``Params``       -- include/edlib/EDParams.h:11-37

``data`` holds the model's datasets under the paths EDLib reads from its INPUT_FILE (see
``edlib_gb300.models``); a text model input can be named by ``params["INPUT_FILE"]`` instead.
All numerical work runs in libedgpu.so on the GPU.
"""
import ctypes
import math

import numpy as np

from . import _abi
from . import models as _models

DEFAULTS = {
    "NSITES": 4, "NSPINS": 2, "INPUT_FILE": "input.h5", "OUTPUT_FILE": "sim.h5",
    "storage.MAX_DIM": 5000, "storage.MAX_SIZE": 70000, "storage.EIGENVALUES_ONLY": 0,
    "spinstorage.ORBITAL_NUMBER": 1, "arpack.NEV": 2, "lanc.NOMEGA": 32, "lanc.EMIN": -3.0, "lanc.EMAX": 3.0,
    "lanc.NLANC": 100, "lanc.BETA": 10.0, "lanc.BOLTZMANN_CUTOFF": 1e-12, "siam.NORBITALS": 1,
}


class Params(dict):
    """EDLib parameters with the defaults of define_parameters (EDParams.h:11-37)."""

    def __init__(self, *a, **kw):
        super().__init__(DEFAULTS)
        self.update(*a, **kw)

    def exists(self, k):
        return k in self

    def num(self, k):
        v = self[k]
        if isinstance(v, str):
            if v.upper() in ("TRUE", "FALSE"):
                return 1.0 if v.upper() == "TRUE" else 0.0
            return float(v)
        return float(v)


def define_parameters(p=None):
    p = Params() if p is None else p
    for k, v in DEFAULTS.items():
        p.setdefault(k, v)
    return p


_ctx = {}


def context(device=0):
    """The process-wide GPU context of a device (one stream)."""
    if device not in _ctx:
        L = _abi.lib()
        h = ctypes.c_void_p()
        rc = L.edgpu_ctx_create(ctypes.byref(h), device, 0)
        if rc != 0:
            raise _abi.EdgpuError(rc, "cannot create a context on device %d" % device)
        _ctx[device] = h
    return _ctx[device]


def _check(rc, ctx):
    if rc < 0:
        raise _abi.EdgpuError(rc, _abi.lib().edgpu_last_error(ctx).decode())
    return rc


class EigenPair:
    def __init__(self, ham, index, value, sector, ident):
        self._ham = ham
        self._index = index
        self.value = value
        self._sector = sector
        self.id = ident

    def eigenvalue(self):
        return self.value

    def sector(self):
        return self._sector

    def eigenvector(self):
        n = self._ham.vector_size(self._sector)
        out = np.zeros(n)
        _check(_abi.lib().edgpu_eigenvector(self._ham._m, self._index, _abi.dptr(out), n), self._ham._ctx)
        return out

    def __repr__(self):
        return "EigenPair(E=%.14g, sector=%s, id=%d)" % (self.value, self._sector, self.id)


class Storage:
    """The Storage concept of the reference (Storage.h, CRSStorage.h, SpinResolvedStorage.h, SOCRSStorage.h)."""

    def __init__(self, ham, kind):
        self._ham = ham
        self.kind = kind
        self.sector = None

    def fill(self, nup=None, ndn=None):
        if nup is None:
            nup, ndn = self.sector
        dim = ctypes.c_longlong(0)
        _check(_abi.lib().edgpu_fill(self._ham._m, _abi.STORAGES[self.kind], nup, ndn, ctypes.byref(dim)),
               self._ham._ctx)
        self.sector = (nup, ndn)
        return dim.value

    def av(self, v, w=None, clear=True, precision=None):
        v = np.ascontiguousarray(v, dtype=np.float64)
        w = np.zeros_like(v) if w is None else np.ascontiguousarray(w, dtype=np.float64).copy()
        prec = _abi.PRECISIONS[precision or self._ham.precision]
        _check(_abi.lib().edgpu_av(self._ham._m, _abi.dptr(v), _abi.dptr(w), v.size, 1 if clear else 0, prec),
               self._ham._ctx)
        return w

    def a_adag(self, spin_orbital, vin, sector, next_sector, annihilate):
        vin = np.ascontiguousarray(vin, dtype=np.float64)
        out = np.zeros(self._ham.vector_size(next_sector))
        _check(_abi.lib().edgpu_a_adag(self._ham._m, spin_orbital, sector[0], sector[1], next_sector[0],
                                       next_sector[1], _abi.dptr(vin), _abi.dptr(out), 1 if annihilate else 0),
               self._ham._ctx)
        return out

    def vv(self, v, w):
        v = np.ascontiguousarray(v, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        r = ctypes.c_double(0)
        _check(_abi.lib().edgpu_vv(self._ham._m, _abi.dptr(v), _abi.dptr(w), v.size, ctypes.byref(r)), self._ham._ctx)
        return r.value


def _gf_precision(precision):
    """Vector precision of the Green's-function recurrences for a Hamiltonian precision: "mixed" runs them on
    float-float vectors (pairs of FP32, about 2^-48 relative; spin-resolved storage, FP64 on the others) from
    FP64 start vectors."""
    return precision


class Hamiltonian:
    """EDLib::Hamiltonian<Storage> on the GPU.  storage in {"CRS", "SRS", "SOCRS"}, precision in
    {"fp64", "fp32", "mixed"} (vectors; dot products, projected matrices and fractions stay FP64).  "mixed"
    solves every sector with FP32 vectors, then continues the sectors of the Boltzmann-weighted pairs in FP64
    before Green's functions, susceptibilities and static observables, whose recurrences run in FP64."""

    def __init__(self, params, data=None, storage="SRS", precision="fp64", device=0):
        self.p = params if isinstance(params, Params) else Params(params)
        if data is None:
            fp, data = _models.read_input(self.p["INPUT_FILE"])
            for k, v in fp.items():
                self.p.setdefault(k, v)
        self.data = data
        self.kind = _models.model_kind(data)
        self.precision = precision
        self._ctx = context(device)
        L = _abi.lib()
        ns = int(self.p.num("NSITES"))
        if int(self.p.num("NSPINS")) != 2:
            raise ValueError("Incorrect values for the number of spins. Please check input file.")
        self.ns = ns
        h = ctypes.c_void_p()
        if self.kind == _models.HUBBARD:
            t = np.ascontiguousarray(data["hopping/values"], dtype=np.float64).reshape(ns, ns)
            U = np.ascontiguousarray(data["interaction/values"], dtype=np.float64).reshape(ns)
            mu = np.ascontiguousarray(data["chemical_potential/values"], dtype=np.float64).reshape(ns)
            hm = data.get("magnetic_field/values")
            J = data.get("exchange/values")
            hm = None if hm is None else np.ascontiguousarray(hm, dtype=np.float64).reshape(ns)
            J = None if J is None else np.ascontiguousarray(J, dtype=np.float64).reshape(ns, ns)
            rc = L.edgpu_model_hubbard(self._ctx, ns, _abi.dptr(t), _abi.dptr(U), _abi.dptr(mu),
                                       _abi.dptr(hm) if hm is not None else None,
                                       _abi.dptr(J) if J is not None else None, ctypes.byref(h))
            self.nint = ns
        else:
            ml = int(self.p.num("siam.NORBITALS"))
            nk = ns - ml
            epsk = np.ascontiguousarray(data["Bath/Epsk/values"], dtype=np.float64).reshape(nk, 2)
            vk = np.ascontiguousarray(np.stack([np.asarray(data["Bath/Vk_%d/values" % m], dtype=np.float64)
                                                for m in range(ml)]).reshape(ml, nk, 2))
            h0 = np.ascontiguousarray(np.stack([np.asarray(data["H0_%d/values" % m], dtype=np.float64)
                                                for m in range(ml)]).reshape(ml, ml, 2))
            U = np.ascontiguousarray(data["interaction/values"], dtype=np.float64).reshape(-1)
            rc = L.edgpu_model_siam(self._ctx, ns, ml, _abi.dptr(epsk), _abi.dptr(vk), _abi.dptr(h0),
                                    float(data["mu"]), _abi.dptr(U), ctypes.byref(h))
            self.nint = ml
        _check(rc, self._ctx)
        self._m = h
        L.edgpu_model_set_limits(self._m, int(self.p.num("storage.MAX_DIM")), int(self.p.num("storage.MAX_SIZE")))
        self.storage = Storage(self, storage)
        self._pairs = None
        self.info = 0
        self.multiplicity_check = 0
        # sectors per lock-step eigen-solver batch and recurrences per Green's-function batch: 0 = all at
        # once, 1 = the plain path (one sector / one start vector at a time); results do not depend on it
        self.max_batch = 0

    def close(self):
        if getattr(self, "_m", None):
            _abi.lib().edgpu_model_destroy(self._m)
            self._m = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_limits(self, max_dim=0, max_size=0):
        _abi.lib().edgpu_model_set_limits(self._m, int(max_dim), int(max_size))

    # symmetry helpers
    def vector_size(self, sector):
        L = _abi.lib()
        return int(L.edgpu_binom(self._m, self.ns, sector[0]) * L.edgpu_binom(self._m, self.ns, sector[1]))

    def sector_order(self):
        L = _abi.lib()
        sec = None
        n_in = 0
        if self.p.exists("arpack.SECTOR") and self.p.num("arpack.SECTOR"):
            sec = np.ascontiguousarray(np.asarray(self.data["sectors/values"]).reshape(-1, 2), dtype=np.int32)
            n_in = sec.shape[0]
        out = np.zeros((max(n_in, (self.ns + 1) ** 2), 2), dtype=np.int32)
        n = ctypes.c_int(0)
        _check(L.edgpu_sector_order(self._m, _abi.iptr(sec) if sec is not None else None, n_in, _abi.iptr(out),
                                    ctypes.byref(n)), self._ctx)
        return [tuple(int(x) for x in r) for r in out[:n.value]]

    def basis(self, k):
        out = np.zeros(int(_abi.lib().edgpu_binom(self._m, self.ns, k)), dtype=np.int32)
        _check(_abi.lib().edgpu_basis(self._m, k, _abi.iptr(out)), self._ctx)
        return out

    def ninv(self, k):
        out = np.zeros(1 << self.ns, dtype=np.int32)
        _check(_abi.lib().edgpu_ninv(self._m, k, _abi.iptr(out)), self._ctx)
        return out

    def diag(self, tol=0.0, maxitr=0, multiplicity_check=None):
        """Hamiltonian::diag: all sectors (or arpack.SECTOR's list) in the reference order.
        multiplicity_check: 0 full (default), 1 off, c >= 2 a check of c - 1 restart cycles."""
        p = self.p
        dp = _abi.DiagParams()
        dp.storage = _abi.STORAGES[self.storage.kind]
        dp.precision = _abi.PRECISIONS[self.precision]
        dp.nev = int(p.num("arpack.NEV"))
        dp.ncv = int(p.num("arpack.NCV")) if p.exists("arpack.NCV") else 0
        dp.eigenvalues_only = int(p.num("storage.EIGENVALUES_ONLY"))
        dp.tol = tol
        dp.maxitr = maxitr
        dp.multiplicity_check = int(multiplicity_check if multiplicity_check is not None else self.multiplicity_check)
        dp.max_batch = int(self.max_batch)
        sec = None
        if p.exists("arpack.SECTOR") and p.num("arpack.SECTOR"):
            sec = np.ascontiguousarray(np.asarray(self.data["sectors/values"]).reshape(-1, 2), dtype=np.int32)
            dp.sectors = _abi.iptr(sec)
            dp.n_sectors = sec.shape[0]
        n = ctypes.c_int(0)
        self.info = _check(_abi.lib().edgpu_diag(self._m, ctypes.byref(dp), ctypes.byref(n)), self._ctx)
        self._load_pairs(n.value)
        return self.info

    def _load_pairs(self, n):
        ev = np.zeros(max(n, 1))
        sec = np.zeros((max(n, 1), 2), dtype=np.int32)
        ids = np.zeros(max(n, 1), dtype=np.int32)
        _check(_abi.lib().edgpu_eigenpairs(self._m, _abi.dptr(ev), _abi.iptr(sec), _abi.iptr(ids), n), self._ctx)
        self._pairs = [EigenPair(self, i, float(ev[i]), (int(sec[i, 0]), int(sec[i, 1])), int(ids[i]))
                       for i in range(n)]

    def eigenpairs(self):
        if self._pairs is None:
            raise RuntimeError("diag() has not been run")
        return self._pairs

    def stats(self):
        """Counters since the last diag(): operator applications, Lanczos steps, restart cycles and
        element-steps (operator applications weighted by sector dimension)."""
        a, b, c = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        w = ctypes.c_double()
        _abi.lib().edgpu_stats(self._m, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(w))
        return {"spmv": a.value, "lanczos_steps": b.value, "restarts": c.value, "element_steps": w.value}

    def operator_tuning(self):
        """{'blocks_per_sm', 'staged', 'ms'}: the eigen-step operator variant the tuner chose for this model's
        first eigen batch (ms -1 when not tuned)."""
        return _operator_tuning(self)


def _operator_tuning(ham):
    """The operator variant the library's tuner chose for this model (edgpu_operator_tuning)."""
    mb, st = ctypes.c_int(), ctypes.c_int()
    ms = ctypes.c_double()
    _abi.lib().edgpu_operator_tuning(ham._m, 0 if ham.precision == "fp64" else 1, ctypes.byref(mb), ctypes.byref(st),
                                     ctypes.byref(ms))
    return {"blocks_per_sm": mb.value, "staged": bool(st.value), "ms": ms.value}


def _orbital_array(data, key):
    if key in data:
        return np.ascontiguousarray(np.asarray(data[key]).reshape(-1, 2), dtype=np.int32)
    return None


def _gf_params(p, precision, orbs, max_batch=0, mesh="matsubara"):
    g = _abi.GfParams()
    g.max_batch = int(max_batch)
    g.mesh = 1 if mesh == "real" else 0
    if mesh == "real":
        g.emin = p.num("lanc.EMIN")
        g.emax = p.num("lanc.EMAX")
    g.beta = p.num("lanc.BETA")
    g.nomega = int(p.num("lanc.NOMEGA"))
    g.nlanc = int(p.num("lanc.NLANC"))
    g.cutoff = p.num("lanc.BOLTZMANN_CUTOFF")
    g.precision = _abi.PRECISIONS[precision]
    if orbs is not None:
        g.orbitals = _abi.iptr(orbs)
        g.n_orbitals = orbs.shape[0]
    return g


class GreensFunction:
    """G(i w_n) on the positive Matsubara mesh, fermionic (GreensFunction.h:109-159); mesh="real": G(w + i pi /
    beta) on the linear lanc.EMIN..lanc.EMAX grid (RealFreqMeshFactory, MeshFactory.h:27-34)."""

    def __init__(self, params, ham, precision=None, mesh="matsubara"):
        self.p = params if isinstance(params, Params) else Params(params)
        self.ham = ham
        self.precision = precision or _gf_precision(ham.precision)
        self.mesh = mesh
        if int(self.p.num("storage.EIGENVALUES_ONLY")) == 1:
            raise RuntimeError("Eigenvectors have not been computed. Green's function can not be evaluated.")
        self._orbs = _orbital_array(ham.data, "GreensFunction_orbitals/values")

    def compute(self):
        nw = int(self.p.num("lanc.NOMEGA"))
        n = self.ham.nint
        G = np.zeros((nw, n, 2, 2))
        Gij = np.zeros((nw, n * n, 2, 2))
        Z = ctypes.c_double(0)
        g = _gf_params(self.p, self.precision, self._orbs, self.ham.max_batch, self.mesh)
        _check(_abi.lib().edgpu_greens_function(self.ham._m, ctypes.byref(g), _abi.dptr(G), _abi.dptr(Gij),
                                                ctypes.byref(Z)), self.ham._ctx)
        self.G = G[..., 0] + 1j * G[..., 1]
        self.G_ij = Gij[..., 0] + 1j * Gij[..., 1]
        self.Z = Z.value
        self._set_omega(nw)
        return self.G

    def compute_weighted(self, weights):
        """G of orbital combinations c_w = sum_j w_j c_j, one per row of weights [nrows, n_int_orb]:
        returns [nomega, nrows, 2 spins] complex (edgpu_greens_function_weighted)."""
        w = np.ascontiguousarray(np.atleast_2d(weights), dtype=np.float64)
        if w.shape[1] != self.ham.nint:
            raise ValueError("weights need one column per interacting orbital")
        nw = int(self.p.num("lanc.NOMEGA"))
        G = np.zeros((nw, w.shape[0], 2, 2))
        Z = ctypes.c_double(0)
        g = _gf_params(self.p, self.precision, None, self.ham.max_batch, self.mesh)
        _check(_abi.lib().edgpu_greens_function_weighted(self.ham._m, ctypes.byref(g), _abi.dptr(w), w.shape[0],
                                                         _abi.dptr(G), ctypes.byref(Z)), self.ham._ctx)
        self.Z = Z.value
        self._set_omega(nw)
        return G[..., 0] + 1j * G[..., 1]

    def compute_selfenergy(self):
        """GreensFunction::compute_selfenergy (GreensFunction.h:202-222) on the mesh of the last compute():
        the model's bare G0 (HubbardModel.h:180-201, SingleImpurityAndersonModel.h:377-391) and
        Sigma = G0^-1 - G_ij^-1 per frequency and spin (FermionicModel.h:83-108), both [nomega, n^2, 2 spins]
        complex; G0 is kept as .G0, Sigma returned and kept as .Sigma (edgpu_self_energy)."""
        if not hasattr(self, "G_ij"):
            raise RuntimeError("compute() the Green's function before the self-energy")
        nw = self.G_ij.shape[0]
        if self.G_ij.shape != (nw, self.ham.nint ** 2, 2):
            raise ValueError("G_ij must be [nomega, n_int_orb^2, 2 spins]")
        gij = np.ascontiguousarray(np.stack([self.G_ij.real, self.G_ij.imag], axis=-1))
        G0 = np.zeros_like(gij)
        S = np.zeros_like(gij)
        g = _gf_params(self.p, self.precision, self._orbs, self.ham.max_batch, self.mesh)
        g.nomega = nw
        _check(_abi.lib().edgpu_self_energy(self.ham._m, ctypes.byref(g), _abi.dptr(gij), _abi.dptr(G0),
                                            _abi.dptr(S)), self.ham._ctx)
        self.G0 = G0[..., 0] + 1j * G0[..., 1]
        self.Sigma = S[..., 0] + 1j * S[..., 1]
        return self.Sigma

    def _set_omega(self, nw):
        beta = self.p.num("lanc.BETA")
        if self.mesh == "real":
            emin, emax = self.p.num("lanc.EMIN"), self.p.num("lanc.EMAX")
            self.omega = emin + (emax - emin) * np.arange(nw) / float(nw - 1)
        else:
            self.omega = (2.0 * np.arange(nw) + 1) * math.pi / beta


class ChiLoc:
    """Local susceptibility chi(i W_n), bosonic (ChiLoc.h:180-233); mesh="real": chi(w + i pi / beta) on the
    linear lanc.EMIN..lanc.EMAX grid, without the zero-frequency correction (ChiLoc.h:384-390)."""

    def __init__(self, params, ham, precision=None, mesh="matsubara"):
        self.p = params if isinstance(params, Params) else Params(params)
        self.ham = ham
        self.precision = precision or _gf_precision(ham.precision)
        self.mesh = mesh
        if int(self.p.num("storage.EIGENVALUES_ONLY")) == 1:
            raise RuntimeError("Eigenvectors have not been computed. Green's function can not be evaluated.")
        self._orbs = _orbital_array(ham.data, "ChiLoc_orbitals/values")

    def compute(self, op="Sz", avg=None):
        if avg is None:
            avg = 0.0 if op == "Sz" else 1.0
        nw = int(self.p.num("lanc.NOMEGA"))
        n = self.ham.nint
        chi = np.zeros((nw, n, 2))
        chij = np.zeros((nw, n * n, 2))
        Z = ctypes.c_double(0)
        g = _gf_params(self.p, self.precision, self._orbs, self.ham.max_batch, self.mesh)
        _check(_abi.lib().edgpu_chiloc(self.ham._m, ctypes.byref(g), _abi.OPERATORS[op], float(avg), _abi.dptr(chi),
                                       _abi.dptr(chij), ctypes.byref(Z)), self.ham._ctx)
        self.G = chi[..., 0] + 1j * chi[..., 1]
        self.G_ij = chij[..., 0] + 1j * chij[..., 1]
        self.Z = Z.value
        return self.G


class StaticObservables:
    """Boltzmann-averaged static observables (StaticObservables.h:106-158)."""

    def __init__(self, params):
        self.p = params if isinstance(params, Params) else Params(params)
        if int(self.p.num("storage.EIGENVALUES_ONLY")) == 1:
            raise RuntimeError("Eigenvectors have not been computed. StaticObservables can not continue.")

    def calculate_static_observables(self, ham):
        if ham.precision == "mixed":
            refine_eigenpairs([ham], self.p.num("lanc.BETA"), self.p.num("lanc.BOLTZMANN_CUTOFF"))
        n = ham.nint
        arr = {k: np.zeros(n) for k in ("N", "N_up", "N_dn", "M", "D_occ")}
        mimj = np.zeros(n * n)
        neff = ctypes.c_double(0)
        en = ctypes.c_double(0)
        _check(_abi.lib().edgpu_static_observables(ham._m, self.p.num("lanc.BETA"), self.p.num("lanc.BOLTZMANN_CUTOFF"),
                                                   _abi.dptr(arr["N"]), _abi.dptr(arr["N_up"]), _abi.dptr(arr["N_dn"]),
                                                   _abi.dptr(arr["M"]), _abi.dptr(arr["D_occ"]), _abi.dptr(mimj),
                                                   ctypes.byref(neff), ctypes.byref(en)), ham._ctx)
        arr["M_i M_j"] = mimj
        arr["N_eff"] = np.array([neff.value])
        arr["E"] = np.array([en.value])
        return arr


def _diag_params(ham, tol=0.0, maxitr=0):
    p = ham.p
    dp = _abi.DiagParams()
    dp.multiplicity_check = int(ham.multiplicity_check)
    dp.max_batch = int(ham.max_batch)
    dp.storage = _abi.STORAGES[ham.storage.kind]
    dp.precision = _abi.PRECISIONS[ham.precision]
    dp.nev = int(p.num("arpack.NEV"))
    dp.ncv = int(p.num("arpack.NCV")) if p.exists("arpack.NCV") else 0
    dp.eigenvalues_only = int(p.num("storage.EIGENVALUES_ONLY"))
    dp.tol = tol
    dp.maxitr = maxitr
    return dp


def _model_array(hams):
    arr = (ctypes.c_void_p * len(hams))()
    for i, h in enumerate(hams):
        arr[i] = h._m
    return arr


def diag_many(hams, tol=0.0, maxitr=0):
    """Hamiltonian::diag of several models (same context, storage, precision and NEV/NCV) in one batched
    eigen-solve; every Hamiltonian afterwards holds its own eigen-pairs."""
    h0 = hams[0]
    if h0.p.exists("arpack.SECTOR") and h0.p.num("arpack.SECTOR"):
        raise ValueError("diag_many solves all sectors of every model")
    dp = _diag_params(h0, tol, maxitr)
    n = (ctypes.c_int * len(hams))()
    rc = _check(_abi.lib().edgpu_diag_many(_model_array(hams), len(hams), ctypes.byref(dp), n), h0._ctx)
    for i, h in enumerate(hams):
        h.info = rc
        h._load_pairs(n[i])
    return rc


def _many_outputs(count, shape):
    arrs = [np.zeros(shape) for _ in range(count)]
    ptrs = (ctypes.POINTER(ctypes.c_double) * count)(*[_abi.dptr(a) for a in arrs])
    return arrs, ptrs


def greens_function_many(params, hams, precision=None):
    """GreensFunction::compute for several models in one batched Lanczos run: list of G arrays."""
    p = params if isinstance(params, Params) else Params(params)
    h0 = hams[0]
    nw = int(p.num("lanc.NOMEGA"))
    n = h0.nint
    G, gp = _many_outputs(len(hams), (nw, n, 2, 2))
    Gij, gijp = _many_outputs(len(hams), (nw, n * n, 2, 2))
    Z = np.zeros(len(hams))
    g = _gf_params(p, precision or _gf_precision(h0.precision),
                   _orbital_array(h0.data, "GreensFunction_orbitals/values"), h0.max_batch)
    _check(_abi.lib().edgpu_greens_function_many(_model_array(hams), len(hams), ctypes.byref(g), gp, gijp,
                                                 _abi.dptr(Z)), h0._ctx)
    return [a[..., 0] + 1j * a[..., 1] for a in G], [a[..., 0] + 1j * a[..., 1] for a in Gij], Z


def chiloc_many(params, hams, op="Sz", avgs=None, precision=None):
    """ChiLoc::compute<Op> for several models in one batched Lanczos run: list of chi arrays."""
    p = params if isinstance(params, Params) else Params(params)
    h0 = hams[0]
    nw = int(p.num("lanc.NOMEGA"))
    n = h0.nint
    if avgs is None:
        avgs = [0.0 if op == "Sz" else 1.0] * len(hams)
    av = np.ascontiguousarray(avgs, dtype=np.float64)
    C, cp = _many_outputs(len(hams), (nw, n, 2))
    Cij, cijp = _many_outputs(len(hams), (nw, n * n, 2))
    Z = np.zeros(len(hams))
    g = _gf_params(p, precision or _gf_precision(h0.precision), _orbital_array(h0.data, "ChiLoc_orbitals/values"),
                   h0.max_batch)
    _check(_abi.lib().edgpu_chiloc_many(_model_array(hams), len(hams), ctypes.byref(g), _abi.OPERATORS[op],
                                        _abi.dptr(av), cp, cijp, _abi.dptr(Z)), h0._ctx)
    return [a[..., 0] + 1j * a[..., 1] for a in C], [a[..., 0] + 1j * a[..., 1] for a in Cij], Z


def refine_eigenpairs(hams, beta, cutoff):
    """FP64 continuation of an FP32 diag for the pairs kept at inverse temperature beta (Boltzmann weight not
    below cutoff), for several Hamiltonians of one context at once (edgpu_refine_eigenpairs).  Returns the
    status (1 when a sector's continuation did not converge and its pairs kept their FP32 vectors)."""
    return _check(_abi.lib().edgpu_refine_eigenpairs(_model_array(hams), len(hams), float(beta), float(cutoff)),
                  hams[0]._ctx)


def lanczos(ham, sector, starts, nlanc, storage=None, precision=None):
    """Lanczos recurrences (Lanczos.h:36-77) of normalised start vectors in one sector: (alpha, beta, nlanc)."""
    starts = np.ascontiguousarray(np.atleast_2d(starts), dtype=np.float64)
    cnt = starts.shape[0]
    a = np.zeros((cnt, nlanc))
    b = np.zeros((cnt, nlanc + 1))
    nl = np.zeros(cnt, dtype=np.int32)
    _check(_abi.lib().edgpu_lanczos(ham._m, _abi.STORAGES[storage or ham.storage.kind], sector[0], sector[1],
                                    _abi.dptr(starts), cnt, nlanc,
                                    _abi.PRECISIONS[precision or _gf_precision(ham.precision)],
                                    _abi.dptr(a), _abi.dptr(b), _abi.iptr(nl)), ham._ctx)
    return a, b, nl


def frac_points(alpha, beta, nlanc, isign, expectation, expb, ener, device=0):
    """get_frac_point (Lanczos.h:201-224) evaluated on the GPU for complex energies `ener`."""
    ctx = context(device)
    ener = np.asarray(ener, dtype=complex)
    e = np.ascontiguousarray(np.stack([ener.real, ener.imag], -1).reshape(-1))
    out = np.zeros(e.size)
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    b = np.ascontiguousarray(beta, dtype=np.float64)
    _check(_abi.lib().edgpu_frac_points(ctx, _abi.dptr(a), _abi.dptr(b), nlanc, isign, expectation, expb,
                                        _abi.dptr(e), ener.size, _abi.dptr(out)), ctx)
    return out[0::2] + 1j * out[1::2]


class Server:
    """Continuous-batching request loop (edgpu_server_*): Hamiltonian::diag (+ GreensFunction::compute)
    requests of any size are admitted in arrival order while their eigen-solver footprint fits the
    device-memory budget; their sectors join one running lock-step eigen-solver batch between restart
    cycles and leave it as they converge; a request's Green's function runs when its spectrum is complete.
    Each result equals the same solve alone.  Drive it with step(); poll() / done() report progress."""

    DONE = 2

    def __init__(self, precision="fp32", hbm_budget=0, device=0):
        self._ctx = context(device)
        h = ctypes.c_void_p()
        _check(_abi.lib().edgpu_server_create(self._ctx, _abi.PRECISIONS[precision], int(hbm_budget),
                                              ctypes.byref(h)), self._ctx)
        self._s = h
        self.precision = precision
        self._reqs = {}

    def submit(self, ham, gf=True):
        """Queue ham (a Hamiltonian of this device) for diag and, with gf, its Green's function; returns a
        ticket.  The Hamiltonian's multiplicity_check applies."""
        p = ham.p
        dp = _diag_params(ham)
        keep = []
        if p.exists("arpack.SECTOR") and p.num("arpack.SECTOR"):
            sec = np.ascontiguousarray(np.asarray(ham.data["sectors/values"]).reshape(-1, 2), dtype=np.int32)
            dp.sectors = _abi.iptr(sec)
            dp.n_sectors = sec.shape[0]
            keep.append(sec)
        G = Gij = None
        Z = np.zeros(1)
        gptr = None
        if gf:
            nw, n = int(p.num("lanc.NOMEGA")), ham.nint
            G = np.zeros((nw, n, 2, 2))
            Gij = np.zeros((nw, n * n, 2, 2))
            orbs = _orbital_array(ham.data, "GreensFunction_orbitals/values")
            keep.append(orbs)
            g = _gf_params(p, _gf_precision(self.precision), orbs)
            keep.append(g)
            gptr = ctypes.byref(g)
        t = ctypes.c_longlong(0)
        _check(_abi.lib().edgpu_server_submit(self._s, ham._m, ctypes.byref(dp), gptr,
                                              _abi.dptr(G) if G is not None else None,
                                              _abi.dptr(Gij) if Gij is not None else None, _abi.dptr(Z),
                                              ctypes.byref(t)), self._ctx)
        self._reqs[t.value] = {"ham": ham, "G": G, "Gij": Gij, "Z": Z, "keep": keep + [dp], "state": 0}
        return t.value

    def step(self):
        """One scheduling round; returns (running, queued)."""
        r, q = ctypes.c_int(0), ctypes.c_int(0)
        _check(_abi.lib().edgpu_server_step(self._s, ctypes.byref(r), ctypes.byref(q)), self._ctx)
        return r.value, q.value

    def poll(self, ticket):
        """0 queued, 1 running, 2 done, < 0 failed (edgpu status)."""
        req = self._reqs[ticket]
        if req["state"] == self.DONE or req["state"] < 0:
            return req["state"]
        st, n = ctypes.c_int(0), ctypes.c_int(0)
        _check(_abi.lib().edgpu_server_poll(self._s, ticket, ctypes.byref(st), ctypes.byref(n)), self._ctx)
        req["state"] = st.value
        if st.value == self.DONE:
            req["ham"]._load_pairs(n.value)
        return st.value

    def result(self, ticket):
        """(Hamiltonian with its eigen-pairs, G, G_ij, Z) of a finished request."""
        req = self._reqs[ticket]
        if self.poll(ticket) != self.DONE:
            raise RuntimeError("request %d is not done" % ticket)
        G = req["G"][..., 0] + 1j * req["G"][..., 1] if req["G"] is not None else None
        Gij = req["Gij"][..., 0] + 1j * req["Gij"][..., 1] if req["Gij"] is not None else None
        return req["ham"], G, Gij, float(req["Z"][0])

    def close(self):
        if getattr(self, "_s", None):
            _abi.lib().edgpu_server_destroy(self._s)
            self._s = None
