"""Model inputs in EDLib's dataset vocabulary.

A model input is a pair ``(params, data)``: ``params`` maps EDLib parameter names
(include/edlib/EDParams.h:11-37, e.g. ``NSITES``, ``arpack.NEV``, ``lanc.BETA``) to values and
``data`` maps the dataset paths EDLib reads from its INPUT_FILE to numpy arrays:

* Hubbard (include/edlib/HubbardModel.h:55-67): ``hopping/values`` [Ns][Ns] (t_ij with
  H = -sum t_ij c+_j c_i), ``interaction/values`` [Ns], ``chemical_potential/values`` [Ns]
  (only entries 0 and 1 are read, indexed by spin), optional ``magnetic_field/values`` [Ns]
  and ``exchange/values`` [Ns][Ns].
* Single-impurity Anderson (include/edlib/SingleImpurityAndersonModel.h:199-222):
  ``Bath/Epsk/values`` [Nk][2], ``Bath/Vk_<m>/values`` [Nk][2], ``H0_<m>/values`` [ml][2],
  ``mu`` (scalar), ``interaction/values`` [2][2][ml][ml][ml][ml].
* optional ``sectors/values`` [n][2] (with ``arpack.SECTOR``), ``GreensFunction_orbitals/values``
  and ``ChiLoc_orbitals/values`` [n][2].

HDF5 is not available, so the same content is exchanged as a small text file
(``write_input`` / ``read_input``): lines ``param KEY VALUE`` and
``data PATH NDIM DIM... VALUES...``.
"""
import numpy as np

HUBBARD = "HUBBARD"
SIAM = "SIAM"


def model_kind(data):
    return SIAM if "Bath/Epsk/values" in data else HUBBARD


def write_input(path, params, data):
    with open(path, "w") as f:
        for k, v in params.items():
            f.write("param %s %s\n" % (k, v))
        for k, v in data.items():
            a = np.asarray(v, dtype=np.float64)
            f.write("data %s %d %s %s\n" % (k, a.ndim, " ".join(str(s) for s in a.shape),
                                            " ".join(repr(float(x)) for x in a.reshape(-1))))


def read_input(path):
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
            raise ValueError("bad token in model input: %r" % t)
    return params, data


# ------------------------------------------------------------------------------ Hubbard
def hubbard(t, U, mu, hmag=None, J=None):
    """Dataset dict for a Hubbard cluster with hopping matrix t (EDLib sign convention)."""
    t = np.asarray(t, dtype=np.float64)
    ns = t.shape[0]
    d = {"hopping/values": t,
         "interaction/values": np.broadcast_to(np.asarray(U, dtype=np.float64), (ns,)).copy(),
         "chemical_potential/values": np.broadcast_to(np.asarray(mu, dtype=np.float64), (ns,)).copy()}
    if hmag is not None:
        d["magnetic_field/values"] = np.broadcast_to(np.asarray(hmag, dtype=np.float64), (ns,)).copy()
    if J is not None:
        d["exchange/values"] = np.asarray(J, dtype=np.float64)
    return d


def ring_hopping(n, t=1.0):
    """Periodic 1D ring with nearest-neighbour hopping value t."""
    h = np.zeros((n, n))
    for i in range(n):
        h[i, (i + 1) % n] = t
        h[(i + 1) % n, i] = t
    return h


def square_hopping(nrows, ncols, t=1.0, tp=0.0):
    """Periodic nrows x ncols square lattice: value t on nearest-neighbour bonds and tp on both
    diagonals (the layout of the reference's plaquette input generators)."""
    n = nrows * ncols
    h = np.zeros((n, n))
    for r in range(nrows):
        for c in range(ncols):
            i = r * ncols + c
            for (dr, dc, v) in ((0, 1, t), (1, 0, t), (1, 1, tp), (1, -1, tp)):
                if v == 0.0:
                    continue
                j = ((r + dr) % nrows) * ncols + (c + dc) % ncols
                h[i, j] = v
                h[j, i] = v
    return h


def lattice_gk(G_ij, nrows, ncols, k):
    """G(k) = (1/N) sum_ij e^{i k (r_i - r_j)} G_ij of a translation-invariant cluster from the row G_0j
    (G_ij as returned for GreensFunction_orbitals (0, j): [nw, N*N, spin]); inversion symmetry leaves the
    cosine part."""
    n = nrows * ncols
    out = 0.0
    for j in range(n):
        r, c = divmod(j, ncols)
        out = out + np.cos(k[0] * r + k[1] * c) * G_ij[:, j, :]
    return out


def lattice_k_weights(nrows, ncols, k):
    """Weight rows cos(k r_j), sin(k r_j) of the orbital combinations whose Green's functions give
    G(k) = (G_cos + G_sin) / N (edgpu_greens_function_weighted)."""
    r = [divmod(j, ncols) for j in range(nrows * ncols)]
    return np.array([[np.cos(k[0] * a + k[1] * b) for a, b in r], [np.sin(k[0] * a + k[1] * b) for a, b in r]])


def plaquette_2x2_gf_chi():
    """2x2 plaquette with t = -1, t' = 0.3, U = 3, mu = 1 (hopping values +1 and -0.3), G and chi
    on orbital 0: the model of the reference's Lanczos golden test."""
    data = hubbard(square_hopping(2, 2, 1.0, -0.3), 3.0, 1.0)
    data["GreensFunction_orbitals/values"] = np.array([[0, 0]], dtype=np.float64)
    data["ChiLoc_orbitals/values"] = np.array([[0, 0]], dtype=np.float64)
    params = {"NSITES": 4, "NSPINS": 2, "arpack.SECTOR": 0, "storage.MAX_SIZE": 864, "storage.MAX_DIM": 36,
              "storage.EIGENVALUES_ONLY": 0, "arpack.NEV": 100, "lanc.BETA": 20, "lanc.EMIN": -4.0,
              "lanc.EMAX": 4.0, "lanc.NOMEGA": 1000}
    return params, data


def ring4_magnetic():
    """4-site ring, t = -1 (value -1 with the reference's sign convention of its input), U = 5,
    mu = 2.5, field H = 0.01: the model of the reference's Hubbard known-answer test."""
    h = -ring_hopping(4, 1.0)
    data = hubbard(h, 5.0, 2.5, hmag=0.01)
    data["sectors/values"] = np.array([[2, 2]], dtype=np.float64)
    params = {"NSITES": 4, "NSPINS": 2, "arpack.SECTOR": 0, "storage.MAX_SIZE": 576, "storage.MAX_DIM": 36,
              "storage.EIGENVALUES_ONLY": 0, "arpack.NEV": 1}
    return params, data


def hubbard_ring8():
    """8-site ring, t = 1 nearest neighbour, U = 4, mu = U/2, all Sz sectors, 10 lowest eigenpairs
    per sector, beta = 50, 200 Matsubara points, 100 Lanczos steps (CRS, FP64)."""
    data = hubbard(ring_hopping(8, 1.0), 4.0, 2.0)
    params = {"NSITES": 8, "NSPINS": 2, "arpack.NEV": 10, "lanc.BETA": 50.0, "lanc.NOMEGA": 200,
              "lanc.NLANC": 100, "lanc.BOLTZMANN_CUTOFF": 1e-12, "storage.MAX_DIM": 4900,
              "storage.MAX_SIZE": 4900 * 17}
    return params, data


def hubbard_4x4(U=8.0, t=1.0, tp=-0.3):
    """Periodic 4x4 Hubbard cluster at half filling, sector (8, 8) only, 4 eigenpairs, NCV 20; G_0j for
    every site j (GreensFunction_orbitals (0, j)), from which G(k) = sum_j cos(k r_j) G_0j."""
    data = hubbard(square_hopping(4, 4, t, tp), U, U / 2.0)
    data["sectors/values"] = np.array([[8, 8]], dtype=np.float64)
    data["GreensFunction_orbitals/values"] = np.array([[0, j] for j in range(16)], dtype=np.float64)
    params = {"NSITES": 16, "NSPINS": 2, "arpack.SECTOR": 1, "arpack.NEV": 4, "arpack.NCV": 20,
              "lanc.BETA": 100.0, "lanc.NOMEGA": 512, "lanc.BOLTZMANN_CUTOFF": 1e-4}
    return params, data


# ------------------------------------------------------------------------------ Anderson
def kanamori(norb, U, J):
    """Kanamori tensor U[i][j][k][l]: U on iiii, U-2J on ijij, J on ijji and iijj (i != j),
    the convention of the reference's Anderson input generator."""
    T = np.zeros((norb,) * 4)
    for i in range(norb):
        T[i, i, i, i] = U
        for j in range(norb):
            if i != j:
                T[i, j, i, j] = U - 2 * J
                T[i, j, j, i] = J
                T[i, i, j, j] = J
    return T


def siam(epsk, vk, h0, mu, U4):
    """Dataset dict for a single-impurity Anderson model.

    epsk [Nk][2]; vk [ml][Nk][2]; h0 [ml][ml][2]; U4 [ml]^4 (spin-independent, copied to all
    four spin blocks as the reference's generator does)."""
    epsk = np.asarray(epsk, dtype=np.float64)
    vk = np.asarray(vk, dtype=np.float64)
    h0 = np.asarray(h0, dtype=np.float64)
    ml = h0.shape[0]
    UU = np.zeros((2, 2) + (ml,) * 4)
    for a in range(2):
        for b in range(2):
            UU[a, b] = U4
    d = {"Bath/Epsk/values": epsk, "mu": float(mu), "interaction/values": UU}
    for m in range(ml):
        d["Bath/Vk_%d/values" % m] = vk[m]
        d["H0_%d/values" % m] = h0[m]
    return d


def random_siam(seed, nbath, U=3.0, eps_range=(-2.0, 2.0), v_range=(0.1, 0.5)):
    """Single-orbital Anderson impurity with nbath bath sites: eps_d = -U/2 (H0 = -U/2, mu = 0),
    bath energies ~ U[eps_range], hybridisations ~ U[v_range] (spin-symmetric), from seed."""
    rng = np.random.default_rng(seed)
    eps = rng.uniform(*eps_range, size=nbath)
    v = rng.uniform(*v_range, size=nbath)
    epsk = np.stack([eps, eps], axis=1)
    vk = np.stack([v, v], axis=1)[None]
    h0 = np.full((1, 1, 2), -U / 2.0)
    data = siam(epsk, vk, h0, 0.0, np.full((1, 1, 1, 1), U))
    params = {"NSITES": 1 + nbath, "NSPINS": 2, "siam.NORBITALS": 1}
    return params, data


def anderson_12(seed=0):
    """Single-orbital Anderson impurity with 11 bath sites (12 orbitals, 24 spin-orbitals), U = 3,
    eps_d = -U/2, eps_k ~ U[-2, 2], V_k ~ U[0.1, 0.5]; all sectors, 8 eigenpairs, beta = 100,
    G and chi on 1024 Matsubara points."""
    params, data = random_siam(seed, 11, U=3.0)
    params.update({"arpack.NEV": 8, "lanc.BETA": 100.0, "lanc.NOMEGA": 1024, "lanc.NLANC": 100,
                   "lanc.BOLTZMANN_CUTOFF": 1e-12})
    return params, data


def random_kanamori_siam(seed, nbath_per_orb=None, norb=3):
    """Three-orbital Kanamori impurity: U ~ U[2, 5], J = U/6, 2-4 bath sites per orbital, bath
    energies ~ U[-2, 2], hybridisations ~ U[0.1, 0.5]; mu at the half-filling point 2.5U - 5J."""
    rng = np.random.default_rng(seed)
    U = rng.uniform(2.0, 5.0)
    J = U / 6.0
    if nbath_per_orb is None:
        nbath_per_orb = [int(x) for x in rng.integers(2, 5, size=norb)]
    nk = int(sum(nbath_per_orb))
    epsk = np.zeros((nk, 2))
    vk = np.zeros((norb, nk, 2))
    k = 0
    for m in range(norb):
        for _ in range(nbath_per_orb[m]):
            e = rng.uniform(-2.0, 2.0)
            v = rng.uniform(0.1, 0.5)
            epsk[k] = (e, e)
            vk[m, k] = (v, v)
            k += 1
    h0 = np.zeros((norb, norb, 2))
    data = siam(epsk, vk, h0, 2.5 * U - 5.0 * J, kanamori(norb, U, J))
    params = {"NSITES": norb + nk, "NSPINS": 2, "siam.NORBITALS": norb}
    return params, data
