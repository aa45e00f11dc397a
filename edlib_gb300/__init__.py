"""GB300-native exact diagonalisation: the hot path of EDLib (Hamiltonian x vector for the CRS,
SOCRS and spin-resolved storages, the eigen-solver that replaces ARPACK, the Lanczos continued
fraction for G(i w_n) and chi(i w_n), and the symmetry-sector tables) as sm_103a kernels behind the
C ABI of include/edgpu.h.

``edlib_gb300.models`` needs no GPU; everything in ``edlib_gb300.ed`` runs in libedgpu.so.
"""
from . import models  # noqa: F401

__all__ = ["models", "ed", "Params", "Hamiltonian", "GreensFunction", "ChiLoc", "StaticObservables",
           "define_parameters"]


def __getattr__(name):
    if name in ("ed", "Params", "Hamiltonian", "GreensFunction", "ChiLoc", "StaticObservables", "EigenPair",
                "define_parameters", "lanczos", "frac_points", "context"):
        import importlib
        mod = importlib.import_module(__name__ + ".ed")
        return mod if name == "ed" else getattr(mod, name)
    raise AttributeError(name)
