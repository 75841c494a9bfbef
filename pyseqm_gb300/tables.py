"""Element tables, MNDO/AM1/PM3/PM6_SP parameters and the PM6 diatomic core-core parameters
(loaded once from ``data/*.json``)."""

import functools
import json
import os

import numpy as np

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")

EV = 27.21  # eV per hartree used by MOPAC (seqm/seqm_functions/constants.py:4)
A0 = 0.529167  # bohr radius in Angstrom (constants.py:9)
EV_KCALPMOL = 23.061  # constants.py:10

# parameters each method reads (seqm/basics.py:35-95)
METHOD_FIELDS = {
    "MNDO": ["U_ss", "U_pp", "zeta_s", "zeta_p", "beta_s", "beta_p", "g_ss", "g_sp", "g_pp", "g_p2", "h_sp", "alpha"],
    "AM1": ["U_ss", "U_pp", "zeta_s", "zeta_p", "beta_s", "beta_p", "g_ss", "g_sp", "g_pp", "g_p2", "h_sp", "alpha",
            "Gaussian1_K", "Gaussian2_K", "Gaussian3_K", "Gaussian4_K", "Gaussian1_L", "Gaussian2_L", "Gaussian3_L",
            "Gaussian4_L", "Gaussian1_M", "Gaussian2_M", "Gaussian3_M", "Gaussian4_M"],
    "PM3": ["U_ss", "U_pp", "zeta_s", "zeta_p", "beta_s", "beta_p", "g_ss", "g_sp", "g_pp", "g_p2", "h_sp", "alpha",
            "Gaussian1_K", "Gaussian2_K", "Gaussian1_L", "Gaussian2_L", "Gaussian1_M", "Gaussian2_M"],
    # PM6 parameters on the sp basis (basics.py:132-162); the fields its sp path reads
    "PM6_SP": ["U_ss", "U_pp", "zeta_s", "zeta_p", "beta_s", "beta_p", "g_ss", "g_sp", "g_pp", "g_p2", "h_sp",
               "rho_core", "alpha",
               "Gaussian1_K", "Gaussian2_K", "Gaussian3_K", "Gaussian4_K", "Gaussian1_L", "Gaussian2_L", "Gaussian3_L",
               "Gaussian4_L", "Gaussian1_M", "Gaussian2_M", "Gaussian3_M", "Gaussian4_M"],
}
# methods whose core-core repulsion reads diatomic (alpha, chi) parameters (parameters.py:49-87)
PAIR_METHODS = ("PM6_SP",)
SUPPORTED = ", ".join(METHOD_FIELDS)


@functools.lru_cache(maxsize=None)
def elements():
    with open(os.path.join(_DATA, "elements.json")) as f:
        d = json.load(f)
    return {k: np.asarray(v, dtype=np.float64) for k, v in d.items()}


@functools.lru_cache(maxsize=None)
def method_table(method):
    """(fields, rows[Zmax+1, nfields]) of the method's MOPAC parameter file."""
    if method not in METHOD_FIELDS:
        raise ValueError(f"unsupported method {method!r}; supported: {SUPPORTED}")
    with open(os.path.join(_DATA, f"params_{method}.json")) as f:
        d = json.load(f)
    return tuple(d["fields"]), np.asarray(d["rows"], dtype=np.float64)


@functools.lru_cache(maxsize=None)
def pair_table(method):
    """(alp, chi), each (zmax+1, zmax+1), indexed [Z of the pair's first (heavier or equal) atom,
    Z of the second] as the PM6 core-core term reads them (energy.py:135-171); None for methods
    without diatomic parameters."""
    if method not in PAIR_METHODS:
        return None
    with open(os.path.join(_DATA, f"pwcct_{method}.json")) as f:
        d = json.load(f)
    n = int(d["zmax"]) + 1
    alp, chi = np.zeros((n, n)), np.zeros((n, n))
    for z1, z2, a, c in d["entries"]:
        alp[int(z1), int(z2)], chi[int(z1), int(z2)] = a, c
    return alp, chi


def pair_par(method):
    """Device table of the PM6 core-core pair terms, (zmax+1)^2 x 3 doubles: (alp, chi,
    atomic_num(Z1)^(1/3) + atomic_num(Z2)^(1/3)) at [Z1 * (zmax+1) + Z2]; None if unused."""
    t = pair_table(method)
    if t is None:
        return None
    alp, chi = t
    n = alp.shape[0]
    an = np.zeros(n)
    src = elements()["atomic_num"]
    an[: min(n, src.size)] = src[: min(n, src.size)]
    c = an ** (1.0 / 3.0)
    return np.stack([alp, chi, c[:, None] + c[None, :]], axis=-1).reshape(-1), n - 1
