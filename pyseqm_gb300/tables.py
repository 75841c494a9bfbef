"""Element tables and MNDO/AM1/PM3 parameters (loaded once from ``data/*.json``)."""

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
}


@functools.lru_cache(maxsize=None)
def elements():
    with open(os.path.join(_DATA, "elements.json")) as f:
        d = json.load(f)
    return {k: np.asarray(v, dtype=np.float64) for k, v in d.items()}


@functools.lru_cache(maxsize=None)
def method_table(method):
    """(fields, rows[Zmax+1, nfields]) of the method's MOPAC parameter file."""
    if method not in METHOD_FIELDS:
        raise ValueError(f"unsupported method {method!r}; supported: MNDO, AM1, PM3")
    with open(os.path.join(_DATA, f"params_{method}.json")) as f:
        d = json.load(f)
    return tuple(d["fields"]), np.asarray(d["rows"], dtype=np.float64)
