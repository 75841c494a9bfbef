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
# PM6_SP with parameters from the user's parameter_file_dir (no packaged table; the reference's
# PWCCT gives it no diatomic parameters, parameters.py:77)
METHOD_FIELDS["PM6_SP_STAR"] = METHOD_FIELDS["PM6_SP"]
# methods with the PM6 core-core repulsion and its (alpha, chi) table
PAIR_METHODS = ("PM6_SP", "PM6_SP_STAR")
SUPPORTED = ", ".join(METHOD_FIELDS)


def read_parameter_csv(path, fields):
    """A MOPAC-format parameter file as parameters.py:4-46 reads it: header names with spaces
    removed, one row per element (first column Z), the requested columns as float64; rows that
    do not parse are left out (the reference only parses the requested elements' rows)."""
    table = {}
    with open(path) as f:
        header = f.readline().strip().replace(" ", "").split(",")
        col = [header.index(x) for x in fields]
        for line in f:
            t = line.strip().replace(" ", "").split(",")
            if not t or not t[0]:
                continue
            try:
                table[int(t[0])] = [float(t[c]) for c in col]
            except ValueError:
                continue
    zmax = max(table) if table else 0
    rows = np.zeros((zmax + 1, len(fields)))
    for z, v in table.items():
        rows[z] = v
    return tuple(fields), rows


def read_pwcct_csv(path):
    """PWCCT_<method>_MOPAC.csv as parameters.py:49-87 reads it: alp[Z1][Z2] the third column,
    chi[Z1][Z2] the fourth, for the listed (Z1, Z2) order."""
    entries = []
    with open(path) as f:
        for line in f:
            t = line.strip().replace(" ", "").split(",")
            if len(t) >= 4 and t[0]:
                entries.append((int(t[0]), int(t[1]), float(t[2]), float(t[3])))
    n = max(max(e[0], e[1]) for e in entries) + 1 if entries else 1
    alp, chi = np.zeros((n, n)), np.zeros((n, n))
    for z1, z2, a, c in entries:
        alp[z1, z2], chi[z1, z2] = a, c
    return alp, chi


@functools.lru_cache(maxsize=None)
def elements():
    with open(os.path.join(_DATA, "elements.json")) as f:
        d = json.load(f)
    return {k: (list(v) if k == "label" else np.asarray(v, dtype=np.float64)) for k, v in d.items()}


@functools.lru_cache(maxsize=None)
def method_table(method, param_dir=None):
    """(fields, rows[Zmax+1, nfields]) of the method's MOPAC parameter file: the packaged table,
    or parameters_<method>_MOPAC.csv in param_dir (seqm_parameters['parameter_file_dir'],
    basics.py:420-427)."""
    if method not in METHOD_FIELDS:
        raise ValueError(f"unsupported method {method!r}; supported: {SUPPORTED}")
    if param_dir is not None:
        return read_parameter_csv(os.path.join(param_dir, f"parameters_{method}_MOPAC.csv"), METHOD_FIELDS[method])
    if method == "PM6_SP_STAR":
        raise FileNotFoundError("PM6_SP_STAR reads its parameters from seqm_parameters['parameter_file_dir']")
    with open(os.path.join(_DATA, f"params_{method}.json")) as f:
        d = json.load(f)
    return tuple(d["fields"]), np.asarray(d["rows"], dtype=np.float64)


@functools.lru_cache(maxsize=None)
def pair_table(method, param_dir=None):
    """(alp, chi), each (zmax+1, zmax+1), indexed [Z of the pair's first (heavier or equal) atom,
    Z of the second] as the PM6 core-core term reads them (energy.py:135-171): the packaged
    table, PWCCT_<method>_MOPAC.csv in param_dir, zeros for PM6_SP_STAR; None for methods
    without the PM6 core-core term."""
    if method not in PAIR_METHODS:
        return None
    if method == "PM6_SP_STAR":
        n = int(elements()["tore"].size)
        return np.zeros((n, n)), np.zeros((n, n))
    if param_dir is not None:
        return read_pwcct_csv(os.path.join(param_dir, f"PWCCT_{method}_MOPAC.csv"))
    with open(os.path.join(_DATA, f"pwcct_{method}.json")) as f:
        d = json.load(f)
    n = int(d["zmax"]) + 1
    alp, chi = np.zeros((n, n)), np.zeros((n, n))
    for z1, z2, a, c in d["entries"]:
        alp[int(z1), int(z2)], chi[int(z1), int(z2)] = a, c
    return alp, chi


def pair_par(method, param_dir=None):
    """Device table of the PM6 core-core pair terms, (zmax+1)^2 x 3 doubles: (alp, chi,
    atomic_num(Z1)^(1/3) + atomic_num(Z2)^(1/3)) at [Z1 * (zmax+1) + Z2]; None if unused."""
    t = pair_table(method, param_dir)
    if t is None:
        return None
    alp, chi = t
    n = alp.shape[0]
    an = np.zeros(n)
    src = elements()["atomic_num"]
    an[: min(n, src.size)] = src[: min(n, src.size)]
    c = an ** (1.0 / 3.0)
    return np.stack([alp, chi, c[:, None] + c[None, :]], axis=-1).reshape(-1), n - 1


@functools.lru_cache(maxsize=None)
def grimme_c6_r0():
    """(C6 [J nm^6 / mol], R0 [Angstrom]) per atomic number of Grimme's 2006 dispersion
    correction (the table AM1-FS1 reads, dispersion_am1_fs1.py:77-113)."""
    with open(os.path.join(_DATA, "grimme_2006_b97d.json")) as f:
        rows = np.asarray(json.load(f)["rows"], dtype=np.float64)
    return rows[:, 0], rows[:, 1]
