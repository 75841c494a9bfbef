"""Regenerate the element and method-parameter tables shipped in this folder.

The MNDO/AM1/PM3/PM6_SP parameter values, the PM6 diatomic core-core parameters and the
per-element constants (valence charge, principal quantum number, isolated-atom energy
coefficients, experimental atomic heats of formation, masses, the atomic numbers of the
PM6 core-core term) are published semi-empirical data.  Reproducing the
reference energies bit-for-bit requires the very same numbers, so this script
reads them from a PYSEQM checkout and writes them as JSON:

  * ``elements.json``      <- seqm/seqm_functions/constants.py:68-216 (tables only)
  * ``params_<M>.json``    <- seqm/params/parameters_<M>_MOPAC.csv, parsed the way
                              seqm/seqm_functions/parameters.py:4-46 parses them
                              (float64 here; the reference parses into the torch
                              default dtype).
  * ``grimme_2006_b97d.json`` <- seqm/params/grimme_2006_b97-d.csv (C6, R0 of AM1-FS1)
  * ``pwcct_<M>.json``     <- seqm/params/PWCCT_<M>_MOPAC.csv (PM6_SP), parsed the way
                              PWCCT (parameters.py:49-87) parses it: alp[Z1][Z2] is the
                              third column, chi[Z1][Z2] the fourth, for the listed (Z1, Z2)
                              order only (the nonzero entries are stored).

Usage:  python pyseqm_gb300/data/make_tables.py /path/to/PYSEQM
The script is only needed when the tables change; the JSON files are committed.
"""

import json
import os
import sys

METHOD_FIELDS = {
    # seqm/basics.py:35-95 (parameterlist for the sp methods)
    "MNDO": ["U_ss", "U_pp", "zeta_s", "zeta_p", "beta_s", "beta_p", "g_ss", "g_sp", "g_pp", "g_p2",
             "h_sp", "alpha"],
    "AM1": ["U_ss", "U_pp", "zeta_s", "zeta_p", "beta_s", "beta_p", "g_ss", "g_sp", "g_pp", "g_p2",
            "h_sp", "alpha",
            "Gaussian1_K", "Gaussian2_K", "Gaussian3_K", "Gaussian4_K",
            "Gaussian1_L", "Gaussian2_L", "Gaussian3_L", "Gaussian4_L",
            "Gaussian1_M", "Gaussian2_M", "Gaussian3_M", "Gaussian4_M"],
    "PM3": ["U_ss", "U_pp", "zeta_s", "zeta_p", "beta_s", "beta_p", "g_ss", "g_sp", "g_pp", "g_p2",
            "h_sp", "alpha",
            "Gaussian1_K", "Gaussian2_K", "Gaussian1_L", "Gaussian2_L", "Gaussian1_M", "Gaussian2_M"],
    # seqm/basics.py:132-162: the fields of PM6_SP its sp-basis path reads (the orbital
    # exponent tails, F0SD, G2SD and EISOL only enter the d-orbital method)
    "PM6_SP": ["U_ss", "U_pp", "zeta_s", "zeta_p", "beta_s", "beta_p", "g_ss", "g_sp", "g_pp", "g_p2",
               "h_sp", "rho_core", "alpha",
               "Gaussian1_K", "Gaussian2_K", "Gaussian3_K", "Gaussian4_K",
               "Gaussian1_L", "Gaussian2_L", "Gaussian3_L", "Gaussian4_L",
               "Gaussian1_M", "Gaussian2_M", "Gaussian3_M", "Gaussian4_M"],
}
PAIR_METHODS = ("PM6_SP",)


def read_csv(path, fields):
    with open(path) as f:
        header = f.readline().strip().replace(" ", "").split(",")
        col = [header.index(x) for x in fields]
        table = {}
        for line in f:
            t = line.strip().replace(" ", "").split(",")
            if not t or not t[0]:
                continue
            try:
                table[int(t[0])] = [float(t[c]) for c in col]
            except ValueError:
                # a malformed row (PM6_SP's Re row merges two fields); the reference only
                # fails on it when that element is requested, and it is outside the sp set
                continue
    return table


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    for method, fields in METHOD_FIELDS.items():
        tab = read_csv(os.path.join(ref_root, "seqm", "params", f"parameters_{method}_MOPAC.csv"), fields)
        zmax = max(tab)
        rows = [tab.get(z, [0.0] * len(fields)) for z in range(zmax + 1)]
        with open(os.path.join(here, f"params_{method}.json"), "w") as f:
            json.dump({"method": method, "fields": fields, "rows": rows}, f, indent=0)
    for method in PAIR_METHODS:
        entries = []
        with open(os.path.join(ref_root, "seqm", "params", f"PWCCT_{method}_MOPAC.csv")) as f:
            for line in f:
                t = line.strip().replace(" ", "").split(",")
                if len(t) >= 4 and t[0]:
                    entries.append((int(t[0]), int(t[1]), float(t[2]), float(t[3])))
        nonzero = [list(e) for e in entries if e[2] != 0.0 or e[3] != 0.0]
        with open(os.path.join(here, f"pwcct_{method}.json"), "w") as f:
            json.dump({"method": method, "zmax": max(max(e[0], e[1]) for e in entries),
                       "columns": ["Z1", "Z2", "alp", "chi"], "entries": nonzero}, f, separators=(",", ":"))

    # C6 (J nm^6 / mol) and R0 (Angstrom) of Grimme's 2006 dispersion correction, which AM1-FS1
    # reads (dispersion_am1_fs1.py:77-113); the file starts with a byte-order mark
    c6r0 = {}
    with open(os.path.join(ref_root, "seqm", "params", "grimme_2006_b97-d.csv"), encoding="utf-8-sig") as f:
        f.readline()
        for line in f:
            t = line.strip().replace(" ", "").split(",")
            if len(t) >= 4 and t[0]:
                c6r0[int(t[0])] = [float(t[2]), float(t[3])]
    zmax = max(c6r0)
    with open(os.path.join(here, "grimme_2006_b97d.json"), "w") as f:
        json.dump({"columns": ["C_6", "R_0"], "rows": [c6r0.get(z, [0.0, 0.0]) for z in range(zmax + 1)]}, f)

    sys.path.insert(0, ref_root)
    import types

    import torch

    # the reference package imports h5py at load time (trajectory files); a stub suffices here
    h5 = types.ModuleType("h5py")
    h5.Group = h5.File = h5.Dataset = type("Stub", (), {})
    sys.modules.setdefault("h5py", h5)

    # the tables are built with the torch default dtype; the reference's own tests
    # run with float64 (tests/conftest.py:29), which is what the energies assume
    torch.set_default_dtype(torch.float64)
    from seqm.seqm_functions.constants import Constants

    c = Constants()
    out = {}
    for name in ["tore", "qn", "ussc", "uppc", "gssc", "gspc", "hspc", "gp2c", "gppc", "mass", "atomic_num", "iso",
                 "qnD_int"]:
        out[name] = [float(v) for v in getattr(c, name).tolist()]
    # heats of formation are stored in kcal/mol; the reference divides by 23.061 at load
    out["label"] = list(c.label)  # element symbols as the reference's tables spell them
    out["eheat_kcal"] = [float(v) * 23.061 for v in c.eheat.tolist()]
    out["eheat_ev"] = [float(v) for v in c.eheat.tolist()]
    with open(os.path.join(here, "elements.json"), "w") as f:
        json.dump(out, f, indent=0)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_tables.py <path to the PYSEQM source tree>")
    main(sys.argv[1])
