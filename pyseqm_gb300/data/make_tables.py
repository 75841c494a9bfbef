"""Regenerate the element and method-parameter tables shipped in this folder.

The MNDO/AM1/PM3 parameter values and the per-element constants (valence charge,
principal quantum number, isolated-atom energy coefficients, experimental atomic
heats of formation, masses) are published semi-empirical data.  Reproducing the
reference energies bit-for-bit requires the very same numbers, so this script
reads them from a PYSEQM checkout and writes them as JSON:

  * ``elements.json``      <- seqm/seqm_functions/constants.py:68-216 (tables only)
  * ``params_<M>.json``    <- seqm/params/parameters_<M>_MOPAC.csv, parsed the way
                              seqm/seqm_functions/parameters.py:4-46 parses them
                              (float64 here; the reference parses into the torch
                              default dtype).

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
}


def read_csv(path, fields):
    with open(path) as f:
        header = f.readline().strip().replace(" ", "").split(",")
        col = [header.index(x) for x in fields]
        table = {}
        for line in f:
            t = line.strip().replace(" ", "").split(",")
            if not t or not t[0]:
                continue
            table[int(t[0])] = [float(t[c]) for c in col]
    return table


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    for method, fields in METHOD_FIELDS.items():
        tab = read_csv(os.path.join(ref_root, "seqm", "params", f"parameters_{method}_MOPAC.csv"), fields)
        zmax = max(tab)
        rows = [tab.get(z, [0.0] * len(fields)) for z in range(zmax + 1)]
        with open(os.path.join(here, f"params_{method}.json"), "w") as f:
            json.dump({"method": method, "fields": fields, "rows": rows}, f, indent=0)

    sys.path.insert(0, ref_root)
    import torch

    # the tables are built with the torch default dtype; the reference's own tests
    # run with float64 (tests/conftest.py:29), which is what the energies assume
    torch.set_default_dtype(torch.float64)
    from seqm.seqm_functions.constants import Constants

    c = Constants()
    out = {}
    for name in ["tore", "qn", "ussc", "uppc", "gssc", "gspc", "hspc", "gp2c", "gppc", "mass"]:
        out[name] = [float(v) for v in getattr(c, name).tolist()]
    # heats of formation are stored in kcal/mol; the reference divides by 23.061 at load
    out["eheat_kcal"] = [float(v) * 23.061 for v in c.eheat.tolist()]
    out["eheat_ev"] = [float(v) for v in c.eheat.tolist()]
    with open(os.path.join(here, "elements.json"), "w") as f:
        json.dump(out, f, indent=0)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
