import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built native library")


def load_golden(name):
    with open(os.path.join(GOLDEN, f"{name}.json")) as f:
        g = json.load(f)
    g["species_np"] = np.asarray(g["species"], dtype=np.int64)
    g["coords_np"] = np.asarray(g["coords"], dtype=np.float64)
    return g


# single-point fixtures (molecular dynamics trajectories, md_*, and excited states, cis_* / rpa_*,
# have their own tests)
GOLDEN_NAMES = sorted(f[:-5] for f in os.listdir(GOLDEN)
                      if f.endswith(".json") and not f.startswith(("md_", "cis_", "rpa_", "pdir_", "disp_", "io_")))


def write_param_dir(g, path):
    """The parameter files a parameter_file_dir fixture carries, written into path."""
    import os

    for fn, text in g["param_files"].items():
        with open(os.path.join(path, fn), "w") as f:
            f.write(text + "\n")
    return str(path) + os.sep
