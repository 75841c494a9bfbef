"""The xyz helpers against the reference's own read_xyz / save_xyz output (no GPU)."""

import json
import os
from types import SimpleNamespace

import numpy as np
import torch

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden():
    with open(os.path.join(GOLDEN, "io_xyz.json")) as f:
        return json.load(f)


def test_read_xyz_matches_reference(tmp_path):
    """Symbols and the reference's atom ordering (decreasing Z, stable) and zero padding."""
    from pyseqm_gb300 import read_xyz

    g = _golden()
    for n, text in g["xyz"].items():
        (tmp_path / n).write_text(text)
    for group, ref in g["read"].items():
        sp, c = read_xyz([str(tmp_path / n) for n in group.split("+")])
        np.testing.assert_array_equal(sp, np.asarray(ref["species"]))
        np.testing.assert_array_equal(c, np.asarray(ref["coords"]))
    # sort=False keeps the file's order
    (tmp_path / "hoc.xyz").write_text("3\n\nH 0 0 1\nO 0 0 0\nC 1 0 0\n")
    sp, c = read_xyz([str(tmp_path / "hoc.xyz")], sort=False)
    assert sp.tolist() == [[1, 8, 6]] and c[0, 2, 0] == 1.0
    sp, _ = read_xyz([str(tmp_path / "hoc.xyz")])
    assert sp.tolist() == [[8, 6, 1]]


def test_save_xyz_writes_the_reference_files(tmp_path):
    """Byte-identical files to the reference's save_xyz, with and without forces."""
    from pyseqm_gb300 import Constants, save_xyz

    g = _golden()
    f64 = dict(dtype=torch.float64)
    mol = SimpleNamespace(species=torch.as_tensor(g["species"]), coordinates=torch.as_tensor(g["coords"], **f64),
                          Etot=torch.as_tensor(g["Etot"], **f64), force=torch.as_tensor(g["force"], **f64),
                          const=Constants())
    for forces in (False, True):
        save_xyz(mol, str(tmp_path / "out"), Forces=forces)
        for i in range(len(g["species"])):
            assert (tmp_path / f"out.{i}.xyz").read_text() == g["saved"][f"{int(forces)}.{i}"]


def test_read_xyz_trajectory_matches_reference(tmp_path):
    """read_xyz_trajectory against the reference's outputs: slices, evenly spaced frames,
    explicit (negative, repeated) indices, velocities, unsorted, symbol and numeric columns; and
    the argument checks."""
    import pytest

    from pyseqm_gb300 import read_xyz_trajectory

    with open(os.path.join(GOLDEN, "io_traj.json")) as f:
        g = json.load(f)
    for fn, text in g["texts"].items():
        (tmp_path / fn).write_text(text)
    for case in g["cases"]:
        got = read_xyz_trajectory(str(tmp_path / case["file"]), **case["kwargs"])
        assert len(got) == len(case["result"]), case["kwargs"]
        for a, b in zip(got, case["result"]):
            np.testing.assert_array_equal(a, np.asarray(b).reshape(a.shape), err_msg=str(case["kwargs"]))
    full = read_xyz_trajectory(str(tmp_path / "coords.xyz"))
    assert full[0].shape == (6, 5)  # stop None: to the end of the file
    with pytest.raises(ValueError):
        read_xyz_trajectory(str(tmp_path / "coords.xyz"), indices=[0], num=2)
    with pytest.raises(ValueError):
        read_xyz_trajectory(str(tmp_path / "coords.xyz"), num=2, step=2)
    with pytest.raises(FileNotFoundError):
        read_xyz_trajectory(str(tmp_path / "coords.xyz"), stop=2, return_vel=True, vel_file=str(tmp_path / "x"))
