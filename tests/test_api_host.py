"""Host-side logic of the drop-in API (no GPU): parser outputs, option checks, errors."""

import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import seqm_oracle as O


def test_parser_matches_oracle_parse():
    from pyseqm_gb300 import Constants, Molecule

    g = load_golden("mixed_am1")
    s = dict(g["settings"])
    mol = Molecule(Constants(), s, torch.as_tensor(g["coords_np"]), torch.as_tensor(g["species_np"]))
    ref = O.parse(g["species_np"], g["coords_np"])
    for a, b in [("idxi", "idxi"), ("idxj", "idxj"), ("ni", "ni"), ("nj", "nj"), ("mask", "mask"),
                 ("maskd", "maskd"), ("Z", "Z"), ("atom_molid", "atom_molid"), ("pair_molid", "pair_molid"),
                 ("nHeavy", "nheavy"), ("nHydro", "nhyd"), ("nocc", "nocc")]:
        np.testing.assert_array_equal(getattr(mol, a).cpu().numpy(), ref[b])
    np.testing.assert_allclose(mol.rij.cpu().numpy(), ref["rij"], rtol=1e-15, atol=1e-14)
    np.testing.assert_allclose(mol.xij.cpu().numpy(), ref["xij"], rtol=1e-14, atol=1e-15)
    # written into the caller's dict exactly like the reference (padding 0 included, Molecule.py:51-53)
    assert s["elements"] == [0] + sorted(set(g["species_np"].reshape(-1).tolist()))


def test_layout_reference_pair_order_roundtrip():
    from pyseqm_gb300.layout import Layout

    g = load_golden("mixed_am1")
    L = Layout.from_padded(g["species_np"], g["coords_np"], "AM1")
    ri, rj = L.reference_pair_atoms()
    ref = O.parse(g["species_np"], g["coords_np"])
    np.testing.assert_array_equal(ri, ref["idxi"])
    np.testing.assert_array_equal(rj, ref["idxj"])


def test_rejects_unsorted_species_and_odd_electrons():
    from pyseqm_gb300 import Constants, Molecule

    with pytest.raises(ValueError, match="non-increasing"):
        Molecule(Constants(), {"method": "AM1", "scf_eps": 1e-6, "scf_converger": [1]},
                 torch.zeros(1, 2, 3, dtype=torch.float64), torch.tensor([[1, 6]]))
    with pytest.raises(ValueError, match="closed shell"):
        Molecule(Constants(), {"method": "AM1", "scf_eps": 1e-6, "scf_converger": [1]},
                 torch.rand(1, 4, 3, dtype=torch.float64), torch.tensor([[6, 1, 1, 1]]))


@pytest.mark.parametrize("opt", [{"UHF": True}, {"method": "PM6"}, {"scf_backward": 1}, {"scf_converger": [2]},
                                 {"excited_states": {"n_states": 2}}])
def test_unsupported_options_raise(opt):
    from pyseqm_gb300 import Constants, Molecule

    s = {"method": "AM1", "scf_eps": 1e-6, "scf_converger": [1]}
    s.update(opt)
    with pytest.raises(NotImplementedError):
        Molecule(Constants(), s, torch.rand(1, 5, 3, dtype=torch.float64), torch.tensor([[6, 1, 1, 1, 1]]))


def test_unsupported_element_raises():
    from pyseqm_gb300.layout import Layout

    with pytest.raises(ValueError):
        Layout.from_padded(np.array([[35, 1]]), np.array([[[0, 0, 0], [1.4, 0, 0.0]]]), "AM1")


def test_workload_generators_are_seeded_and_sorted():
    from pyseqm_gb300 import workloads

    a = workloads.mixed_batch(6, seed=9)
    b = workloads.mixed_batch(6, seed=9)
    for (s1, c1), (s2, c2) in zip(a, b):
        np.testing.assert_array_equal(s1, s2)
        np.testing.assert_array_equal(c1, c2)
        assert np.all(s1[:-1] >= s1[1:])
