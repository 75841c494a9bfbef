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
    with pytest.raises(ValueError) as exc:
        Molecule(Constants(), {"method": "AM1", "scf_eps": 1e-6, "scf_converger": [1]},
                 torch.rand(1, 4, 3, dtype=torch.float64), torch.tensor([[6, 1, 1, 1]]))
    # the reference's committed message (tests/reference/rhf_odd_electron_error.json)
    assert str(exc.value) == "RHF setting requires closed shell systems (even number of electrons)"


@pytest.mark.parametrize("opt", [{"UHF": True, "scf_converger": [2]}, {"UHF": True, "sp2": [True, 1e-5]},
                                 {"method": "PM6"}, {"scf_backward": 1}, {"scf_converger": [3]},
                                 {"excited_states": {"n_states": 2}, "UHF": True}])
def test_unsupported_options_raise(opt):
    from pyseqm_gb300 import Constants, Molecule

    s = {"method": "AM1", "scf_eps": 1e-6, "scf_converger": [1]}
    s.update(opt)
    with pytest.raises(NotImplementedError):
        Molecule(Constants(), s, torch.rand(1, 5, 3, dtype=torch.float64), torch.tensor([[6, 1, 1, 1, 1]]))


def test_uhf_occupations_from_multiplicity():
    """Alpha / beta occupations (basics.py:279-294): (nel + mult - 1) / 2 and (nel - mult + 1) / 2,
    a ValueError for an impossible combination, doublets by rounding with HIPNN_automatic_doublet."""
    from pyseqm_gb300 import Constants, Molecule

    s = {"method": "AM1", "scf_eps": 1e-6, "scf_converger": [1], "UHF": True}
    xyz = torch.tensor([[[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]],
                        [[0.0, 0.0, 0.0], [1.2, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]], dtype=torch.float64)
    sp = torch.tensor([[6, 1, 1, 1], [8, 8, 0, 0]])
    mol = Molecule(Constants(), s, xyz, sp, mult=torch.tensor([2.0, 3.0]))
    assert mol.nocc.tolist() == [[4, 3], [7, 5]]
    with pytest.raises(ValueError, match="Invalid charge/multiplicity"):
        Molecule(Constants(), s, xyz, sp, mult=torch.tensor([1.0, 3.0]))
    mol = Molecule(Constants(), dict(s, HIPNN_automatic_doublet=True), xyz, sp, mult=torch.tensor([1.0, 1.0]))
    assert mol.nocc.tolist() == [[4, 3], [6, 6]]


def test_unsupported_element_raises():
    from pyseqm_gb300.layout import Layout

    with pytest.raises(ValueError):
        Layout.from_padded(np.array([[35, 1]]), np.array([[[0, 0, 0], [1.4, 0, 0.0]]]), "AM1")


def test_pm6_pair_table_and_super_heavy_count():
    """The PM6_SP diatomic table the kernels read: (alp, chi, cbrt Z1 + cbrt Z2) at [Z1, Z2] as the
    oracle reads PWCCT; Pack_Parameters returns the same alp/chi for the listed elements; the
    convergence-test count of 13 <= Z <= 17 atoms per molecule."""
    from pyseqm_gb300 import tables
    from pyseqm_gb300.basics import Pack_Parameters
    from pyseqm_gb300.layout import Layout

    flat, zmax = tables.pair_par("PM6_SP")
    tab = flat.reshape(zmax + 1, zmax + 1, 3)
    alp, chi = O.load_pair_params("PM6_SP", zmax)
    np.testing.assert_array_equal(tab[..., 0], alp)
    np.testing.assert_array_equal(tab[..., 1], chi)
    an = O.load_elements()["atomic_num"]
    assert tab[6, 1, 2] == pytest.approx(6.0 ** (1 / 3) + 1.0)
    assert tab[10, 1, 2] == pytest.approx(an[10] ** (1 / 3) + 1.0)  # the reference's atomic_num[10] is 0
    assert alp[6, 1] > 0 and alp[1, 6] == 0  # the listed (heavier, lighter) order only
    assert tables.pair_par("AM1") is None
    pp = Pack_Parameters({"elements": [0, 1, 6, 8], "method": "PM6_SP"})
    _, a, c = pp(torch.tensor([8, 6, 1]))
    assert a.shape == (9, 9)
    assert float(a[8, 1]) == alp[8, 1] and float(c[6, 6]) == chi[6, 6] and float(a[7, 1]) == 0.0
    sp = np.array([[17, 14, 8, 6, 1, 1, 1], [8, 1, 1, 0, 0, 0, 0]])
    xyz = np.random.default_rng(0).normal(size=sp.shape + (3,)) * 2.0
    L = Layout.from_padded(sp, xyz, "PM6_SP")
    assert L.nsuper.tolist() == [2, 0]
    assert L.pair_par[1] == zmax
    with pytest.raises(NotImplementedError):
        from pyseqm_gb300.basics import _check_options
        _check_options({"method": "PM6"})


def test_parameter_files_read_like_the_packaged_tables(tmp_path):
    """parameter_file_dir: MOPAC-format files (header with spaces, N and symbol columns) read back
    into the packaged values, PWCCT included; PM6_SP_STAR has no packaged table."""
    from pyseqm_gb300 import tables

    fields, rows = tables.method_table("AM1")
    with open(tmp_path / "parameters_AM1_MOPAC.csv", "w") as f:
        f.write("N, sym, " + ", ".join(reversed(fields)) + "\n")
        for z in range(1, rows.shape[0]):
            f.write(f"{z}, X{z}, " + ", ".join(repr(float(v)) for v in reversed(rows[z])) + "\n")
    f2, r2 = tables.method_table("AM1", str(tmp_path))
    assert f2 == fields
    np.testing.assert_array_equal(r2, rows)
    alp, chi = tables.pair_table("PM6_SP")
    with open(tmp_path / "PWCCT_PM6_SP_MOPAC.csv", "w") as f:
        for z1, z2 in zip(*np.nonzero(alp)):
            f.write(f"{z1},{z2},{float(alp[z1, z2])!r},{float(chi[z1, z2])!r}\n")
    a2, c2 = tables.pair_table("PM6_SP", str(tmp_path))
    n = a2.shape[0]
    np.testing.assert_array_equal(a2, alp[:n, :n])
    np.testing.assert_array_equal(c2, chi[:n, :n])
    with pytest.raises(FileNotFoundError):
        tables.method_table("PM6_SP_STAR")
    a3, _ = tables.pair_table("PM6_SP_STAR")
    assert not a3.any()


def test_workload_generators_are_seeded_and_sorted():
    from pyseqm_gb300 import workloads

    a = workloads.mixed_batch(6, seed=9)
    b = workloads.mixed_batch(6, seed=9)
    for (s1, c1), (s2, c2) in zip(a, b):
        np.testing.assert_array_equal(s1, s2)
        np.testing.assert_array_equal(c1, c2)
        assert np.all(s1[:-1] >= s1[1:])


def test_large_molecule_view_for_sp2():
    """SP2 over a mixed batch runs on a compact view of the molecules above the Jacobi limit:
    gathered sizes and occupations, matrix offsets into the full batch ending with its total."""
    from pyseqm_gb300 import workloads
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF

    rng = np.random.default_rng(0)
    mols = [workloads.alkane(3, rng, 0.03), workloads.water_cluster(30, rng), workloads.alkane(2, rng, 0.03),
            workloads.alkane(30, rng, 0.03)]
    L = Layout.from_padded(*workloads.pad_batch(mols), "PM3").to_device("cpu")
    v = BatchSCF(L)._large
    np.testing.assert_array_equal(v["idx"].numpy(), [1, 3])
    np.testing.assert_array_equal(v["norb"].numpy(), L.norb[[1, 3]])
    np.testing.assert_array_equal(v["nocc"].numpy(), L.nocc[[1, 3]])
    np.testing.assert_array_equal(v["mat_off"].numpy(), [L.mat_off[1], L.mat_off[3], L.mat_off[-1]])
    assert v["struct"].nmol == 2 and v["struct"].max_norb == 182
    assert v["struct"].mol_mat_off == v["mat_off"].data_ptr()
    # a batch of large molecules only needs no view
    L2 = Layout.from_padded(*workloads.pad_batch(mols[1::2]), "PM3").to_device("cpu")
    assert BatchSCF(L2)._large is None


def test_size_classes_of_scheduling_order():
    """Per-molecule kernels launch once per size class of mol_order (descending norb): class
    ends and the largest norb of each class, empty classes dropped."""
    from pyseqm_gb300 import native
    from pyseqm_gb300.layout import set_size_classes

    b = native.SeqmBatch()
    set_size_classes(b, np.array([144, 120, 97, 96, 70, 40, 33, 8, 6]))
    assert b.nclass == 4
    assert list(b.class_end) == [2, 3, 5, 9]
    assert list(b.class_norb) == [144, 97, 96, 40]
    set_size_classes(b, np.array([120, 60, 50, 12]))
    assert b.nclass == 2 and list(b.class_end)[:2] == [1, 4] and list(b.class_norb)[:2] == [120, 60]
    set_size_classes(b, np.zeros(0, dtype=np.int64))
    assert b.nclass == 0


def test_md_host_logic_matches_oracle():
    """MD driver host logic on the CPU: momentum removal (centre of mass and rotation, pseudo-
    inverse of the inertia tensor), kinetic energy, temperature and the Langevin factors against
    the oracle's restatement; file outputs are refused."""
    from pyseqm_gb300 import Constants, Molecular_Dynamics_Basic, Molecular_Dynamics_Langevin, Molecule
    from oracle import seqm_md as MD

    g = load_golden("md_am1_verlet")
    s = dict(g["settings"])
    mol = Molecule(Constants(), s, torch.as_tensor(g["coords_np"]), torch.as_tensor(g["species_np"]))
    v0 = np.asarray(g["velocities0"])
    mol.velocities = torch.as_tensor(v0.copy())
    md = Molecular_Dynamics_Basic(s, timestep=0.5, output={"print every": 0, "checkpoint every": 0})
    md.set_dof(mol)
    md._zero_com(mol, restore_kinetic_energy=False)
    mass = MD.masses(g["species_np"])
    want = MD.zero_com(mass, g["coords_np"], v0, restore_kinetic_energy=False)
    np.testing.assert_allclose(mol.velocities.numpy(), want, atol=1e-14, rtol=0)
    ek = md._kinetic_energy(mol).numpy()
    np.testing.assert_allclose(ek, MD.kinetic_energy(mass, want), rtol=1e-13)
    np.testing.assert_allclose(md._calc_temperature(torch.as_tensor(ek)).numpy(),
                               MD.temperature(ek, 3.0 * (g["species_np"] > 0).sum(1)), rtol=1e-13)
    lg = Molecular_Dynamics_Langevin(damp=5.0, seqm_parameters=s, timestep=0.5, Temp=300.0,
                                     output={"print every": 0, "checkpoint every": 0})
    dt, damp = 0.5, 5.0
    s_ = torch.as_tensor(-dt / damp, dtype=torch.float64)
    lg.langevin_c1 = torch.exp(0.5 * s_)
    assert abs(float(lg.langevin_c1) - np.exp(-0.5 * dt / damp)) < 1e-15
    with pytest.raises(NotImplementedError):
        Molecular_Dynamics_Basic(s, output={"xyz": 10})


def test_layout_edge_cases_match_the_oracle_parse():
    """Single-atom molecules, hydrogen-only and hydrogen-free molecules, and a pair cutoff that
    removes every pair of one molecule: the kept pairs in the reference's order equal the oracle
    parser's, counts and offsets stay consistent."""
    from pyseqm_gb300.layout import Layout

    species = np.array([[6, 0, 0, 0], [1, 1, 0, 0], [8, 8, 0, 0], [7, 6, 1, 0], [8, 1, 1, 0]])
    rng = np.random.default_rng(3)
    coords = rng.normal(size=species.shape + (3,)) * 1.2
    coords[2, 1] = coords[2, 0] + [6.0, 0.0, 0.0]  # the O2 pair lies beyond the 3 A cutoff
    for cutoff in (None, 3.0):
        L = Layout.from_padded(species, coords, "AM1", pair_cutoff=cutoff)
        ref = O.parse(species, coords, cutoff=cutoff)
        ri, rj = L.reference_pair_atoms()
        np.testing.assert_array_equal(ri, ref["idxi"])
        np.testing.assert_array_equal(rj, ref["idxj"])
        assert L.nref == ref["idxi"].size
        assert L.npairs == int(np.sum(L.natoms_m * (L.natoms_m - 1) // 2))
        np.testing.assert_array_equal(L.norb, 4 * ref["nheavy"] + ref["nhyd"])
        assert L.mat_off[-1] == int(np.sum(L.norb ** 2))
    assert L.pair_skip is not None and L.pair_skip.sum() >= 1
