"""The seqm drop-in API (Molecule / Electronic_Structure / Energy / Force) on the GPU:
energies, autograd forces and parameter gradients against golden outputs of the
reference, finite differences and rotation invariance."""

import math

import numpy as np
import pytest
import torch

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _molecule(g, settings=None, learned=None):
    from pyseqm_gb300 import Constants, Molecule

    s = dict(settings or g["settings"])
    const = Constants().cuda()
    species = torch.as_tensor(g["species_np"], dtype=torch.int64, device="cuda")
    coords = torch.as_tensor(g["coords_np"], dtype=torch.float64, device="cuda")
    kw = {}
    if "charges" in g:
        kw["charges"] = torch.as_tensor(g["charges"], dtype=torch.float64, device="cuda")
    return Molecule(const, s, coords, species, **kw).cuda(), s


@pytest.mark.parametrize("name", ["force_methane_am1", "force_methanal_am1", "force_mixed_am1"])
@pytest.mark.parametrize("mode", [{}, {"analytical_gradient": [True]}, {"analytical_gradient": [True, "numerical"]}])
def test_force_modes_match_reference_test_values(name, mode):
    """The reference's force-method suite (test_force_methods.py): autograd, analytical and
    semi-numerical gradient settings all give the forces of its committed values (1e-5)."""
    from pyseqm_gb300 import Electronic_Structure

    g = load_golden(name)
    s = dict(g["settings"], **mode)
    mol, s = _molecule(g, s)
    Electronic_Structure(s).cuda()(mol)
    rj = g["reference_test_json"]
    np.testing.assert_allclose(mol.force.cpu().numpy(), np.asarray(rj["force"]), atol=1e-5, rtol=1e-5)
    if mode:
        np.testing.assert_allclose(mol.analytical_gradient.cpu().numpy(), -np.asarray(rj["force"]), atol=1e-5,
                                   rtol=1e-5)


@pytest.mark.parametrize("name", ["smoke_MNDO", "smoke_AM1", "smoke_PM3", "batch_am1", "force_methanal_am1",
                                  "force_mixed_am1", "force_methane_am1", "mixed_am1_cutoff", "disp_am1_fs1", "mixed_pm6sp", "ions_pm6sp", "hetero_pm6sp", "hetero_am1",
                                  "hetero_pm3"])
def test_electronic_structure_matches_reference(name):
    from pyseqm_gb300 import Electronic_Structure

    g = load_golden(name)
    ref = g["ref"]
    mol, s = _molecule(g)
    Electronic_Structure(s).cuda()(mol)
    for key in ("Etot", "Eelec", "Enuc", "Hf", "Eiso"):
        np.testing.assert_allclose(getattr(mol, key).detach().cpu().numpy(), ref[key], atol=1e-6, rtol=0)
    # forces: adjoint kernel vs the reference's autograd
    np.testing.assert_allclose(mol.force.cpu().numpy(), np.asarray(ref["force"]), atol=1e-6, rtol=0)
    np.testing.assert_allclose(mol.q.cpu().numpy(), np.asarray(ref["q"]), atol=1e-7, rtol=0)
    if "reference_test_json" in g:  # the reference's own committed values
        rj = g["reference_test_json"]
        np.testing.assert_allclose(mol.force.cpu().numpy(), np.asarray(rj["force"]), atol=1e-5, rtol=1e-5)


def test_parameter_gradients_match_reference():
    from pyseqm_gb300 import Constants, Energy, Molecule

    g = load_golden("mndo_param_grads")
    ref = g["ref"]
    s = dict(g["settings"], learned=["U_ss", "U_pp", "beta_s", "beta_p"])
    const = Constants().cuda()
    species = torch.as_tensor(g["species_np"], device="cuda")
    coords = torch.as_tensor(g["coords_np"], device="cuda")
    from pyseqm_gb300 import tables

    fields, rows = tables.method_table("MNDO")
    Z = np.asarray(ref["Z"])
    lp = {k: torch.as_tensor(rows[Z, fields.index(k)], device="cuda").requires_grad_(True)
          for k in ("U_ss", "U_pp", "beta_s", "beta_p")}
    mol = Molecule(const, s, coords, species, learned_parameters=lp).cuda()
    out = Energy(s).cuda()(mol, learned_parameters=lp, all_terms=True)
    Etot = out[1]
    Etot.sum().backward()
    np.testing.assert_allclose(Etot.detach().cpu().numpy(), ref["Etot"], atol=1e-6)
    for k in lp:
        np.testing.assert_allclose(mol.parameters[k].grad.cpu().numpy(), np.asarray(ref["param_grads"][k]),
                                   atol=1e-6, rtol=1e-7)
    np.testing.assert_allclose(mol.coordinates.grad.cpu().numpy(), np.asarray(ref["dEtot_dR"]), atol=1e-6)


def test_forces_match_central_differences():
    """-dHf/dR against central differences of the full SCF energy (h = 1e-4 A)."""
    from pyseqm_gb300 import workloads
    from pyseqm_gb300.api import single_point

    rng = np.random.default_rng(3)
    species, coords = workloads.pad_batch([workloads.alkane(3, rng, 0.05), workloads.water_cluster(3, rng)])
    g = {"species_np": species, "coords_np": coords,
         "settings": {"method": "PM3", "scf_eps": 1e-10, "scf_converger": [1]}}
    from pyseqm_gb300 import Electronic_Structure

    mol, s = _molecule(g)
    Electronic_Structure(s).cuda()(mol)
    f = mol.force.cpu().numpy()
    h = 1e-4
    picks = [(0, 0, 0), (0, 3, 2), (0, 7, 1), (1, 0, 1), (1, 4, 0)]
    for (m, a, x) in picks:
        vals = []
        for sgn in (1.0, -1.0):
            c = coords.copy()
            c[m, a, x] += sgn * h
            vals.append(single_point(species, c, "PM3", 1e-10, (1,))["Hf"][m])
        fd = -(vals[0] - vals[1]) / (2 * h)
        assert abs(fd - f[m, a, x]) < 2e-5, (m, a, x, fd, f[m, a, x])


def test_rotation_invariance():
    """Energy invariant and forces covariant under a rotation (reference tests/unit/test_invariants.py:26-51)."""
    from pyseqm_gb300 import Electronic_Structure

    g = load_golden("smoke_AM1")
    mol, s = _molecule(g)
    Electronic_Structure(s).cuda()(mol)
    th = 0.7
    Rz = np.array([[math.cos(th), -math.sin(th), 0], [math.sin(th), math.cos(th), 0], [0, 0, 1.0]])
    g2 = dict(g, coords_np=g["coords_np"] @ Rz.T)
    mol2, s2 = _molecule(g2)
    Electronic_Structure(s2).cuda()(mol2)
    assert abs(float(mol.Etot[0]) - float(mol2.Etot[0])) < 1e-8
    np.testing.assert_allclose(mol2.force.cpu().numpy()[0], mol.force.cpu().numpy()[0] @ Rz.T, atol=1e-7)


def test_hamiltonian_tuple_shapes():
    from pyseqm_gb300 import Hamiltonian

    g = load_golden("batch_am1")
    mol, s = _molecule(g)
    F, e, P, H, w, charge, r0i, r0j, riXH, ri, nc, v = Hamiltonian(s)(mol, s["method"])
    n4 = 4 * mol.molsize
    assert F.shape == P.shape == H.shape == (mol.nmol, n4, n4)
    assert w.shape == (mol.idxi.numel(), 10, 10)
    assert e.shape == (mol.nmol, n4)
    assert torch.allclose(F, F.transpose(1, 2))


@pytest.mark.parametrize("name", ["pdir_pm6sp_star_params", "pdir_pm6sp_star"])
def test_parameter_file_dir_matches_reference(name, tmp_path):
    """seqm_parameters['parameter_file_dir']: the reference's STAR parameter set of PM6_SP read
    from MOPAC-format files (as PM6_SP with its PWCCT file, and as PM6_SP_STAR): energies,
    forces and charges against the reference's run on the same files."""
    from conftest import write_param_dir
    from pyseqm_gb300 import Electronic_Structure

    g = load_golden(name)
    s = dict(g["settings"], parameter_file_dir=write_param_dir(g, tmp_path))
    mol, s = _molecule(g, s)
    Electronic_Structure(s).cuda()(mol)
    ref = g["ref"]
    for key in ("Etot", "Eelec", "Enuc", "Hf", "Eiso"):
        np.testing.assert_allclose(getattr(mol, key).detach().cpu().numpy(), ref[key], atol=1e-6, rtol=0)
    np.testing.assert_allclose(mol.force.cpu().numpy(), np.asarray(ref["force"]), atol=1e-6, rtol=0)
    np.testing.assert_allclose(mol.q.cpu().numpy(), np.asarray(ref["q"]), atol=1e-7, rtol=0)
