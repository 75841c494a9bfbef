"""Unrestricted (open-shell) SCF on the GPU against the reference's UHF outputs: energies,
per-spin orbital energies and densities, iteration counts, and through the seqm API the
forces, charges and HOMO-LUMO gaps (needs a GB300).

Where a spin occupies one of two exactly degenerate orbitals of the symmetric guess (the
fixtures' ``density_ambiguous`` molecules, e.g. the OH and NO radicals), any rotation within
the degenerate pair is an equally converged density; energies and orbital energies are
compared for every molecule, densities and forces only where the density is unique."""

import numpy as np
import pytest
import torch

from conftest import load_golden

pytestmark = pytest.mark.gpu

UHF_CASES = ["uhf_mndo", "uhf_am1", "uhf_pm3"]


def _run(g, **kw):
    from pyseqm_gb300.scf import run_energy

    s = g["settings"]
    return run_energy(g["species_np"], g["coords_np"], s["method"], eps=s["scf_eps"],
                      converger=tuple(s["scf_converger"]), charges=g.get("charges"), device="cuda",
                      mult=g["mult"], **kw)


@pytest.mark.parametrize("want_vectors", [True, False])
@pytest.mark.parametrize("name", UHF_CASES)
def test_uhf_matches_reference(name, want_vectors):
    g = load_golden(name)
    ref = g["ref"]
    out = _run(g, want_vectors=want_vectors)
    L, s = out["layout"], out["solver"]
    assert not out["notconverged"].any()
    np.testing.assert_allclose(out["Etot"].cpu().numpy(), ref["Etot"], atol=1e-6, rtol=0)
    np.testing.assert_allclose(out["Eelec"].cpu().numpy(), ref["Eelec"], atol=1e-6, rtol=0)
    np.testing.assert_allclose(out["Enuc"].cpu().numpy(), ref["Enuc"], atol=1e-6, rtol=0)
    assert abs(int(out["iters"].max()) - ref["loop_count"]) <= 1
    evs = (s.evals.cpu().numpy(), s.evals_b.cpu().numpy())
    dens = (s.P, s.Pb)
    for m in range(L.nmol):
        n = int(L.norb[m])
        r0 = int(L.row_off[m])
        for spin in range(2):
            np.testing.assert_allclose(evs[spin][r0: r0 + n], np.asarray(ref["e"][m][spin])[:n], atol=1e-6, rtol=0)
            if m not in g["density_ambiguous"]:
                np.testing.assert_allclose(L.block(dens[spin], m).cpu().numpy(), np.asarray(ref["P"][m][spin]),
                                           atol=1e-7, rtol=0)


@pytest.mark.parametrize("name", UHF_CASES)
def test_uhf_seqm_api_forces_charges_gaps(name):
    from pyseqm_gb300 import Constants, Electronic_Structure, Molecule

    g = load_golden(name)
    ref = g["ref"]
    s = dict(g["settings"])
    const = Constants().cuda()
    species = torch.as_tensor(g["species_np"], device="cuda")
    coords = torch.as_tensor(g["coords_np"], device="cuda")
    mult = torch.as_tensor(g["mult"], dtype=torch.float64, device="cuda")
    mol = Molecule(const, s, coords, species, mult=mult).cuda()
    Electronic_Structure(s).cuda()(mol)
    for key in ("Etot", "Eelec", "Enuc", "Hf", "Eiso"):
        np.testing.assert_allclose(getattr(mol, key).detach().cpu().numpy(), ref[key], atol=1e-6, rtol=0)
    assert mol.dm.shape[1] == 2 and mol.e_mo.shape[1] == 2
    keep = [m for m in range(len(ref["Etot"])) if m not in g["density_ambiguous"]]
    np.testing.assert_allclose(mol.force.cpu().numpy()[keep], np.asarray(ref["force"])[keep], atol=1e-6, rtol=0)
    np.testing.assert_allclose(mol.q.cpu().numpy()[keep], np.asarray(ref["q"])[keep], atol=1e-6, rtol=0)
    # per-spin HOMO-LUMO gaps from the reference's orbital energies (empty when a spin has
    # no occupied orbital)
    nocc = mol.nocc.cpu().numpy()
    if (nocc == 0).any():
        assert mol.e_gap.numel() == 0
    else:
        e = np.asarray(ref["e"])
        want = np.stack([[e[m, sp, nocc[m, sp]] - e[m, sp, nocc[m, sp] - 1] for sp in range(2)]
                         for m in range(e.shape[0])])
        np.testing.assert_allclose(mol.e_gap.cpu().numpy(), want, atol=1e-6, rtol=0)


def test_uhf_singlet_equals_rhf():
    """A closed-shell molecule run unrestricted as a singlet gives the restricted result."""
    g = load_golden("smoke_AM1")
    s = g["settings"]
    from pyseqm_gb300.scf import run_energy

    r = run_energy(g["species_np"], g["coords_np"], s["method"], eps=1e-8, device="cuda")
    u = run_energy(g["species_np"], g["coords_np"], s["method"], eps=1e-8, device="cuda",
                   mult=np.ones(g["species_np"].shape[0]))
    np.testing.assert_allclose(u["Etot"].cpu().numpy(), r["Etot"].cpu().numpy(), atol=1e-7, rtol=0)
    np.testing.assert_allclose((u["solver"].P + u["solver"].Pb).cpu().numpy(), r["solver"].P.cpu().numpy(),
                               atol=1e-7, rtol=0)


def test_uhf_ch3_matches_reference_test_value():
    """The reference's UHF known answer (test_uhf.py: planar CH3 doublet, AM1): Etot to its 1e-5
    and the spin-resolved density shape (nmol, 2, 4 molsize, 4 molsize)."""
    from pyseqm_gb300 import Constants, Electronic_Structure, Molecule

    g = load_golden("uhf_ch3_ref_am1")
    s = dict(g["settings"])
    mol = Molecule(Constants().cuda(), s, torch.as_tensor(g["coords_np"], device="cuda"),
                   torch.as_tensor(g["species_np"], device="cuda"),
                   mult=torch.as_tensor(g["mult"], device="cuda")).cuda()
    Electronic_Structure(s).cuda()(mol)
    rj = g["reference_test_json"]
    np.testing.assert_allclose(float(mol.Etot.item()), rj["Etot"], atol=1e-5, rtol=1e-5)
    assert list(mol.dm.shape) == rj["dm_shape"]
