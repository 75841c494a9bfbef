"""CIS / RPA excited states on the GPU (needs a GB300): the general-density two-electron
contraction against the oracle; excitation energies, transition densities, transition dipoles
and oscillator strengths through the seqm API against the reference's Davidson solvers and its
own committed test values."""

import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import seqm_excited as X
from oracle import seqm_oracle as O

pytestmark = pytest.mark.gpu

CASES = ["cis_am1_mixed", "cis_pm3_same", "rpa_am1_same"]


def test_general_density_contraction_matches_oracle():
    """seqm_fock_general on random non-symmetric densities (three sets) against the oracle's
    restatement of makeA_pi (symmetric and antisymmetric parts) to 1e-11."""
    from pyseqm_gb300 import native
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF

    g = load_golden("cis_am1_mixed")
    sp, xyz = g["species_np"], g["coords_np"]
    L = Layout.from_padded(sp, xyz, "AM1").to_device("cuda")
    s = BatchSCF(L)
    s.hcore()
    T = int(L.mat_off[-1])
    rng = np.random.default_rng(3)
    nset = 3
    P = rng.normal(size=(nset, T))
    Pd = torch.as_tensor(P, device="cuda")
    G = torch.empty_like(Pd)
    native.check(s.lib.seqm_fock_general(L.struct, nset, native.ptr(Pd), native.ptr(s.w_xx), native.ptr(s.w_xh),
                                         native.ptr(s.w_hh), native.ptr(G), T, None, s._s()), "seqm_fock_general")
    G = G.cpu().numpy()
    mol = O.parse(sp, xyz)
    p = O.atom_params("AM1", mol["Z"])
    ints = O.integrals(mol, p, O.load_elements())
    n4 = 4 * mol["molsize"]
    for v in range(nset):
        Ppad = np.zeros((mol["nmol"], n4, n4))
        for m in range(mol["nmol"]):
            idx = O.packed_index(mol["nheavy"][m], mol["nhyd"][m])
            n = idx.size
            Ppad[m][np.ix_(idx, idx)] = P[v, L.mat_off[m]: L.mat_off[m] + n * n].reshape(n, n)
        Gref = X.g_transition(mol, p, ints, Ppad)
        for m in range(mol["nmol"]):
            idx = O.packed_index(mol["nheavy"][m], mol["nhyd"][m])
            n = idx.size
            np.testing.assert_allclose(G[v, L.mat_off[m]: L.mat_off[m] + n * n].reshape(n, n),
                                       Gref[m][np.ix_(idx, idx)], atol=1e-11, rtol=1e-12)


@pytest.mark.parametrize("name", CASES)
def test_excited_states_match_reference(name):
    """Electronic_Structure with excited_states: excitation energies to 1e-6 eV and transition
    densities C_occ X C_virt^T (for RPA also of Y) to 1e-5 up to one sign per state, against the
    reference run through its own seqm API."""
    from pyseqm_gb300 import Constants, Electronic_Structure, Molecule

    g = load_golden(name)
    s = dict(g["settings"])
    s["excited_states"] = dict(s["excited_states"])
    mol = Molecule(Constants().cuda(), s, torch.as_tensor(g["coords_np"], device="cuda"),
                   torch.as_tensor(g["species_np"], device="cuda")).cuda()
    Electronic_Structure(s).cuda()(mol)
    ref = g["ref"]
    np.testing.assert_allclose(mol.cis_energies.cpu().numpy(), ref["cis_energies"], atol=1e-6, rtol=0)
    np.testing.assert_allclose(mol.Etot.detach().cpu().numpy(), ref["Etot"], atol=1e-6, rtol=0)
    ex = mol._excited
    amps = mol.cis_amplitudes.cpu().numpy()
    rpa = s["excited_states"]["method"] == "rpa"
    sets = [amps[0], amps[1]] if rpa else [amps]
    Co, Cv = ex.Co.cpu().numpy(), ex.Cv.cpu().numpy()
    norb, nocc = ex.norb, ex.nocc
    for m in range(ex.nmol):
        n = int(norb[m])
        signs = None
        for which, a in enumerate(sets):
            Xm = a[m].reshape(a.shape[1], ex.no, ex.nv)
            Tm = np.einsum("mi,ria,na->rmn", Co[m, :n], Xm, Cv[m, :n])
            Tr = np.asarray(ref["transition_densities"][which][m])
            if signs is None:
                signs = np.sign((Tm * Tr).sum((1, 2)))[:, None, None]
            np.testing.assert_allclose(signs * Tm, Tr, atol=1e-5, rtol=0)
    # transition dipoles (atomic units, one sign per state) and oscillator strengths
    np.testing.assert_allclose(mol.oscillator_strength.cpu().numpy(), ref["oscillator_strength"], atol=1e-6, rtol=0)
    np.testing.assert_allclose(np.abs(mol.transition_dipole.cpu().numpy()), np.abs(np.asarray(ref["transition_dipole"])),
                               atol=1e-5, rtol=0)


@pytest.mark.parametrize("name", ["cis_ref_cis_am1_methane", "cis_ref_rpa_am1_methane", "cis_ref_cis_am1_methanal",
                                  "cis_ref_rpa_am1_methanal", "cis_ref_cis_am1_mixed"])
def test_excited_states_match_reference_test_values(name):
    """The seqm API on the inputs of the reference's own excited-state tests
    (test_excited_states.py) against its committed energies and oscillator strengths, at that
    test's tolerance (rtol = atol = 1e-5)."""
    from pyseqm_gb300 import Constants, Electronic_Structure, Molecule

    g = load_golden(name)
    s = dict(g["settings"])
    s["excited_states"] = dict(s["excited_states"])
    mol = Molecule(Constants().cuda(), s, torch.as_tensor(g["coords_np"], device="cuda"),
                   torch.as_tensor(g["species_np"], device="cuda")).cuda()
    Electronic_Structure(s).cuda()(mol)
    rj = g["reference_test_json"]
    np.testing.assert_allclose(mol.cis_energies.cpu().numpy(), rj["cis_energies"], atol=1e-5, rtol=1e-5)
    np.testing.assert_allclose(mol.oscillator_strength.cpu().numpy(), rj["oscillator_strength"], atol=1e-5, rtol=1e-5)
