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

CASES = ["cis_am1_mixed", "cis_pm3_same", "rpa_am1_same", "cis_pm3_window"]


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
    for m in range(ex.nmol):
        n = int(ex.L.norb[m])  # AOs (the excitation space may be an orbital window)
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


REF_EXCITED = ["cis_ref_cis_am1_methane", "cis_ref_rpa_am1_methane", "cis_ref_cis_am1_methanal",
               "cis_ref_rpa_am1_methanal", "cis_ref_cis_am1_mixed"]


def _excited_molecule(g, excited=None, **extra):
    from pyseqm_gb300 import Constants, Molecule

    s = dict(g["settings"], **extra)
    s["excited_states"] = dict(s["excited_states"], **(excited or {}))
    mol = Molecule(Constants().cuda(), s, torch.as_tensor(g["coords_np"], device="cuda"),
                   torch.as_tensor(g["species_np"], device="cuda")).cuda()
    return mol, s


@pytest.mark.parametrize("name", REF_EXCITED)
@pytest.mark.parametrize("mode", [{}, {"analytical_gradient": [True]}])
def test_excited_state_forces_match_reference_test_values(name, mode):
    """active_state 1: the relaxed forces of the first excited state (Z-vector response and the
    excited-state derivative kernel) against the reference's committed values (its
    test_excited_states.py / test_force_methods.py tolerance rtol = atol = 1e-5), and Etot
    carrying the state's excitation energy."""
    from pyseqm_gb300 import Electronic_Structure

    g = load_golden(name)
    mol, s = _excited_molecule(g, active_state=1, **mode)
    Electronic_Structure(s).cuda()(mol)
    rj = g["reference_test_json"]
    # the ragged batch's committed forces come from the reference's autograd through its SCF at
    # scf_eps 1e-7: they sit up to 8.6e-6 eV/A from the converged central differences, ours (same
    # loose settings) up to 4e-6 on the other side, so that one case is compared at 2e-5
    tol = 2e-5 if name == "cis_ref_cis_am1_mixed" else 1e-5
    np.testing.assert_allclose(mol.force.cpu().numpy(), np.asarray(rj["force"]), atol=tol, rtol=1e-5)
    E1 = mol.cis_energies[:, 0].cpu().numpy()
    np.testing.assert_allclose((mol.Etot - mol.Eelec - mol.Enuc).detach().cpu().numpy(), E1, atol=1e-10, rtol=0)
    np.testing.assert_allclose(E1, np.asarray(rj["cis_energies"])[:, 0], atol=1e-5, rtol=1e-5)


@pytest.mark.parametrize("name", ["cis_ref_cis_am1_methanal", "cis_ref_rpa_am1_methane"])
def test_excited_state_forces_match_oracle_differences(name):
    """Tight settings (excited-state tolerance 1e-8, so scf_eps 1e-9): the analytic relaxed
    forces against the oracle's Richardson-extrapolated central differences of E_ground + omega_1
    to 1e-6 eV/A."""
    from pyseqm_gb300 import Electronic_Structure

    g = load_golden(name)
    mol, s = _excited_molecule(g, active_state=1, excited={"tolerance": 1e-8})
    Electronic_Structure(s).cuda()(mol)
    es = g["settings"]["excited_states"]
    f = X.excited_forces_fd(g["settings"]["method"], g["species_np"], g["coords_np"], 1e-11, 1,
                            rpa=es["method"] == "rpa")
    np.testing.assert_allclose(mol.force.cpu().numpy(), f, atol=1e-6, rtol=0)


def test_mixed_ground_and_excited_active_states():
    """A per-molecule active_state tensor: molecules in the ground state keep the ground-state
    energy and forces, the others those of their state."""
    from pyseqm_gb300 import Electronic_Structure

    g = load_golden("cis_ref_cis_am1_methanal")
    mol0, s0 = _excited_molecule(g)
    Electronic_Structure(s0).cuda()(mol0)
    mol1, s1 = _excited_molecule(g, active_state=1)
    Electronic_Structure(s1).cuda()(mol1)
    mix, sm = _excited_molecule(g)
    mix.active_state = torch.tensor([1, 0, 2], device="cuda")
    Electronic_Structure(sm).cuda()(mix)
    f = mix.force.cpu().numpy()
    np.testing.assert_allclose(f[0], mol1.force[0].cpu().numpy(), atol=1e-9, rtol=0)
    np.testing.assert_allclose(f[1], mol0.force[1].cpu().numpy(), atol=1e-9, rtol=0)
    E = mix.Etot.detach().cpu().numpy()
    np.testing.assert_allclose(E[1], mol0.Etot[1].item(), atol=1e-9, rtol=0)
    np.testing.assert_allclose(E[2] - mol0.Etot[2].item(), mol0.cis_energies[2, 1].item(), atol=1e-9, rtol=0)


def test_nac_matches_reference():
    """CIS nonadiabatic couplings (seqm_parameters['nonadiabatic']): every state pair's
    (nmol, molsize, 3) vectors against the reference's calc_nac to 1e-6, up to one sign per
    molecule and pair (the sign of the state-to-state density follows the amplitudes')."""
    from pyseqm_gb300 import Electronic_Structure

    g = load_golden("cis_nac_am1_methanal")
    mol, s = _excited_molecule(g)
    s["nonadiabatic"] = dict(g["settings"]["nonadiabatic"])
    Electronic_Structure(s).cuda()(mol)
    np.testing.assert_allclose(mol.cis_energies.cpu().numpy(), g["ref"]["cis_energies"], atol=1e-6, rtol=0)
    assert sorted(mol.nac) == sorted((a, b) for a, b, _ in g["ref"]["nac"])
    for a, b, v in g["ref"]["nac"]:
        ours = mol.nac[(a, b)].cpu().numpy()
        v = np.asarray(v)
        for m in range(v.shape[0]):
            sg = np.sign((ours[m] * v[m]).sum())
            np.testing.assert_allclose(sg * ours[m], v[m], atol=1e-6, rtol=0)


def test_phase_alignment_and_saved_transition_densities():
    """A second excited-state call on a displaced geometry keeps every root's sign continuous
    with the previous amplitudes (non-negative overlaps), and save_tdm stores the per-root
    transition densities C_occ X C_virt^T."""
    from pyseqm_gb300 import Electronic_Structure

    g = load_golden("cis_ref_cis_am1_methanal")
    mol, s = _excited_molecule(g, excited={"save_tdm": True})
    es = Electronic_Structure(s).cuda()
    es(mol)
    a0 = mol.cis_amplitudes.clone()
    tdm = mol.transition_density_matrices.cpu().numpy()
    ex = mol._excited
    Co, Cv = ex.Co.cpu().numpy(), ex.Cv.cpu().numpy()
    X = a0.cpu().numpy().reshape(ex.nmol, -1, ex.no, ex.nv)
    np.testing.assert_allclose(tdm, np.einsum("bmi,bria,bna->brmn", Co, X, Cv), atol=1e-12, rtol=0)
    with torch.no_grad():
        mol.coordinates.add_(0.002 * torch.randn_like(mol.coordinates))
    es(mol)
    ov = (mol.cis_amplitudes * a0).sum(-1)
    assert bool((ov >= 0).all()), ov



@pytest.mark.parametrize("name", ["cis_allforces_cis_am1_methanal", "cis_allforces_rpa_am1_methanal"])
def test_all_state_forces_match_reference(name):
    """do_all_forces: the ground state's and every excited state's forces, and the states'
    relaxed and unrelaxed dipoles, against the reference (tight settings: 1e-6)."""
    from pyseqm_gb300 import Electronic_Structure

    g = load_golden(name)
    mol, s = _excited_molecule(g)
    Electronic_Structure(s).cuda()(mol)
    ref = g["ref"]
    np.testing.assert_allclose(mol.cis_energies.cpu().numpy(), ref["cis_energies"], atol=1e-6, rtol=0)
    np.testing.assert_allclose(mol.all_forces.cpu().numpy(), np.asarray(ref["all_forces"]), atol=1e-6, rtol=0)
    np.testing.assert_allclose(mol.all_cis_relaxed_diploles.cpu().numpy(), ref["relaxed"], atol=1e-6, rtol=0)
    np.testing.assert_allclose(mol.all_cis_unrelaxed_diploles.cpu().numpy(), ref["unrelaxed"], atol=1e-6, rtol=0)
