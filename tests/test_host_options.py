"""Host logic of the seqm options added on top of the SCF (no GPU): the nonadiabatic-coupling
pair resolution, the CIS phase alignment, active states, and the AM1-FS1 dispersion expression
against the oracle (energies and its autograd gradient against central differences)."""

import numpy as np
import pytest
import torch

from oracle import seqm_oracle as O


def test_nac_pairs_follow_the_reference_resolution():
    """resolve_nac_config (dynamics/nac_utils.py:29-63): off unless compute_nac; all pairs of the
    states when enabled alone; 'states' gives all their pairs; 'pairs' explicit, sorted,
    deduplicated, out-of-range and diagonal ones dropped."""
    from pyseqm_gb300.basics import nac_pairs

    assert nac_pairs({}, 3) is None
    assert nac_pairs({"nonadiabatic": {"compute_nac": False, "pairs": [(1, 2)]}}, 3) is None
    assert nac_pairs({"nonadiabatic": {"compute_nac": True}}, 3) == [(1, 2), (1, 3), (2, 3)]
    assert nac_pairs({"nonadiabatic": {"compute_nac": True, "states": [3, 1, 3]}}, 4) == [(1, 3)]
    got = nac_pairs({"nonadiabatic": {"compute_nac": True, "pairs": [(2, 1), (1, 2), (2, 2), (1, 5), [3, 2]]}}, 3)
    assert got == [(1, 2), (2, 3)]


def test_phase_alignment_flips_roots_with_negative_overlap():
    """_phase_align_cis (basics.py:567-593): each root's sign makes its overlap with the previous
    amplitudes non-negative; RPA amplitudes (X, Y) flip together; shape changes leave them."""
    from pyseqm_gb300.basics import _phase_align

    rng = np.random.default_rng(0)
    ref = torch.as_tensor(rng.normal(size=(2, 3, 6)))
    sign = torch.tensor([[1.0, -1.0, 1.0], [-1.0, -1.0, 1.0]])
    new = ref * sign[:, :, None] + 0.01 * torch.as_tensor(rng.normal(size=(2, 3, 6)))
    out = _phase_align(new, ref)
    assert bool(((out * ref).sum(-1) >= 0).all())
    np.testing.assert_array_equal(out.abs().numpy(), new.abs().numpy())
    rpa_new, rpa_ref = torch.stack((new, new)), torch.stack((ref, ref))
    out2 = _phase_align(rpa_new, rpa_ref, rpa=True)
    np.testing.assert_array_equal(out2[0].numpy(), out.numpy())
    np.testing.assert_array_equal(out2[1].numpy(), out.numpy())
    assert _phase_align(new, ref[:, :, :4]) is new
    assert _phase_align(new, None) is new


def test_active_states_from_int_or_tensor():
    from types import SimpleNamespace

    from pyseqm_gb300.basics import _active_states

    assert _active_states(SimpleNamespace(active_state=2), 3, "cpu").tolist() == [2, 2, 2]
    assert _active_states(SimpleNamespace(active_state=None), 2, "cpu").tolist() == [0, 0]
    assert _active_states(SimpleNamespace(active_state=torch.tensor(1)), 2, "cpu").tolist() == [1, 1]
    assert _active_states(SimpleNamespace(active_state=torch.tensor([0, 3])), 2, "cpu").tolist() == [0, 3]


@pytest.mark.parametrize("cutoff", [None, 3.0])
def test_dispersion_expression_matches_oracle_and_differences(cutoff):
    """AM1-FS1 dispersion on the device expression (run here on the CPU): per-molecule energies
    equal the oracle's (with and without a pair cutoff), and its autograd gradient equals
    central differences of itself."""
    from pyseqm_gb300 import workloads
    from pyseqm_gb300.basics import _dispersion_am1_fs1
    from pyseqm_gb300.layout import Layout

    species, coords = workloads.pad_batch(workloads.mixed_batch(4, seed=7, alkane_range=(2, 6),
                                                                water_range=(3, 6)))
    L = Layout.from_padded(species, coords, "AM1", pair_cutoff=cutoff)
    xyz = torch.as_tensor(L.xyz.copy(), dtype=torch.float64).requires_grad_(True)
    E = _dispersion_am1_fs1(L, xyz)
    ref = O.dispersion_am1_fs1(O.parse(species, coords, cutoff=cutoff))
    np.testing.assert_allclose(E.detach().numpy(), ref, atol=1e-12, rtol=1e-10)
    g, = torch.autograd.grad(E.sum(), xyz)
    h = 1e-5
    for a in (0, 3, L.natoms - 1):
        for x in range(3):
            xp, xm = L.xyz.copy(), L.xyz.copy()
            xp[a, x] += h
            xm[a, x] -= h
            fd = (_dispersion_am1_fs1(L, torch.as_tensor(xp)).sum() - _dispersion_am1_fs1(L, torch.as_tensor(xm)).sum())
            np.testing.assert_allclose(g[a, x].item(), fd.item() / (2 * h), atol=1e-8, rtol=1e-6)


def test_resolve_nac_config_like_the_reference():
    """The public resolve_nac_config / NACConfig: pairs are resolved whether or not enabled."""
    from pyseqm_gb300 import resolve_nac_config

    c = resolve_nac_config({"nonadiabatic": {"pairs": [(2, 1), (3, 3)]}}, nroots=3)
    assert not c.enabled and c.pairs == [(1, 2)]
    c = resolve_nac_config({"nonadiabatic": {"compute_nac": True, "states": [1, 2, 9]}}, nroots=None)
    assert c.enabled and c.pairs == [(1, 2), (1, 9), (2, 9)]
    c = resolve_nac_config({}, nroots=2, default_enabled=True)
    assert c.enabled and c.pairs == [(1, 2)]


def test_geometric_optimization_glue(tmp_path, monkeypatch):
    """The geomeTRIC wrapper with a stand-in geomeTRIC and a stand-in driver (no GPU): coordinates
    come in bohr and are set in Angstrom, energy and gradient go out in hartree and hartree/bohr,
    one trajectory frame per step, the last geometry in optimized.xyz; ImportError without it."""
    import sys
    import types

    import pyseqm_gb300
    from pyseqm_gb300 import Constants, Molecule, basics, optimization

    for name in [k for k in sys.modules if k == "geometric" or k.startswith("geometric.")]:
        monkeypatch.delitem(sys.modules, name)
    with pytest.raises(ImportError):
        optimization.geomeTRIC_optimization(None)

    calls = []
    bohr2ang, ev2au = 0.529177210903, 1.0 / 27.211386245988

    class Engine:
        def __init__(self, molecule):
            self.M = molecule

    class GeomMolecule:
        pass

    def run_optimizer(customengine, input, qccnv, **kw):
        x0 = customengine.M.xyzs[0].reshape(-1) / bohr2ang
        for k in range(2):
            calls.append(customengine.calc_new(x0 + 0.01 * k))
        return types.SimpleNamespace(write_xyz=lambda selection: ["5", "last", "C 0 0 0"])

    mods = {"geometric": types.ModuleType("geometric"), "geometric.engine": types.SimpleNamespace(Engine=Engine),
            "geometric.molecule": types.SimpleNamespace(Elements=["X", "H", "He", "Li", "Be", "B", "C"],
                                                       Molecule=GeomMolecule),
            "geometric.nifty": types.SimpleNamespace(bohr2ang=bohr2ang, ev2au=ev2au),
            "geometric.optimize": types.SimpleNamespace(run_optimizer=run_optimizer)}
    for k, v in mods.items():
        monkeypatch.setitem(sys.modules, k, v)

    class FakeDriver:
        def __init__(self, seqm_parameters):
            pass

        def __call__(self, m, P0=None, dm_prop="SCF"):
            x = m.coordinates.detach()
            m.Etot = (x * x).sum((1, 2))
            m.force = -2.0 * x
            m.dm = torch.zeros(1, 20, 20, dtype=torch.float64)

    monkeypatch.setattr(basics, "Electronic_Structure", FakeDriver)
    monkeypatch.chdir(tmp_path)
    xyz = torch.tensor([[[0.0, 0.0, 0.0], [0.63, 0.63, 0.63], [-0.63, -0.63, 0.63], [-0.63, 0.63, -0.63],
                         [0.63, -0.63, -0.63]]], dtype=torch.float64)
    mol = Molecule(Constants(), {"method": "AM1", "scf_eps": 1e-6, "scf_converger": [1]}, xyz,
                   torch.tensor([[6, 1, 1, 1, 1]]))
    pyseqm_gb300.geomeTRIC_optimization(mol, traj_file=str(tmp_path / "traj.xyz"))
    x1 = mol.coordinates.detach().numpy()[0]
    np.testing.assert_allclose(x1, xyz.numpy()[0] + 0.01 * bohr2ang, atol=1e-12)
    assert calls[1]["energy"] == pytest.approx(float((x1 ** 2).sum()) * ev2au)
    np.testing.assert_allclose(calls[1]["gradient"], (2.0 * x1 * ev2au * bohr2ang).reshape(-1), atol=1e-12)
    traj = (tmp_path / "traj.xyz").read_text().splitlines()
    assert traj[0] == "5" and traj[1].startswith("Step 1, E = ") and traj[1].endswith(" eV") and len(traj) == 14
    assert traj[2].split()[0] == "C"
    assert (tmp_path / "optimized.xyz").read_text() == "5\nlast\nC 0 0 0"
