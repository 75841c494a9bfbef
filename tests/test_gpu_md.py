"""Device-resident SCF across MD-like steps (the reference's MD passes P0 = the previous
density): resuming from the current density and eigenvectors gives the cold-start energies
and needs fewer iterations."""

import numpy as np
import pytest

from pyseqm_gb300 import workloads

pytestmark = pytest.mark.gpu


def test_resume_matches_cold_start_and_saves_iterations():
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF, run_energy

    rng = np.random.default_rng(17)
    mols = workloads.mixed_batch(12, seed=5, alkane_range=(1, 8), water_range=(2, 8))
    species, coords = workloads.pad_batch(mols)
    L = Layout.from_padded(species, coords, "AM1").to_device("cuda")
    s = BatchSCF(L)
    s.hcore()
    s.scf(1e-8, (1,))
    xyz = L.xyz.copy()
    for _ in range(3):
        xyz = xyz + rng.normal(0.0, 0.01, size=xyz.shape)
        nc = s.resume(xyz, 1e-8, (1,))
        assert not nc.any()
        warm_iters = s.iters[: L.nmol].cpu().numpy()
        E, En = s.final(want_vectors=False)
        pad = np.zeros((L.nmol * L.molsize, 3))
        pad[L.real_index] = xyz
        cold = run_energy(species, pad.reshape(L.nmol, L.molsize, 3), "AM1", eps=1e-8, converger=(1,))
        np.testing.assert_allclose((E + En).cpu().numpy(), cold["Etot"].cpu().numpy(), atol=1e-6, rtol=0)
        assert warm_iters.mean() < cold["iters"].mean()
