"""Tensor-core (tcgen05, FP16 hi+lo) SP2 with FP64 McWeeny refinement, and the Jacobi / SP2
dispatch for molecules above the Jacobi limit.  Mixed-precision form: |dE| <= 1e-4 eV per
molecule against the FP64 oracle, idempotency of P/2 to FP64 level."""

import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import seqm_oracle as O

pytestmark = pytest.mark.gpu

TOL_E_MIXED = 1e-4  # eV, the mixed-precision form's energy tolerance
TOL_P_MIXED = 1e-4  # density max-abs
SCF_EPS_MIXED = 1e-5  # SCF threshold of the mixed-precision (serving) form


def _solve(species, coords, method, eps, sp2=(False,), large="tc"):
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF

    L = Layout.from_padded(species, coords, method).to_device("cuda")
    s = BatchSCF(L)
    s.large_density = large
    s.hcore()
    nc = s.scf(eps, (1,), sp2)
    E, En = s.final(want_vectors=False)
    return L, s, (E + En).cpu().numpy(), nc


def _idempotency(L, P, m):
    X = 0.5 * L.block(P, m)
    return float((X @ X - X).abs().max())


def test_tc_sp2_matches_reference_sp2_option():
    """sp2 = [True, eps, "tc"] on the golden mixed AM1 batch (the reference ran SP2 there)."""
    g = load_golden("mixed_am1_sp2")
    # the mixed-precision density carries ~1e-7 noise: SCF to the serving threshold 1e-5
    L, s, E, nc = _solve(g["species_np"], g["coords_np"], "AM1", SCF_EPS_MIXED, (True, 1e-7, "tc"))
    assert not nc.any()
    np.testing.assert_allclose(E, g["ref"]["Etot"], atol=TOL_E_MIXED, rtol=0)
    for m in range(L.nmol):
        np.testing.assert_allclose(L.block(s.P, m).cpu().numpy(), np.asarray(g["ref"]["P"][m]), atol=TOL_P_MIXED)
        assert _idempotency(L, s.P, m) < 1e-9


@pytest.mark.parametrize("large", ["tc", "fp64"])
def test_large_molecules_take_sp2_and_match_oracle(large):
    """Molecules above 160 AOs (water 30 = 180 AOs, C30 alkane = 182 AOs) next to small ones."""
    from pyseqm_gb300 import workloads

    rng = np.random.default_rng(21)
    mols = [workloads.water_cluster(30, rng), workloads.alkane(4, rng, 0.03), workloads.alkane(30, rng, 0.03),
            workloads.water_cluster(5, rng)]
    species, coords = workloads.pad_batch(mols)
    L, s, E, nc = _solve(species, coords, "PM3", SCF_EPS_MIXED if large == "tc" else 1e-8, large=large)
    assert not nc.any()
    ref = O.single_point("PM3", species, coords, 1e-8, (1,))
    tol = TOL_E_MIXED if large == "tc" else 1e-6
    np.testing.assert_allclose(E, ref["Etot"], atol=tol, rtol=0)
    for m in (0, 2):
        assert int(L.norb[m]) > 160
        assert _idempotency(L, s.P, m) < 1e-9


@pytest.mark.parametrize("large", ["tc", "fp64"])
def test_captured_sp2_iteration_matches_eager(large):
    """One SCF iteration of a batch of molecules above the Jacobi limit captured in a CUDA graph
    (the SP2 step loop becomes a conditional WHILE node that the device ends, no host
    synchronisation) and replayed to convergence gives the eager solve's iterations and
    energies."""
    from pyseqm_gb300 import workloads
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF

    rng = np.random.default_rng(33)
    mols = [workloads.water_cluster(30, rng), workloads.alkane(28, rng, 0.03), workloads.water_cluster(40, rng)]
    species, coords = workloads.pad_batch(mols)
    eps = SCF_EPS_MIXED if large == "tc" else 1e-7
    L = Layout.from_padded(species, coords, "PM3").to_device("cuda")
    eager = BatchSCF(L)
    eager.large_density = large
    eager.hcore()
    assert not eager.scf(eps, (1,)).any()
    E_eager = eager.final(want_vectors=False)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        s = BatchSCF(L, stream=stream)
        s.large_density = large
        s.hcore()
        s.start(eps, (1,))
        s.step()  # eager first iteration: scratch buffers and kernel attributes
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            s.step()
        for _ in range(200):
            g.replay()
            if not bool(s.active[: L.nmol].any()):
                break
        E = s.final(want_vectors=False)
    torch.cuda.synchronize()
    assert not bool(s.active[: L.nmol].any())
    np.testing.assert_array_equal(s.iters[: L.nmol].cpu().numpy(), eager.iters[: L.nmol].cpu().numpy())
    # the tensor-core form sums its traces with atomics: two eager solves differ at ~1e-9 eV too
    np.testing.assert_allclose((E[0] + E[1]).cpu().numpy(), (E_eager[0] + E_eager[1]).cpu().numpy(),
                               atol=1e-7 if large == "tc" else 1e-9, rtol=0)
    assert bool((s.status[: L.nmol] > 0).all())


def test_mixing_at_the_48kb_shared_memory_edge():
    """A 3072-AO molecule ((H2O)512): the adaptive mixer's diagonal history is exactly 48 KB of
    dynamic shared memory, which with the kernel's static shared memory exceeds the default
    limit; two SCF iterations run without a launch failure."""
    from pyseqm_gb300 import workloads
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF

    species, coords = workloads.pad_batch([workloads.big_water(seed=0, n_side=8)])
    L = Layout.from_padded(species, coords, "PM3").to_device("cuda")
    assert L.max_norb == 3072
    s = BatchSCF(L)
    s.large_density = "tc"
    s.hcore()
    s.scf(1e-5, (1,), max_iter=2)
    torch.cuda.synchronize()
    assert int(s.iters[0]) == 2 and bool(torch.isfinite(s.Eout[:1]).all())


def test_refinement_gate_matches_refining_every_iteration():
    """(H2O)125 (750 AOs), tensor-core SP2: starting at active = 2, the early iterations keep the
    FP32-level density (the FP64-accurate McWeeny step waits until |dE| < 1 eV) and the molecule
    is never retired on such a density; the converged energy matches the run that refines every
    iteration and the FP64 oracle, with idempotency at FP64 level."""
    from pyseqm_gb300 import workloads
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF

    species, coords = workloads.pad_batch([workloads.big_water(seed=3, n_side=5)])
    L = Layout.from_padded(species, coords, "PM3").to_device("cuda")
    out = {}
    for gate in (True, False):
        s = BatchSCF(L)
        s.large_density = "tc"
        s.refine_near_convergence = gate
        s.hcore()
        s.start(SCF_EPS_MIXED, (1,))
        assert int(s.active[0]) == (2 if gate else 1)
        s.step()
        if gate:  # the first iteration moves the energy by far more than 1 eV
            assert abs(float(s.err[0])) > 1.0 and int(s.active[0]) == 2
        nc = s.iterate()
        E, En = s.final(want_vectors=False)
        assert not nc.any()
        out[gate] = (float(E[0] + En[0]), int(s.iters[0]), _idempotency(L, s.P, 0))
    (e1, it1, id1), (e0, it0, id0) = out[True], out[False]
    assert abs(e1 - e0) < 5e-5 and abs(it1 - it0) <= 2
    assert id1 < 1e-9 and id0 < 1e-9
    ref = O.single_point("PM3", species, coords, 1e-8, (1,))
    assert abs(e1 - float(ref["Etot"][0])) < TOL_E_MIXED
