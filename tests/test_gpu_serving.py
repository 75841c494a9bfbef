"""Serving loop on the GPU: each result is the same alone and in the mix (cohorts admitted
while others run), and within the mixed-precision tolerance of the FP64 oracle / plain form."""

import numpy as np
import pytest

from oracle import seqm_oracle as O
from pyseqm_gb300 import serving, workloads

pytestmark = pytest.mark.gpu

TOL_E_SMALL = 1e-7  # eV: Jacobi-sized molecules, same kernels alone and in the mix
TOL_E_MIXED = 1e-4  # eV: tensor-core SP2 molecules (and any molecule against the FP64 oracle)
TOL_F_MIXED = 1e-3  # eV/A: forces of the serving form against the FP64 plain form
EPS = 1e-5


def _mols():
    rng = np.random.default_rng(5)
    mols = [workloads.alkane(k, rng, 0.03) for k in (1, 3, 5, 8)]
    mols += [workloads.water_cluster(k, rng) for k in (2, 4, 7)]
    mols += [workloads.water_cluster(30, rng), workloads.alkane(28, rng, 0.03)]  # 180 and 170 AOs: SP2
    return [(s, c, i % 3 == 0) for i, (s, c) in enumerate(mols)]


@pytest.fixture(scope="module")
def mix():
    mols = _mols()
    loop = serving.ServingLoop("PM3", eps=EPS)
    res = loop.run(serving.make_requests(mols, np.arange(len(mols)) * 0.003))
    return mols, loop, res


def test_same_alone_and_in_the_mix(mix):
    mols, loop, res = mix
    assert loop.max_concurrent >= 2, "later requests were not admitted while earlier ones were on the GPU"
    for i, m in enumerate(mols):
        alone = serving.ServingLoop("PM3", eps=EPS).run(serving.make_requests([m]))[0]
        large = serving.norb_of(m[0]) > 160
        assert alone.converged and res[i].converged
        assert abs(alone.Etot - res[i].Etot) <= (TOL_E_MIXED if large else TOL_E_SMALL)
        if m[2]:
            np.testing.assert_allclose(res[i].forces, alone.forces, atol=TOL_F_MIXED if large else 1e-6)


def test_serving_within_tolerance_of_fp64(mix):
    mols, _, res = mix
    species, coords = workloads.pad_batch([(s, c) for s, c, _ in mols])
    ref = O.single_point("PM3", species, coords, 1e-8, (1,))
    np.testing.assert_allclose([r.Etot for r in res], ref["Etot"], atol=TOL_E_MIXED, rtol=0)
    plain = serving.ServingLoop("PM3", eps=1e-8, form="plain").run(serving.make_requests(mols))
    np.testing.assert_allclose([r.Etot for r in plain], ref["Etot"], atol=1e-6, rtol=0)
    for r, p, m in zip(res, plain, mols):
        if m[2]:
            np.testing.assert_allclose(r.forces, p.forces, atol=TOL_F_MIXED)


def test_graph_replay_matches_eager_launches(mix):
    """Cohorts replaying their captured SCF iteration give the eager results: Jacobi-sized ones
    bit for bit (the same kernels in the same order), SP2-sized ones, whose captured step loop is
    a conditional node ended on the device, to 1e-7 eV (their traces are summed with atomics, so
    two eager runs differ at that level too)."""
    mols = _mols()
    eager = serving.ServingLoop("PM3", eps=EPS, graphs=False).run(serving.make_requests(mols))
    graph = serving.ServingLoop("PM3", eps=EPS, graphs=True).run(serving.make_requests(mols))
    for m, a, g in zip(mols, eager, graph):
        assert a.converged and g.converged
        assert a.iterations == g.iterations
        if serving.norb_of(m[0]) > 160:
            assert abs(a.Etot - g.Etot) <= 1e-7
            if a.forces is not None:
                np.testing.assert_allclose(a.forces, g.forces, atol=1e-5, rtol=0)
            continue
        assert a.Etot == g.Etot, (serving.norb_of(m[0]), a.Etot - g.Etot)
        if a.forces is not None:
            np.testing.assert_array_equal(a.forces, g.forces)
