"""The allocation-free Jacobi entry point, through the C ABI (needs a GB300).

seqm_density_jacobi_noalloc serves callers that cannot allocate device memory (a
host that owns a fixed device-memory pool, or one that must not stall the GPU with
cudaMalloc mid-pipeline): its eigenvector scratch is a fixed 16 MiB array inside
the library.  This file is collected last so that, if it fails, a run that stops
at the first failure has already run every other test.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-10  # the two entry points run the same kernel on the same inputs


def _fock_batch(mols, method="AM1"):
    from pyseqm_gb300 import workloads
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF

    species, coords = workloads.pad_batch(mols)
    L = Layout.from_padded(species, coords, method).to_device("cuda")
    s = BatchSCF(L)
    s.hcore()
    s.scf(1e-6, (1,), max_iter=2)  # any symmetric Fock matrices will do; two SCF steps make them non-trivial
    s.fock()
    torch.cuda.synchronize()
    return L, s


def _call(fn_name, L, F, with_work):
    from pyseqm_gb300 import native

    lib = native.load()
    T, R = int(L.mat_off[-1]), int(L.row_off[-1])
    P = torch.full((T,), np.nan, dtype=torch.float64, device="cuda")
    ev = torch.full((R,), np.nan, dtype=torch.float64, device="cuda")
    vec = torch.full((T,), np.nan, dtype=torch.float64, device="cuda")
    st = torch.zeros(L.nmol, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = [L.struct, native.ptr(F), native.ptr(P), native.ptr(ev), native.ptr(vec)]
    if with_work:
        work = torch.empty(T, dtype=torch.float64, device="cuda")
        args.append(native.ptr(work))
    # the allocating entry point also takes (warm, mixed_threshold): cold FP64 sweeps, like the variant
    args += [native.ptr(L.dev["row_off"]), None, native.ptr(st), 50] + ([None, 0, 0] if with_work else []) + [stream]
    rc = getattr(lib, fn_name)(*args)
    torch.cuda.synchronize()
    return rc, P, ev, vec, st


def test_noalloc_matches_allocating_entry_point_twice():
    from pyseqm_gb300 import native, workloads

    rng = np.random.default_rng(7)
    mols = [workloads.alkane(int(k), rng, 0.03) for k in (1, 3, 6)] + \
           [workloads.water_cluster(int(k), rng) for k in (2, 5, 9)]
    L, s = _fock_batch(mols)
    rc, P0, e0, v0, st0 = _call("seqm_density_jacobi", L, s.F, True)
    assert rc == native.SEQM_OK
    for _ in range(2):  # two calls in a row share (and reuse) the fixed scratch array
        rc, P1, e1, v1, st1 = _call("seqm_density_jacobi_noalloc", L, s.F, False)
        assert rc == native.SEQM_OK
        torch.testing.assert_close(P1, P0, atol=TOL, rtol=0)
        torch.testing.assert_close(e1, e0, atol=TOL, rtol=0)
        for m in range(L.nmol):  # eigenvectors up to sign
            a, b = L.block(v1, m), L.block(v0, m)
            sgn = torch.sign((a * b).sum(dim=1, keepdim=True))
            torch.testing.assert_close(a * sgn, b, atol=1e-8, rtol=0)
        assert torch.equal(st1, st0) and bool((st1 > 0).all())


def test_noalloc_rejects_batches_beyond_its_scratch():
    from pyseqm_gb300 import native, workloads

    rng = np.random.default_rng(8)
    # 120 x (H2O)_24: 120 * 144^2 = 2.49 M doubles > 2^21
    mols = [workloads.water_cluster(24, rng) for _ in range(120)]
    from pyseqm_gb300.layout import Layout

    species, coords = workloads.pad_batch(mols)
    L = Layout.from_padded(species, coords, "PM3").to_device("cuda")
    assert int(L.mat_off[-1]) > 2**21
    F = torch.zeros(int(L.mat_off[-1]), dtype=torch.float64, device="cuda")
    rc, P, *_ = _call("seqm_density_jacobi_noalloc", L, F, False)
    assert rc == native.SEQM_E_TOO_LARGE
    assert bool(torch.isnan(P).all())  # nothing was launched


def test_noalloc_rejects_molecules_above_the_jacobi_limit():
    """A batch holding one molecule above 160 AOs is refused as a whole before any launch."""
    from pyseqm_gb300 import native, workloads
    from pyseqm_gb300.layout import Layout

    rng = np.random.default_rng(9)
    mols = [workloads.alkane(2, rng, 0.03), workloads.water_cluster(30, rng)]  # 30 waters: 180 AOs
    species, coords = workloads.pad_batch(mols)
    L = Layout.from_padded(species, coords, "PM3").to_device("cuda")
    assert L.max_norb > 160 and int(L.mat_off[-1]) <= 2**21
    F = torch.zeros(int(L.mat_off[-1]), dtype=torch.float64, device="cuda")
    rc, P, ev, vec, st = _call("seqm_density_jacobi_noalloc", L, F, False)
    assert rc == native.SEQM_E_TOO_LARGE
    assert bool(torch.isnan(P).all()) and bool(torch.isnan(ev).all()) and bool(torch.isnan(vec).all())
    assert bool((st == 0).all())
