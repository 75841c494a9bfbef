"""Index arithmetic the kernels rely on, checked on the host: the division-free row / diagonal
tests (common.cuh FastDivU32 / DiagTest) and the incremental (row, column) walk of the fused
mixer's stream (fock.cu fused_stream)."""

import numpy as np


def _umulhi64(j, M):
    return (j * M) >> 64


def test_multiply_high_division_is_exact():
    """j / d == umulhi64(j, ceil(2^64 / d)) for 32-bit j: every j of the small molecules' matrices,
    a dense sample plus every row boundary of the large ones."""
    rng = np.random.default_rng(0)
    for d in list(range(2, 200)) + [361, 362, 363, 1001, 6001, 12801]:
        M = (2**64 - 1) // d + 1
        n2 = (d - 1) ** 2
        js = range(n2) if d <= 161 else rng.integers(0, max(1, n2), 20000).tolist()
        for j in js:
            assert _umulhi64(int(j), M) == int(j) // d
        for r in range(1, min(d, 4000)):
            j = r * d
            assert _umulhi64(j, M) == r and _umulhi64(j - 1, M) == r - 1
        assert _umulhi64(2**32 - 1, M) == (2**32 - 1) // d


def test_diagonal_walk_of_the_fused_stream():
    """A thread's elements i0, i0 + S, ... of an n x n matrix: the (row, column) advanced by
    S // n and S % n with one wrap per step marks exactly the diagonal elements."""
    rng = np.random.default_rng(1)
    for n in list(range(1, 170)) + [362, 1000, 6000]:
        for stride in (32, 256, 512):
            for i0 in rng.integers(0, stride, 4).tolist() + ([(n * n // 3 // 512) * 512 + 7] if stride == 512 else []):
                if i0 >= n * n:
                    continue
                row, col = i0 // n, i0 % n
                drow, dcol = stride // n, stride % n
                for j in range(i0, min(n * n, i0 + 3000 * stride), stride):
                    assert (row == col) == (j % (n + 1) == 0)
                    col += dcol
                    row += drow
                    if col >= n:
                        col -= n
                        row += 1


def test_single_rotation_scratch_fits():
    """jacobi.cu rotate_orth: for every basis size the Jacobi step takes (<= 160) and every
    occupation, its G scratch (Theta^T, Theta Theta^T and Theta^T Theta in [0, n^2 - st); a_ST and
    two Theta buffers in [n^2, n^2 + 3 st), st = |S| |T|) fits P's n^2 doubles = 2 n^2 floats, and
    the gathered A'_TT, A'_SS fit the n^2 floats of the sweeps' rotation buffer behind A32
    (n lda floats) in the launch's cap lda doubles of shared memory."""
    for n in range(2, 161):
        lda = n | 1
        for nocc in range(1, n):
            use_occ = nocc <= n - nocc
            nsel = nocc if use_occ else n - nocc
            ncomp = n - nsel
            st = nsel * ncomp
            assert st + ncomp * ncomp + nsel * nsel == n * n - st
            assert n * n + 3 * st <= 2 * n * n
            assert ncomp * ncomp + nsel * nsel <= n * n
            assert n * lda + n * n <= 2 * n * lda
