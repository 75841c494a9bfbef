"""The first-order occupied-virtual density of the Jacobi kernel (k_jacobi, newton_density)
restated in NumPy: from eigenvector rows perturbed by small rotations, the Loewdin-
orthonormalised first-order rotation of the smaller set gives the density to second order in
the largest occupied-virtual ratio |a_uo| / gap, and an idempotent P."""

import numpy as np
import pytest


def _first_order_density(A, V, nocc):
    n = A.shape[0]
    dg = np.diag(A)
    order = np.argsort(dg, kind="stable")
    use_occ = nocc <= n - nocc
    S, T = (order[:nocc], order[nocc:]) if use_occ else (order[nocc:], order[:nocc])
    theta = A[np.ix_(T, S)].T / (dg[S][:, None] - dg[T][None, :])
    C1 = V[S] + theta @ V[T]
    E = C1 @ C1.T - np.eye(len(S))
    U = C1 - 0.5 * E @ C1
    return 2.0 * U.T @ U if use_occ else 2.0 * (np.eye(n) - U.T @ U), \
        np.abs(A[np.ix_(order[nocc:], order[:nocc])]).max() / (dg[order[nocc]] - dg[order[nocc - 1]])


@pytest.mark.parametrize("n,nocc", [(60, 20), (144, 48), (100, 70)])
@pytest.mark.parametrize("rot", [1e-5, 1e-6, 1e-7])
def test_first_order_density_error_is_second_order(n, nocc, rot):
    rng = np.random.default_rng(n + nocc)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    ev = np.sort(np.r_[rng.uniform(-40, -5, nocc), rng.uniform(0, 30, n - nocc)])
    F = (Q * ev) @ Q.T
    F = 0.5 * (F + F.T)
    w, C = np.linalg.eigh(F)
    P_exact = 2.0 * C[:, :nocc] @ C[:, :nocc].T
    K = rng.normal(size=(n, n)) * rot
    V = (C @ np.linalg.qr(np.eye(n) + K - K.T)[0]).T  # eigenvector rows, slightly rotated
    A = V @ F @ V.T
    P, theta = _first_order_density(A, V, nocc)
    assert np.abs(P - P_exact).max() <= 10.0 * theta**2 + 1e-13
    X = 0.5 * P
    assert np.abs(X @ X - X).max() < 1e-13
    if theta <= 1e-5:  # the kernel's threshold: density error well below the 1e-7 parity bound
        assert np.abs(P - P_exact).max() < 1e-9


def _ov_block_density(V, F, nocc, dg):
    """newton_density_ov: the coupling block alone in FP64, small products in FP32."""
    n = F.shape[0]
    order = np.argsort(dg, kind="stable")
    use_occ = nocc <= n - nocc
    S, T = (order[:nocc], order[nocc:]) if use_occ else (order[nocc:], order[:nocc])
    a_st = (V[S] @ F) @ V[T].T
    theta = a_st / (dg[S][:, None] - dg[T][None, :])
    f32 = np.float32
    C1 = V[S] + (theta.astype(f32) @ V[T].astype(f32)).astype(np.float64)
    E = (theta.astype(f32) @ theta.T.astype(f32)).astype(np.float64)
    U = C1 - 0.5 * (E.astype(f32) @ C1.astype(f32)).astype(np.float64)
    P = 2.0 * U.T @ U if use_occ else 2.0 * (np.eye(n) - U.T @ U)
    return P, np.abs(theta).max()


@pytest.mark.parametrize("n,nocc", [(60, 20), (144, 48), (100, 70), (8, 4)])
def test_fp32_sweeps_then_coupling_block_density(n, nocc):
    """fp32_sweeps_orth + newton_density_ov: eigenvectors good to FP32 only (W from an FP32
    diagonalisation of the rotated F), X = W V formed in FP32, one Newton-Schulz step with
    D = X X^T - I accumulated in FP64 from the FP32 values, then the first-order density
    from the FP64 coupling block: density error ~1e-10, far below the 1e-7 parity bound."""
    rng = np.random.default_rng(7 * n + nocc)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    ev = np.sort(np.r_[rng.uniform(-40, -5, nocc), rng.uniform(0, 30, n - nocc)])
    F = (Q * ev) @ Q.T
    F = 0.5 * (F + F.T)
    w, C = np.linalg.eigh(F)
    P_exact = 2.0 * C[:, :nocc] @ C[:, :nocc].T
    K = rng.normal(size=(n, n)) * 1e-2
    V = (C @ np.linalg.qr(np.eye(n) + K - K.T)[0]).T  # warm start, rotations ~1e-2
    f32 = np.float32
    A32 = (V.astype(f32) @ F.astype(f32)) @ V.T.astype(f32)
    d32, W = np.linalg.eigh(0.5 * (A32 + A32.T))  # FP32 sweeps: rotations W (rows)
    W = W.T.astype(f32)
    X = (W @ V.astype(f32)).astype(np.float64)  # FP32 values
    D = X @ X.T - np.eye(n)  # exact products, FP64 sums
    V2 = X - 0.5 * (D.astype(f32) @ X.astype(f32)).astype(np.float64)
    assert np.abs(V2 @ V2.T - np.eye(n)).max() < 5e-13  # second order in |D| ~ 2e-7
    dg = np.zeros(n)
    dg[:] = d32  # swept diagonal in row order
    P, theta = _ov_block_density(V2, F, nocc, dg)
    assert theta <= 1e-5
    assert np.abs(P - P_exact).max() < 1e-9
    X2 = 0.5 * P
    assert np.abs(X2 @ X2 - X2).max() < 1e-12


def _single_rotation(V, F, nocc, passes=3):
    """rotate_orth restated: Theta from the fixed-point passes of the block Sylvester equation
    on A32 = V F V^T (FP32), W = I + K + K^2 / 2 in FP32, then the lift of the FP32 sweeps
    (X = W V in FP32, D = X X^T - I from exact products, one Newton-Schulz step)."""
    n = F.shape[0]
    f32 = np.float32
    A32 = (V.astype(f32) @ F.astype(f32)) @ V.T.astype(f32)
    A32 = np.triu(A32) + np.triu(A32, 1).T
    dg = np.diag(A32).astype(np.float64)
    order = np.argsort(dg, kind="stable")
    use_occ = nocc <= n - nocc
    S, T = (order[:nocc], order[nocc:]) if use_occ else (order[nocc:], order[:nocc])
    a = A32[np.ix_(S, T)]
    Att = A32[np.ix_(T, T)].copy()
    Ass = A32[np.ix_(S, S)].copy()
    np.fill_diagonal(Att, 0.0)
    np.fill_diagonal(Ass, 0.0)
    d = (dg[S][:, None] - dg[T][None, :]).astype(f32)
    th = (a / d).astype(f32)
    for _ in range(passes - 1):
        th = ((a + th @ Att - Ass @ th) / d).astype(f32)
    W = np.eye(n, dtype=f32)
    W[np.ix_(S, S)] -= f32(0.5) * (th @ th.T)
    W[np.ix_(T, T)] -= f32(0.5) * (th.T @ th)
    W[np.ix_(S, T)] = th
    W[np.ix_(T, S)] = -th.T
    X = (W @ V.astype(f32)).astype(np.float64)
    D = X @ X.T - np.eye(n)
    V2 = X - 0.5 * (D.astype(f32) @ X.astype(f32)).astype(np.float64)
    return V2, dg, float(np.sqrt((th.astype(np.float64) ** 2).sum()))


@pytest.mark.parametrize("n,nocc", [(144, 96), (98, 49), (60, 20), (12, 8)])
@pytest.mark.parametrize("dF", [1e-4, 1e-3])
def test_single_rotation_then_coupling_block_density(n, nocc, dF):
    """rotate_orth + newton_density_ov: a warm start (eigenvector rows of an earlier Fock matrix,
    mixed within the occupied and the virtual blocks as earlier rotations leave them) whose
    occupied-virtual ratio is <= 1e-3 is brought to block-diagonal form by one rotation in place
    of FP32 sweeps; what coupling is left is at A32's FP32 rounding, the rows stay orthonormal to
    FP64 accuracy, and the density is good to < 1e-8 (the parity bound is 1e-7)."""
    from scipy.linalg import expm

    rng = np.random.default_rng(3 * n + nocc)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    ev = np.sort(np.r_[rng.uniform(-40, -10, nocc), rng.uniform(0, 30, n - nocc)])
    F0 = (Q * ev) @ Q.T
    F0 = 0.5 * (F0 + F0.T)
    w0, C0 = np.linalg.eigh(F0)
    K = rng.normal(size=(n, n)) * dF
    K = K - K.T
    M = np.zeros((n, n))
    M[:nocc, :nocc] = K[:nocc, :nocc]
    M[nocc:, nocc:] = K[nocc:, nocc:]
    V = expm(M) @ C0.T  # rows: the occupied and virtual subspaces of F0, mixed within each
    Pert = rng.normal(size=(n, n))
    Pert = 0.5 * (Pert + Pert.T)
    F = F0 + Pert * (10.0 * dF / np.abs(Pert).max())
    w, C = np.linalg.eigh(F)
    P_exact = 2.0 * C[:, :nocc] @ C[:, :nocc].T
    A = V @ F @ V.T
    dga = np.diag(A)
    o = np.argsort(dga)
    ratio = np.abs(A[np.ix_(o[nocc:], o[:nocc])]).max() / (dga[o[nocc]] - dga[o[nocc - 1]])
    assert 5e-6 < ratio <= 1e-3  # the range the kernel takes this path for
    V2, dg, norm = _single_rotation(V, F, nocc)
    assert norm <= 1e-2  # ROT_NORM
    assert np.abs(V2 @ V2.T - np.eye(n)).max() < 5e-13
    P, theta = _ov_block_density(V2, F, nocc, dg)
    assert theta <= 1e-6  # well inside the first-order density's 1e-5
    assert np.abs(P - P_exact).max() < 1e-8
    X2 = 0.5 * P
    assert np.abs(X2 @ X2 - X2).max() < 1e-12
