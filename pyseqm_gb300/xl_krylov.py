"""Fermi-Dirac density and the rank-m Krylov kernel of KSA-XL-BOMD, batched on the device.

Mirrors Fermi_Q (seqm/seqm_functions/fermi_q.py:8-72), Canon_DM_PRT (canon_dm_prt.py:6-39;
Alg. 2 of J. Chem. Theory Comput. 16, 3628 (2020)) and the Krylov loop of EnergyXL
(dynamics/xlbomd.py:200-341).  Molecules are held as zero-padded per-molecule matrices in their
packed basis (orbitals past norb inert); the two-electron response of each Krylov vector comes
from the CUDA kernel seqm_fock_general.
"""

import numpy as np
import torch

from . import native

KB_EV = 8.61739e-5  # eV/K (dynamics/xlbomd.py:206)
CANON_DM_PRT_ITER = 10  # dynamics/xlbomd.py:55


class PaddedBasis:
    """Ragged per-molecule blocks <-> zero-padded (nmol, nmax, nmax) tensors."""

    def __init__(self, L):
        self.L = L
        norb = L.norb.astype(np.int64)
        self.nmax = int(norb.max())
        nm = self.nmax
        gidx = np.concatenate([m * nm * nm + (np.arange(n)[:, None] * nm + np.arange(n)[None, :]).reshape(-1)
                               for m, n in enumerate(norb)])
        self.gidx = torch.as_tensor(gidx, dtype=torch.int64, device=L.device)
        rows = np.concatenate([m * nm + np.arange(n) for m, n in enumerate(norb)])
        self.rows = torch.as_tensor(rows, dtype=torch.int64, device=L.device)
        self.mask = torch.arange(nm, device=L.device)[None, :] < torch.as_tensor(norb, device=L.device)[:, None]

    def to_padded(self, flat):
        out = torch.zeros(self.L.nmol * self.nmax * self.nmax, dtype=flat.dtype, device=flat.device)
        out[self.gidx] = flat[: self.gidx.numel()]
        return out.view(self.L.nmol, self.nmax, self.nmax)

    def to_ragged(self, pad):
        return pad.reshape(-1)[self.gidx].contiguous()

    def vector_to_padded(self, flat):
        out = torch.zeros(self.L.nmol * self.nmax, dtype=flat.dtype, device=flat.device)
        out[self.rows] = flat[: self.rows.numel()]
        return out.view(self.L.nmol, self.nmax)


def fermi_density(e, Q, nocc, mask, T):
    """Fermi-Dirac occupations at T with mu from Newton iterations on sum_i f_i = nocc (at most 64,
    tolerance 1e-9), D = 2 Q f Q^T and the entropy S (fermi_q.py:8-72)."""
    beta = 1.0 / (KB_EV * T)
    m = mask.to(e.dtype)
    nocc_t = torch.as_tensor(nocc, dtype=e.dtype, device=e.device)
    idx = torch.as_tensor(nocc, dtype=torch.int64, device=e.device)[:, None]
    mu = 0.5 * (e.gather(1, idx - 1) + e.gather(1, idx))
    fe = None
    for _ in range(64):
        fe = torch.sigmoid(-beta * (e - mu)) * m
        occ = fe.sum(1)
        if bool(((nocc_t - occ).abs() <= 1e-9).all()):
            break
        d = (beta * fe * (1.0 - fe)).sum(1).clamp_min(1e-30)
        mu = mu + ((nocc_t - occ) / d)[:, None]
    D = 2.0 * (Q * fe[:, None, :]) @ Q.transpose(1, 2)
    ok = (fe > 1e-14) & ((1.0 - fe) > 1e-14)
    p = fe.masked_fill(~ok, 0.5)
    S = (-KB_EV * (p * torch.log(p) + (1.0 - p) * torch.log(1.0 - p)) * ok.to(e.dtype)).sum(1)
    return D, S, fe, mu


def canon_dm_prt(F1, T, Q, e, mu0, mask, m=CANON_DM_PRT_ITER):
    """First-order density response to F1 (canon_dm_prt.py:6-39), batched."""
    beta = 1.0 / (KB_EV * T)
    cnst = 2.0 ** (-2 - m) * beta
    p0 = ((0.5 - cnst * (e - mu0)) * mask.to(e.dtype))[:, :, None]
    P1 = -cnst * (Q.transpose(1, 2) @ F1 @ Q)
    for _ in range(m):
        p02 = p0 * p0
        dX1 = p0 * P1 + P1 * p0.transpose(1, 2)
        iD0 = 1.0 / (2.0 * (p02 - p0) + 1.0)
        p0 = iD0 * p02
        P1 = iD0 * (dX1 + 2.0 * (P1 - dX1) * p0.transpose(1, 2))
    dpdmu = beta * p0 * (1.0 - p0)
    dmu1 = -torch.diagonal(P1, dim1=1, dim2=2).sum(1) / dpdmu.sum((1, 2))
    P1 = P1 + torch.diag_embed(dpdmu[:, :, 0]) * dmu1[:, None, None]
    return Q @ P1 @ Q.transpose(1, 2)


def krylov_kernel(s, basis, D, P, Q, e, mu, T, rank, err_threshold):
    """dP2dt2 = -V alpha from the rank-m Krylov approximation of the kernel acting on D - P
    (dynamics/xlbomd.py:240-341); matrices padded per molecule.  Returns dP2dt2 and the
    relative residual per molecule."""
    L = basis.L
    lib = native.load()
    dDS = D - P
    nrm = torch.linalg.norm(dDS, dim=(1, 2))
    V, W = [], []
    dW = dDS
    err = torch.full((L.nmol,), 10.0, dtype=D.dtype, device=D.device)
    alpha = None
    k = -1
    T_el = int(basis.gidx.numel())
    while k < rank - 1 and float(err.max()) > err_threshold:
        k += 1
        v = dW.clone()
        for vj in V:
            v = v - (v.transpose(1, 2) * vj).sum((1, 2))[:, None, None] * vj
        v = v / torch.linalg.norm(v, dim=(1, 2), keepdim=True)
        V.append(v)
        vr = basis.to_ragged(v)
        g = torch.empty_like(vr)
        s.launches += 1
        native.check(lib.seqm_fock_general(L.struct, 1, native.ptr(vr), native.ptr(s.w_xx), native.ptr(s.w_xh),
                                           native.ptr(s.w_hh), native.ptr(g), T_el, None, s._s()), "seqm_fock_general")
        P1 = canon_dm_prt(basis.to_padded(g), T, Q, e, mu, basis.mask)
        w = P1 - v
        W.append(w)
        dW = w
        Wm = torch.stack(W, dim=-1)
        Om = torch.einsum("bjir,bijq->brq", Wm, Wm)
        rhs = torch.einsum("bjir,bij->br", Wm, dDS)
        alpha = torch.linalg.solve(Om, rhs[..., None])[..., 0]
        err = torch.linalg.norm(torch.einsum("bijr,br->bij", Wm, alpha) - dDS, dim=(1, 2)) / nrm
    Vm = torch.stack(V, dim=-1)
    return -torch.einsum("bijr,br->bij", Vm, alpha), err
