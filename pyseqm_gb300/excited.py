"""Excited states of the ground-state SCF: CIS (Tamm-Dancoff) and RPA (TDHF) by Davidson
iterations, on the GPU.

Mirrors rcis_batch (seqm/seqm_functions/rcis_batch.py:13-247), rcis_any_batch
(rcis_new.py:19-200) and rpa (rpa.py:12-210): the same guesses (unit vectors on the smallest
orbital-energy differences, the requested roots widened over degenerate differences, up to 7
extra vectors), preconditioned residual corrections orthogonalised twice against the subspace,
subspace collapse, convergence on the infinity norm of every root's residual, and the same
amplitude layout (occupied x virtual, padded to the batch's largest).  The matrix-vector
product

    (A V)_ia = (e_a - e_i) V_ia + 2 (C_occ^T G(C_occ V C_virt^T) C_virt)_ia,
    (B V)_ia = 2 (C_occ^T G(C_occ V C_virt^T)^T C_virt)_ia

forms the AO transition densities with batched GEMMs and contracts them with the two-electron
integrals in the CUDA kernel seqm_fock_general.  Molecules of a batch are independent: every
one keeps its own subspace (shorter ones padded with inert slots) and stops on its own test.
RPA is also available for batches of different molecules (the reference has it for batches of
one species only).
"""

import math

import numpy as np
import torch

from . import native

INERT = 1.0e6  # diagonal of the subspace matrix at padding slots: never among the lowest roots
A0_ANGSTROM = 0.529167  # bohr radius (seqm/seqm_functions/constants.py:9)
HARTREE_NEXMD = 27.2113962  # eV per hartree of the oscillator strength (rcis_batch.py:705)


class ExcitedStates:
    """Davidson solver bound to a converged BatchSCF whose final step kept the eigenvectors."""

    def __init__(self, s, window=None):
        """window: (n, m) the n highest occupied and m lowest virtual orbitals span the
        excitations (orbital_window, get_occ_virt rcis_batch.py:900-925; a batch of one species);
        None: all of them."""
        if s.evecs is None:
            raise ValueError("excited states need the ground state's eigenvectors (final(want_vectors=True))")
        L = s.L
        self.s, self.L = s, L
        dev = L.device
        f64 = dict(dtype=torch.float64, device=dev)
        self.nmol = L.nmol
        norb = L.norb.astype(np.int64)
        nocc = L.nocc.astype(np.int64)
        occ_lo = np.zeros_like(nocc)  # first occupied orbital of the excitation space
        self.window = None
        if window is not None:
            nb, ma = map(int, window)
            if not (np.all(norb == norb[0]) and np.all(nocc == nocc[0])):
                raise ValueError("orbital_window requires uniform nocc/norb across the batch.")
            if not (0 <= nb <= nocc[0] and 0 <= ma <= norb[0] - nocc[0]):
                raise ValueError("orbital_window out of bounds.")
            self.window = (nb, ma)
            occ_lo = nocc - nb
            norb, nocc = nocc + ma - occ_lo, nocc - occ_lo  # the window as a molecule of its own
        self.norb, self.nocc, self.nvirt = norb, nocc, norb - nocc
        nmax, self.no, self.nv = int(L.norb.max()), int(nocc.max()), int((norb - nocc).max())
        self.nmax = nmax
        # ragged element (m, r, c) <-> padded position m nmax^2 + r nmax + c (r, c over the AOs)
        nao = L.norb.astype(np.int64)
        gidx = np.concatenate([m * nmax * nmax + (np.arange(n)[:, None] * nmax + np.arange(n)[None, :]).reshape(-1)
                               for m, n in enumerate(nao)])
        self.gidx = torch.as_tensor(gidx, dtype=torch.int64, device=dev)
        self.T = int(gidx.size)
        Vp = torch.zeros(self.nmol * nmax * nmax, **f64)
        Vp[self.gidx] = s.evecs[: self.T]
        C = Vp.view(self.nmol, nmax, nmax).transpose(1, 2)  # columns: orbitals (eigenvector k = row k)
        ep = torch.zeros(self.nmol * nmax, **f64)
        rows = np.concatenate([m * nmax + np.arange(n) for m, n in enumerate(nao)])
        ep[torch.as_tensor(rows, device=dev)] = s.evals[: int(nao.sum())]
        e = ep.view(self.nmol, nmax)
        # occupied / virtual coefficients and orbital energies, padded with zeros
        io = torch.arange(self.no, device=dev)
        iv = torch.arange(self.nv, device=dev)
        no_t = torch.as_tensor(nocc, device=dev)
        nv_t = torch.as_tensor(norb - nocc, device=dev)
        lo_t = torch.as_tensor(occ_lo, device=dev)
        vo = io[None, :] < no_t[:, None]
        vv = iv[None, :] < nv_t[:, None]
        cols_o = (lo_t[:, None] + io[None, :]).clamp(max=nmax - 1)
        cols_v = (lo_t[:, None] + no_t[:, None] + iv[None, :]).clamp(max=nmax - 1)
        self.Co = torch.gather(C, 2, cols_o[:, None, :].expand(-1, nmax, -1)) * vo[:, None, :]
        self.Cv = torch.gather(C, 2, cols_v[:, None, :].expand(-1, nmax, -1)) * vv[:, None, :]
        eo = torch.gather(e, 1, cols_o)
        ev = torch.gather(e, 1, cols_v)
        self.valid = (vo[:, :, None] & vv[:, None, :]).reshape(self.nmol, -1)
        self.dE = (ev[:, None, :] - eo[:, :, None]).reshape(self.nmol, -1) * self.valid
        self.nov = torch.as_tensor(nocc * (norb - nocc), device=dev)

    # -------------------------------------------------------------- products
    def products(self, X, want_b=False):
        """A X (and B X) for trial vectors X (nmol, k, no*nv), zero outside each molecule's block."""
        nmol, k = X.shape[0], X.shape[1]
        Xm = X.view(nmol, k, self.no, self.nv)
        P = self.Co[:, None] @ Xm @ self.Cv[:, None].transpose(2, 3)  # (nmol, k, nmax, nmax)
        Pr = P.permute(1, 0, 2, 3).reshape(k, -1)[:, self.gidx].contiguous()
        G = torch.empty_like(Pr)
        s, L = self.s, self.L
        s.launches += 1
        native.check(s.lib.seqm_fock_general(L.struct, k, native.ptr(Pr), native.ptr(s.w_xx), native.ptr(s.w_xh),
                                             native.ptr(s.w_hh), native.ptr(G), self.T, None, s._s()),
                     "seqm_fock_general")
        Gp = torch.zeros(k, nmol * self.nmax * self.nmax, dtype=G.dtype, device=G.device)
        Gp[:, self.gidx] = G
        Gp = Gp.view(k, nmol, self.nmax, self.nmax).permute(1, 0, 2, 3)
        CoT = self.Co.transpose(1, 2)[:, None]
        AX = (2.0 * (CoT @ Gp @ self.Cv[:, None])).reshape(nmol, k, -1) + self.dE[:, None, :] * X
        AX = AX * self.valid[:, None, :]
        if not want_b:
            return AX
        BX = (2.0 * (CoT @ Gp.transpose(2, 3) @ self.Cv[:, None])).reshape(nmol, k, -1) * self.valid[:, None, :]
        return AX, BX

    # ------------------------------------------------------------------ guess
    def _targets(self, nroots):
        """Roots per molecule: nroots widened over degenerate orbital-energy differences (uniform
        batch: only where every molecule is degenerate there, rcis_batch.py:777-806; otherwise per
        molecule, rcis_new.py make_guess_any_batch), and the sorted candidate order."""
        d = torch.where(self.valid, self.dE, torch.full_like(self.dE, math.inf))
        srt, order = torch.sort(d, dim=1, stable=True)
        nov = self.nov.cpu().numpy()
        if int(nov.min()) < nroots:
            raise ValueError(f"Maximum number of roots for this batch of molecules is {int(nov.min())}. "
                             "Reduce the requested number of roots")
        s = srt.cpu().numpy()
        uniform = np.all(self.norb == self.norb[0]) and np.all(self.nocc == self.nocc[0])
        k = np.full(self.nmol, nroots, dtype=np.int64)
        if uniform:
            kk = nroots
            while kk < s.shape[1] and np.all(s[:, kk] - s[:, kk - 1] < 1e-4):
                kk += 1
            k[:] = kk
        else:
            for m in range(self.nmol):
                while k[m] < nov[m] and abs(s[m, k[m]] - s[m, k[m] - 1]) < 1e-4:
                    k[m] += 1
        return k, order

    # ------------------------------------------------------------------ solver
    def solve(self, nroots, tol, rpa=False, max_iter=None, max_subspace=None):
        """Lowest roots: energies (nmol, kmax) and amplitudes (nmol, kmax, no*nv), or for RPA
        (2, nmol, kmax, no*nv) with X, Y normalised to X.X - Y.Y = 1.  Every molecule keeps its own
        subspace (cnt[m] orthonormal vectors, no holes); the padding slots past cnt[m] are inert."""
        nmol, dev = self.nmol, self.dE.device
        k, order = self._targets(nroots)
        self.roots = k
        kmax = int(k.max())
        k_t = torch.as_tensor(k, device=dev)
        nov_np = self.nov.cpu().numpy()
        nstart = k + np.minimum(nov_np - k, 7)
        width = self.no * self.nv
        if max_subspace is None:
            # as getMaxSubspacesize (rcis_batch.py:542-566): 40 % of the free memory for the
            # subspace and its products, at most the full occupied-virtual space
            free = torch.cuda.mem_get_info(dev)[0] if dev.type == "cuda" else 8 << 30
            max_subspace = min(width, int(0.4 * free // (width * nmol * 8 * (3 if rpa else 2))))
        msub = max(int(max_subspace), int(nstart.max()) + 2 * kmax)
        cap = msub + 2 * kmax  # room for one iteration's new vectors past the collapse threshold
        max_iter = int(max_iter or (100 if rpa else 200))
        vec_tol = tol * (0.02 if rpa else 0.01 * math.sqrt(width))
        ar = torch.arange(cap, device=dev)
        V = torch.zeros(nmol, cap, width, dtype=torch.float64, device=dev)
        ns = torch.as_tensor(nstart, device=dev)
        n0 = int(nstart.max())
        sel = ar[None, :n0] < ns[:, None]
        V[:, :n0].scatter_(2, order[:, :n0, None], sel[..., None].double())
        AV = torch.zeros_like(V)
        BV = torch.zeros_like(V) if rpa else None
        cnt = ns.clone()  # subspace size per molecule
        new_lo = torch.zeros_like(cnt)  # the new vectors of a molecule: slots new_lo .. cnt - 1
        done = torch.zeros(nmol, dtype=torch.bool, device=dev)
        E = torch.zeros(nmol, kmax, dtype=torch.float64, device=dev)
        amp = torch.zeros((2, nmol, kmax, width) if rpa else (nmol, kmax, width), dtype=torch.float64, device=dev)
        root_ok = torch.arange(kmax, device=dev)[None, :] < k_t[:, None]
        rows = torch.arange(nmol, device=dev)
        self.iterations = 0
        for it in range(max_iter + 1):
            # products of the new vectors, gathered into one block
            nnew = cnt - new_lo
            b = int(nnew.max())
            if b > 0:
                pos = new_lo[:, None] + ar[None, :b]
                keep = ar[None, :b] < nnew[:, None]
                blk = torch.gather(V, 1, pos[..., None].expand(-1, -1, width)) * keep[..., None]
                out = self.products(blk, want_b=rpa)
                for dst, val in ((AV, out[0]), (BV, out[1])) if rpa else ((AV, out),):
                    old = torch.gather(dst, 1, pos[..., None].expand(-1, -1, width))
                    dst.scatter_(1, pos[..., None].expand(-1, -1, width), torch.where(keep[..., None], val, old))
            self.iterations = it + 1
            hi = int(cnt.max())
            Vs = V[:, :hi]
            inert = torch.diag_embed((ar[None, :hi] >= cnt[:, None]).double() * INERT)
            if rpa:
                As = Vs @ AV[:, :hi].transpose(1, 2) + inert
                Bs = Vs @ BV[:, :hi].transpose(1, 2)
                w, Xs, Ys = _rpa_subspace(As + Bs, As - Bs, kmax)
                Xa = Xs.transpose(1, 2) @ Vs
                Ya = Ys.transpose(1, 2) @ Vs
                AX, AY = Xs.transpose(1, 2) @ AV[:, :hi], Ys.transpose(1, 2) @ AV[:, :hi]
                BX, BY = Xs.transpose(1, 2) @ BV[:, :hi], Ys.transpose(1, 2) @ BV[:, :hi]
                resX = AX + BY - w[..., None] * Xa
                resY = AY + BX + w[..., None] * Ya
                rR, rL = resX - resY, resX + resY
                rn = torch.maximum(rR.abs().amax(2), rL.abs().amax(2))
            else:
                H = Vs @ AV[:, :hi].transpose(1, 2) + inert
                w_all, U = torch.linalg.eigh(H)
                w, Us = w_all[:, :kmax], U[:, :, :kmax]
                Xa = Us.transpose(1, 2) @ Vs
                R = Us.transpose(1, 2) @ AV[:, :hi] - w[..., None] * Xa
                rn = R.abs().amax(2)
            bad = (rn > tol) & root_ok
            conv_now = (~done) & ~bad.any(1)
            self._store(E, amp, w, Xa, Ya if rpa else None, conv_now)
            done |= conv_now
            if bool(done.all()) or it == max_iter:
                break
            # corrections of the unconverged roots, preconditioned (rcis_batch.py:213-216, rpa.py:112-113)
            den = w[..., None] - self.dE[:, None, :]
            if rpa:
                cand = torch.cat([rR / den, rL / den], dim=1) * self.valid[:, None, :]
                cmask = torch.cat([bad, bad], dim=1) & ~done[:, None]
            else:
                cand = (R / den) * self.valid[:, None, :]
                cmask = bad & ~done[:, None]
            cand = torch.nan_to_num(cand, nan=0.0, posinf=0.0, neginf=0.0) * cmask[..., None]
            nadd = cmask.sum(1)
            # collapse onto the current roots where the subspace would outgrow its limit
            # (rcis_batch.py:184-200, rpa.py:134-158); never where it already spans the space
            coll = (~done) & (cnt + nadd > msub) & (cnt < self.nov) & (msub < width)
            if bool(coll.any()):
                keep_v = torch.cat([Xa, Ya], 1) if rpa else Xa
                Q = torch.linalg.qr(keep_v.transpose(1, 2)).Q.transpose(1, 2) * self.valid[:, None, :]
                nk = Q.shape[1]
                coef = Q @ Vs.transpose(1, 2)
                cm = coll[:, None, None]
                AV[:, :nk] = torch.where(cm, coef @ AV[:, :hi], AV[:, :nk])
                AV[:, nk:] = torch.where(cm, torch.zeros_like(AV[:, nk:]), AV[:, nk:])
                if rpa:
                    BV[:, :nk] = torch.where(cm, coef @ BV[:, :hi], BV[:, :nk])
                    BV[:, nk:] = torch.where(cm, torch.zeros_like(BV[:, nk:]), BV[:, nk:])
                V[:, :nk] = torch.where(cm, Q, V[:, :nk])
                V[:, nk:] = torch.where(cm, torch.zeros_like(V[:, nk:]), V[:, nk:])
                cnt = torch.where(coll, torch.full_like(cnt, nk), cnt)
            # orthonormalise the kept candidates into each molecule's subspace, twice
            # (orthogonalize_to_current_subspace, rcis_batch.py:510-539)
            idx = torch.argsort((~cmask).to(torch.int8), dim=1, stable=True)[:, : int(nadd.max())]
            cand = torch.gather(cand, 1, idx[..., None].expand(-1, -1, width))
            cm = torch.gather(cmask, 1, idx)
            new_lo = cnt.clone()
            for j in range(cand.shape[1]):
                hi = int(cnt.max())
                v = cand[:, j]
                for _ in range(2):
                    v = v - ((v[:, None, :] @ V[:, :hi].transpose(1, 2)) @ V[:, :hi]).squeeze(1)
                nrm = v.norm(dim=1)
                ok = cm[:, j] & (nrm > vec_tol) & ~done & (cnt < cap)
                slot = cnt.clamp(max=cap - 1)
                V[rows, slot] = torch.where(ok[:, None], v / nrm.clamp_min(1e-300)[:, None], V[rows, slot])
                cnt = cnt + ok.long()
            stalled = (~done) & (cnt == new_lo)
            if bool(stalled.any()):  # no new direction: the subspace holds the roots (rcis_batch.py:232-236)
                self._store(E, amp, w, Xa, Ya if rpa else None, stalled)
                done |= stalled
                if bool(done.all()):
                    break
        self.converged = done.cpu().numpy()
        return E, amp

    # ------------------------------------------------------- excited-state densities
    def _G(self, Xp):
        """Two-electron part G(X) (seqm_fock_general) of padded general densities
        Xp (nmol, k, nmax, nmax); the reference's makeA_pi_batched (rcis_batch.py:296-388)."""
        nmol, k = Xp.shape[0], Xp.shape[1]
        Xr = Xp.permute(1, 0, 2, 3).reshape(k, -1)[:, self.gidx].contiguous()
        G = torch.empty_like(Xr)
        s, L = self.s, self.L
        s.launches += 1
        native.check(s.lib.seqm_fock_general(L.struct, k, native.ptr(Xr), native.ptr(s.w_xx), native.ptr(s.w_xh),
                                             native.ptr(s.w_hh), native.ptr(G), self.T, None, s._s()),
                     "seqm_fock_general")
        Gp = torch.zeros(k, nmol * self.nmax * self.nmax, dtype=G.dtype, device=G.device)
        Gp[:, self.gidx] = G
        return Gp.view(k, nmol, self.nmax, self.nmax).permute(1, 0, 2, 3)

    def _hessian(self, z):
        """Orbital-rotation Hessian on z (nmol, no*nv): (e_a - e_i) z + 2 C_occ^T G(Z + Z^T) C_virt
        with Z = C_occ z C_virt^T (make_A_times_zvector_batched, rcis_batch.py:951-965)."""
        nmol = self.nmol
        Z = self.Co @ z.view(nmol, self.no, self.nv) @ self.Cv.transpose(1, 2)
        G = self._G((Z + Z.transpose(1, 2))[:, None])[:, 0]
        Az = (2.0 * (self.Co.transpose(1, 2) @ G @ self.Cv)).reshape(nmol, -1) + self.dE * z
        return Az * self.valid

    def _cg(self, b, tol, max_iter=100):
        """Z-vector: batched conjugate gradients on the Hessian, preconditioned by e_a - e_i,
        stopping per molecule when the largest residual element is below tol
        (conjugate_gradient_batch, cg_solver.py:6-95)."""
        Minv = 1.0 / torch.where(self.valid, self.dE, torch.ones_like(self.dE))
        x = torch.zeros_like(b)
        r = b.clone()
        z = r * Minv
        p = z.clone()
        rs_old = (r * z).sum(1)
        active = r.abs().amax(1) >= tol
        for _ in range(max_iter):
            if not bool(active.any()):
                return x
            Ap = self._hessian(p)
            alpha = rs_old / (p * Ap).sum(1).clamp(min=1e-20) * active
            x = x + alpha[:, None] * p
            r = r - alpha[:, None] * Ap
            active = r.abs().amax(1) >= tol
            z = r * Minv
            rs_new = (r * z).sum(1)
            beta = rs_new / rs_old.clamp(min=1e-20) * active
            p = z + beta[:, None] * p
            rs_old = rs_new
        if bool(active.any()):
            raise RuntimeError(f"Conjugate gradient did not converge in {max_iter} steps")
        return x

    def state_densities(self, X, Y=None, tol=1e-6):
        """Transition density R, unrelaxed difference density B and relaxed difference density
        D = B + Z + Z^T of one state per molecule (make_cis_densities, rcis_batch.py:971-1059),
        padded (nmol, nmax, nmax).  X (and Y for RPA): the state's amplitudes (nmol, no*nv).
        Z solves the CPSCF equations H z = rhs built from G(B) and G(R)."""
        if self.window is not None:
            raise NotImplementedError("excited-state forces with an orbital_window are not supported")
        nmol, no, nv = self.nmol, self.no, self.nv
        Co, Cv = self.Co, self.Cv
        CoT = Co.transpose(1, 2)
        Xm = X.view(nmol, no, nv)
        R = Co @ Xm @ Cv.transpose(1, 2)
        Bv = Cv @ Xm.transpose(1, 2)  # (nmol, nmax, no)
        Bo = Co @ Xm  # (nmol, nmax, nv)
        B = Bv @ Bv.transpose(1, 2) - Bo @ Bo.transpose(1, 2)
        if Y is not None:
            Ym = Y.view(nmol, no, nv)
            R = R + Cv @ Ym.transpose(1, 2) @ CoT
            BvY, BoY = Cv @ Ym.transpose(1, 2), Co @ Ym
            B = B + BvY @ BvY.transpose(1, 2) - BoY @ BoY.transpose(1, 2)
        G2 = 2.0 * self._G(torch.stack((B, R), dim=1))
        Bpi, Rpi = G2[:, 0], G2[:, 1]
        rhs = -(CoT @ Bpi.transpose(1, 2) @ Cv)
        rhs = rhs - Bv.transpose(1, 2) @ Rpi.transpose(1, 2) @ Cv
        rhs = rhs + CoT @ Rpi.transpose(1, 2) @ Bo
        if Y is not None:
            rhs = rhs - BvY.transpose(1, 2) @ Rpi @ Cv
            rhs = rhs + CoT @ Rpi @ BoY
        z = self._cg(rhs.reshape(nmol, -1) * self.valid, tol)
        Zao = Co @ z.view(nmol, no, nv) @ Cv.transpose(1, 2)
        return R, B, B + Zao + Zao.transpose(1, 2)

    def transition_densities(self, amp, rpa=False):
        """C_occ X C_virt^T (+ C_virt Y^T C_occ^T for RPA) per root, (nmol, kmax, nmax, nmax) in
        the packed basis of each molecule (zero past its norb)."""
        nmol = self.nmol
        X = amp[0] if rpa else amp
        k = X.shape[1]
        R = self.Co[:, None] @ X.view(nmol, k, self.no, self.nv) @ self.Cv.transpose(1, 2)[:, None]
        if rpa:
            Y = amp[1].view(nmol, k, self.no, self.nv)
            R = R + self.Cv[:, None] @ Y.transpose(2, 3) @ self.Co.transpose(1, 2)[:, None]
        return R

    def nac_densities(self, X, pairs):
        """Unrelaxed CIS state-to-state densities B_ij = sym(V_i V_j^T - O_i O_j^T) with
        V = C_virt X^T and O = C_occ X (calc_nac, nac.py:142-171), padded, one per 0-based
        state pair."""
        nmol, no, nv = self.nmol, self.no, self.nv
        out = []
        for i, j in pairs:
            Xi, Xj = X[:, i].view(nmol, no, nv), X[:, j].view(nmol, no, nv)
            B = (self.Cv @ Xi.transpose(1, 2)) @ (self.Cv @ Xj.transpose(1, 2)).transpose(1, 2) \
                - (self.Co @ Xi) @ (self.Co @ Xj).transpose(1, 2)
            out.append(0.5 * (B + B.transpose(1, 2)))
        return out

    def to_ragged(self, Mp):
        """Padded (nmol, nmax, nmax) -> the ragged per-molecule blocks of the batch."""
        return Mp.reshape(-1)[self.gidx].contiguous()

    # ------------------------------------------------------- transition properties
    def _dipole_geometry(self):
        """Per AO of the packed basis (padded to nmax): the owning atom's position (Angstrom), and
        per heavy atom the flat (s, p_d) / (p_d, s) positions of its one-centre dipole integrals
        with dd (Angstrom); padding entries carry zero weight."""
        L = self.L
        nmax, nmol = self.nmax, self.nmol
        nhmax = max(1, int(L.nheavy.max()))
        ao_atom = np.full((nmol, nmax), -1, dtype=np.int64)
        sp_a = np.zeros((nmol, nhmax, 3), dtype=np.int64)
        sp_b = np.zeros((nmol, nhmax, 3), dtype=np.int64)
        heavy = np.full((nmol, nhmax), -1, dtype=np.int64)
        d3 = np.arange(3)
        for m in range(nmol):
            a0, nh, ny = int(L.atom_off[m]), int(L.nheavy[m]), int(L.nhyd[m])
            ao_atom[m, : 4 * nh] = a0 + np.repeat(np.arange(nh), 4)
            ao_atom[m, 4 * nh: 4 * nh + ny] = a0 + nh + np.arange(ny)
            o = 4 * np.arange(nh)
            sp_a[m, :nh] = o[:, None] * nmax + o[:, None] + 1 + d3[None, :]
            sp_b[m, :nh] = (o[:, None] + 1 + d3[None, :]) * nmax + o[:, None]
            heavy[m, :nh] = a0 + np.arange(nh)
        dev = self.dE.device
        xyz = torch.as_tensor(L.xyz, dtype=torch.float64, device=dev)
        par = L.dev["par"].view(native.NPAR, -1)
        dd = par[native.PAR["_dd"]] * A0_ANGSTROM  # bohr -> Angstrom (dipole.py:40-41)
        at = torch.as_tensor(ao_atom, device=dev)
        hv = torch.as_tensor(heavy, device=dev)
        return dict(ao_xyz=torch.where(at[..., None] >= 0, xyz[at.clamp(min=0)], 0.0),
                    sp_a=torch.as_tensor(sp_a.reshape(nmol, -1), device=dev),
                    sp_b=torch.as_tensor(sp_b.reshape(nmol, -1), device=dev),
                    dd=torch.where(hv >= 0, dd[hv.clamp(min=0)], 0.0))

    def dipole_contract(self, R):
        """sum_mn R_mn D^d_mn for padded matrices R (nmol, k, nmax, nmax) with the one-centre
        dipole integrals of calc_dipole_matrix (dipole.py:7-82): (nmol, k, 3), Angstrom x charge."""
        g = self._dipole_geometry()
        nmol, k = R.shape[0], R.shape[1]
        mu = -torch.einsum("bkn,bnd->bkd", torch.diagonal(R, dim1=2, dim2=3), g["ao_xyz"])
        Rf = R.reshape(nmol, k, -1)
        sp = Rf.gather(2, g["sp_a"][:, None, :].expand(-1, k, -1)) + Rf.gather(2, g["sp_b"][:, None, :].expand(-1, k, -1))
        return mu - torch.einsum("bkhd,bh->bkd", sp.view(nmol, k, -1, 3), g["dd"])

    def transition_properties(self, E, amp, rpa=False):
        """Transition dipoles (atomic units, (nmol, kmax, 3)) and oscillator strengths (nmol, kmax)
        of the roots, as calc_transition_dipoles (rcis_batch.py:679-710, rcis_new.py:547-585):
        the transition density R = C_occ X C_virt^T (+ C_virt Y^T C_occ^T for RPA) against the
        one-centre dipole integrals of calc_dipole_matrix (dipole.py:7-82: -R_A on the diagonal of
        atom A's AOs, -dd_A between its s and p_d), mu = sqrt(2)/a0 sum R.D and
        f = 2/3 (E / 27.2113962) |mu|^2; zero for the padding roots of a molecule."""
        k = (amp[0] if rpa else amp).shape[1]
        mu = self.dipole_contract(self.transition_densities(amp, rpa)) * (math.sqrt(2.0) / A0_ANGSTROM)
        ok = (torch.arange(k, device=E.device)[None, :] < torch.as_tensor(self.roots, device=E.device)[:, None])
        mu = mu * ok[..., None]
        f = (2.0 / 3.0) * E / HARTREE_NEXMD * (mu * mu).sum(-1) * ok
        return mu, f

    @staticmethod
    def _store(E, amp, w, Xa, Ya, mask):
        if not bool(mask.any()):
            return
        E[mask] = w[mask]
        if Ya is None:
            amp[mask] = Xa[mask]
        else:
            amp[0, mask] = Xa[mask]
            amp[1, mask] = Ya[mask]


def _rpa_subspace(ApB, AmB, k):
    """Lowest k RPA roots of the subspace problem (rpa.py:213-278): w^2 from
    (A-B)^1/2 (A+B) (A-B)^1/2, X + Y = (A-B)^1/2 z, X - Y = (A+B)(X+Y)/w, X.X - Y.Y = 1."""
    ev, U = torch.linalg.eigh(AmB)
    if bool((ev < 0.0).any()):
        raise ValueError("A-B matrix has negative eigenvalues, cannot compute sqrt of A-B matrix")
    S = (U * ev.sqrt()[:, None, :]) @ U.transpose(1, 2)
    w2, Z = torch.linalg.eigh(S @ ApB @ S)
    if bool((w2[:, :k] < 0.0).any()):
        raise ValueError("negative RPA eigenvalues w^2: imaginary roots (the SCF solution may not be a minimum)")
    w = w2[:, :k].sqrt()
    XpY = S @ Z[:, :, :k]
    XmY = (ApB @ XpY) / w[:, None, :]
    X, Y = XpY + XmY, XpY - XmY
    nrm = ((X ** 2).sum(1) - (Y ** 2).sum(1)).sqrt()
    return w, X / nrm[:, None, :], Y / nrm[:, None, :]
