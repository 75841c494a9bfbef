"""Device-resident batched SCF driver over the native kernels.

``BatchSCF`` owns every device buffer of one ragged batch and runs the
reference's SCF semantics (seqm/seqm_functions/scf_loop.py:2034-2394):

    hcore -> initial diagonal density -> F(P0), E(P0)
    repeat for molecules still active:
        density step (Jacobi eigensolver, or SP2)  -> Pnew
        mixing (linear scf_forward0 / adaptive scf_forward1 / Pulay DIIS scf_forward2) -> P, Pold
        F(P), Eelec(P) and the get_error test, which retires converged molecules
    final eigen-decomposition of F (orbital energies and vectors)

Converged molecules are retired on the device (their ``active`` flag drops)
and every kernel skips them, so a molecule's trajectory does not depend on its
batch mates.  The host reads one byte count per iteration to stop the loop.
"""

import ctypes
import time

import numpy as np
import torch

from . import native
from .layout import Layout

MAX_ITER = 1000  # scf_loop.py:29
JACOBI_MAX_N = 160


class BatchSCF:
    def __init__(self, layout: Layout, stream=None, jacobi_max_n=JACOBI_MAX_N):
        if layout.dev is None:
            raise ValueError("layout must be uploaded with to_device() first")
        self.L = layout
        self.lib = native.load()
        dev = layout.device
        f64 = dict(dtype=torch.float64, device=dev)
        T = int(layout.mat_off[-1])
        R = int(layout.row_off[-1])
        nm = layout.nmol
        self.w_xx = torch.empty(max(1, 100 * layout.nxx), **f64)
        self.w_xh = torch.empty(max(1, 10 * layout.nxh), **f64)
        self.w_hh = torch.empty(max(1, layout.nhh), **f64)
        self.enuc_pair = torch.empty(max(1, layout.npairs), **f64)
        self.H = torch.empty(max(1, T), **f64)
        self.F = torch.empty(max(1, T), **f64)
        self.P = torch.zeros(max(1, T), **f64)
        self.Pnew = torch.empty(max(1, T), **f64)
        self.Pold = torch.empty(max(1, T), **f64)
        self.work = torch.empty(max(1, T), **f64)
        self.evals = torch.zeros(max(1, R), **f64)
        self.old2 = torch.zeros(max(1, R), **f64)
        self.Eelec = torch.zeros(max(1, nm), **f64)
        self.Eout = torch.zeros(max(1, nm), **f64)
        self.err = torch.ones(max(1, nm), **f64)
        self.dm_err = torch.ones(max(1, nm), **f64)
        self.dm_el = torch.ones(max(1, nm), **f64)
        self.Enuc = torch.zeros(max(1, nm), **f64)
        self.active = torch.ones(max(1, nm), dtype=torch.uint8, device=dev)
        self.nactive = torch.zeros(1, dtype=torch.int32, device=dev)  # molecules active after an iteration
        # scratch of the fused iteration (dP terms, energy partials of the Fock build, slice sums)
        self.step_scratch = torch.empty(max(1, native.scf_scratch_doubles(nm, layout.natoms, layout.npairs, R)),
                                        **f64)
        self.h_nactive = torch.zeros(2, dtype=torch.int32, pin_memory=dev.type == "cuda")
        self.iters = torch.zeros(max(1, nm), dtype=torch.int32, device=dev)
        self.status = torch.zeros(max(1, nm), dtype=torch.int32, device=dev)
        # 1 once the molecule's eigenvector rows in `work` are valid (warm-started Jacobi)
        self.warm = torch.zeros(max(1, nm), dtype=torch.uint8, device=dev)
        # molecules starting cold or whose last solve took >= this many sweeps presweep in FP32 (0 = never)
        self.mixed_threshold = 5
        # SCF iterations take the first-order density once A = V F V^T is nearly diagonal
        self.first_order_density = True
        self.sp2_work = None
        self.sp2_tc_work = None
        self._diis_hist = None
        self._diis = False
        self._diis_err = None
        # molecules above the Jacobi limit take SP2: "fp64" (plain) or "tc" (tensor cores + FP64 McWeeny)
        self.large_density = "fp64"
        self.mcweeny_steps = 1  # FP64-accurate McWeeny steps after the tensor-core SP2 (and one FP32 step)
        # tensor-core SP2 molecules skip the FP64-accurate McWeeny step while their energy still moves
        # by 1 eV or more per iteration (at most 8 iterations) and are never retired on such a density
        self.refine_near_convergence = True
        # molecules above jacobi_max_n basis functions (at most the kernel's 160) take SP2
        if not 0 <= int(jacobi_max_n) <= JACOBI_MAX_N:
            raise ValueError(f"jacobi_max_n must lie in [0, {JACOBI_MAX_N}]")
        self.jacobi_max_n = int(jacobi_max_n)
        self.large_mask = torch.as_tensor((layout.norb > self.jacobi_max_n).astype(np.uint8), device=dev)
        self.n_large = int((layout.norb > self.jacobi_max_n).sum())
        self.n_small = layout.nmol - self.n_large
        self.small_mask = 1 - self.large_mask
        # SP2 runs over a compact view of the large molecules when the batch also holds small ones
        self._large = self._large_view() if self.n_large and self.n_small else None
        self.stream = stream
        self.launches = 0  # kernels of this library launched (for reporting)
        self.profile_density = False  # record CUDA events around every density launch
        self.density_events = []
        # FP64 multiply-adds of the Jacobi density step per molecule (jacobi.cu): the first-order
        # density from the coupling block, (V_S F) n^2 nsel + (coupling) nsel ncomp n + (U^T U,
        # upper) n^2 nsel / 2; after FP32 sweeps also D = X X^T - I (upper) n^3 / 2; the
        # eigenvalue-only final step D + V F V^T (n^3 + n^3 / 2)
        n = layout.norb.astype(np.float64)
        nsel = np.minimum(layout.nocc, layout.norb - layout.nocc).astype(np.float64)
        fma_newton = nsel * n * n + nsel * (n - nsel) * n + 0.5 * n * n * nsel
        self._fma = {k: torch.as_tensor(v, dtype=torch.float64, device=dev)
                     for k, v in (("newton", fma_newton), ("orth", 0.5 * n ** 3), ("final", 2.0 * n ** 3))}
        # algorithmic units of the measurement: an eigensolve with vectors and the density,
        # 9 n^3 + 2 n^2 nocc flops per molecule and density call (symmetric QR convention,
        # independent of the sweeps taken); a Fock build, 8 (W_c + 3 N_blk) bytes per molecule
        # (W_c = 100 XX + 10 XH + 1 HH integrals read, N_blk = 16 XX + 4 XH + 1 HH + 10 heavy + 1 H
        # block elements of P read, of Hcore read and of F written)
        nocc = layout.nocc.astype(np.float64)
        self._eig_unit = torch.as_tensor(9.0 * n ** 3 + 2.0 * n * n * nocc, dtype=torch.float64, device=dev)
        wc = 100.0 * layout.nxx_m + 10.0 * layout.nxh_m + layout.nhh_m
        nblk = 16.0 * layout.nxx_m + 4.0 * layout.nxh_m + layout.nhh_m + 10.0 * layout.nheavy + layout.nhyd
        self._fock_unit = torch.as_tensor(8.0 * (wc + 3.0 * nblk), dtype=torch.float64, device=dev)
        self.profile_fock = False  # record CUDA events around every Fock build
        self.fock_events = []

    # ------------------------------------------------------------------ calls
    def _s(self):
        s = self.stream if self.stream is not None else torch.cuda.current_stream(self.L.device)
        return ctypes_stream(s)

    def hcore(self):
        self.launches += 4
        b = self.L.struct
        native.check(self.lib.seqm_hcore(b, native.ptr(self.w_xx), native.ptr(self.w_xh), native.ptr(self.w_hh),
                                         native.ptr(self.H), native.ptr(self.enuc_pair), self._s()), "seqm_hcore")
        native.check(self.lib.seqm_pair_sum(b, native.ptr(self.enuc_pair), native.ptr(self.Enuc), self._s()),
                     "seqm_pair_sum")

    def fock(self, active=None):
        self.launches += 1
        ev = None
        if self.profile_fock:
            stream = self.stream if self.stream is not None else torch.cuda.current_stream(self.L.device)
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            unit = self._fock_unit if active is None else self._fock_unit * active[: self.L.nmol].double()
            ev[0].record(stream)
        native.check(self.lib.seqm_fock(self.L.struct, native.ptr(self.P), native.ptr(self.H), native.ptr(self.w_xx),
                                        native.ptr(self.w_xh), native.ptr(self.w_hh), native.ptr(self.F),
                                        native.ptr(active), self._s()), "seqm_fock")
        if ev is not None:
            ev[1].record(stream)
            self.fock_events.append((ev[0], ev[1], unit.sum()))

    def density(self, out, sp2=(False,), active=None, evecs=None, max_sweeps=50, density_only=False):
        if self.profile_density:
            stream = self.stream if self.stream is not None else torch.cuda.current_stream(self.L.device)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            act = None if active is None else active[: self.L.nmol].clone()
            e0.record(stream)
            self._density(out, sp2, active, evecs, max_sweeps, density_only)
            e1.record(stream)
            small = self.small_mask[: self.L.nmol].double() if self.n_large else 1.0
            unit = self._eig_unit * small * (1.0 if act is None else act.double())
            self.density_events.append((e0, e1, self._fp64_flops(act, int(density_only), evecs is not None),
                                        unit.sum()))
            return
        self._density(out, sp2, active, evecs, max_sweeps, density_only)

    def _fp64_flops(self, act, density_only, vectors):
        """FP64 flops of one Jacobi density call (device scalar), from the path each molecule
        took: the status (sweeps) written by the call tells an SCF step with FP32 sweeps (or the
        single FP32 rotation, reported as one sweep: the same lift follows) from one without."""
        n = self.L.nmol
        if vectors or density_only == 0:
            fma = self._fma["final"] * 0  # eigenpairs for output: not counted
        elif density_only == 2:
            fma = self._fma["final"]
        else:
            swept = (self.status[:n] > 0).double()
            fma = self._fma["newton"] + swept * self._fma["orth"]
        if act is not None:
            fma = fma * act.double()
        return 2.0 * fma.sum()

    def _large_view(self):
        """Batch struct over the molecules above the Jacobi limit only (the fields SP2 reads:
        nmol, max_norb, mol_norb, mol_nocc, mol_mat_off; the matrix offsets point into the
        full batch's matrices and end with the full size)."""
        L = self.L
        idx = np.nonzero(L.norb > self.jacobi_max_n)[0]
        dev = L.device
        v = dict(idx=torch.as_tensor(idx, dtype=torch.int64, device=dev),
                 norb=torch.as_tensor(L.norb[idx].astype(np.int32), device=dev),
                 nocc=torch.as_tensor(L.nocc[idx].astype(np.int32), device=dev),
                 mat_off=torch.as_tensor(np.append(L.mat_off[idx], L.mat_off[-1]).astype(np.int64), device=dev),
                 active=torch.zeros(idx.size, dtype=torch.uint8, device=dev),
                 status=torch.zeros(idx.size, dtype=torch.int32, device=dev))
        b = native.SeqmBatch.from_buffer_copy(L.struct)
        b.nmol = int(idx.size)
        b.nclass = 0  # no per-molecule size classes in this view
        b.max_norb = int(L.norb[idx].max())
        b.mol_norb = v["norb"].data_ptr()
        b.mol_nocc = v["nocc"].data_ptr()
        b.mol_mat_off = v["mat_off"].data_ptr()
        v["struct"] = b
        return v

    def _sp2_target(self, active, subset):
        """(struct, nmol, max_norb, active, status) of an SP2 call over all molecules or the large view."""
        L = self.L
        if not subset or self._large is None:
            return L.struct, L.nmol, L.max_norb, active, self.status
        v = self._large
        if active is None:
            v["active"].fill_(1)
        else:
            torch.index_select(active[: L.nmol], 0, v["idx"], out=v["active"])
        return v["struct"], v["struct"].nmol, v["struct"].max_norb, v["active"], v["status"]

    def _sp2_fp64(self, out, eps, active, subset=False):
        b, nm, maxn, act, status = self._sp2_target(active, subset)
        T = int(self.L.mat_off[-1])
        nd = 2 * T + (11 + 2 * maxn) * nm + 2  # SEQM_SP2_WORK_DOUBLES
        if self.sp2_work is None or self.sp2_work.numel() < nd:
            self.sp2_work = torch.empty(nd, dtype=torch.float64, device=self.L.device)
        self.launches += 1
        native.check(self.lib.seqm_density_sp2(b, native.ptr(self.F), native.ptr(out), native.ptr(self.sp2_work),
                                               eps, native.ptr(act), native.ptr(status), 1000, self._s()),
                     "seqm_density_sp2")
        if status is not self.status:
            self.status.index_copy_(0, self._large["idx"], status)

    def _sp2_tc(self, out, eps, active, subset=False):
        b, nm, maxn, act, status = self._sp2_target(active, subset)
        T = int(self.L.mat_off[-1])
        nbytes = int(self.lib.seqm_sp2_tc_work_bytes(T, nm, maxn))
        if self.sp2_tc_work is None or self.sp2_tc_work.numel() < nbytes:
            self.sp2_tc_work = torch.empty(nbytes, dtype=torch.uint8, device=self.L.device)
        self.launches += 1
        native.check(self.lib.seqm_density_sp2_tc(b, native.ptr(self.F), native.ptr(out),
                                                  native.ptr(self.sp2_tc_work), eps, native.ptr(act),
                                                  native.ptr(status), 1000, self.mcweeny_steps, self._s()),
                     "seqm_density_sp2_tc")
        if status is not self.status:
            self.status.index_copy_(0, self._large["idx"], status)

    def _density(self, out, sp2=(False,), active=None, evecs=None, max_sweeps=50, density_only=False):
        """Density step.  sp2[0] set: the reference's SP2 option for every molecule (plain FP64
        SP2, or tensor-core SP2 + FP64 McWeeny when sp2[2] == "tc").  Otherwise the Jacobi
        eigensolver for norb <= 160 and, for larger molecules, the SP2 form chosen by
        ``large_density`` ("fp64" by default, "tc")."""
        L = self.L
        if sp2[0]:
            if len(sp2) > 2 and sp2[2] == "tc":
                self._sp2_tc(out, float(sp2[1]), active)
            else:
                self._sp2_fp64(out, float(sp2[1]), active)
            return
        if self.n_large:
            if self.large_density == "tc":
                self._sp2_tc(out, 1.0e-7, active, subset=True)
            else:
                self._sp2_fp64(out, 1.0e-7, active, subset=True)
            if not self.n_small:
                return
        act_s = active if not self.n_large else (self.small_mask if active is None else active & self.small_mask)
        self.launches += 1
        native.check(self.lib.seqm_density_jacobi(L.struct, native.ptr(self.F), native.ptr(out),
                                                  native.ptr(self.evals), native.ptr(evecs), native.ptr(self.work),
                                                  native.ptr(L.dev["row_off"]), native.ptr(act_s),
                                                  native.ptr(self.status), max_sweeps, native.ptr(self.warm),
                                                  self.mixed_threshold,
                                                  int(density_only) if self.first_order_density else 0,
                                                  self._s()),
                     "seqm_density_jacobi")  # sets warm[m] for the molecules it solved

    def energy_error(self, eps, first=False):
        self.launches += 1
        b = self.L.struct
        if first:
            native.check(self.lib.seqm_energy_error(b, native.ptr(self.P), None, native.ptr(self.H),
                                                    native.ptr(self.F), native.ptr(self.Eelec), native.ptr(self.Eout),
                                                    native.ptr(self.err), native.ptr(self.dm_err),
                                                    native.ptr(self.dm_el), None, float(eps), None, self._s()),
                         "seqm_energy_error")
            return
        native.check(self.lib.seqm_energy_error(b, native.ptr(self.P), native.ptr(self.Pold), native.ptr(self.H),
                                                native.ptr(self.F), native.ptr(self.Eelec), native.ptr(self.Eout),
                                                native.ptr(self.err), native.ptr(self.dm_err), native.ptr(self.dm_el),
                                                native.ptr(self.active), float(eps), native.ptr(self._diis_err),
                                                self._s()), "seqm_energy_error")

    # --------------------------------------------------------------- drivers
    def start(self, eps, converger=(1,), sp2=(False,), P0=None, keep_warm=False):
        """Initial density, F(P0), E(P0) and the per-molecule SCF state; no host synchronisation.
        P0: packed density guess (None: the diagonal guess); keep_warm: keep the eigenvector
        rows of the previous solve as the Jacobi warm start (same molecules, nearby geometry)."""
        L = self.L
        b = L.struct
        if int(converger[0]) not in (0, 1, 2):
            raise NotImplementedError("scf_converger must be [0, alpha] (linear), [1] (adaptive) or [2] (DIIS)")
        if P0 is None:
            self.P.zero_()
            self.launches += 1
            native.check(self.lib.seqm_initial_density(b, native.ptr(self.P), self._s()), "seqm_initial_density")
        elif P0 is not self.P:
            self.P.copy_(P0)
        self.fock()
        self.energy_error(eps, first=True)
        self.Eelec.copy_(self.Eout)
        self.err.fill_(1.0)
        self.dm_err.fill_(1.0)
        self.dm_el.fill_(1.0)
        self.active.fill_(1)
        gated = self._refine_gated(sp2)
        if gated is not None:
            self.active[: L.nmol] += gated  # 2: the FP64-accurate McWeeny step may wait (see seqm_scf_step)
        self.iters.zero_()
        if not keep_warm:
            self.warm.zero_()
        self.old2.zero_()
        self._eps = float(eps)
        self._linear = int(converger[0]) == 0
        self._alpha = float(converger[1]) if self._linear else 0.0
        self._sp2 = tuple(sp2)
        self._diis = int(converger[0]) == 2
        self._diis_err = None
        self._state = self._scf_state()
        if self._diis:
            dev = L.device
            if self._diis_hist is None:
                self._diis_hist = torch.empty(max(1, 21 * int(L.mat_off[-1])), dtype=torch.float64, device=dev)
                self._diis_state = torch.empty(max(1, native.DIIS_STATE * L.nmol), dtype=torch.float64, device=dev)
                self._diis_err_buf = torch.empty(max(1, L.nmol), dtype=torch.float64, device=dev)
            self._diis_err = self._diis_err_buf
            self._state.diis_err = self._diis_err.data_ptr()
            self._state.mixing = -1
            self.launches += 1
            native.check(self.lib.seqm_diis_init(b, native.ptr(self._diis_state), native.ptr(self._diis_err),
                                                 self._s()), "seqm_diis_init")

    def _refine_gated(self, sp2):
        """uint8 mask of the molecules whose tensor-core SP2 density may skip the FP64-accurate
        McWeeny step early in the SCF (None: no molecule)."""
        if not self.refine_near_convergence:
            return None
        if sp2[0]:
            return self.large_mask.new_ones(self.L.nmol) if len(sp2) > 2 and sp2[2] == "tc" else None
        if self.n_large and self.large_density == "tc":
            return self.large_mask[: self.L.nmol]
        return None

    def _scf_state(self):
        """seqm_scf_state of this solver's buffers and the current converger."""
        st = native.ScfState()
        for name in ("P", "Pnew", "Pold", "old2", "H", "F", "w_xx", "w_xh", "w_hh", "Eelec", "Eout", "err", "dm_err",
                     "dm_el", "iters", "active", "nactive"):
            setattr(st, name, getattr(self, name).data_ptr())
        st.mol_row_off = self.L.dev["row_off"].data_ptr()
        st.scratch = self.step_scratch.data_ptr()
        st.diis_err = None
        st.mixing = 0 if self._linear else 1
        st.alpha, st.occupation, st.eps = self._alpha, 2.0, self._eps
        return st

    def step(self):
        """One SCF iteration of every still-active molecule (density, mixing, F(P), E(P), get_error);
        molecules that pass the test are retired on the device.  No host synchronisation (except
        inside the SP2 density step)."""
        L = self.L
        if self._diis:
            # store F and its commutator, F <- DIIS extrapolation (scf_forward2, scf_loop.py:974-1033)
            self.launches += 4
            native.check(self.lib.seqm_diis_extrapolate(L.struct, native.ptr(self.F), native.ptr(self.P),
                                                        native.ptr(self._diis_hist), native.ptr(self._diis_state),
                                                        native.ptr(self._diis_err), native.ptr(self.active),
                                                        native.ptr(self.iters), self._s()), "seqm_diis_extrapolate")
        self.density(self.Pnew, self._sp2, active=self.active, density_only=True)
        if self._diis:
            self.launches += 1
            native.check(self.lib.seqm_diis_mix(L.struct, native.ptr(self.P), native.ptr(self.Pnew),
                                                native.ptr(self.Pold), native.ptr(self._diis_state),
                                                native.ptr(self.active), self._s()), "seqm_diis_mix")
        if self.profile_fock:
            # the same kernels as seqm_scf_step, called one by one so that the Fock build is timed alone
            if not self._diis:
                self.launches += 1
                native.check(self.lib.seqm_mix(L.struct, native.ptr(self.P), native.ptr(self.Pnew),
                                               native.ptr(self.Pold), native.ptr(self.old2),
                                               native.ptr(L.dev["row_off"]), native.ptr(self.iters), int(self._linear),
                                               self._alpha, 2.0, native.ptr(self.active), self._s()), "seqm_mix")
            self.fock(self.active)
            self.energy_error(self._eps)
            self.nactive.copy_(self.active[: L.nmol].sum())
            return
        # mixing, Fock build, energy and convergence test, count of the molecules still active (fused:
        # adaptive diagonal step(s), two mixer streams (+ the grid one), Fock build, energy finish;
        # DIIS: Fock build, energy pass(es))
        large = 1 if self.L.max_norb > 160 else 0
        if self._diis:
            self.launches += 2 + large
        else:
            self.launches += 4 + large + (0 if self._linear else 1 + large)
        native.check(self.lib.seqm_scf_step(L.struct, ctypes.byref(self._state), self._s()), "seqm_scf_step")

    def max_loops(self, max_iter=MAX_ITER):
        """Iterations the reference's loop allows: MAX_ITER + 1 for linear mixing (scf_loop.py:250)
        and DIIS (:974), MAX_ITER adaptive (:505)."""
        return max_iter + 1 if (self._linear or self._diis) else max_iter

    def iterate(self, max_iter=MAX_ITER):
        """SCF iterations until no molecule is active or the cap.  The host keeps one iteration
        queued ahead of the one whose active count it reads (copied to pinned memory behind each
        iteration), so the GPU does not wait for the host between iterations; the iteration queued
        after the last molecule retired finds nothing active and every kernel of it returns at
        once.  Returns the per-molecule not-converged mask (host numpy)."""
        stream = self.stream if self.stream is not None else torch.cuda.current_stream(self.L.device)
        queued = []
        for it in range(self.max_loops(max_iter)):
            self.step()
            slot = it & 1
            self.h_nactive[slot].copy_(self.nactive[0], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
            queued.append((ev, slot))
            if len(queued) == 2:
                ev0, s0 = queued.pop(0)
                ev0.synchronize()
                if int(self.h_nactive[s0]) == 0:
                    break
        for ev, _ in queued:
            ev.synchronize()
        return self.active[: self.L.nmol].bool().cpu().numpy()

    def scf(self, eps, converger=(1,), sp2=(False,), P0=None, max_iter=MAX_ITER):
        """Run the SCF; returns the per-molecule not-converged mask (host numpy)."""
        self.start(eps, converger, sp2, P0)
        return self.iterate(max_iter)

    def resume(self, xyz, eps, converger=(1,), sp2=(False,), max_iter=MAX_ITER):
        """Next geometry of the same molecules (an MD step, cf. MolecularDynamics.py:815-825,
        which passes P0 = molecule.dm): new coordinates (natoms x 3, Angstrom), integrals and
        Hcore recomputed, the SCF started from the current density with the current
        eigenvectors as the Jacobi warm start; everything stays on the device."""
        self.L.set_coordinates(xyz)
        self.hcore()
        self.start(eps, converger, sp2, P0=self.P, keep_warm=True)
        return self.iterate(max_iter)

    def final(self, want_vectors=True):
        """Fock matrix of the converged density, orbital energies / vectors, energies."""
        self.fock()
        evecs = torch.empty_like(self.work) if want_vectors else None
        # orbital energies without vectors may come from second-order perturbation of the
        # nearly diagonal rotated Fock matrix (density_only 2)
        self.density(self.Pnew, (False,), active=None if not self.n_large else self.small_mask, evecs=evecs,
                     density_only=2 if evecs is None else 0)
        self.energy_error(0.0, first=True)
        self.evecs = evecs
        return self.Eout[: self.L.nmol].clone(), self.Enuc[: self.L.nmol].clone()


class BatchUHF(BatchSCF):
    """Unrestricted SCF (UHF) of a batch of molecules with given spin multiplicities: the
    reference's scf_forward0/1 with unrestricted=True (scf_loop.py:194-635).  Each spin has its
    own density (starting at half the restricted guess, scf_loop.py:2083-2085), Fock matrix
    (seqm_fock_u), Jacobi density step with occupation 1 (the eigensolver's 2 C C^T halved,
    scf_loop.py:259-260 / 515-516), warm-start vectors and mixing state (occupation 1); the
    energy and the convergence test cover both spins (seqm_energy_error_u).  The inherited
    buffers (P, F, Pnew, Pold, work, evals, ...) hold the alpha spin.  SP2 has no open-shell
    form in the reference (SP2.py raises), so molecules above the Jacobi limit are rejected."""

    def __init__(self, layout, stream=None):
        if not getattr(layout, "uhf", False):
            raise ValueError("BatchUHF needs a layout built with spin multiplicities (mult)")
        super().__init__(layout, stream)
        if self.n_large:
            raise NotImplementedError(f"unrestricted SCF is limited to {JACOBI_MAX_N} basis functions per molecule "
                                      "(the reference has no open-shell SP2)")
        L, dev = layout, layout.device
        f64 = dict(dtype=torch.float64, device=dev)
        T, R, nm = int(L.mat_off[-1]), int(L.row_off[-1]), L.nmol
        self.Pb = torch.zeros(max(1, T), **f64)
        self.Fb = torch.empty(max(1, T), **f64)
        self.Pnewb = torch.empty(max(1, T), **f64)
        self.Poldb = torch.empty(max(1, T), **f64)
        self.workb = torch.empty(max(1, T), **f64)
        self.evals_b = torch.zeros(max(1, R), **f64)
        self.old2b = torch.zeros(max(1, R), **f64)
        self.warm_b = torch.zeros(max(1, nm), dtype=torch.uint8, device=dev)
        self.status_b = torch.zeros(max(1, nm), dtype=torch.int32, device=dev)
        self.iters_b = torch.zeros(max(1, nm), dtype=torch.int32, device=dev)
        self._spin_struct = []
        for key in ("nocc_a", "nocc_b"):  # batch views whose occupations are one spin's
            v = native.SeqmBatch.from_buffer_copy(L.struct)
            v.mol_nocc = L.dev[key].data_ptr()
            self._spin_struct.append(v)

    def fock(self, active=None):
        L = self.L
        self.launches += 1
        native.check(self.lib.seqm_fock_u(L.struct, native.ptr(self.P), native.ptr(self.Pb), native.ptr(self.H),
                                          native.ptr(self.w_xx), native.ptr(self.w_xh), native.ptr(self.w_hh),
                                          native.ptr(self.F), native.ptr(self.Fb), native.ptr(active), self._s()),
                     "seqm_fock_u")

    def energy_error(self, eps, first=False):
        L = self.L
        self.launches += 1
        olds = (None, None) if first else (native.ptr(self.Pold), native.ptr(self.Poldb))
        native.check(self.lib.seqm_energy_error_u(L.struct, native.ptr(self.P), native.ptr(self.Pb), olds[0], olds[1],
                                                  native.ptr(self.H), native.ptr(self.F), native.ptr(self.Fb),
                                                  native.ptr(self.Eelec), native.ptr(self.Eout), native.ptr(self.err),
                                                  native.ptr(self.dm_err), native.ptr(self.dm_el),
                                                  None if first else native.ptr(self.active), float(eps), self._s()),
                     "seqm_energy_error_u")

    def density(self, out=None, sp2=(False,), active=None, evecs=None, max_sweeps=50, density_only=False,
                evecs_b=None):
        """Both spins' density steps into Pnew / Pnewb (occupation 1)."""
        L = self.L
        if sp2[0]:
            raise NotImplementedError("SP2 has no open-shell form (SP2.py)")
        spins = ((self._spin_struct[0], self.F, self.Pnew, self.evals, evecs, self.work, self.status, self.warm),
                 (self._spin_struct[1], self.Fb, self.Pnewb, self.evals_b, evecs_b, self.workb, self.status_b,
                  self.warm_b))
        for struct, F, Pn, ev, vec, work, status, warm in spins:
            self.launches += 1
            native.check(self.lib.seqm_density_jacobi(struct, native.ptr(F), native.ptr(Pn), native.ptr(ev),
                                                      native.ptr(vec), native.ptr(work), native.ptr(L.dev["row_off"]),
                                                      native.ptr(active), native.ptr(status), max_sweeps,
                                                      native.ptr(warm), self.mixed_threshold,
                                                      int(density_only) if self.first_order_density else 0,
                                                      self._s()), "seqm_density_jacobi")
            Pn.mul_(0.5)

    def start(self, eps, converger=(1,), sp2=(False,), P0=None, keep_warm=False):
        """P0: (Pa, Pb) packed spin densities, or None for half the restricted guess each."""
        L = self.L
        if int(converger[0]) not in (0, 1):
            raise NotImplementedError("unrestricted SCF supports scf_converger [0, alpha] and [1] "
                                      "(the reference has no open-shell DIIS)")
        if sp2[0]:
            raise NotImplementedError("SP2 has no open-shell form (SP2.py)")
        if P0 is None:
            self.P.zero_()
            self.launches += 1
            native.check(self.lib.seqm_initial_density(L.struct, native.ptr(self.P), self._s()), "seqm_initial_density")
            self.P.mul_(0.5)
            self.Pb.copy_(self.P)
        else:
            self.P.copy_(P0[0])
            self.Pb.copy_(P0[1])
        self.fock()
        self.energy_error(eps, first=True)
        self.Eelec.copy_(self.Eout)
        self.err.fill_(1.0)
        self.dm_err.fill_(1.0)
        self.dm_el.fill_(1.0)
        self.active.fill_(1)
        self.iters.zero_()
        self.iters_b.zero_()
        if not keep_warm:
            self.warm.zero_()
            self.warm_b.zero_()
        self.old2.zero_()
        self.old2b.zero_()
        self._eps = float(eps)
        self._linear = int(converger[0]) == 0
        self._alpha = float(converger[1]) if self._linear else 0.0
        self._sp2 = (False,)
        self._diis = False
        self._diis_err = None

    def step(self):
        L = self.L
        self.density(active=self.active, density_only=True)
        for P, Pn, Po, o2, it in ((self.P, self.Pnew, self.Pold, self.old2, self.iters),
                                  (self.Pb, self.Pnewb, self.Poldb, self.old2b, self.iters_b)):
            self.launches += 1
            native.check(self.lib.seqm_mix(L.struct, native.ptr(P), native.ptr(Pn), native.ptr(Po), native.ptr(o2),
                                           native.ptr(L.dev["row_off"]), native.ptr(it), int(self._linear),
                                           self._alpha, 1.0, native.ptr(self.active), self._s()), "seqm_mix")
        self.fock(self.active)
        self.energy_error(self._eps)
        self.nactive.copy_(self.active[: L.nmol].sum())

    def resume(self, xyz, eps, converger=(1,), sp2=(False,), max_iter=MAX_ITER):
        self.L.set_coordinates(xyz)
        self.hcore()
        self.start(eps, converger, sp2, P0=(self.P.clone(), self.Pb.clone()), keep_warm=True)
        return self.iterate(max_iter)

    def final(self, want_vectors=True):
        """Fock matrices of the converged spin densities, orbital energies (and vectors) per spin,
        energies."""
        self.fock()
        evecs = torch.empty_like(self.work) if want_vectors else None
        evecs_b = torch.empty_like(self.workb) if want_vectors else None
        self.density(active=None, evecs=evecs, evecs_b=evecs_b, density_only=2 if evecs is None else 0)
        self.energy_error(0.0, first=True)
        self.evecs, self.evecs_b = evecs, evecs_b
        return self.Eout[: self.L.nmol].clone(), self.Enuc[: self.L.nmol].clone()


def ctypes_stream(s):
    return ctypes.c_void_p(s.cuda_stream)


def run_energy(species, coords, method, eps=1e-6, converger=(1,), sp2=(False,), charges=None, device="cuda",
               want_vectors=False, mult=None, pair_cutoff=None):
    """One batched single point: returns a dict of device tensors and host arrays.  mult: spin
    multiplicities for an unrestricted solve; pair_cutoff: the parser's pair_outer_cutoff (A)."""
    t0 = time.perf_counter()
    L = Layout.from_padded(species, coords, method, charges, mult=mult, pair_cutoff=pair_cutoff).to_device(device)
    s = BatchUHF(L) if mult is not None else BatchSCF(L)
    s.hcore()
    nc = s.scf(eps, converger, sp2)
    Eelec, Enuc = s.final(want_vectors)
    return dict(layout=L, solver=s, Eelec=Eelec, Enuc=Enuc, Etot=Eelec + Enuc, notconverged=nc,
                iters=s.iters[: L.nmol].cpu().numpy(), wall=time.perf_counter() - t0)
