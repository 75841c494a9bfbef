"""Continuous-batching SCF service on one GPU.

Requests (closed-shell molecules, some also asking for forces) arrive over time.
The loop admits whatever has arrived as a *cohort* -- a ragged, unpadded batch
with its own CUDA stream and device-resident SCF state (Hcore, F, P, mixing
history, eigenvector warm starts) -- as soon as a cohort slot and the device
memory budget allow, and advances every live cohort one SCF iteration at a time
on worker threads, so cohorts admitted at different times overlap on the
device.  Molecules retire individually: each iteration's convergence flags come
back to the host, and a molecule's result is final from the iteration in which
it passed the test (every kernel skips retired molecules, so its density no
longer changes).  Forces of a retiring molecule come from the adjoint kernel at
that density.  Molecules above the Jacobi limit are admitted in cohorts of their
own, so the SP2 grids cover only their tiles.

Two forms share the request format and the result record:

* ``ServingLoop(form="serving")``: tensor-core SP2 with FP64-accurate McWeeny refinement
  above the Jacobi limit, FP32-presweep + FP64 Jacobi below, continuous admission;
  every cohort captures its SCF iteration once as a CUDA graph after its first iteration and
  replays it (an SP2 cohort's step loop is a conditional node ended on the device).
* ``ServingLoop(form="plain")``: FP64 kernels only, one batch at a time: the
  batch is everything that has arrived when the previous batch finished, solved
  to completion (its force requests, converged tighter, as a second solve)
  before the next one is taken.

The SCF semantics per molecule are the reference's (seqm/seqm_functions/
scf_loop.py:350-635 with get_error :106-147); only the batching changes.
"""

import collections
import threading
import time
from concurrent.futures import FIRST_COMPLETED, ThreadPoolExecutor, wait
from dataclasses import dataclass

import numpy as np
import torch

from . import native, workloads
from .layout import Layout
from .scf import JACOBI_MAX_N, MAX_ITER, BatchSCF


# torch.cuda.graph synchronises the device when a capture starts, which is not allowed while
# another thread's stream is capturing: cohorts capture one at a time
_CAPTURE_LOCK = threading.Lock()


@dataclass
class Request:
    rid: int
    species: np.ndarray  # (natoms,) atomic numbers, non-increasing
    coords: np.ndarray  # (natoms, 3) Angstrom
    forces: bool = False
    arrival: float = 0.0  # seconds after the start of the stream


@dataclass
class Result:
    rid: int
    Etot: float  # eV
    Eelec: float
    Enuc: float
    iterations: int
    converged: bool
    forces: np.ndarray  # (natoms, 3) eV/Angstrom, or None
    arrival: float
    done: float  # seconds after the start of the stream

    @property
    def latency(self):
        return self.done - self.arrival


def make_requests(molecules, arrivals=None):
    """[(species, coords, forces)] (+ arrival times) -> [Request]."""
    arrivals = np.zeros(len(molecules)) if arrivals is None else arrivals
    return [Request(i, np.asarray(s), np.asarray(c, dtype=np.float64), bool(f), float(t))
            for i, ((s, c, f), t) in enumerate(zip(molecules, arrivals))]


def norb_of(species):
    s = np.asarray(species)
    return int(4 * (s > 1).sum() + (s == 1).sum())


def footprint(req, form="serving"):
    """Device bytes a request holds while it is in a cohort (matrices, SP2 work, integrals)."""
    s = np.asarray(req.species)
    n, nh = norb_of(s), int((s > 1).sum())
    ny = s.size - nh
    nxx, nxh, nhh = nh * (nh - 1) // 2, nh * ny, ny * (ny - 1) // 2
    dense = 6 * 8 * n * n
    if n > JACOBI_MAX_N:
        dense += (24 if form == "serving" else 16) * n * n
    pairs = 8 * (100 * nxx + 10 * nxh + nhh) + 8 * 8 * (nxx + nxh + nhh)
    return dense + pairs + 4096


def _configure(solver, form):
    if form == "serving":
        solver.large_density = "tc"
        solver.mixed_threshold = 5
    else:
        solver.large_density = "fp64"
        solver.mixed_threshold = 0


class _Cohort:
    """One admitted batch: layout, solver and stream; its methods run on one worker thread at a time."""

    def __init__(self, reqs, method, eps, form, device, large, stream, graphs=False):
        self.reqs = reqs
        self.graphs = graphs
        self.graph = None
        self.method = method
        self.eps = eps
        self.form = form
        self.device = device
        self.large = large
        self.bytes = sum(footprint(r, form) for r in reqs)
        self.stream = stream
        self.iteration = 0
        self.future = None
        self.finished = False

    def admit(self):
        with torch.cuda.stream(self.stream):
            species, coords = workloads.pad_batch([(r.species, r.coords) for r in self.reqs])
            self.L = Layout.from_padded(species, coords, self.method).to_device(self.device)
            s = BatchSCF(self.L, stream=self.stream)
            _configure(s, self.form)
            s.hcore()
            s.start(self.eps, (1,))
            self.s = s
            nm = self.L.nmol
            pin = dict(pin_memory=True)
            self.h_active = torch.empty(nm, dtype=torch.uint8, **pin)
            self.h_E = torch.empty(3, nm, dtype=torch.float64, **pin)
            self.h_iters = torch.empty(nm, dtype=torch.int32, **pin)
            self.retired = np.zeros(nm, dtype=bool)
            self.want_forces = np.array([r.forces for r in self.reqs])
            self._grad_buf = None
        return []

    def iterate(self, t0):
        """One SCF iteration; returns the Results of the molecules that retired in it."""
        s, L = self.s, self.L
        nm = L.nmol
        with torch.cuda.stream(self.stream):
            if self.graph is not None:
                self.graph.replay()
                s.launches += self.graph_launches
            else:
                s.step()
                if self.graphs:
                    self._capture()
            self.iteration += 1
            self.h_active.copy_(s.active[:nm], non_blocking=True)
            self.h_E[0].copy_(s.Eout[:nm], non_blocking=True)
            self.h_E[1].copy_(s.Enuc[:nm], non_blocking=True)
            self.h_iters.copy_(s.iters[:nm], non_blocking=True)
            self.stream.synchronize()
        act = self.h_active.numpy().astype(bool)
        last = self.iteration >= s.max_loops(MAX_ITER)
        new = np.nonzero(~self.retired & (~act | last))[0]
        if new.size == 0:
            return []
        forces = self._forces() if self.want_forces[new].any() else None
        t = time.perf_counter() - t0
        E = self.h_E.numpy()
        its = self.h_iters.numpy()
        out = []
        for m in new:
            r = self.reqs[m]
            f = None
            if r.forces:
                a0, a1 = int(L.atom_off[m]), int(L.atom_off[m + 1])
                f = -forces[a0:a1].copy()
            out.append(Result(r.rid, float(E[0, m] + E[1, m]), float(E[0, m]), float(E[1, m]), int(its[m]),
                              bool(not act[m]), f, r.arrival, t))
        self.retired[new] = True
        self.finished = bool(self.retired.all())
        return out

    def launches(self):
        return self.s.launches

    def _capture(self):
        """Record one SCF iteration (density step, mixing, Fock build, energy and test) as a CUDA
        graph, replayed for every later iteration: buffers and retirement flags stay on the device,
        and an SP2 density step's loop is a conditional node the device ends.  Capture follows the
        first, eager iteration, which has set up everything done once (scratch buffers, kernel
        attributes); capturing records the launches without running them."""
        s = self.s
        self.graph = torch.cuda.CUDAGraph()
        before = s.launches
        with _CAPTURE_LOCK, torch.cuda.graph(self.graph, stream=self.stream, capture_error_mode="thread_local"):
            s.step()
        self.graph_launches = s.launches - before
        s.launches = before  # counted at every replay

    def _forces(self):
        """dE_tot/dR (natoms, 3) of the whole cohort at the current densities (host array)."""
        L, s = self.L, self.s
        with torch.cuda.stream(self.stream):
            if self._grad_buf is None:
                f64 = dict(dtype=torch.float64, device=self.device)
                self._grad_buf = (torch.ones(L.nmol, **f64), torch.empty(3 * max(1, L.natoms), **f64),
                                  torch.empty(4 * max(1, L.natoms), **f64), torch.empty(7 * max(1, L.npairs), **f64))
            g, dR, dpar, work = self._grad_buf
            s.launches += 2
            native.check(s.lib.seqm_energy_grad(L.struct, native.ptr(s.P), None, native.ptr(g), native.ptr(g),
                                                native.ptr(dR), native.ptr(dpar), native.ptr(work), s._s()),
                         "seqm_energy_grad")
            host = dR[: 3 * L.natoms].cpu()  # synchronises this stream
        return host.numpy().reshape(-1, 3)


class ServingLoop:
    """Request loop over one GPU (see the module docstring).

    graphs: every cohort replays its SCF iteration as a CUDA graph after the first (serving form);
    eps: SCF threshold (get_error) of energy requests; eps_forces: of force requests (forces
    are linear in the density error where the energy is quadratic, so they converge tighter
    and are admitted in cohorts of their own); budget_bytes: device memory the live cohorts
    may hold;
    max_live: concurrent cohorts per size class (Jacobi-sized, SP2-sized);
    max_cohort: most molecules admitted into one cohort; cohort_factory: the cohort class
    (arguments of ``_Cohort``), replaceable to exercise the scheduling on the host."""

    def __init__(self, method="PM3", eps=1.0e-5, form="serving", budget_bytes=100e9, max_live=(4, 4),
                 max_cohort=(4096, 256), device="cuda", cohort_factory=None, eps_forces=1.0e-6, graphs=True):
        if form not in ("serving", "plain"):
            raise ValueError("form must be 'serving' or 'plain'")
        self.method = method
        self.eps = float(eps)
        self.eps_forces = min(float(eps_forces), self.eps)
        self.form = form
        self.budget = float(budget_bytes)
        self.max_live = tuple(max_live)
        self.max_cohort = tuple(max_cohort)
        self.device = torch.device(device)
        self.cohort_factory = cohort_factory or _Cohort
        self.graphs = bool(graphs) and form == "serving"
        self.launches = 0
        self.cohorts = 0
        self.max_concurrent = 0  # most cohorts live at once (overlap on the device)
        self.max_bytes = 0.0  # most budgeted bytes held at once

    # ----------------------------------------------------------------- serving
    def run(self, requests):
        """Serve `requests` (their arrival times are relative to the call); returns [Result] by rid."""
        if self.form == "plain":
            return self._run_plain(requests)
        for r in requests:
            if footprint(r, self.form) > self.budget:
                raise ValueError(f"request {r.rid} needs more device memory than the budget")
        reqs = sorted(requests, key=lambda r: r.arrival)
        n = len(reqs)
        # FIFO queues by (size class: Jacobi-sized 0 / SP2-sized 1, forces requested)
        queues = {(k, f): collections.deque() for k in (0, 1) for f in (False, True)}
        live = ([], [])
        results = {}
        used = 0.0
        nxt = 0
        pool = ThreadPoolExecutor(max_workers=sum(self.max_live))
        # one stream per cohort slot: the caching allocator reuses a finished cohort's memory
        # for the next cohort on the same stream
        mk = (lambda: torch.cuda.Stream(device=self.device)) if self.device.type == "cuda" else (lambda: None)
        free_streams = tuple([mk() for _ in range(k)] for k in self.max_live)
        t0 = time.perf_counter()
        try:
            while len(results) < n:
                now = time.perf_counter() - t0
                while nxt < n and reqs[nxt].arrival <= now:
                    r = reqs[nxt]
                    queues[(int(norb_of(r.species) > JACOBI_MAX_N), r.forces)].append(r)
                    nxt += 1
                # admission: new cohorts within the size class's slots and the budget
                for k, f in ((1, True), (1, False), (0, True), (0, False)):
                    q = queues[(k, f)]
                    if not q or len(live[k]) >= self.max_live[k]:
                        continue
                    take, nbytes = [], 0.0
                    while q and len(take) < self.max_cohort[k] and used + nbytes + footprint(q[0], self.form) <= self.budget:
                        nbytes += footprint(q[0], self.form)
                        take.append(q.popleft())
                    if take:
                        c = self.cohort_factory(take, self.method, self.eps_forces if f else self.eps, self.form,
                                                self.device, bool(k), free_streams[k].pop(), self.graphs)
                        c.future = pool.submit(c.admit)
                        live[k].append(c)
                        used += c.bytes
                        self.cohorts += 1
                        self.max_concurrent = max(self.max_concurrent, len(live[0]) + len(live[1]))
                        self.max_bytes = max(self.max_bytes, used)
                # advance: every cohort whose previous task finished gets its next iteration
                pending = []
                for k in (0, 1):
                    for c in list(live[k]):
                        if c.future is not None and c.future.done():
                            for res in c.future.result():
                                results[res.rid] = res
                            c.future = None
                            if c.finished:
                                live[k].remove(c)
                                free_streams[k].append(c.stream)
                                used -= c.bytes
                                self.launches += c.launches()
                                continue
                        if c.future is None:
                            c.future = pool.submit(c.iterate, t0)
                        pending.append(c.future)
                if len(results) >= n:
                    break
                timeout = None
                if nxt < n:
                    timeout = max(0.0, reqs[nxt].arrival - (time.perf_counter() - t0))
                if pending:
                    wait(pending, timeout=timeout, return_when=FIRST_COMPLETED)
                elif timeout:
                    time.sleep(timeout)
        finally:
            pool.shutdown(wait=True)
        return [results[r.rid] for r in sorted(requests, key=lambda r: r.rid)]

    # ------------------------------------------------------------------- plain
    def _run_plain(self, requests):
        reqs = sorted(requests, key=lambda r: r.arrival)
        n = len(reqs)
        results = {}
        nxt = 0
        t0 = time.perf_counter()
        while nxt < n:
            now = time.perf_counter() - t0
            if reqs[nxt].arrival > now:
                time.sleep(reqs[nxt].arrival - now)
                continue
            batch, nbytes = [], 0.0
            while nxt < n and reqs[nxt].arrival <= now and len(batch) < self.max_cohort[0]:
                fb = footprint(reqs[nxt], self.form)
                if batch and nbytes + fb > self.budget:
                    break
                batch.append(reqs[nxt])
                nbytes += fb
                nxt += 1
            for group, eps in (([r for r in batch if not r.forces], self.eps), ([r for r in batch if r.forces],
                                                                                  self.eps_forces)):
                if group:
                    for res in self._solve_batch(group, t0, eps):
                        results[res.rid] = res
            self.cohorts += 1
        return [results[r.rid] for r in sorted(requests, key=lambda r: r.rid)]

    def _solve_batch(self, batch, t0, eps):
        species, coords = workloads.pad_batch([(r.species, r.coords) for r in batch])
        L = Layout.from_padded(species, coords, self.method).to_device(self.device)
        s = BatchSCF(L)
        _configure(s, self.form)
        s.hcore()
        nc = s.scf(eps, (1,))
        E = torch.stack([s.Eout[: L.nmol], s.Enuc[: L.nmol]]).cpu().numpy()
        its = s.iters[: L.nmol].cpu().numpy()
        forces = None
        if any(r.forces for r in batch):
            f64 = dict(dtype=torch.float64, device=self.device)
            g = torch.ones(L.nmol, **f64)
            dR = torch.empty(3 * max(1, L.natoms), **f64)
            dpar = torch.empty(4 * max(1, L.natoms), **f64)
            work = torch.empty(7 * max(1, L.npairs), **f64)
            s.launches += 2
            native.check(s.lib.seqm_energy_grad(L.struct, native.ptr(s.P), None, native.ptr(g), native.ptr(g),
                                                native.ptr(dR), native.ptr(dpar), native.ptr(work), s._s()),
                         "seqm_energy_grad")
            forces = dR[: 3 * L.natoms].cpu().numpy().reshape(-1, 3)
        t = time.perf_counter() - t0
        self.launches += s.launches
        out = []
        for m, r in enumerate(batch):
            f = None
            if r.forces:
                f = -forces[int(L.atom_off[m]): int(L.atom_off[m + 1])].copy()
            out.append(Result(r.rid, float(E[0, m] + E[1, m]), float(E[0, m]), float(E[1, m]), int(its[m]),
                              bool(not nc[m]), f, r.arrival, t))
        return out


def summarize(results):
    """solves/s over the makespan (first arrival to last completion) and latency percentiles (ms)."""
    lat = np.array([r.latency for r in results])
    t_first = min(r.arrival for r in results)
    t_last = max(r.done for r in results)
    span = max(t_last - t_first, 1e-9)
    return dict(solves_per_s=len(results) / span, makespan_s=span, p50_ms=float(np.percentile(lat, 50) * 1e3),
                p99_ms=float(np.percentile(lat, 99) * 1e3), mean_ms=float(lat.mean() * 1e3),
                notconverged=int(sum(not r.converged for r in results)))
