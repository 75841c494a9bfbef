#!/usr/bin/env python
"""Benchmark: batched semi-empirical single-point SCF throughput (SCF solves/s).

Workload (one "step"): the AM1 batched single point of 4096 molecules drawn
50/50 from n-alkanes C_nH_{2n+2} (n uniform 1..16, N(0, 0.03 A) jitter) and
water clusters (H2O)_k (k uniform 2..24, jittered 2.9 A lattice, random
orientations), seeded; scf_eps 1e-8, adaptive mixing [1]; integrals + Hcore +
SCF to convergence + final energies.  Synthetic inputs, generated here.

Arms:
  default            this library on N GPUs (one process per GPU, replicas: every
                     rank solves its own 4096-molecule batch, no collective on the
                     data path; weak scaling).  Rank 0 adds to the line: the same
                     batch with the strictly FP64 density step (fp64_only), with
                     SP2 above 128 AOs as the workload's specification writes it
                     (c2_as_written), end to end through api.single_point (e2e), the
                     CPU oracle on a bounded sample (cpu_baseline), and the other
                     workloads below as sub-objects c1, c3, c4, c5 (--configs).
  --impl reference   the CPU oracle (NumPy restatement of the reference path) on
                     the host cores of rank 0 over a bounded sample per step.

Other workloads (sub-objects of the default line, or one line each with --config):
  c1   16 perturbed n-butanes, PM3, plain FP64, linear mixing (alpha 0.1), eps 1e-8
  c3   (H2O)1000 PM3: plain FP64 SP2 vs tensor-core SP2 + McWeeny (dE, max|dP|, ||X^2 - X||);
       --c3-side 6 runs (H2O)216, --c3-modes tc only the tensor-core form
  c4   MNDO forces and parameter gradients: 256 octanes + 256 (H2O)16, central
       differences (h = 1e-4 A) on seeded coordinates
  c5   the serving stream (--requests, default 4000) at several Poisson arrival rates
       (--rates), the plain FP64 form one batch at a time at the lowest and highest rate

Prints one JSON line.
"""

import argparse
import gc
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

WORKLOAD = {"workload": "AM1 batched single-point SCF, 4096 molecules 50/50 n-alkanes C1-C16 / (H2O)2-24, seed 0",
            "method": "AM1", "nmol": 4096, "scf_eps": 1e-8, "scf_converger": [1], "seed": 0,
            "density_step": "Jacobi for all molecules (norb <= 144): FP32 sweeps (one FP32 rotation for a warm "
                            "start whose occupied-virtual ratio is <= 1e-3), FP64 orthonormalisation, "
                            "coupling block and first-order density; FP64-accurate"}
METRIC = "SCF solves/s"
# DRAM bytes of one density call (all size-class launches) of the default workload, from ncu
# captures of the norb > 114 class of the 2048-molecule batch (92 MB with FP32 sweeps, 74 MB for
# a warm first-order step, for 37 % of that batch's matrix elements), scaled to the 4096-molecule
# batch and weighted by the calls of a solve that take FP32 sweeps or the single FP32 rotation (73 %;
# both end in the same lift of the rotations to FP64, which writes what the warm step does not)
JACOBI_TRAFFIC_BYTES = 4.7e8


def _oracle_chunk(args):
    """Run the CPU oracle on a list of molecules (worker of the spawned pool)."""
    method, mols, eps, conv = args
    sys.path.insert(0, HERE)
    from oracle import seqm_oracle as O
    from pyseqm_gb300 import workloads

    E = []
    for s, c in mols:
        sp, cc = workloads.pad_batch([(s, c)])
        E.append(float(O.single_point(method, sp, cc, eps, tuple(conv))["Etot"][0]))
    return E


def oracle_pool(procs):
    """Spawned worker pool, one single-threaded BLAS per worker (children inherit the env)."""
    for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[k] = "1"
    return mp.get_context("spawn").Pool(procs)


def cpu_oracle_rate(pool, procs, mols, method, eps, conv):
    chunks = [mols[i::procs] for i in range(procs)]
    t0 = time.perf_counter()
    pool.map(_oracle_chunk, [(method, ch, eps, conv) for ch in chunks if ch])
    dt = time.perf_counter() - t0
    return len(mols) / dt, dt


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, bus_id):
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", bus_id], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(nmol, seed):
    from pyseqm_gb300 import workloads

    return workloads.mixed_batch(nmol, seed=seed)


def run_reference(args):
    """--impl reference: the CPU oracle over a bounded sample per step, all host cores of rank 0."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    mols = make_workload(WORKLOAD["nmol"], WORKLOAD["seed"])[: args.cpu_sample]
    with oracle_pool(procs) as pool:
        for _ in range(args.warmup):
            cpu_oracle_rate(pool, procs, mols, WORKLOAD["method"], WORKLOAD["scf_eps"], WORKLOAD["scf_converger"])
        times = []
        for _ in range(args.steps):
            _, dt = cpu_oracle_rate(pool, procs, mols, WORKLOAD["method"], WORKLOAD["scf_eps"],
                                    WORKLOAD["scf_converger"])
            times.append(dt)
    value = len(mols) / min(times)  # best step after the warm-up (min of the timed steps)
    sample = (f"first {len(mols)} molecules of the 4096-molecule workload per step (NumPy oracle, {procs} "
              f"processes); value from the best of {len(times)} steps after {args.warmup} warm-up steps, mean "
              f"{len(mols) * len(times) / sum(times):.1f} solves/s")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(WORKLOAD, sample=len(mols)),
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def fp64_peak_tflops(torch, dev):
    """Measured FP64 dense throughput (cuBLAS DGEMM 4096^3, best of 5)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    best = 1e9
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2.0 * n**3 / best / 1e12


def gpu_bus_id(torch, dev, local):
    """nvidia-smi -i selector of the GPU we run on (PCI bus id when torch exposes it)."""
    p = torch.cuda.get_device_properties(dev)
    if all(hasattr(p, k) for k in ("pci_domain_id", "pci_bus_id", "pci_device_id")):
        return f"{p.pci_domain_id:08X}:{p.pci_bus_id:02X}:{p.pci_device_id:02X}.0"
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    ids = [v for v in vis.split(",") if v.strip()]
    return ids[local].strip() if local < len(ids) else str(local)


def serving_sample(torch, dev, n, rate, seed=0, forms=("serving", "plain"), mols=None):
    """Bounded sample of the serving stream: the forms on the same requests and arrivals."""
    from pyseqm_gb300 import serving, workloads

    mols = mols if mols is not None else workloads.request_molecules(n, seed=seed)
    arr = workloads.poisson_arrivals(n, rate, seed=seed)
    for form in forms:  # warm-up: library, kernel attributes, allocator
        serving.ServingLoop("PM3", eps=1e-5, form=form, device=dev).run(serving.make_requests(mols[:8]))
    torch.cuda.synchronize()
    out = {}
    for form in forms:
        loop = serving.ServingLoop("PM3", eps=1e-5, form=form, device=dev)
        res = loop.run(serving.make_requests(mols, arr))
        sm = serving.summarize(res)
        sm.update(cohorts=loop.cohorts, max_live_cohorts=loop.max_concurrent, gpu_launches=loop.launches)
        out[form] = (sm, res)
    line = {"workload": f"{n} PM3 requests, 3-600 atoms log-uniform (alkanes / water clusters), 10% with forces, "
                        f"Poisson {rate:.0f} req/s, seed {seed}",
            "scf_eps": 1e-5, "scf_eps_forces": 1e-6, "budget_bytes": 100e9}
    if "serving" in out:
        line["serving"] = out["serving"][0]
    if "plain" in out:
        line["plain_fp64_one_batch_at_a_time"] = out["plain"][0]
    if "serving" in out and "plain" in out:
        dE = max(abs(a.Etot - b.Etot) for a, b in zip(out["serving"][1], out["plain"][1]))
        dF = [float(np.abs(a.forces - b.forces).max()) for a, b in zip(out["serving"][1], out["plain"][1])
              if a.forces is not None]
        line.update(solves_per_s_ratio=out["serving"][0]["solves_per_s"] / out["plain"][0]["solves_per_s"],
                    max_abs_dE_eV=dE, max_abs_dF_eV_per_A=max(dF) if dF else None)
    return line


def _events_sum(events):
    """(total seconds, total algorithmic units) of recorded (start, end, ..., units) events."""
    dur = sum(ev[0].elapsed_time(ev[1]) / 1e3 for ev in events)
    return dur, sum(float(ev[-1]) for ev in events)


def run_ours(args):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pool = None
    procs = os.cpu_count() or 1
    if rank == 0 and not args.no_cpu_baseline:
        pool = oracle_pool(procs)  # before the first GPU call
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    from pyseqm_gb300 import api, native, workloads
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF

    native.load()
    mols = make_workload(args.nmol, WORKLOAD["seed"] + rank)
    species, coords = workloads.pad_batch(mols)
    L = Layout.from_padded(species, coords, WORKLOAD["method"]).to_device(dev)
    s = BatchSCF(L)

    def step(solver=s):
        solver.hcore()
        solver.scf(WORKLOAD["scf_eps"], tuple(WORKLOAD["scf_converger"]))
        return solver.final(want_vectors=False)

    for w in range(args.warmup):
        s.profile_density = s.profile_fock = w == args.warmup - 1  # the last warm-up loads the bookkeeping too
        step()
    torch.cuda.synchronize()
    peak_fp64 = fp64_peak_tflops(torch, dev)
    bus = gpu_bus_id(torch, dev, local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(bus)
    # the timed steps run the production iteration (seqm_scf_step); events around the density step
    # do not change its path, the Fock build is timed alone in one profiled step after the region
    s.profile_density, s.profile_fock = True, False
    s.density_events, s.fock_events = [], []
    launches0 = s.launches
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    step_ms = []
    gc.collect()
    gc.disable()  # no collector pause inside the timed region
    e0.record(stream)
    for _ in range(args.steps):
        a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        Eel, Enu = step()
        c.record(stream)
        step_ms.append((a, c))
    e1.record(stream)
    torch.cuda.synchronize()
    gc.enable()
    if world > 1:
        dist.barrier()
    clocks = sampler.stop()
    s.profile_density = False
    elapsed = e0.elapsed_time(e1) / 1e3
    # one more step with the Fock build called on its own between events (the split entry points)
    s.profile_fock = True
    step()
    torch.cuda.synchronize()
    s.profile_fock = False
    launches = s.launches - launches0
    step_ms = [a.elapsed_time(c) for a, c in step_ms]
    if world > 1:
        t = torch.tensor([elapsed], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    total_solves = args.nmol * args.steps * world
    value = total_solves / elapsed
    # dominant kernel: the batched Jacobi density step.  Algorithmic work per launch = sum over the
    # molecules it solves of 9 n^3 + 2 n^2 nocc flops (an eigensolve with vectors + the density);
    # the FP64 products the kernel's path actually executes are reported beside it
    t_jac, unit_jac = _events_sum(s.density_events)
    exec_jac = sum(float(ev[2]) for ev in s.density_events)
    achieved = unit_jac / t_jac / 1e12 if t_jac else None
    roofline = {"kernel": "k_jacobi (batched Jacobi density step: FP32 sweeps, FP64 coupling block and density)",
                "bound": "fp64", "achieved": achieved, "peak": peak_fp64, "unit": "TFLOP/s",
                "frac": (achieved / peak_fp64) if achieved else None, "traffic": JACOBI_TRAFFIC_BYTES,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the norb > 114 class launch "
                                  "of the 2048-molecule batch (92 MB with FP32 sweeps, 74 MB warm, for 37 % of its "
                                  "matrix elements), scaled to this batch and weighted by the calls with sweeps "
                                  "(73 %)",
                "peak_source": "measured in this run: cuBLAS DGEMM 4096^3 (the measured-peaks file has no FP64 "
                               "figure); the unit counts FP64-accurate eigensolve work, which the kernel runs as FP32 "
                               "sweeps, a first-order density step and double-float products on the FP32 pipe, so "
                               "the fraction can exceed 1",
                "algorithmic_unit": "9 n^3 + 2 n^2 nocc flops per molecule and density call (eigensolve with "
                                    "vectors, symmetric QR convention, + density), summed over the molecules "
                                    "each call solves",
                "algorithmic_tflop": unit_jac / 1e12,
                "executed_fp64": {"achieved": exec_jac / t_jac / 1e12 if t_jac else None,
                                  "frac": (exec_jac / t_jac / 1e12 / peak_fp64) if t_jac else None,
                                  "what": "FP64-accurate products the path executes (double-float on the FP32 "
                                          "pipe), as FP64 flops: SCF step 2 (n^2 s + s (n - s) n + n^2 s / 2), "
                                          "s = min(nocc, n - nocc), + n^3 after FP32 sweeps; final eigenvalue step "
                                          "4 n^3 (FP32 sweep work not counted)"},
                "launches": len(s.density_events), "avg_launch_ms": 1e3 * t_jac / max(1, len(s.density_events)),
                "share_of_step_time": t_jac / elapsed}
    t_fock, unit_fock = _events_sum(s.fock_events)
    hbm = measured_hbm_gbs()
    fock_gbs = unit_fock / t_fock / 1e9 if t_fock else None
    roofline_fock = {"kernel": "k_fock (Fock build, a9)", "bound": "fp64",
                     "achieved_hbm": fock_gbs, "hbm_peak": hbm[0], "hbm_unit": "GB/s",
                     "hbm_frac": fock_gbs / hbm[0] if fock_gbs and hbm[0] else None, "hbm_peak_source": hbm[1],
                     "algorithmic_unit": "8 (W_c + 3 N_blk) bytes per molecule and build: W_c = 100 XX + 10 XH + "
                                         "1 HH integrals, N_blk = 16 XX + 4 XH + 1 HH + 10 heavy + 1 H block "
                                         "elements (P read, Hcore read, F written)",
                     "algorithmic_gb": unit_fock / 1e9, "launches": len(s.fock_events),
                     "avg_launch_ms": 1e3 * t_fock / max(1, len(s.fock_events)),
                     "share_of_step_time": t_fock / (elapsed / args.steps),
                     "measured": "one step after the timed region with the Fock build called on its own"}
    iters = s.iters[: args.nmol].cpu().numpy()
    E_default = (Eel + Enu).clone()
    # the same batch with a strictly FP64 density step (no FP32 sweeps: mixed_threshold 0)
    fp64_only = None
    if rank == 0 and not args.skip_fp64_only:
        mixed_default = s.mixed_threshold
        s.mixed_threshold = 0
        step()
        torch.cuda.synchronize()
        ms64 = []
        for _ in range(args.steps):
            a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            Eel64, Enu64 = step()
            c.record(stream)
            ms64.append((a, c))
        torch.cuda.synchronize()
        ms64 = [a.elapsed_time(c) for a, c in ms64]
        fp64_only = {"value": args.nmol * len(ms64) / (sum(ms64) / 1e3), "unit": "solves/s",
                     "ms_per_step": statistics.mean(ms64), "steps": len(ms64), "step_ms": [round(x, 2) for x in ms64],
                     "max_abs_dE_vs_default_eV": float((Eel64 + Enu64 - E_default).abs().max()),
                     "what": "density step with FP64 arithmetic only (FP64 rotation, first-order density and "
                             "sweeps; no FP32 stage)"}
        s.mixed_threshold = mixed_default
    # the workload as its specification writes it: Jacobi up to 128 AOs, plain FP64 SP2 above
    as_written = None
    if rank == 0 and args.as_written_steps > 0:
        s128 = BatchSCF(L, jacobi_max_n=128)
        step(s128)
        torch.cuda.synchronize()
        ms128 = []
        for _ in range(args.as_written_steps):
            a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            E1, E2 = step(s128)
            c.record(stream)
            ms128.append((a, c))
        torch.cuda.synchronize()
        ms128 = [a.elapsed_time(c) for a, c in ms128]
        as_written = {"value": args.nmol * len(ms128) / (sum(ms128) / 1e3), "unit": "solves/s",
                      "ms_per_step": statistics.mean(ms128), "steps": len(ms128),
                      "molecules_on_sp2": int(s128.n_large),
                      "max_abs_dE_vs_default_eV": float((E1 + E2 - E_default).abs().max()),
                      "what": "Jacobi density step up to 128 AOs, plain FP64 SP2 above (the headline runs the "
                              "Jacobi step up to 160 AOs)"}
        del s128
    # end to end through the public API with host buffers
    e2e = None
    if rank == 0 and args.e2e_steps > 0:
        torch.cuda.synchronize()
        api.single_point(species, coords, WORKLOAD["method"], WORKLOAD["scf_eps"], WORKLOAD["scf_converger"],
                         device=dev)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            r = api.single_point(species, coords, WORKLOAD["method"], WORKLOAD["scf_eps"], WORKLOAD["scf_converger"],
                                 device=dev)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / args.e2e_steps
        h2d = L.h2d_bytes
        d2h = 2 * 8 * args.nmol + 4 * args.nmol + args.nmol  # energies, iteration counts, flags
        e2e = {"value": args.nmol / dt, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": 1e3 * dt, "includes": "host layout build (NumPy; the pair list and the per-atom parameters are built on the GPU), H2D, hcore+SCF+energies, D2H"}
        assert not r["notconverged"].any()
    configs = {}
    if rank == 0:
        for cid in [c for c in args.configs.split(",") if c and c != "none"]:
            t0 = time.perf_counter()
            configs[cid] = CONFIGS[cid](torch, dev, args)
            configs[cid]["wall_s"] = round(time.perf_counter() - t0, 1)
            torch.cuda.empty_cache()
    cpu = None
    if pool is not None:
        sample = mols[: args.cpu_sample]
        cpu = cpu_baseline(pool, procs, sample)
        pool.close()
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(WORKLOAD, nmol=args.nmol, parallelism=f"replicas x{world}",
                               l2="working set (>1 GB of F/P/Hcore/integrals) exceeds L2; no flush needed",
                               scf_iterations_max=int(iters.max()), scf_iterations_mean=float(iters.mean()),
                               deviation="Jacobi density step up to 160 AOs where the specification says SP2 above "
                                         "128; the as-written form is timed in c2_as_written"),
                "p50_ms": statistics.median(step_ms), "p99_ms": float(np.percentile(step_ms, 99)),
                "step_ms": [round(x, 2) for x in step_ms],
                "roofline": roofline, "roofline_fock": roofline_fock, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": launches, "clocks": clocks, "fp64_only": fp64_only, "c2_as_written": as_written}
        line.update(configs)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def cpu_baseline(pool, procs, sample, runs=3):
    """The CPU oracle on a bounded sample of the workload: one warm-up pass, then the best of
    `runs` passes (the same estimator as the reference arm)."""
    cpu_oracle_rate(pool, procs, sample, WORKLOAD["method"], WORKLOAD["scf_eps"], WORKLOAD["scf_converger"])
    times = [cpu_oracle_rate(pool, procs, sample, WORKLOAD["method"], WORKLOAD["scf_eps"],
                             WORKLOAD["scf_converger"])[1] for _ in range(runs)]
    return {"value": len(sample) / min(times), "unit": "solves/s", "cores": procs, "kind": "port",
            "sample": f"first {len(sample)} molecules of the workload, NumPy oracle, {procs} processes; one warm-up "
                      f"pass, best of {runs} ({', '.join(f'{t:.2f}' for t in times)} s)"}


def measured_hbm_gbs():
    """(HBM copy bandwidth GB/s, source) from the measured-peaks file, else the machine's fallback."""
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        for k in ("hbm_gbs", "hbm_GBs", "hbm"):
            if k in d:
                v = d[k]
                v = v.get("value", v.get("gbs")) if isinstance(v, dict) else v
                return float(v), "MEASURED_PEAKS.json (measured copy)"
    except (OSError, ValueError, TypeError, AttributeError):
        pass
    return 6800.0, "fallback 6.8 TB/s (no measured-peaks file on this box)"


# ------------------------------------------------------------------ other workloads
def _timed(torch, fn, steps, warmup):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        out = fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3 / steps, out


def config_c1(torch, dev, args):
    """16 perturbed n-butanes, PM3, plain FP64 (Jacobi eigensolver), linear mixing alpha 0.1, eps 1e-8."""
    from pyseqm_gb300 import api, workloads
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF

    species, coords = workloads.pad_batch(workloads.butane_batch(16, seed=0))
    L = Layout.from_padded(species, coords, "PM3").to_device(dev)
    s = BatchSCF(L)
    s.mixed_threshold = 0

    def step():
        s.hcore()
        nc = s.scf(1e-8, (0, 0.1))
        s.final(want_vectors=False)
        return nc

    dt, nc = _timed(torch, step, args.steps, args.warmup)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        api.single_point(species, coords, "PM3", 1e-8, (0, 0.1), device=dev)
    e2e = (time.perf_counter() - t0) / args.steps
    it = s.iters[: L.nmol].cpu().numpy()
    return {"metric": "SCF solves/s", "value": 16 / dt, "unit": "solves/s", "ms_per_step": 1e3 * dt,
            "config": {"workload": "16 n-butanes C4H10 (sigma 0.03 A), PM3, plain FP64, converger [0, 0.1], eps 1e-8",
                       "iterations": [int(it.min()), int(it.max())], "notconverged": int(nc.sum())},
            "e2e": {"value": 16 / e2e, "unit": "solves/s", "ms_per_step": 1e3 * e2e}}


def config_c3(torch, dev, args):
    """(H2O)1000, PM3: plain FP64 SP2 vs tensor-core SP2 + McWeeny refinement."""
    from pyseqm_gb300 import workloads
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF

    side = args.c3_side
    species, coords = workloads.pad_batch([workloads.big_water(seed=0, n_side=side)])
    L = Layout.from_padded(species, coords, "PM3").to_device(dev)
    out = {}
    for mode in args.c3_modes.split(","):
        s = BatchSCF(L)
        s.large_density = mode
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.hcore()
        nc = s.scf(1e-5, (1,))
        s.final(want_vectors=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        X = 0.5 * L.block(s.P, 0)
        idem = float((X @ X - X).abs().max())
        it = int(s.iters[0])
        out[mode] = dict(Etot=float(s.Eout[0] + s.Enuc[0]), seconds=dt, iterations=it, ms_per_iteration=1e3 * dt / it,
                         idempotency_max_abs=idem, converged=not bool(nc[0]), P=s.P.clone())
        del s, X
        torch.cuda.empty_cache()
    both = "tc" in out and "fp64" in out
    dP = float((out["tc"]["P"] - out["fp64"]["P"]).abs().max()) if both else None
    for v in out.values():
        v.pop("P")
    first = next(iter(out.values()))
    k = side**3
    return {"metric": "seconds per single point", "value": first["seconds"], "unit": "s", "higher_is_better": False,
            "config": {"workload": f"(H2O){k} PM3, {3 * k} atoms / {6 * k} AOs, {side}^3 lattice 3.1 A, jitter 0.25 A, "
                                   f"seed 0", "scf_eps": 1e-5},
            "tensor_core_sp2": out.get("tc"), "plain_fp64_sp2": out.get("fp64"),
            "dE_tc_minus_fp64_eV": out["tc"]["Etot"] - out["fp64"]["Etot"] if both else None,
            "density_max_abs_diff": dP, "speedup": out["fp64"]["seconds"] / out["tc"]["seconds"] if both else None}


def config_c4(torch, dev, args):
    """MNDO forces + parameter gradients (adjoint kernels) of 256 octanes + 256 (H2O)16; central
    differences (h = 1e-4 A) on 32 seeded coordinates per molecule, all molecules at once."""
    from pyseqm_gb300 import native, workloads
    from pyseqm_gb300.layout import Layout
    from pyseqm_gb300.scf import BatchSCF

    rng = np.random.default_rng(0)
    mols = [workloads.alkane(8, rng, 0.05) for _ in range(256)] + [workloads.water_cluster(16, rng) for _ in range(256)]
    species, coords = workloads.pad_batch(mols)
    eps = 1e-8
    L = Layout.from_padded(species, coords, "MNDO").to_device(dev)
    s = BatchSCF(L)
    nm, na = L.nmol, L.natoms
    f64 = dict(dtype=torch.float64, device=dev)
    g = torch.ones(nm, **f64)
    dR, dpar = torch.empty(3 * na, **f64), torch.empty(4 * na, **f64)
    work = torch.empty(7 * max(1, L.npairs), **f64)

    def solve_and_grad():
        s.hcore()
        s.scf(eps, (1,))
        s.final(want_vectors=False)
        native.check(s.lib.seqm_energy_grad(L.struct, native.ptr(s.P), None, native.ptr(g), native.ptr(g), native.ptr(dR),
                                            native.ptr(dpar), native.ptr(work), s._s()), "seqm_energy_grad")
        return dR

    dt_all, _ = _timed(torch, solve_and_grad, args.steps, args.warmup)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    native.check(s.lib.seqm_energy_grad(L.struct, native.ptr(s.P), None, native.ptr(g), native.ptr(g), native.ptr(dR),
                                        native.ptr(dpar), native.ptr(work), s._s()), "seqm_energy_grad")
    e1.record()
    torch.cuda.synchronize()
    dt_grad = e0.elapsed_time(e1) / 1e3
    force = -dR.view(na, 3).cpu().numpy()
    xyz0 = L.xyz.copy()
    h = 1e-4
    worst = 0.0
    for _ in range(32):
        pick = np.array([L.atom_off[m] + rng.integers(0, L.natoms_m[m]) for m in range(nm)])
        dim = rng.integers(0, 3, size=nm)
        E = []
        for sign in (1.0, -1.0):
            xyz = xyz0.copy()
            xyz[pick, dim] += sign * h
            L.set_coordinates(xyz)
            s.hcore()
            s.scf(eps, (1,))
            s.final(want_vectors=False)
            E.append((s.Eout[:nm] + s.Enuc[:nm]).cpu().numpy())
        fd = -(E[0] - E[1]) / (2 * h)
        worst = max(worst, float(np.abs(fd - force[pick, dim]).max()))
    L.set_coordinates(xyz0)
    return {"metric": "solves+gradients/s", "value": nm / dt_all, "unit": "molecules/s", "ms_per_step": 1e3 * dt_all,
            "config": {"workload": "MNDO, 256 n-octanes (sigma 0.05 A) + 256 (H2O)16, seed 0", "scf_eps": eps,
                       "gradients": "all coordinates; U_ss, U_pp, beta_s, beta_p per atom"},
            "gradient_kernel_ms": 1e3 * dt_grad,
            "fd_check": {"h_A": h, "coordinates_per_molecule": 32, "max_abs_force_error_eV_per_A": worst}}


def config_c5(torch, dev, args):
    """The serving stream at each rate; the plain form (about a minute per rate at 4000 requests) at
    the lowest and the highest rate, or at every rate with --c5-plain-all."""
    from pyseqm_gb300 import workloads

    mols = workloads.request_molecules(args.requests, seed=0)
    rates = [float(x) for x in args.rates.split(",")]
    lines = []
    for k, rate in enumerate(rates):
        plain = args.c5_plain_all or k in (0, len(rates) - 1)
        lines.append(serving_sample(torch, dev, args.requests, rate, forms=("serving", "plain") if plain else
                                    ("serving",), mols=mols))
    worst = {}
    for ln in lines:
        if "plain_fp64_one_batch_at_a_time" in ln:
            sv, pl = ln["serving"], ln["plain_fp64_one_batch_at_a_time"]
            worst = {"min_solves_per_s_ratio": min(worst.get("min_solves_per_s_ratio", 1e30), ln["solves_per_s_ratio"]),
                     "p99_lower_at_every_compared_rate": worst.get("p99_lower_at_every_compared_rate", True)
                     and sv["p99_ms"] < pl["p99_ms"],
                     "max_abs_dE_eV": max(worst.get("max_abs_dE_eV", 0.0), ln["max_abs_dE_eV"]),
                     "max_abs_dF_eV_per_A": max(worst.get("max_abs_dF_eV_per_A", 0.0), ln["max_abs_dF_eV_per_A"] or 0.0)}
    return {"metric": "SCF solves/s + p50/p99 latency vs plain FP64 one batch at a time", "requests": args.requests,
            "rates_req_per_s": rates, "summary": worst, "rates": lines}


CONFIGS = {}  # filled below: id -> function(torch, dev, args) returning the config's JSON object


def run_config(args):
    import torch

    if int(os.environ.get("RANK", "0")) != 0:
        return
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    line = CONFIGS[args.config](torch, dev, args)
    line.update({"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "dtype": "f64", "data": "synthetic",
                 "config_id": args.config})
    print(json.dumps(line), flush=True)


CONFIGS.update(c1=config_c1, c3=config_c3, c4=config_c4, c5=config_c5)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nmol", type=int, default=WORKLOAD["nmol"])
    ap.add_argument("--cpu-sample", type=int, default=256)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-fp64-only", action="store_true",
                    help="default workload: do not also time it with the strictly FP64 density step")
    ap.add_argument("--as-written-steps", type=int, default=3,
                    help="default workload: steps timed with SP2 above 128 AOs (0: skip)")
    ap.add_argument("--configs", default="c1,c3,c4,c5",
                    help="default run: the other workloads reported as sub-objects of the line ('none': skip)")
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5"])
    ap.add_argument("--requests", type=int, default=4000)
    ap.add_argument("--rates", default="1000,5000,20000,50000")
    ap.add_argument("--c5-plain-all", action="store_true", help="--config c5: the plain form at every rate")
    ap.add_argument("--c3-side", type=int, default=10, help="water cluster lattice side of --config c3")
    ap.add_argument("--c3-modes", default="tc,fp64", help="SP2 forms run by --config c3")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        run_reference(args)
    elif args.config != "c2":
        run_config(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
