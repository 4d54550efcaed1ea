"""AC-CAS correlation energies per second on one GB300.

Workload (batched uneven instances): 64 synthetic systems, nbasis ~ U[50,250],
inactive ~ U[5,25], CAS(2,2)..CAS(6,6), ERI factor rank 6*nbasis, 8
Gauss-Legendre lambda points each. A step is one pass of the AC-CAS path over
the whole batch (64 energies). Inputs (MO coefficients, ERI factors) are
resident in HBM for `value`; `e2e` copies them from pinned host memory inside
the timed region. The per-system working set (ERI factor, FFOO/FOFO, A+-B) is
larger than L2 for all but the smallest systems.

The measured step is the mixed + batched + learned form: FP64-accurate
sliced-BF16 tensor-core transform, ERPA products and integrand, Cholesky ERPA on
an affine A+-B with the eigensolve in FP32 refined to FP64 accuracy, concurrent
worker streams, and the integrand surrogate (ERPA at the two end nodes of the
8-point rule, an ensemble estimate, and the six interior nodes where the
estimate exceeds 1 microhartree, on integrals and A+-B kept on the device by a
batch session between the two passes). After the timed steps the plain FP64
GPU path (ERPASYMM1 with FP64 products, A+-B reassembled per point) runs on the
whole batch with the same worker streams, timed with CUDA events, and every
energy of the last timed step is checked against it (1 microhartree).

--impl reference times the reference's algorithm on the host cores (the
reference itself cannot be compiled here: no Fortran compiler, no MKL): the
multi-threaded CPU port oracle/cpu_port.py (A+-B reassembled at every point,
ERPASYMM1 with two LAPACK dsyevd, the integrand as one GEMM) on a stratified
sample of the same batch: ordered by ERPA dimension, the 64 systems form 8
strata of 8, each step runs the median system of the next stratum, and the
batch rate is 8 / (sum over strata of the mean time of its representative), the
stratified estimate of 64 energies over the batch's CPU time. Strata not reached
in the timed steps are left out of the sum (the line says which).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "AC-CAS energies/s at <=1 uEh vs FP64 oracle: mixed+batched+learned vs plain GPU"
WORKLOAD = "batched-uneven-64: nbasis U[50,250], inactive U[5,25], CAS(2,2)-(6,6), rank 6n, 8 lambda"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nsys", type=int, default=64)
    ap.add_argument("--ngrid", type=int, default=8)
    ap.add_argument("--nstreams", type=int, default=8,
                    help="worker streams of the batch; 0 chooses them with api.autotune_streams")
    ap.add_argument("--precision", default="fp64tc5")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--eig-emulation", type=int, default=0)
    ap.add_argument("--erpa", default="refined", choices=["cholesky", "refined"],
                    help="ERPA form of the measured step: FP64 dsyevd of L^T A- L, or an FP32 "
                         "eigensolve refined to FP64 accuracy")
    ap.add_argument("--eig-refine", type=int, default=2)
    ap.add_argument("--surrogate", type=int, default=1)
    ap.add_argument("--threshold", type=float, default=1e-6)
    ap.add_argument("--gen", default="device", choices=["device", "cpu"],
                    help="input generator: FP64 torch on the GPU, or numpy on the host")
    ap.add_argument("--no-subset", action="store_true",
                    help="skip the plain FP64 GPU path on the whole batch (comparison and check)")
    ap.add_argument("--plain-energies", default=None,
                    help="file of the plain FP64 energies of this batch: read when it exists "
                         "(the check runs without the plain timing), written otherwise")
    ap.add_argument("--tile", type=int, default=0,
                    help="column tile of the sliced GEMMs (0: chosen per product; 64/96/128)")
    ap.add_argument("--kernel-only", type=int, default=0,
                    help="time only the tensor-core GEMM at this size (for profiling)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="batched", choices=["batched", "precision", "large"],
                    help="batched: the 64-system batch (the headline); precision: the "
                         "transform-scale precision study (n=400, 40 inactive, CAS(8,8), rank "
                         "2400); large: the large single system (n=500, 30 inactive, CAS(8,8), "
                         "rank 3000)")
    ap.add_argument("--plain", type=int, default=0,
                    help="large workload: also time the plain FP64 GPU path (ERPASYMM1)")
    ap.add_argument("--erpa-once", action="store_true",
                    help="time one ERPA solve (the --erpa form) of the largest batch system, "
                         "inside a profiler range (for profiling)")
    ap.add_argument("--acecorr-once", action="store_true",
                    help="one ACECORR point (A+-B assembly at lambda = 0 and 1, ERPA, integrand) "
                         "of the largest batch system inside a profiler range (for profiling the "
                         "assembly and integrand kernels)")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def rank_shapes(nsys: int, seed: int, rank: int):
    """One rank's batch: the shared shape distribution with the rank's own seeds.
    Systems are independent and no system is on two ranks, so the ranks exchange
    no data (weak scaling); only the timing reduction is collective."""
    from gammcor_gb300 import synth
    return synth.batched_shapes(count=nsys, seed=seed + 7919 * rank)


def max_over_ranks(values, world: int, device):
    """Element-wise maximum of per-rank timings over all ranks."""
    if world == 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def whole_job_rate(world: int, nsys: int, ms: float) -> float:
    """Energies per second of the whole job: every rank's systems over the slowest rank."""
    return world * nsys / (ms / 1000.0)


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the sliced
# GEMM at the bench's roofline shape, from a one-launch ncu capture of
# `bench.py --kernel-only N --precision P` (summarised under profiles/).
GEMM_TRAFFIC: dict = {("fp64tc5", 6290): 4511958528 + 319232512}


def read_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_batch(nsys, seed, device, run, rank_offset=0, log=print, gen="device"):
    """Generate the batch. Systems whose A+B is not positive definite at a
    quadrature point are reported by the GPU path itself (Cholesky status) and
    resampled; the final check run is the first warm-up step on the final batch."""
    from gammcor_gb300 import api, synth
    shapes = rank_shapes(nsys, seed, rank_offset)
    if gen == "device":
        make = lambda n, a, b, r, sd: synth.make_system_device(n, a, b, r, sd, device=device)  # noqa
    else:
        make = lambda n, a, b, r, sd: synth.make_system(n, a, b, r, sd)  # noqa
    t0 = time.time()
    systems = [make(sh["n"], sh["nin"], sh["nact"], sh["rank"], sh["seed"]) for sh in shapes]
    log(f"generated {nsys} systems in {time.time() - t0:.1f}s")
    for attempt in range(1, 8):
        batch = api.BatchInputs(systems, device=device)
        status = run(batch)[3]
        bad = [int(i) for i in (status != 0).nonzero()[0]]
        if not bad:
            return batch
        log(f"resampling {len(bad)} systems (A+B not positive definite): {bad}")
        for i in bad:
            sh = shapes[i]
            systems[i] = make(sh["n"], sh["nin"], sh["nact"], sh["rank"],
                              sh["seed"] + 100000 * attempt)
    raise RuntimeError("could not find positive-definite systems")


# The CPU baseline's stratified sample: the batch ordered by ERPA dimension is cut
# into strata of 8 systems and each stratum is represented by its median system
# (positions 4, 12, ..., 60). The batch's CPU time is estimated without a model as
# 8 x the sum over strata of the representative's time.
CPU_STRATUM = 8
CPU_SAMPLE = tuple(range(CPU_STRATUM // 2, 64, CPU_STRATUM))


def pair_count(sh) -> int:
    """NDimX of a shape (accas.f:58-99: all pairs minus inactive-inactive and virtual-virtual)."""
    n, nin, na = sh["n"], sh["nin"], sh["nact"]
    nv = n - nin - na
    return n * (n - 1) // 2 - nin * (nin - 1) // 2 - nv * (nv - 1) // 2


def workload_config(args) -> dict:
    """The workload both arms report (the method is reported separately)."""
    return {"workload": WORKLOAD, "nsys": args.nsys, "lambda_points": args.ngrid,
            "seed": args.seed, "l2": "inputs larger than L2 (per-system factor + FFOO/FOFO)"}


def cpu_port_energies(systems, ngrid, log=print):
    """Time the CPU port of the reference algorithm on the given systems; returns
    (seconds per system, energies, ERPA dimensions)."""
    from oracle import ac_cas_ref as R
    from oracle import cpu_port
    cpu_port.load()
    times, energies, dims = [], [], []
    for s in systems:
        t0 = time.perf_counter()
        _, ecorr, _ = cpu_port.energy_of_system(s, ngrid=ngrid)
        times.append(time.perf_counter() - t0)
        energies.append(ecorr)
        dims.append(len(R.pair_space(s.occ, s.nele)))
        log(f"cpu port: N={dims[-1]} {times[-1]:.2f}s")
    return times, energies, dims


def batch_estimate(times, dims, all_dims):
    """Whole-batch energies/s from a t = c N^3 least-squares fit of the sample."""
    import numpy as np
    t, n3 = np.asarray(times), np.asarray(dims, dtype=float) ** 3
    c = float((t * n3).sum() / (n3 * n3).sum())
    total = c * float((np.asarray(all_dims, dtype=float) ** 3).sum())
    return len(all_dims) / total, c


def cpu_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def run_reference(args):
    """The reference's algorithm on the host cores, on a stratified sample of the batch."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    from gammcor_gb300 import synth
    from oracle import ac_cas_ref as R
    from oracle import cpu_port
    log = lambda *a: print(*a, file=sys.stderr, flush=True)  # noqa: E731
    shapes = synth.batched_shapes(count=args.nsys, seed=args.seed)
    dims = [pair_count(sh) for sh in shapes]
    order = np.argsort(dims, kind="stable")
    picks = [int(order[k]) for k in CPU_SAMPLE if k < len(order)]
    x, w = R.gauleg(0.0, 1.0, args.ngrid)
    systems = []
    for i in picks:
        sh = shapes[i]
        # the same inputs as the GPU arm: a seed whose A+B is not positive definite at a
        # quadrature point is replaced as make_batch replaces it
        for attempt in range(8):
            seed = sh["seed"] + 100000 * attempt
            s = synth.make_system(sh["n"], sh["nin"], sh["nact"], sh["rank"], seed)
            indn = R.pair_space(s.occ, s.nele)
            ffoo, fofo = cpu_port.transform_factored(s.cmo, s.lfac, s.nin, s.nact)
            ok = True
            for lam in x:
                abp, _, _ = cpu_port.ab_cas_fofo(s.occ, s.xone, indn, s.nin, s.nact, ffoo, fofo,
                                                 s.rdm2act, lam)
                try:
                    np.linalg.cholesky(0.5 * (abp + abp.T))
                except np.linalg.LinAlgError:
                    ok = False
                    break
            if ok:
                break
        systems.append(s)
    log(f"reference sample: systems {picks}, N {[len(R.pair_space(s.occ, s.nele)) for s in systems]}")
    for _ in range(args.warmup):  # thread pools and libraries warmed on the smallest stratum
        cpu_port_energies([systems[0]], args.ngrid, log=lambda *a: None)
    per = [[] for _ in systems]
    sdims = [0] * len(systems)
    nrev = min(4, len(systems))  # strata revisited after the first pass: the cheapest ones
    for k in range(args.steps):
        # one pass over all strata, then the cheapest strata again, so that a long --steps
        # run stays within minutes (the value uses each stratum's mean time)
        j = k if k < len(systems) else (k - len(systems)) % nrev
        t, _, d = cpu_port_energies([systems[j]], args.ngrid, log=log)
        per[j] += t
        sdims[j] = d[0]
    reached = [j for j in range(len(systems)) if per[j]]
    strata_s = sum(statistics.mean(per[j]) for j in reached)
    value = len(reached) / strata_s
    times = [t for j in reached for t in per[j]]
    est, c = batch_estimate([statistics.mean(per[j]) for j in reached], [sdims[j] for j in reached],
                            dims)
    threads = cpu_threads()
    sample = (f"CPU port of the reference algorithm (oracle/cpu_port.py: A+-B reassembled per "
              f"point with OpenMP, ERPASYMM1 with two LAPACK dsyevd, BLAS products), "
              f"{args.ngrid} points; the batch ordered by ERPA dimension in {len(systems)} strata "
              f"of {CPU_STRATUM}, one step = the median system of the next stratum (N "
              f"{[sdims[j] for j in reached]}; after one pass the {nrev} smallest strata are "
              f"revisited); value = strata reached / sum of their mean "
              f"times" + ("" if len(reached) == len(systems) else
                          f" ({len(reached)} of {len(systems)} strata reached: biased to the "
                          f"smaller systems)"))
    line = {"metric": METRIC, "value": value, "unit": "energies/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference", "config": workload_config(args),
            "method": "reference algorithm on the host cores (CPU port; the Fortran reference "
                      "cannot be compiled here)",
            "cpu_baseline": {"value": value, "unit": "energies/s", "cores": threads, "kind": "port",
                             "sample": sample,
                             "batch_estimate": {"value": est, "unit": "energies/s",
                                                "model": f"t = {c:.3e} s * N^3 fitted to the "
                                                         "sample, summed over the 64 systems"}},
            "e2e": {"value": value, "unit": "energies/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    log = (lambda *a: print(*a, file=sys.stderr, flush=True)) if rank == 0 else (lambda *a: None)

    import __graft_entry__
    __graft_entry__.build()
    from gammcor_gb300 import api, surrogate

    if args.erpa_once or args.acecorr_once:
        from gammcor_gb300 import synth
        shapes = synth.batched_shapes(args.nsys, args.seed)

        def pairs(sh):
            nv = sh["n"] - sh["nin"] - sh["nact"]
            return sh["n"] * (sh["n"] - 1) // 2 - sh["nin"] * (sh["nin"] - 1) // 2 - nv * (nv - 1) // 2
        sh = max(shapes, key=pairs)
        s = synth.make_system_device(sh["n"], sh["nin"], sh["nact"], sh["rank"], sh["seed"],
                                     device=dev)
        C = torch.as_tensor(np.asfortranarray(s.cmo), device=dev)
        L = torch.as_tensor(np.asfortranarray(s.lfac), device=dev)
        co = C[:, :s.nocc].contiguous()
        indn = api.pair_space(s.occ, s.nele)
        fofo = api.tran4_factored(s.n, L, C, co, C, co, precision=args.precision)
        ffoo = api.tran4_factored(s.n, L, co, co, C, C, precision=args.precision)
        if args.acecorr_once:
            run = lambda: api.acecorr(s.occ, s.xone, indn, s.nact, s.nin, ffoo, fofo,  # noqa: E731
                                      s.rdm2act, ngrid=1, erpa_mode=args.erpa,
                                      precision=args.precision)
            run()  # warm-up
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.cudart().cudaProfilerStart()
            e0.record()
            run()
            e1.record()
            torch.cuda.synchronize()
            torch.cuda.cudart().cudaProfilerStop()
            ctx = api.default_context(0)
            ctx.set_phase_timing(True)
            ph0 = ctx.phase_times()
            run()
            ph1 = ctx.phase_times()
            ctx.set_phase_timing(False)
            print(json.dumps({"acecorr_point": args.erpa, "precision": args.precision,
                              "N": len(indn), "n": s.n, "nocc": s.nocc,
                              "ms": e0.elapsed_time(e1),
                              "phases_ms": {k: ph1[k][0] - ph0[k][0] for k in ph1}}))
            return
        abp, abm, _ = api.ab_cas_fofo(s.occ, s.xone, indn, s.nact, s.nin, ffoo, fofo, s.rdm2act, 0.5)
        api.erpasymm1(abp.clone(), abm.clone(), mode=args.erpa, precision=args.precision)  # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.cudart().cudaProfilerStart()
        e0.record()
        api.erpasymm1(abp, abm, mode=args.erpa, precision=args.precision)
        e1.record()
        torch.cuda.synchronize()
        torch.cuda.cudart().cudaProfilerStop()
        print(json.dumps({"erpa": args.erpa, "precision": args.precision, "N": len(indn),
                          "ms": e0.elapsed_time(e1)}))
        return

    if args.kernel_only:
        n = args.kernel_only
        api.default_context(0).set_gemm_tile(args.tile)
        ms_k = api.tc_gemm_time(n, n, n, args.precision, reps=3)
        print(json.dumps({"kernel": f"tcgen05 GEMM {args.precision} {n}^3", "tile": args.tile,
                          "ms_per_launch": ms_k}))
        return

    ens = surrogate.Ensemble.load(surrogate.MODEL) if args.surrogate else None
    kw = dict(nstreams=args.nstreams or 8, precision=args.precision,
              eig_emulation=bool(args.eig_emulation), erpa_mode=args.erpa)

    def step(b):
        """One pass over a batch: (energies, fallback mask, error estimate, status)."""
        if ens is not None:
            return surrogate.energies(b, ens, threshold=args.threshold,
                                      eig_refine=args.eig_refine, **kw)
        e, _, _, st = api.ac_energy_batched(b, ngrid=args.ngrid, affine=True,
                                            eig_refine=args.eig_refine, **kw)
        return e, np.ones(len(e), bool), np.zeros(len(e)), st

    t0 = time.time()
    batch = make_batch(args.nsys, args.seed, dev, step, rank_offset=rank, log=log, gen=args.gen)
    log(f"batch ready in {time.time() - t0:.1f}s (includes the first warm-up step)")
    ctx = api.default_context(local)
    Ns = batch.ndimx()
    tuned = None
    if args.nstreams == 0:
        best, times = api.autotune_streams(batch, precision=args.precision, erpa_mode=args.erpa)
        tuned = {"streams": best, "seconds": {str(k): v for k, v in times.items()}}
        kw["nstreams"] = best
        args.nstreams = best
        log(f"autotuned worker streams: {best} ({times})")
    log(f"N range {min(Ns)}..{max(Ns)}, mean {sum(Ns) / len(Ns):.0f}")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(max(0, args.warmup - 1)):
        step(batch)
    # Timed steps. Each step first copies the inputs (MO coefficients, ERI
    # factors) from pinned host memory (e2e); `value` is timed from the end of
    # those copies, with the inputs resident in HBM.
    host_c = [t.cpu().pin_memory() for t in batch.cmo]
    host_l = [t.cpu().pin_memory() for t in batch.lfac]
    h2d = sum(t.numel() * 8 for t in host_c) + sum(t.numel() * 8 for t in host_l)
    d2h = args.nsys * 8 * 2
    barrier()
    stream = torch.cuda.current_stream()
    l0 = ctx.launches()
    eig0 = ctx.eig_time()
    ctx.set_phase_timing(True)
    ph0 = ctx.phase_times()
    ms = ems = 0.0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            for i in range(args.nsys):
                batch.cmo[i].copy_(host_c[i], non_blocking=True)
                batch.lfac[i].copy_(host_l[i], non_blocking=True)
            e1.record(stream)
            ecorr, fb, est, status = step(batch)
            e2.record(stream)
            barrier()
            ms += e1.elapsed_time(e2)
            ems += e0.elapsed_time(e2)
    ms /= args.steps
    ems /= args.steps
    launches = (ctx.launches() - l0) // args.steps
    eig1 = ctx.eig_time()
    ph1 = ctx.phase_times()
    ctx.set_phase_timing(False)
    eig = {"device_ms_per_step": (eig1[0] - eig0[0]) / args.steps,
           "calls_per_step": (eig1[1] - eig0[1]) // args.steps,
           "what": "cuSOLVER FP32 eigensolves of the refined form (one cusolverDnXsyevBatched "
                   "call per system for all its points; ssyevd / dsyevd fallbacks), CUDA events "
                   "around each call, summed over the concurrent worker streams; calls = "
                   "matrices solved"}
    phases = {k: {"device_ms_per_step": (ph1[k][0] - ph0[k][0]) / args.steps,
                  "calls_per_step": (ph1[k][1] - ph0[k][1]) // args.steps} for k in ph1}
    phases["what"] = ("CUDA events around each phase on its worker stream, summed over the "
                      "concurrent workers (a phase's time includes the slowdown from the "
                      "others running beside it)")
    ms, ems = max_over_ranks([ms, ems], world, dev)
    value = whole_job_rate(world, args.nsys, ms)
    e2e = {"value": whole_job_rate(world, args.nsys, ems), "unit": "energies/s",
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    log(f"step: {ms:.0f} ms, {value:.3f} energies/s (e2e {e2e['value']:.3f}), fallback "
        f"{fb.mean():.2f}, {launches} kernels/step, eigensolves {eig['device_ms_per_step']:.0f} "
        f"ms in {eig['calls_per_step']} calls")

    # The plain FP64 GPU path (ERPASYMM1 with FP64 products, A+-B reassembled at every
    # point) on the whole batch with the same worker streams, timed with CUDA events; every
    # energy of the last timed step is checked against it.
    plain = None
    key = np.array([args.nsys, args.seed, args.ngrid, rank], dtype=np.int64)
    cached = args.plain_energies and Path(args.plain_energies).exists()
    if cached:
        d = np.load(args.plain_energies)
        if "key" not in d or not np.array_equal(d["key"], key):
            raise SystemExit(f"{args.plain_energies} holds plain energies of another workload "
                             "(systems, seed, points or rank differ)")
    if not args.no_subset and cached:
        pe, pst, t_plain, pclk = d["ecorr"], d["status"], float(d["ms"]), None
    elif not args.no_subset:
        pl = dict(ngrid=args.ngrid, precision="fp64", erpa_mode="symm1", affine=False,
                  nstreams=args.nstreams)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as pclk:
            p0.record(stream)
            pe, _, _, pst = api.ac_energy_batched(batch, **pl)
            p1.record(stream)
            torch.cuda.synchronize()
        t_plain = p0.elapsed_time(p1)
        if args.plain_energies:
            np.savez(args.plain_energies, ecorr=pe, status=pst, ms=t_plain, key=key)
    if not args.no_subset:
        good = (pst == 0) & (status == 0)
        err = np.abs(ecorr - pe)[good]
        worst = int(np.nonzero(good)[0][np.argmax(err)]) if err.size else None
        plain = {"systems": int(good.sum()), "plain_ms": t_plain, "step_ms": ms,
                 "worst_system": worst, "worst_ndimx": Ns[worst] if worst is not None else None,
                 "median_abs_err_eh": float(np.median(err)) if err.size else None,
                 "speedup": t_plain / ms, "streams": args.nstreams,
                 "max_abs_err_eh": float(err.max()) if err.size else None,
                 "within_1ueh": bool(err.size and err.max() <= 1e-6),
                 "timing": ("CUDA events on the calling stream, whole batch" +
                            (" (energies and time read from an earlier run)" if cached else "")),
                 "clocks": pclk.summary() if pclk else None}
        log(f"plain FP64 on all {int(good.sum())} systems: {t_plain / 1000:.1f}s vs step "
            f"{ms / 1000:.1f}s ({t_plain / ms:.2f}x), max |dE| {plain['max_abs_err_eh']:.2e}")

    # Roofline of this library's dominant kernel: the sliced tcgen05 GEMM at the integrand
    # shape of the largest system (N x N x N), on mixed-magnitude operands, timed alone.
    # Its algorithmic work is 2 N^3 (the FP64-accurate product); the BF16 passes it issues
    # for that are reported beside it.
    hbm, bf16, src = read_peaks()
    Nmax = max(Ns)
    npass = {"bf16x3": 3, "bf16x6": 6, "fp64tc4": 10, "fp64tc5": 15, "fp64tc6": 21}[args.precision]
    ms_k = api.tc_gemm_time(Nmax, Nmax, Nmax, args.precision, reps=5)
    ach = 2.0 * Nmax ** 3 / (ms_k / 1000.0) / 1e12
    roof = {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
            "frac": ach / bf16, "traffic": GEMM_TRAFFIC.get((args.precision, Nmax)),
            "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + write.sum)",
            "peak_source": src,
            "passes": {"count": npass, "achieved": ach * npass, "frac": ach * npass / bf16},
            "kernel": f"k_tc_gemm_oz ({args.precision}) {Nmax}^3, {ms_k:.2f} ms/launch"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        order = np.argsort(Ns, kind="stable")
        picks = [int(order[k]) for k in CPU_SAMPLE[:4] if k < len(order)]
        times, _, dims = cpu_port_energies([batch.systems[i] for i in picks], args.ngrid, log=log)
        est, _ = batch_estimate(times, dims, Ns)
        cpu = {"value": len(times) / sum(times), "unit": "energies/s", "cores": cpu_threads(),
               "kind": "port",
               "sample": f"CPU port of the reference algorithm (oracle/cpu_port.py), "
                         f"{args.ngrid} points, systems {picks} of this batch (N {dims}), "
                         f"{sum(times):.1f}s; energies/s of the sample",
               "batch_estimate": {"value": est, "unit": "energies/s",
                                  "model": "t = c N^3 fitted to the sample"}}

    if rank == 0:
        method = {"precision": args.precision,
                  "erpa": ("cholesky(A+B), affine A+-B, " +
                           ("FP32 eigensolve refined to FP64 accuracy "
                            f"({args.eig_refine} iteration(s)); the Cholesky factors and FP32 "
                            "eigensolves of a system's points batched"
                            if args.erpa == "refined" else "FP64 dsyevd")),
                  "gemm_tile": "chosen per product (oz_tile)",
                  "streams": args.nstreams, "streams_autotune": tuned,
                  "surrogate": (f"ensemble gate at {args.threshold:g} Eh" if ens else "off"),
                  "eig_emulation": bool(args.eig_emulation)}
        line = {"metric": METRIC, "value": value, "unit": "energies/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": workload_config(args), "method": method,
                "surrogate_fallback_rate": float(fb.mean()),
                "erpa_solves_per_energy": float(2 + 6 * fb.mean()) if ens else float(args.ngrid),
                "plain_fp64": plain, "eigensolve": eig, "phases": phases,
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
                "clocks": clk.summary(), "failed_systems": int((status != 0).sum()),
                "eig_refine_stats": ctx.eig_refine_stats()}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_single(args):
    """The single-system configurations.

    precision: the FFOO/FOFO transform in BF16x3, BF16x6 and FP64TC5 against the
    FP64 transform (max abs integral error), and the AC energy of each set of
    integrals with the assembly in FP64 and the ERPA eigenpairs and integrand
    FP64-accurate (refined form, FP64TC6 products), so that the energy error is
    the transform's.

    large: the measured form on one system (FP64TC5 products, refined ERPA, the
    surrogate gate with its fallback), its time per energy, and its error against
    the same quadrature with FP64TC6 products; --plain 1 adds the plain FP64 GPU
    path (ERPASYMM1 with FP64 products, minutes at this size)."""
    import numpy as np
    import torch
    torch.cuda.set_device(0)
    dev = "cuda:0"
    log = lambda *a: print(*a, file=sys.stderr, flush=True)  # noqa: E731
    import __graft_entry__
    __graft_entry__.build()
    from gammcor_gb300 import api, surrogate, synth
    cfg = dict(synth.CFG_PRECISION if args.workload == "precision" else synth.CFG_LARGE)
    t0 = time.time()
    s = synth.make_system_device(**cfg, seed=args.seed, device=dev)
    batch = api.BatchInputs([s], dev)
    N = int(batch.ndimx()[0])
    log(f"system {cfg} N={N} generated in {time.time() - t0:.0f}s")
    x8, w8 = surrogate.gauss8()
    line = {"workload": args.workload, "system": cfg, "ndimx": N, "lambda_points": 8,
            "data": "synthetic", "seed": args.seed}

    def seconds(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        out = fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1000.0, out

    if args.workload == "precision":
        C = torch.as_tensor(np.ascontiguousarray(s.cmo), device=dev)
        L = torch.as_tensor(np.ascontiguousarray(s.lfac), device=dev)
        co = C[:, :s.nocc].contiguous()
        indn = batch.indn[0]

        def transform(p):
            fofo = api.tran4_factored(s.n, L, C, co, C, co, precision=p)
            ffoo = api.tran4_factored(s.n, L, co, co, C, C, precision=p)
            return fofo, ffoo

        def energy(fofo, ffoo):
            ws = []
            for lam in x8:
                abp, abm, ecas = api.ab_cas_fofo(s.occ, s.xone, indn, s.nact, s.nin, ffoo, fofo,
                                                 s.rdm2act, float(lam))
                y, e = api.erpasymm1(abp, abm, mode="refined", precision="fp64tc6")
                ws.append(api.ace_ne_erpa_fofo(y, e, s.occ, indn, s.nact, s.nin, fofo,
                                               precision="fp64tc6"))
            return float(np.dot(w8, ws)), ecas

        t64, (fofo64, ffoo64) = seconds(lambda: transform("fp64"))
        e64, ecas = energy(fofo64, ffoo64)
        res = {"fp64": {"transform_s": t64, "ecorr": e64, "integral_max_abs_err": 0.0,
                        "ecorr_err": 0.0}}
        for p in ("bf16x3", "bf16x6", "fp64tc5"):
            tp, (fofo, ffoo) = seconds(lambda: transform(p))
            err = max(float((fofo - fofo64).abs().max()), float((ffoo - ffoo64).abs().max()))
            ep, _ = energy(fofo, ffoo)
            res[p] = {"transform_s": tp, "ecorr": ep, "integral_max_abs_err": err,
                      "ecorr_err": abs(ep - e64)}
            log(f"{p}: transform {tp:.2f}s, max |d integral| {err:.2e}, |d Ecorr| {abs(ep - e64):.2e}")
            del fofo, ffoo
        line.update({"metric": "AC-CAS transform precision: max abs integral error and energy "
                               "error vs FP64", "ecas": ecas, "results": res})
    else:
        ens = surrogate.Ensemble.load(surrogate.MODEL)
        kw = dict(nstreams=1, precision="fp64tc5", erpa_mode="refined")
        surrogate.energies(batch, ens, threshold=args.threshold, **kw)  # warm-up
        t_fast, (e, fb, est, st) = seconds(lambda: surrogate.energies(batch, ens,
                                                                       threshold=args.threshold,
                                                                       **kw))
        t_ref, ref = seconds(lambda: api.ac_energy_batched(batch, ngrid=8, precision="fp64tc6",
                                                           erpa_mode="refined", nstreams=1))
        line.update({"metric": "AC-CAS seconds per energy, large single system",
                     "seconds_per_energy": t_fast, "ecorr": float(e[0]),
                     "surrogate_fallback": bool(fb[0]), "status": int(st[0]),
                     "reference_fp64tc6_s": t_ref, "ecorr_err_vs_fp64tc6": abs(float(e[0] - ref[0][0]))})
        if args.plain:
            t_plain, pl = seconds(lambda: api.ac_energy_batched(
                batch, ngrid=8, precision="fp64", erpa_mode="symm1", affine=False, nstreams=1))
            line.update({"plain_fp64_s": t_plain, "speedup_vs_plain": t_plain / t_fast,
                         "ecorr_err_vs_plain": abs(float(e[0] - pl[0][0]))})
        log(f"large: {t_fast:.1f}s per energy, fallback {bool(fb[0])}, "
            f"|dE| vs FP64TC6 {line['ecorr_err_vs_fp64tc6']:.2e}")
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload != "batched":
        run_single(a)
    else:
        run_ours(a)
