"""Benchmark: single-orbital Anderson impurity solves on one GB300.

Workload (one "step" = one batch of B complete solves, default B = 8 baths): single-orbital Anderson impurity with 11 bath sites
(12 orbitals, 24 spin-orbitals), U = 3, eps_d = -U/2, eps_k ~ U[-2, 2], V_k ~ U[0.1, 0.5] from a seed;
all 169 (N_up, N_dn) sectors (largest 853,776 states); spin-resolved storage; 8 eigen-pairs per sector;
beta = 100; G(i w_n), chi_Sz and chi_N on 1024 Matsubara points; 100 Lanczos steps per start vector.
Default precision ("mixed"): the eigen-solve of every sector with FP32 vectors (float-float dot
products, FP64 projected matrices, an FP64 Rayleigh-Ritz step), then the sectors holding the
Boltzmann-weighted pairs continued in FP64 from their FP32 Ritz vectors, and the G / chi recurrences on
float-float vectors (pairs of FP32 values, about 2^-48 relative) from FP64 start vectors; alpha / beta,
Boltzmann weights and continued fractions in FP64.  Results meet the FP64 bounds (eigenvalues 1e-10
relative, G and chi 1e-8; tests/test_gpu_parity.py checks this workload at full size).

Arms
* default (``--impl gb300``): the CUDA path.  ``value`` = solves/s of a batch of B models with the models
  resident on the device (sector tables built once), the L2 flushed between steps by a 256 MiB write;
  ``plain_single_solve`` = one model through the plain path (one sector and one start vector at a time);
  ``one_model_batched`` = one model with all its sectors batched; ``e2e`` = the batched solve through the
  public API from host arrays every step (model upload, tables, solve, G and chi copied back);
  ``roofline`` = the dominant kernel of a solve, the SRS H*v, as the eigen step launches it (one vector of
  every sector of the B models per launch); ``roofline_spmv_probe`` = the same operator on 64 vectors of the
  largest sector; ``roofline_cgs_dot`` / ``roofline_cgs_update`` the two Gram-Schmidt passes (16 bases x 15
  columns of the largest sector per launch, well above L2), each timed live with CUDA events on the
  library's stream; ``served`` = a seeded request trace through the continuous-batching server;
  ``kanamori_batch`` = 8 three-orbital Kanamori impurities batched; ``cpu_baseline`` = the eigen-solve of the
  largest sector by the CPU restatement on this host, measured, scaled by the share it took of a complete
  CPU solve measured on the same kind of host.
* probes: ``--spmv-only`` (64 vectors of one sector, ``--spmv-sector NU,ND``), ``--spmv-batch-only`` (the
  eigen step's operator over every sector of ``--batch`` models), ``--cgs-only`` (the Gram-Schmidt passes),
  ``--batch-step-only`` (the benchmark step alone, printing its kernel-launch counts for an ncu launch list),
  ``--serve`` / ``--kanamori N`` (the served trace and the Kanamori batch alone).
* ``--impl reference``: the reference's CPU path on the host cores.  The reference cannot be built on
  the GPU host, so its restatement (oracle/) runs complete solves of the workload's model (every sector's
  eigen-solve through ARPACK, G, static observables, chi_Sz, chi_N) with the faster of its spin-resolved
  (one thread) and SOCRS (OpenMP over every core) H*v, as many as fit in ``--ref-budget`` seconds.
"""
import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Anderson solves/s (12-orbital SIAM, all sectors, G + chi_Sz + chi_N)"
UNIT = "solves/s"


def workload(seed=0):
    from edlib_gb300 import models
    return models.anderson_12(seed)


PRECISION_NOTE = {
    "mixed": "eigen-solve fp32 (float-float dots, fp64 projected matrices, Rayleigh-Ritz); kept sectors "
             "continued in fp64; G/chi recurrences on float-float vectors (fp64-accurate) from fp64 start vectors",
    "fp32": "fp32 vectors throughout (fp64 dots, projected matrices, fractions)",
    "fp64": "fp64 vectors throughout"}
DTYPE = {"mixed": "f32+f64", "fp32": "f32", "fp64": "f64"}


def config(precision, batch=1):
    return {"workload": "single-orbital Anderson impurity, 11 bath sites (12 orbitals), all 169 Sz sectors "
                        "(max 853776 states), SRS, nev 8 (ncv 19), beta 100, G + chi_Sz + chi_N on 1024 Matsubara "
                        "points, 100 Lanczos steps", "seeds": "0..%d (one bath per model)" % (batch - 1),
            "models_per_step": batch, "storage": "SRS", "vectors": PRECISION_NOTE[precision],
            "multiplicity_check": "one restart cycle from a fresh random vector per sector",
            "l2": "flushed between steps (256 MiB write)", "parallelism": "replicas"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits", "-i",
                                          os.environ.get("LOCAL_RANK", "0"), "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        try:
            if self.samples:
                out["sm_mhz"] = float(np.median([float(s[0]) for s in self.samples]))
                out["sm_max_mhz"] = float(self.samples[0][1])
                for k, nm in enumerate(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]):
                    if any(s[3 + k].lower() == "active" for s in self.samples):
                        out["reasons"].append(nm)
                out["samples"] = len(self.samples)
        except Exception:
            pass
        return out


_FLUSH = None


def flush_l2():
    """Overwrite the L2 (129 MB) with a 256 MiB device write."""
    global _FLUSH
    import torch
    if _FLUSH is None:
        _FLUSH = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    _FLUSH.fill_(1)
    torch.cuda.synchronize()


def solve(ham, p):
    """One solve on a resident model: diag, G, static observables, chi_Sz, chi_N."""
    from edlib_gb300 import ed
    ham.diag()
    G = ed.GreensFunction(p, ham).compute()
    so = ed.StaticObservables(p).calculate_static_observables(ham)
    chi = ed.ChiLoc(p, ham)
    cs = chi.compute("Sz", sum(so["M"]) / (2.0 * len(so["M"]))).copy()
    cn = chi.compute("N", sum(so["N"]) / len(so["N"])).copy()
    return G, cs, cn


def solve_many(hams, p):
    """B solves in shared launches: batched diag, batched G, per-model static observables, batched chi."""
    from edlib_gb300 import ed
    ed.diag_many(hams)
    Gs, _, _ = ed.greens_function_many(p, hams)
    obs = [ed.StaticObservables(p).calculate_static_observables(h) for h in hams]
    cs, _, _ = ed.chiloc_many(p, hams, "Sz", [float(sum(o["M"]) / (2.0 * len(o["M"]))) for o in obs])
    cn, _, _ = ed.chiloc_many(p, hams, "N", [float(sum(o["N"]) / len(o["N"])) for o in obs])
    return Gs, cs, cn


def rank_seeds(rank, batch):
    """Seeds of the `batch` models one rank solves: every rank its own disjoint batch (weak scaling, replicas:
    no data is exchanged between ranks)."""
    return [rank * batch + q for q in range(batch)]


def max_over_ranks(total, world, device="cpu"):
    """The timed region's length of the slowest rank (a MAX all-reduce; every rank must call it)."""
    if world <= 1:
        return total
    import torch
    t = torch.tensor([total], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, batch, steps, total):
    """Whole-job solves/s: every rank's models over the slowest rank's time."""
    return world * batch * steps / total


def run_gpu(args, rank, world):
    import torch
    from edlib_gb300 import _abi, build, ed
    build.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    B = args.batch
    specs = [workload(sd) for sd in rank_seeds(rank, B)]
    p = ed.Params(specs[0][0])
    L = _abi.lib()
    ext = torch.cuda.ExternalStream(L.edgpu_ctx_stream(ed.context(local)))

    def timed(fn):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(ext)
        out = fn()
        ev1.record(ext)
        ev1.synchronize()
        return ev0.elapsed_time(ev1) * 1e-3, out

    # one model: the plain path (one sector and one start vector at a time, the reference's loop order),
    # then the same model with all its sectors / start vectors batched
    single = ed.Hamiltonian(ed.Params(specs[0][0]), specs[0][1], storage="SRS", precision=args.precision, device=local)
    single.multiplicity_check = args.multiplicity_check
    solve(single, p)  # builds the sector tables once
    single.max_batch = 1
    flush_l2()
    t_plain, _ = timed(lambda: solve(single, p))
    single.max_batch = 0
    flush_l2()
    t_single, _ = timed(lambda: solve(single, p))
    stats = single.stats()
    single.close()

    # resident batch of B impurity models (seeded bath parameters), all sectors of all models per launch
    hams = [ed.Hamiltonian(ed.Params(pp), dd, storage="SRS", precision=args.precision, device=local) for pp, dd in specs]
    for h in hams:
        h.multiplicity_check = args.multiplicity_check
    for _ in range(max(3, args.warmup)):
        solve_many(hams, p)
    launch0 = L.edgpu_launch_count()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler()
    clocks.start()
    times = []
    for _ in range(args.steps):
        flush_l2()
        dt, _ = timed(lambda: solve_many(hams, p))
        times.append(dt)
    clk = clocks.stop()
    launches = (L.edgpu_launch_count() - launch0) // max(1, args.steps)
    total = max_over_ranks(sum(times), world, device="cuda")
    if world > 1:
        torch.distributed.barrier()
    value = job_throughput(world, B, args.steps, total)
    roof_batch = spmv_batch_roofline(L, hams, args)
    for h in hams:
        h.close()

    # end to end: public API from host arrays every step (B model uploads + tables + batched solve + outputs)
    e2e_t = []
    h2d = d2h = 0
    for _ in range(max(1, min(args.steps, 2))):
        flush_l2()

        def e2e_step():
            hs = [ed.Hamiltonian(ed.Params(pp), dd, storage="SRS", precision=args.precision, device=local)
                  for pp, dd in specs]
            for h in hs:
                h.multiplicity_check = args.multiplicity_check
            out = solve_many(hs, p)
            npairs = sum(len(h.eigenpairs()) for h in hs)
            for h in hs:
                h.close()
            return out, npairs

        dt, ((Gs, cs, cn), npairs) = timed(e2e_step)
        e2e_t.append(dt)
        h2d = int(sum(np.asarray(v).nbytes for _, dd in specs for v in dd.values()))
        d2h = int(sum(a.nbytes for a in Gs) + sum(a.nbytes for a in cs) + sum(a.nbytes for a in cn) + 16 * npairs)
    e2e_total = max_over_ranks(sum(e2e_t), world, device="cuda")
    e2e = {"value": round(job_throughput(world, B, len(e2e_t), e2e_total), 4), "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}
    ham = ed.Hamiltonian(ed.Params(specs[0][0]), specs[0][1], storage="SRS", precision=args.precision, device=local)

    # rooflines: the dominant kernel (the SRS H*v) and the two Gram-Schmidt passes
    roof_dot, roof_upd = cgs_roofline(L, ham, args)
    roof = spmv_roofline(L, ham, args)
    ham.close()

    served = kana = None
    if rank == 0 and not args.no_serve:
        served = serve_line(args)
        for k in ("metric", "impl", "unit", "higher_is_better"):
            served.pop(k, None)
    if rank == 0 and args.with_kanamori > 0:
        kana = kanamori_line(args, args.with_kanamori)
        for k in ("impl", "unit"):
            kana.pop(k, None)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline_sample()
    line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1000.0 * total / args.steps, 3), "higher_is_better": True,
            "batch": B,
            "plain_single_solve": {"value": round(1.0 / t_plain, 4), "unit": UNIT, "ms_per_solve": round(1000.0 * t_plain, 2),
                                   "path": "one model, one sector and one start vector at a time (max_batch 1)",
                                   "batched_speedup": round(value / world * t_plain, 2)},
            "one_model_batched": {"value": round(1.0 / t_single, 4), "unit": UNIT,
                                  "ms_per_solve": round(1000.0 * t_single, 2),
                                  "path": "one model, all sectors / start vectors batched (max_batch 0)",
                                  "batched_speedup": round(value / world * t_single, 2)},
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[args.precision],
            "data": "synthetic (seeded bath parameters)", "config": config(args.precision, B), "e2e": e2e,
            "gpu_launches": int(launches), "roofline": roof_batch, "roofline_spmv_probe": roof,
            "roofline_cgs_dot": roof_dot,
            "roofline_cgs_update": roof_upd,
            "served": served, "kanamori_batch": kana, "cpu_baseline": cpu, "clocks": clk,
            "solver_stats": stats}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def spmv_roofline(L, ham, args, sector=(6, 6), label="853776 states"):
    """Batched SRS H*v over `args.nvec` vectors of one sector (default (6,6) of the 12-orbital Anderson model),
    timed with CUDA events inside the library on its own stream (two untimed launches first).  Algorithmic
    bytes per launch: x read and y written once per element of every vector, the sector's diagonal once
    ((2 x vectors + 1) x states x element size); the hop gathers and the per-spin CSR hit L2."""
    ms, by = ctypes.c_double(0), ctypes.c_double(0)
    rc = L.edgpu_bench_spmv(ham._m, 1, sector[0], sector[1], args.nvec, 0 if args.precision == "fp64" else 1,
                            args.reps, ctypes.byref(ms), ctypes.byref(by))
    peak, src = _peak()
    if rc != 0 or ms.value <= 0:
        return None
    achieved = by.value / (ms.value * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": _traffic().get("k_mv"),
            "kernel": "k_mv<%s> SRS H*v, %d vectors x %s per launch" %
                      ("double" if args.precision == "fp64" else "float", args.nvec, label),
            "bytes_per_launch": by.value, "ms_per_launch": round(ms.value, 4), "peak_source": src}


def spmv_batch_roofline(L, hams, args):
    """The SRS H*v as one eigen-solver step launches it: one vector of every sector (169 per model) of the
    step's models in one launch, timed with CUDA events inside the library on its own stream (two untimed
    launches first).  Algorithmic bytes per launch: per sector x read, y written and its diagonal read
    (3 x states x element size)."""
    import ctypes as ct
    ms, by, st = ct.c_double(0), ct.c_double(0), ct.c_longlong(0)
    arr = (ct.c_void_p * len(hams))(*[h._m for h in hams])
    rc = L.edgpu_bench_spmv_batch(arr, len(hams), 1, 0 if args.precision == "fp64" else 1, args.reps, ct.byref(ms),
                                  ct.byref(by), ct.byref(st))
    if rc != 0 or ms.value <= 0:
        return None
    peak, src = _peak()
    achieved = by.value / (ms.value * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": _traffic().get("k_mv_batch"),
            "kernel": "k_mv<%s> SRS H*v, one vector of each of the %d sectors (%d states) of %d models per launch "
                      "(the eigen step's operator)" % ("double" if args.precision == "fp64" else "float",
                                                       169 * len(hams), st.value, len(hams)),
            "bytes_per_launch": by.value, "ms_per_launch": round(ms.value, 4), "peak_source": src}


def cgs_roofline(L, ham, args):
    """The eigen-solver's two Gram-Schmidt passes (the dominant kernels of a solve): 16 independent bases
    of 15 columns of sector (6,6) per launch, timed with CUDA events inside the library (two untimed rounds
    first).  Algorithmic bytes per basis: the 15 columns and w (dot pass, 16 x 853,776 x element size); the
    columns, w read and w written (update pass, 17 x ...)."""
    md, mu, bd, bu = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
    rc = L.edgpu_bench_cgs(ham._m, 1, 6, 6, args.cgs_columns, args.cgs_tasks, 0 if args.precision == "fp64" else 1,
                           args.reps, ctypes.byref(md), ctypes.byref(mu), ctypes.byref(bd), ctypes.byref(bu))
    if rc != 0 or md.value <= 0 or mu.value <= 0:
        return None, None
    peak, src = _peak()
    traffic = _traffic()
    out = []
    for name, ms, by in (("k_cgs_dot", md.value, bd), ("k_cgs_upd", mu.value, bu)):
        achieved = by.value / (ms * 1e-3) / 1e9
        out.append({"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "traffic": traffic.get(name),
                    "kernel": "%s<%s>, %d bases x %d columns x 853776 states per launch" %
                              (name, "double" if args.precision == "fp64" else "float", args.cgs_tasks,
                               args.cgs_columns),
                    "bytes_per_launch": by.value, "ms_per_launch": round(ms, 4), "peak_source": src})
    return out[0], out[1]


def _peak():
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(peaks["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except Exception:
        return 6800.0, "fallback 6800 GB/s"


def _traffic():
    """DRAM bytes per launch (read + write) of the probe kernels from one ncu capture of the same probe,
    kept in profiles/roofline_traffic.json (written by hand from the capture summarised beside it)."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "roofline_traffic.json")))
    except Exception:
        return {}


def run_cgs_only(args):
    import torch
    from edlib_gb300 import _abi, build, ed
    build.build()
    torch.cuda.set_device(0)
    params, data = workload(0)
    ham = ed.Hamiltonian(ed.Params(params), data, storage="SRS", precision=args.precision, device=0)
    dot, upd = cgs_roofline(_abi.lib(), ham, args)
    ham.close()
    print(json.dumps({"roofline_cgs_dot": dot, "roofline_cgs_update": upd}), flush=True)
    return 0 if dot else 1


def run_spmv_batch_only(args):
    import torch
    from edlib_gb300 import _abi, build, ed
    build.build()
    torch.cuda.set_device(0)
    hams = [ed.Hamiltonian(ed.Params(pp), dd, storage="SRS", precision=args.precision, device=0)
            for pp, dd in (workload(q) for q in range(args.batch))]
    roof = spmv_batch_roofline(_abi.lib(), hams, args)
    for h in hams:
        h.close()
    print(json.dumps({"roofline": roof}), flush=True)
    return 0 if roof else 1


def run_batch_step_only(args):
    """The benchmark step alone (B models, all sectors, G + chi), for a launch list: `--warmup` untimed steps,
    then `--steps` steps; prints the library's kernel launches before and during the steps, so that an ncu
    launch list can skip exactly the warm-up (ncu -s <launches_before> -c <launches_steps>)."""
    import time
    import torch
    from edlib_gb300 import _abi, build, ed
    build.build()
    torch.cuda.set_device(0)
    L = _abi.lib()
    specs = [workload(q) for q in range(args.batch)]
    p = ed.Params(specs[0][0])
    hams = [ed.Hamiltonian(ed.Params(pp), dd, storage="SRS", precision=args.precision, device=0) for pp, dd in specs]
    for h in hams:
        h.multiplicity_check = args.multiplicity_check
    for _ in range(args.warmup):
        solve_many(hams, p)
    torch.cuda.synchronize()
    before = L.edgpu_launch_count()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        solve_many(hams, p)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    print(json.dumps({"launches_before": int(before), "launches_steps": int(L.edgpu_launch_count() - before),
                      "s_per_step": round(dt / max(1, args.steps), 4), "batch": args.batch}), flush=True)
    for h in hams:
        h.close()
    return 0


def run_spmv_only(args):
    import torch
    from edlib_gb300 import _abi, build, ed, models
    build.build()
    torch.cuda.set_device(0)
    if args.spmv_model == "hubbard4x4":  # the 4x4 cluster's sector (8,8): 165,636,900 states, rows of 12870
        params, data = models.hubbard_4x4()
        sector, label = (8, 8), "165636900 states (4x4 Hubbard)"
    else:
        params, data = workload(0)
        sector, label = (6, 6), "853776 states"
        if args.spmv_sector:
            from math import comb
            sector = tuple(int(v) for v in args.spmv_sector.split(","))
            ns = int(params["NSITES"])
            label = "%d states, sector %s" % (comb(ns, sector[0]) * comb(ns, sector[1]), sector)
    ham = ed.Hamiltonian(ed.Params(params), data, storage="SRS", precision=args.precision, device=0)
    ham.set_limits(0, 0)
    roof = spmv_roofline(_abi.lib(), ham, args, sector, label)
    ham.close()
    print(json.dumps({"roofline": roof}), flush=True)
    return 0 if roof else 1


def serve_trace(args):
    """Seeded request trace: Poisson arrivals (rate args.rate per second) of single-orbital Anderson
    impurities with 5..(max_orbitals - 1) bath sites and three-orbital Kanamori impurities with 1..2 bath
    sites per orbital (6..9 orbitals), NEV in [4, 8], beta in {20, 50, 100}, G on 512 Matsubara points."""
    from edlib_gb300 import models
    rng = np.random.default_rng(args.serve_seed)
    t, out = 0.0, []
    for q in range(args.requests):
        t += rng.exponential(1.0 / args.rate)
        if rng.uniform() < 0.25:
            nb = [int(x) for x in rng.integers(1, 3, size=3)]
            params, data = models.random_kanamori_siam(1000 + q, nb)
            kind = "kanamori%d" % (3 + sum(nb))
        else:
            nbath = int(rng.integers(5, args.max_orbitals))
            params, data = models.random_siam(1000 + q, nbath)
            kind = "siam%d" % (1 + nbath)
        params.update({"arpack.NEV": int(rng.integers(4, 9)), "lanc.BETA": float(rng.choice([20.0, 50.0, 100.0])),
                       "lanc.NOMEGA": 512, "lanc.NLANC": 100, "lanc.BOLTZMANN_CUTOFF": 1e-12})
        out.append((t, kind, params, data))
    return out


def _pct(xs, p):
    xs = sorted(xs)
    if not xs:
        return None
    k = min(len(xs) - 1, max(0, int(math.ceil(p / 100.0 * len(xs))) - 1))
    return xs[k]


def run_serve(args):
    print(json.dumps(serve_line(args)), flush=True)
    return 0


def serve_line(args):
    """Served solves: the trace through the continuous-batching server (requests join the running
    eigen-solver batch as they arrive), then the same trace one request at a time through the plain path
    (one sector and one start vector at a time) and through the one-model batched path.  Latency =
    completion - arrival (queueing included), wall clock on the host; throughput = requests / (last
    completion - first arrival)."""
    import torch
    from edlib_gb300 import _abi, build, ed
    build.build()
    torch.cuda.set_device(0)
    trace = serve_trace(args)
    mk = lambda p, d: ed.Hamiltonian(ed.Params(p), d, storage="SRS", precision=args.precision, device=0)
    # warm-up: one request through every path (kernel modules, graph instantiation)
    p0, d0 = trace[0][2], trace[0][3]
    h = mk(p0, d0)
    h.multiplicity_check = args.multiplicity_check
    h.diag()
    ed.GreensFunction(ed.Params(p0), h).compute()
    h.close()

    def served():
        hams = [mk(p, d) for _, _, p, d in trace]
        for hm in hams:
            hm.multiplicity_check = args.multiplicity_check
        srv = ed.Server(precision=args.precision)
        done, tickets, lat = {}, {}, []
        t0 = time.perf_counter()
        nxt = 0
        while len(done) < len(trace):
            now = time.perf_counter() - t0
            while nxt < len(trace) and trace[nxt][0] <= now:
                tickets[nxt] = srv.submit(hams[nxt])
                nxt += 1
            if len(tickets) == len(done):  # idle until the next arrival
                time.sleep(max(0.0, trace[nxt][0] - now))
                continue
            srv.step()
            now = time.perf_counter() - t0
            for q, tk in tickets.items():
                if q not in done and srv.poll(tk) == srv.DONE:
                    done[q] = now
        srv.close()
        for hm in hams:
            hm.close()
        return done

    def one_at_a_time(max_batch):
        done = {}
        t0 = time.perf_counter()
        for q, (ta, _, p, d) in enumerate(trace):
            now = time.perf_counter() - t0
            if now < ta:
                time.sleep(ta - now)
            hm = mk(p, d)
            hm.multiplicity_check = args.multiplicity_check
            hm.max_batch = max_batch
            hm.diag()
            ed.GreensFunction(ed.Params(p), hm).compute()
            hm.close()
            done[q] = time.perf_counter() - t0
        return done

    def summary(done):
        lat = [done[q] - trace[q][0] for q in range(len(trace))]
        span = max(done.values()) - trace[0][0]
        return {"p50_ms": round(1000 * _pct(lat, 50), 1), "p99_ms": round(1000 * _pct(lat, 99), 1),
                "mean_ms": round(1000 * sum(lat) / len(lat), 1), "solves_per_s": round(len(trace) / span, 3),
                "span_s": round(span, 2)}

    res = {"server": summary(served()), "plain_one_at_a_time": summary(one_at_a_time(1)),
           "model_batched_one_at_a_time": summary(one_at_a_time(0))}
    kinds = {}
    for _, k, _, _ in trace:
        kinds[k] = kinds.get(k, 0) + 1
    line = {"metric": "served Anderson solves: p50 / p99 latency and solves/s vs the plain one-at-a-time path",
            "impl": "gb300", "requests": len(trace), "rate_per_s": args.rate, "precision": args.precision,
            "trace": {"seed": args.serve_seed, "kinds": kinds, "max_orbitals": args.max_orbitals,
                      "nomega": 512, "nlanc": 100},
            "value": res["server"]["solves_per_s"], "unit": "solves/s", "higher_is_better": True,
            "speedup_vs_plain": round(res["server"]["solves_per_s"] / res["plain_one_at_a_time"]["solves_per_s"], 2),
            "speedup_vs_model_batched": round(res["server"]["solves_per_s"] /
                                              res["model_batched_one_at_a_time"]["solves_per_s"], 2)}
    line.update(res)
    return line


def kanamori_batch(n, seed0=2000):
    """n three-orbital Kanamori impurities (U ~ U[2, 5], J = U/6, 2-4 bath sites per orbital: 9-15 orbitals,
    mu at 2.5U - 5J), each solved in its half-filling sector(s) (N_up + N_dn = N_s; both Sz = +-1/2 sectors
    for odd N_s): 4 eigen-pairs, beta 50, G of the 3 impurity orbitals on 512 Matsubara points."""
    from edlib_gb300 import models
    out = []
    for q in range(n):
        params, data = models.random_kanamori_siam(seed0 + q)
        ns = int(params["NSITES"])
        secs = [(ns // 2, ns // 2)] if ns % 2 == 0 else [((ns - 1) // 2, (ns + 1) // 2), ((ns + 1) // 2, (ns - 1) // 2)]
        data["sectors/values"] = np.array(secs, dtype=np.float64)
        params.update({"arpack.SECTOR": 1, "arpack.NEV": 4, "lanc.BETA": 50.0, "lanc.NOMEGA": 512, "lanc.NLANC": 100,
                       "lanc.BOLTZMANN_CUTOFF": 1e-12})
        out.append((params, data, ns))
    return out


def run_kanamori(args):
    print(json.dumps(kanamori_line(args, args.kanamori)), flush=True)
    return 0


def kanamori_line(args, count):
    """Batched Kanamori impurities: all of them submitted at once to the request server (one lock-step
    eigen-solver batch over every impurity's sectors, batched Lanczos runs for the Green's functions), against
    the same models one at a time through the one-model batched path and through the plain path (one sector
    and one start vector at a time)."""
    import torch
    from edlib_gb300 import build, ed
    build.build()
    torch.cuda.set_device(0)
    specs = kanamori_batch(count)
    mk = lambda p, d: ed.Hamiltonian(ed.Params(p), d, storage="SRS", precision=args.precision, device=0)
    # warm-up on the smallest model (modules, graphs)
    p0, d0, _ = min(specs, key=lambda s: s[2])
    h = mk(p0, d0)
    h.diag()
    ed.GreensFunction(ed.Params(p0), h).compute()
    h.close()

    def batched():
        # every impurity submitted at once to the request server (per-model sector lists): all their sectors
        # share the eigen-solver launches, their Green's functions one batched Lanczos run
        hams = [mk(p, d) for p, d, _ in specs]
        for hm in hams:
            hm.multiplicity_check = args.multiplicity_check
        srv = ed.Server(precision=args.precision)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tickets = [srv.submit(hm) for hm in hams]
        while not all(srv.poll(t) == srv.DONE for t in tickets):
            srv.step()
        dt = time.perf_counter() - t0
        res = [srv.result(t) for t in tickets]
        E0 = [r[0].eigenpairs()[0].eigenvalue() for r in res]
        Gs = [r[1] for r in res]
        srv.close()
        for hm in hams:
            hm.close()
        return dt, E0, Gs

    def one_at_a_time(max_batch):
        t = 0.0
        E0, Gs = [], []
        for p, d, _ in specs:
            hm = mk(p, d)
            hm.multiplicity_check = args.multiplicity_check
            hm.max_batch = max_batch
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            hm.diag()
            Gs.append(ed.GreensFunction(ed.Params(p), hm).compute())
            t += time.perf_counter() - t0
            E0.append(hm.eigenpairs()[0].eigenvalue())
            hm.close()
        return t, E0, Gs

    tb, eb, gb = batched()
    tm, em, gm = one_at_a_time(0)
    tp, ep, gp = one_at_a_time(1)
    same = all(a == b == c for a, b, c in zip(eb, em, ep)) and all(
        np.array_equal(x, y) and np.array_equal(x, z) for x, y, z in zip(gb, gm, gp))
    sizes = {}
    for _, _, ns in specs:
        sizes[ns] = sizes.get(ns, 0) + 1
    line = {"metric": "batched Kanamori impurity solves/s (half-filling sectors, G of 3 orbitals)", "impl": "gb300",
            "impurities": len(specs), "orbitals": {str(k): v for k, v in sorted(sizes.items())},
            "precision": args.precision, "value": round(len(specs) / tb, 3), "unit": "solves/s",
            "batched_s": round(tb, 2), "one_model_batched_s": round(tm, 2), "plain_s": round(tp, 2),
            "speedup_vs_plain": round(tp / tb, 2), "speedup_vs_one_model_batched": round(tm / tb, 2),
            "results_identical_across_paths": bool(same)}
    return line


def _cpu_model():
    """The host CPU's model name (and core count) for the baseline records."""
    name = None
    try:
        for line in open("/proc/cpuinfo"):
            key = line.split(":")[0].strip().lower()
            if key in ("model name", "hardware") and ":" in line:
                name = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    if not name:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for line in out.splitlines():
                if line.lower().startswith("model name"):
                    name = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    import platform
    return "%s (%s, %d cores)" % (name or "unknown", platform.machine(), os.cpu_count() or 1)


def _timed_solve(args_list, threads, timeout=3600):
    """One run of oracle/timed_solve.py in a fresh process (so that OMP_NUM_THREADS takes effect)."""
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    r = subprocess.run([sys.executable, "-m", "oracle.timed_solve"] + list(args_list), cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("timed solve failed: %s" % r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def _cpu_variant():
    """The reference's faster CPU H*v for this model on this host: SpinResolvedStorage (one thread; it has no
    threading) or SOCRSStorage (OpenMP over every core), one H*v of the largest sector each."""
    ncores = os.cpu_count() or 1
    srs = _timed_solve(["--av", "--storage", "SRS"], 1)
    socrs = _timed_solve(["--av", "--storage", "SOCRS"], ncores)
    pick = ("SRS", 1) if srs["av_s"] <= socrs["av_s"] else ("SOCRS", ncores)
    return pick, {"srs_1_thread_av_ms": round(1000 * srs["av_s"], 2),
                  "socrs_%d_threads_av_ms" % ncores: round(1000 * socrs["av_s"], 2)}


def cpu_baseline_sample():
    """A bounded sample of the reference's CPU path on this host for the default arm's cpu_baseline: the
    eigen-solve of the largest sector (6,6) of seed 0 (853,776 states), measured, scaled to a complete solve by
    the share that sector's eigen-solve took of a complete solve measured on the same kind of host
    (profiles/cpu_solve_anderson12.json, written from oracle/timed_solve.py's output)."""
    try:
        full = json.load(open(os.path.join(ROOT, "profiles", "cpu_solve_anderson12.json")))
    except Exception:
        return None
    storage, threads = full["storage"], full["threads"]
    smp = _timed_solve(["--seed", "0", "--storage", storage, "--sectors", "6,6"], threads)
    share = full["per_sector_s"]["6,6"] / full["seconds"]
    t_solve = smp["per_sector_s"]["6,6"] / share
    return {"value": round(1.0 / t_solve, 6), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "eigen-solve of sector (6,6) of seed 0 (%s H*v, %d thread(s)) measured: %.2f s; scaled by the "
                      "%.2f%% share it took of a complete %.0f s solve (all sectors, G, chi) measured on %s"
                      % (storage, threads, smp["per_sector_s"]["6,6"], 100 * share, full["seconds"],
                         full.get("host", "the same kind of host")),
            "host": _cpu_model()}


def run_reference(args):
    """The reference's CPU path timed on the host cores: complete solves (every sector's eigen-solve, G, static
    observables, chi_Sz, chi_N) of the workload's model, seed 0, by the oracle's restatement of the
    reference (oracle/timed_solve.py) with the faster of its SpinResolvedStorage (one thread) and
    SOCRSStorage (OpenMP, every core) H*v.  Warm-up: one H*v per variant.  Timed: complete solves, as many
    of --steps as fit in --ref-budget seconds (at least one); `steps` reports how many ran."""
    (storage, threads), av = _cpu_variant()
    times, last = [], None
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps)):
        last = _timed_solve(["--seed", "0", "--storage", storage], threads)
        times.append(last["seconds"])
        if time.perf_counter() - t0 + last["seconds"] > args.ref_budget:
            break
    total = sum(times)
    value = len(times) / total
    host = _cpu_model()
    line = {"metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": args.gpus, "steps": len(times),
            "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": round(1000.0 * total / len(times), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded bath parameters)",
            "config": dict(config("fp64"), seeds="0", models_per_step=1, parallelism="host cores (%s)" % storage),
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "measured: %d complete solve(s) of seed 0 (all 169 sectors, G, chi_Sz, chi_N), "
                                       "%s H*v with %d thread(s): diag %.1f s, G %.1f s, chi + observables %.1f s "
                                       "(last run)" % (len(times), storage, threads, last["diag_s"], last["gf_s"],
                                                       last["chi_obs_s"]),
                             "host": host, "h_v_per_variant": av},
            "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp32", "fp64"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-serve", action="store_true", help="skip the served-trace summary in the default line")
    ap.add_argument("--with-kanamori", type=int, default=8,
                    help="batched Kanamori impurities summarised in the default line (0: none)")
    ap.add_argument("--batch", type=int, default=8, help="impurity models solved together per step")
    ap.add_argument("--multiplicity-check", type=int, default=2,
                    help="eigen-solver check for missed degenerate copies: 0 full, 1 none, c >= 2 c - 1 cycles")
    ap.add_argument("--spmv-only", action="store_true",
                    help="only time the batched SRS H*v kernel on sector (6,6) (the roofline leg; used for profiling)")
    ap.add_argument("--spmv-batch-only", action="store_true",
                    help="only time the SRS H*v over every sector of --batch models (the eigen step's operator)")
    ap.add_argument("--nvec", type=int, default=64, help="vectors per H*v launch in the roofline leg")
    ap.add_argument("--spmv-model", default="anderson12", choices=["anderson12", "hubbard4x4"],
                    help="--spmv-only: the model whose largest sector is probed")
    ap.add_argument("--batch-step-only", action="store_true",
                    help="run the benchmark step alone and print its kernel-launch counts (for a launch list)")
    ap.add_argument("--spmv-sector", default="",
                    help="N_up,N_dn of the 12-orbital Anderson sector in the --spmv-only leg (default 6,6)")
    ap.add_argument("--reps", type=int, default=20, help="timed launches in the roofline legs")
    ap.add_argument("--cgs-only", action="store_true",
                    help="only time the two Gram-Schmidt passes (the roofline of the dominant kernel; for profiling)")
    ap.add_argument("--cgs-tasks", type=int, default=16, help="bases per Gram-Schmidt probe launch")
    ap.add_argument("--cgs-columns", type=int, default=15, help="basis columns in the Gram-Schmidt probe")
    ap.add_argument("--serve", action="store_true",
                    help="served solves: a seeded Poisson trace through the continuous-batching server vs "
                         "one request at a time (p50 / p99 latency, solves/s)")
    ap.add_argument("--requests", type=int, default=32, help="requests in the --serve trace")
    ap.add_argument("--rate", type=float, default=200.0, help="mean arrivals per second in the --serve trace")
    ap.add_argument("--max-orbitals", type=int, default=12, help="largest single-orbital impurity in --serve")
    ap.add_argument("--serve-seed", type=int, default=7)
    ap.add_argument("--ref-budget", type=float, default=900.0,
                    help="--impl reference: seconds of complete CPU solves (at least one runs)")
    ap.add_argument("--kanamori", type=int, default=0,
                    help="batched three-orbital Kanamori impurities (this many) vs one at a time")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    if args.serve:
        return run_serve(args) if rank == 0 else 0
    if args.kanamori:
        return run_kanamori(args) if rank == 0 else 0
    if args.spmv_only:
        return run_spmv_only(args)
    if args.spmv_batch_only:
        return run_spmv_batch_only(args)
    if args.batch_step_only:
        return run_batch_step_only(args)
    if args.cgs_only:
        return run_cgs_only(args)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return run_reference(args) if rank == 0 else 0
    return run_gpu(args, rank, world)


if __name__ == "__main__":
    sys.exit(main())
