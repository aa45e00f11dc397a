"""Benchmark: single-orbital Anderson impurity solves on one GB300.

Workload (one "step" = one batch of B complete solves, default B = 8 baths): single-orbital Anderson impurity with 11 bath sites
(12 orbitals, 24 spin-orbitals), U = 3, eps_d = -U/2, eps_k ~ U[-2, 2], V_k ~ U[0.1, 0.5] from a seed;
all 169 (N_up, N_dn) sectors (largest 853,776 states); spin-resolved storage; 8 eigen-pairs per sector;
beta = 100; G(i w_n), chi_Sz and chi_N on 1024 Matsubara points; 100 Lanczos steps per start vector.
Default precision: FP32 vectors with FP64 (float-float) dot products, FP64 projected matrices,
Boltzmann weights and continued fractions.

Arms
* default (``--impl gb300``): the CUDA path.  ``value`` = solves/s of a batch of B models with the models
  resident on the device (sector tables built once), the L2 flushed between steps by a 256 MiB write;
  ``plain_single_solve`` = one model through the plain path (one sector and one start vector at a time);
  ``e2e`` = the batched solve through the public API from host arrays every step (model upload, tables,
  solve, G and chi copied back); ``roofline`` = the dominant kernel of a solve, the SRS H*v (the
  operator of the eigen-solver and Lanczos steps, here 64 vectors of the largest sector per launch),
  ``roofline_cgs_dot`` / ``roofline_cgs_update`` the two Gram-Schmidt passes (16 bases x 15 columns of
  the largest sector per launch, well above L2), each timed live with CUDA events on the library's
  stream; ``cpu_baseline`` = the CPU restatement timed on a bounded sample
  (Lanczos steps of the largest sector, single thread as the reference's SpinResolvedStorage) and
  extrapolated by the element-steps the solve performed.
* ``--impl reference``: the reference's CPU path on the host cores.  The reference cannot be built on
  the GPU host, so its restatement (oracle/) runs: SOCRS H*v with OpenMP over all cores.  Each step is a
  bounded sample (Lanczos steps of the largest sector); the solve's work is the ARPACK (dsaupd, through
  scipy's build) operator count measured on the largest sector in warm-up, applied to every sector,
  plus 100 Lanczos steps per Green's-function / susceptibility start vector.
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


def config(precision, batch=1):
    return {"workload": "single-orbital Anderson impurity, 11 bath sites (12 orbitals), all 169 Sz sectors "
                        "(max 853776 states), SRS, nev 8 (ncv 19), beta 100, G + chi_Sz + chi_N on 1024 Matsubara "
                        "points, 100 Lanczos steps", "seeds": "0..%d (one bath per model)" % (batch - 1),
            "models_per_step": batch, "storage": "SRS", "vectors": precision,
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


def cpu_sample(params, data, threads, steps=3):
    """Seconds per element-step of the CPU restatement: `steps` plain Lanczos steps (H*v, two dot products,
    two vector updates) of the largest sector.  threads == 1: SRS H*v (the reference's SpinResolvedStorage
    has no threading); threads > 1: SOCRS H*v with OpenMP."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle.oracle import OracleED
    storage = "SRS" if threads == 1 else "SOCRS"
    p = dict(params)
    p["lanc.NLANC"] = steps
    o = OracleED(p, data, storage, "SIAM")
    n = o.fill(6, 6)
    v = np.random.default_rng(0).standard_normal(n)
    v /= np.linalg.norm(v)
    t0 = time.perf_counter()
    o.lanczos((6, 6), v)
    dt = time.perf_counter() - t0
    return dt / (steps * n), {"dim": n, "steps": steps, "seconds": dt, "storage": storage}


def run_gpu(args, rank, world):
    import torch
    from edlib_gb300 import _abi, build, ed
    build.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    B = args.batch
    specs = [workload(rank * B + q) for q in range(B)]
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
    total = sum(times)
    if world > 1:
        t = torch.tensor([total], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total = float(t.item())
        torch.distributed.barrier()
    value = world * B * args.steps / total
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
    e2e = {"value": round(world * B * len(e2e_t) / sum(e2e_t), 4), "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}
    ham = ed.Hamiltonian(ed.Params(specs[0][0]), specs[0][1], storage="SRS", precision=args.precision, device=local)

    # rooflines: the dominant kernel (the SRS H*v) and the two Gram-Schmidt passes
    roof_dot, roof_upd = cgs_roofline(L, ham, args)
    roof = spmv_roofline(L, ham, args)
    ham.close()

    cpu = None
    if rank == 0 and not args.no_cpu:
        per, smp = cpu_sample(specs[0][0], specs[0][1], 1)
        work = stats["element_steps"]
        cpu = {"value": round(1.0 / (per * work), 6), "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "%d Lanczos steps of sector (6,6) (dim %d, %s, 1 thread) took %.2f s; extrapolated to the "
                         "%.4g element-steps of one solve" % (smp["steps"], smp["dim"], smp["storage"], smp["seconds"],
                                                             work)}
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
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64",
            "data": "synthetic (seeded bath parameters)", "config": config(args.precision, B), "e2e": e2e,
            "gpu_launches": int(launches), "roofline": roof, "roofline_cgs_dot": roof_dot,
            "roofline_cgs_update": roof_upd,
            "cpu_baseline": cpu, "clocks": clk,
            "solver_stats": stats}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def spmv_roofline(L, ham, args):
    """Batched SRS H*v over `args.nvec` vectors of sector (6,6), timed with CUDA events inside the library on
    its own stream (two untimed launches first).  Algorithmic bytes per launch: x read and y written once per
    element of every vector, the sector's diagonal once ((2 x vectors + 1) x states x element size); the hop
    gathers and the per-spin CSR hit L2."""
    ms, by = ctypes.c_double(0), ctypes.c_double(0)
    rc = L.edgpu_bench_spmv(ham._m, 1, 6, 6, args.nvec, 1 if args.precision == "fp32" else 0, args.reps,
                            ctypes.byref(ms), ctypes.byref(by))
    peak, src = _peak()
    if rc != 0 or ms.value <= 0:
        return None
    achieved = by.value / (ms.value * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": _traffic().get("k_mv"),
            "kernel": "k_mv<%s> SRS H*v, %d vectors x 853776 states per launch" %
                      ("float" if args.precision == "fp32" else "double", args.nvec),
            "bytes_per_launch": by.value, "ms_per_launch": round(ms.value, 4), "peak_source": src}


def cgs_roofline(L, ham, args):
    """The eigen-solver's two Gram-Schmidt passes (the dominant kernels of a solve): 16 independent bases
    of 15 columns of sector (6,6) per launch, timed with CUDA events inside the library (two untimed rounds
    first).  Algorithmic bytes per basis: the 15 columns and w (dot pass, 16 x 853,776 x element size); the
    columns, w read and w written (update pass, 17 x ...)."""
    md, mu, bd, bu = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
    rc = L.edgpu_bench_cgs(ham._m, 1, 6, 6, args.cgs_columns, args.cgs_tasks, 1 if args.precision == "fp32" else 0,
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
                              (name, "float" if args.precision == "fp32" else "double", args.cgs_tasks,
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


def run_spmv_only(args):
    import torch
    from edlib_gb300 import _abi, build, ed
    build.build()
    torch.cuda.set_device(0)
    params, data = workload(0)
    ham = ed.Hamiltonian(ed.Params(params), data, storage="SRS", precision=args.precision, device=0)
    roof = spmv_roofline(_abi.lib(), ham, args)
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
    print(json.dumps(line), flush=True)
    return 0


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
    """Batched Kanamori impurities: all of them submitted at once to the request server (one lock-step
    eigen-solver batch over every impurity's sectors, batched Lanczos runs for the Green's functions), against
    the same models one at a time through the one-model batched path and through the plain path (one sector
    and one start vector at a time)."""
    import torch
    from edlib_gb300 import build, ed
    build.build()
    torch.cuda.set_device(0)
    specs = kanamori_batch(args.kanamori)
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
    print(json.dumps(line), flush=True)
    return 0


def arpack_opx_count(params, data, threads):
    """Operator applications ARPACK (scipy's dsaupd build, which="SA", tol=1e-14, ncv = 2 nev + 3) needs
    on the largest sector with the CPU restatement's H*v."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from scipy.sparse.linalg import LinearOperator, eigsh
    from oracle.oracle import OracleED
    o = OracleED(params, data, "SRS", "SIAM")
    n = o.fill(6, 6)
    cnt = [0]

    def mv(x):
        cnt[0] += 1
        return o.av(np.asarray(x).reshape(-1))

    nev = int(params["arpack.NEV"])
    eigsh(LinearOperator((n, n), matvec=mv, dtype=np.float64), k=nev, which="SA", ncv=2 * nev + 3, tol=1e-14,
          maxiter=1000, v0=np.ones(n) / math.sqrt(n))
    return cnt[0]


def run_reference(args):
    params, data = workload(0)
    ncores = os.cpu_count() or 1
    ns = int(params["NSITES"])
    nev = int(params["arpack.NEV"])
    ncv = 2 * nev + 3
    t0 = time.perf_counter()
    opx = arpack_opx_count(params, data, 1)
    t_arpack = time.perf_counter() - t0
    # the reference's fastest CPU H*v for this model: SpinResolvedStorage (one thread) or SOCRSStorage
    # (OpenMP over all cores); both are sampled in warm-up and the faster is timed
    srs, _ = cpu_sample(params, data, 1, steps=2)
    socrs, _ = cpu_sample(params, data, ncores, steps=2)
    threads = 1 if srs <= socrs else ncores
    for _ in range(max(0, args.warmup - 1)):
        cpu_sample(params, data, threads, steps=2)
    per = []
    info = None
    for _ in range(args.steps):
        x, info = cpu_sample(params, data, threads, steps=3)
        per.append(x)
    per = float(np.median(per))
    work = 0.0
    for nu in range(ns + 1):
        for nd in range(ns + 1):
            d = math.comb(ns, nu) * math.comb(ns, nd)
            if d > 1:
                work += (d if d <= ncv else opx) * d
    # Green's function: 4 start vectors (c+/c, 2 spins) and 2 susceptibility start vectors of the ground
    # state, 100 steps each, in sectors of (6 +- 1, 6) / (6, 6) size
    work += 100 * (4 * math.comb(ns, 7) * math.comb(ns, 6) + 2 * math.comb(ns, 6) ** 2)
    t_solve = per * work
    value = 1.0 / t_solve
    line = {"metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1000.0 * t_solve, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded bath parameters)",
            "config": dict(config("fp64"), parallelism="host cores (OpenMP)"), "impl": "reference",
            "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "per step %d Lanczos steps of sector (6,6) (dim %d, %s H*v, %d threads); "
                                       "solve work = ARPACK operator count %d measured on (6,6) in %.1f s, applied to "
                                       "every sector, + 600 Green's-function Lanczos steps: %.4g element-steps"
                                       % (info["steps"], info["dim"], info["storage"], threads, opx, t_arpack, work)},
            "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--batch", type=int, default=8, help="impurity models solved together per step")
    ap.add_argument("--multiplicity-check", type=int, default=2,
                    help="eigen-solver check for missed degenerate copies: 0 full, 1 none, c >= 2 c - 1 cycles")
    ap.add_argument("--spmv-only", action="store_true",
                    help="only time the batched SRS H*v kernel on sector (6,6) (the roofline leg; used for profiling)")
    ap.add_argument("--nvec", type=int, default=64, help="vectors per H*v launch in the roofline leg")
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
    if args.cgs_only:
        return run_cgs_only(args)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return run_reference(args) if rank == 0 else 0
    return run_gpu(args, rank, world)


if __name__ == "__main__":
    sys.exit(main())
