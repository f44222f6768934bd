"""Benchmark: factorize + logDet + RGFdiag of one block-tridiagonal-arrowhead
matrix on GB300, FP64-equivalent TFLOP/s (algorithmic LAPACK flop count).

Workload (default): ns=2000, nt=100, nd=6 (n = 200006), seeded synthetic SPD
matrix (diagonal blocks A A^T/ns + (ns+2) I, sub-diagonal N(0, 0.1/ns),
arrowhead N(0, 0.1), corner R R^T/nd + (nt+2) I), stored as the lower CSC
the reference's RGF constructor takes.  One step = factorize (ingest of the
device-resident CSC into the block layout, Cholesky recursion, log-sum) +
logDet + RGFdiag (selected inversion, diag left on the device).

Arms:
  --impl rgf (default)  this library through its C ABI; prints one JSON line
                        with value (inputs resident in HBM), e2e (host CSC ->
                        device, diag back to host, through rgf_create/...),
                        roofline of the dominant kernel, cpu_baseline, clocks.
  --impl reference      the CPU restatement of the reference recursion on the
                        host cores (numpy/scipy OpenBLAS, all threads), on a
                        bounded sample of the same workload.
Under torchrun with N > 1 every rank runs an independent replica (the
recursion does not shard); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "ns2000_nt100_nd6": dict(ns=2000, nt=100, nd=6, seed=3, spde=None),
    "ns1000_nt50_nd4": dict(ns=1000, nt=50, nd=4, seed=2, spde=(40, 25)),
    "ns3_nt3_nd2": dict(ns=3, nt=3, nd=2, seed=1, spde=None),
    # a 20-block prefix of the default workload, for profiling runs
    "ns2000_nt20_nd6": dict(ns=2000, nt=20, nd=6, seed=3, spde=None),
    "ns2000_nt5_nd6": dict(ns=2000, nt=5, nd=6, seed=3, spde=None),
}
METRIC = "FP64-equiv TFLOP/s for factorize+logDet+RGFdiag"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def max_over_ranks(x: float, dist, device) -> float:
    """The slowest rank's value (the job's time is the last rank to finish)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(flops_per_replica: float, world_size: int, ms_step: float) -> float:
    """Whole-job FP64-equivalent TFLOP/s of world_size replicas that each did
    flops_per_replica in (at most) ms_step."""
    return flops_per_replica * world_size / (ms_step * 1e-3) / 1e12


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax.append(float(p[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    """bf16 peaks from MEASURED_PEAKS.json (measured on this GPU pool), else the
    documented fallback."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return {"bf16": float(p["bf16_tflops"]),
                "bf16_sustained": float(p["bf16_tflops_sustained"])}, "of measured"
    except Exception:
        return {"bf16": 1900.0, "bf16_sustained": 1700.0}, "of fallback"


def make_inputs(w):
    from rgf_gb300 import gen
    t = time.time()
    ia, ja, a = gen.generate_bta(w["ns"], w["nt"], w["nd"], w["seed"], spde_grid=w["spde"])
    log(f"[bench] generated n={len(ia) - 1} nnz={len(ja)} in {time.time() - t:.1f}s")
    return ia, ja, a


def cpu_port_sample(w, target_s: float = 12.0):
    """Time the oracle's block recursion (numpy/scipy, all host threads) on a
    prefix of the workload's block columns sized for ~target_s seconds.
    Returns (tflops, cores, sample description, seconds)."""
    from oracle import rgf_oracle as O
    from rgf_gb300 import gen
    from rgf_gb300.flops import algorithmic_flops
    ns, nt, nd = w["ns"], w["nt"], w["nd"]

    def run(k):
        ia, ja, a = gen.generate_bta(ns, k, nd, w["seed"], spde_grid=w["spde"])
        L = O.Layout(ns, k, nd)
        t0 = time.perf_counter()
        MF = O.ingest(L, ia, ja, a)
        O.factorize(L, MF)
        O.logdet(L, MF)
        O.selinv_exact(L, MF)
        dt = time.perf_counter() - t0
        return algorithmic_flops(ns, k, nd)["total"], dt

    k = min(nt, 2)
    fl, dt = run(k)
    per = dt / k
    k2 = int(max(k, min(nt, target_s / max(per, 1e-9))))
    if k2 > k:
        fl, dt = run(k2)
        k = k2
    cores = os.cpu_count()
    sample = f"ns={ns}, nt={k} of {nt}, nd={nd}: first {k} block columns, same generator"
    return fl / dt / 1e12, cores, sample, dt


def blas_threads():
    """Threads host LAPACK/BLAS uses for the oracle (threadpoolctl where it is
    installed, else OPENBLAS_NUM_THREADS, else OpenBLAS's default of all cores)."""
    try:
        from threadpoolctl import threadpool_info
        n = [i["num_threads"] for i in threadpool_info() if i.get("user_api") == "blas"]
        if n:
            return max(n), "threadpoolctl"
    except Exception:
        pass
    env = os.environ.get("OPENBLAS_NUM_THREADS") or os.environ.get("OMP_NUM_THREADS")
    if env and env.isdigit():
        return int(env), "OPENBLAS_NUM_THREADS"
    return os.cpu_count(), "OpenBLAS default (all cores)"


def cpu_oracle_full(w, ia, ja, a, rhs=None):
    """The oracle's block recursion (numpy/scipy, host LAPACK on all threads)
    on the WHOLE workload: ingest + factorize + logDet + exact RGFdiag timed
    (the CPU baseline), then, untimed, the solve of `rhs`.  Returns the
    baseline entry and the oracle's results (logdet, diag, x)."""
    from oracle import rgf_oracle as O
    from rgf_gb300.flops import algorithmic_flops
    ns, nt, nd = w["ns"], w["nt"], w["nd"]
    L = O.Layout(ns, nt, nd)
    t0 = time.perf_counter()
    MF = O.ingest(L, ia, ja, a)
    O.factorize(L, MF)
    ld = O.logdet(L, MF)
    diag = O.selinv_exact(L, MF)
    dt = time.perf_counter() - t0
    x = O.solve(L, MF, rhs) if rhs is not None else None
    del MF
    threads, how = blas_threads()
    cpu = {"value": algorithmic_flops(ns, nt, nd)["total"] / dt / 1e12, "unit": "TFLOP/s",
           "cores": threads, "kind": "port",
           "sample": f"the whole workload (ns={ns}, nt={nt}, nd={nd}): ingest + factorize + "
                     f"logDet + exact RGFdiag, once",
           "seconds": dt, "blas_threads": threads, "blas_threads_from": how}
    return cpu, {"logdet": ld, "diag": diag, "x": x}


def rel_errors(ld, diag, ref):
    return {"logdet_rel": abs(ld - ref["logdet"]) / abs(ref["logdet"]),
            "diag_max_rel": float(np.max(np.abs(diag - ref["diag"]) / np.abs(ref["diag"])))}


def run_reference(args, w):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    vals = []
    for i in range(args.warmup + args.steps):
        tf, cores, sample, dt = cpu_port_sample(w, target_s=args.ref_seconds)
        if i >= args.warmup:
            vals.append((tf, dt))
    tf = statistics.median(v[0] for v in vals)
    ms = statistics.median(v[1] for v in vals) * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": tf, "unit": "TFLOP/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": args.workload, **cfg_of(w)},
            "cpu_baseline": {"value": tf, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                             "sample": sample, "blas_threads": blas_threads()[0],
                             "blas_threads_from": blas_threads()[1]},
            "e2e": {"value": tf, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """The batched workload: 256 uneven instances (ns in
    {42,128,256,512}, nt in [3,60], nd in {0,2,6}, seed 4), factorize + logDet
    + RGFdiag of all of them as one captured CUDA graph with a concurrent
    branch per instance, against the same work launched instance by instance."""
    import torch
    import rgf_gb300
    from rgf_gb300 import gen
    from rgf_gb300.flops import algorithmic_flops
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    t = time.time()
    inst = gen.generate_batch(args.batch_count, seed=4)
    log(f"[bench] generated {len(inst)} instances in {time.time() - t:.1f}s")
    flops = sum(algorithmic_flops(ns, nt, nd)["total"] for (_, _, _, ns, nt, nd) in inst)
    b = rgf_gb300.RGFBatch(inst, precision=args.precision, slices=args.slices,
                           device=torch.cuda.current_device(),
                           fp64_diag=not args.no_fp64_diag)
    stream = torch.cuda.ExternalStream(b.stream())

    def timed():
        for _ in range(args.warmup):
            b.run(concurrent=True, want_diag=False)
        k0 = b.kernels()
        clocks = Clocks(torch.cuda.current_device())
        torch.cuda.synchronize()
        clocks.start()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            b.run(concurrent=True, want_diag=False)
        e1.record(stream); e1.synchronize()
        return e0.elapsed_time(e1) / args.steps, (b.kernels() - k0) // args.steps, clocks.stop()

    ms, launches, clk = timed()
    tune = None
    if args.autotune:
        # the same batch again after the autotuner picked each (ns, nd)
        # class's knobs (leaf width, look-ahead, routing bias)
        ms_default = ms
        t0 = time.perf_counter()
        classes = b.autotune()
        tune_s = time.perf_counter() - t0
        ms, launches, clk = timed()
        choices = {}
        for (s_, _, d_), t in zip(b.sizes, b.tunings()):
            choices[f"ns{s_}_nd{d_}"] = [t["leaf_nb"], t["lookahead"], t["split_bias"],
                                         t["splitk_max"], t["fp64_tile"]]
        tune = {"classes": classes, "tune_s": tune_s, "default_ms_per_step": ms_default,
                "default_value": flops / (ms_default * 1e-3) / 1e12,
                "choices_leaf_nb_lookahead_bias_splitk_fp64tile": choices}
    # per-instance launches (each instance's own stage graphs, one after another)
    ms_serial = None
    if not args.no_per_instance:
        b.run(concurrent=False, want_diag=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.run(concurrent=False, want_diag=False)
        ms_serial = (time.perf_counter() - t0) * 1e3
    # end to end: host CSC -> device for every instance, diag back to host
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b2 = rgf_gb300.RGFBatch(inst, precision=args.precision, slices=args.slices,
                            device=torch.cuda.current_device(), fp64_diag=not args.no_fp64_diag)
    if args.autotune:
        b2.autotune()  # the choices cached by the first batch
    _, diags = b2.run(concurrent=True, want_diag=True)
    b2.close()
    ms_e2e = (time.perf_counter() - t0) * 1e3
    h2d = sum(x[0].nbytes + x[1].nbytes + x[2].nbytes for x in inst)
    d2h = sum(d.nbytes for d in diags) + 8 * len(inst)
    b.close()
    if rank == 0:
        line = {"metric": METRIC + f" over {len(inst)} uneven instances", "value": flops / (ms * 1e-3) / 1e12,
                "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None,
                "dtype": "f64" if args.precision == "fp64" else "bf16-slices/f64",
                "data": "synthetic",
                "config": {"workload": "batch", "count": len(inst), "seed": 4,
                           "ns_choices": [42, 128, 256, 512], "nt_range": [3, 60],
                           "nd_choices": [0, 2, 6], "precision": args.precision,
                           "execution": "one captured CUDA graph, one concurrent branch per instance",
                           "autotune": bool(args.autotune),
                           "l2": "inputs larger than L2 (%.1f GB CSC)" % (h2d / 1e9)},
                "per_instance_launches": None if ms_serial is None else {
                    "value": flops / (ms_serial * 1e-3) / 1e12, "ms_per_step": ms_serial},
                "speedup_vs_per_instance": None if ms_serial is None else ms_serial / ms,
                "e2e": {"value": flops / (ms_e2e * 1e-3) / 1e12, "unit": "TFLOP/s",
                        "ms_per_step": ms_e2e, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": launches, "clocks": clk}
        if tune is not None:
            line["autotune"] = tune
        print(json.dumps(line), flush=True)


def run_serve(args):
    """The serving workload: Poisson arrivals at --rate req/s,
    70% new factorize+logDet, 20% solve (1-16 RHS) on a resident factor, 10%
    RGFdiag on a resident factor; ns from {42,128,256,512,1024,1500}, nt in
    [3,100], nd in [0,6].  Requests are admitted by HBM footprint into a
    continuous-batching loop.  Reports p50/p99 latency and throughput for the
    chosen precision and for plain FP64, and the logDet error of split against
    FP64 on the same matrices."""
    import threading
    import torch
    import rgf_gb300
    from rgf_gb300 import gen
    from rgf_gb300.flops import algorithmic_flops
    torch.cuda.set_device(0)
    rng = np.random.default_rng(5)
    pool_shapes = [(int(rng.choice([42, 128, 256, 512, 1024, 1500])), int(rng.integers(3, 101)),
                    int(rng.integers(0, 7))) for _ in range(args.serve_pool)]
    t0 = time.time()
    pool = [gen.generate_bta(ns, nt, nd, 5000 + i) for i, (ns, nt, nd) in enumerate(pool_shapes)]
    log(f"[bench] generated {len(pool)} serving matrices in {time.time() - t0:.1f}s")
    nreq = args.serve_requests
    kinds0 = rng.choice([0, 1, 2], size=nreq, p=[0.7, 0.2, 0.1])
    kinds0[0] = 0
    rng_arrivals = np.random.default_rng(8)
    arrivals = np.cumsum(rng_arrivals.exponential(1.0 / args.rate, size=nreq))
    mats0 = rng.integers(0, len(pool), size=nreq)
    nrhs = rng.integers(1, 17, size=nreq)

    def one_run(precision):
        kinds = kinds0.copy()
        mats = mats0.copy()
        rng = np.random.default_rng(6)
        srv = rgf_gb300.RGFServer(hbm_budget_bytes=int(args.serve_budget_gb * (1 << 30)),
                                  slots=args.serve_slots, precision=precision)
        resident = []          # (factor_id, pool index) of completed factorizations
        # warm start: a few factors already resident when the stream begins, so
        # that solve / RGFdiag requests have targets from the first arrival
        warm = [(srv.submit_factor(*pool[i], *pool_shapes[i]), i)
                for i in range(min(args.serve_warm, len(pool)))]
        for t, i in warm:
            r = srv.wait(t)
            if r["status"] == 0:
                resident.append((r["factor_id"], i))
        lock = threading.Lock()
        results = [None] * nreq
        tickets = []

        def waiter():
            for (i, t) in iter(tickets_q.get, None):
                r = srv.wait(t)
                results[i] = r
                if r["kind"] == 0 and r["status"] == 0:
                    with lock:
                        resident.append((r["factor_id"], int(mats[i])))

        import queue as _q
        tickets_q = _q.Queue()
        th = [threading.Thread(target=waiter) for _ in range(4)]
        for t in th:
            t.start()
        start = time.perf_counter()
        flops = 0.0
        for i in range(nreq):
            delay = arrivals[i] - (time.perf_counter() - start)
            if delay > 0:
                time.sleep(delay)
            kind = int(kinds[i])
            with lock:
                have = list(resident[-16:])
            if kind != 0 and not have:
                kind = 0
            if kind == 0:
                ns, nt, nd = pool_shapes[mats[i]]
                t = srv.submit_factor(*pool[mats[i]], ns, nt, nd)
                flops += algorithmic_flops(ns, nt, nd)["factor"]
            else:
                fid, pi = have[int(rng.integers(0, len(have)))]
                mats[i] = pi
                ns, nt, nd = pool_shapes[pi]
                n = ns * nt + nd
                if kind == 1:
                    t = srv.submit_solve(fid, rng.standard_normal((n, int(nrhs[i]))))
                else:
                    t = srv.submit_diag(fid, n)
                    flops += algorithmic_flops(ns, nt, nd)["selinv"]
            kinds[i] = kind
            tickets_q.put((i, t))
        for _ in th:
            tickets_q.put(None)
        for t in th:
            t.join()
        makespan = time.perf_counter() - start
        stats = srv.stats()
        srv.close()
        lat = np.array([r["latency_ms"] for r in results if r and r["status"] == 0])
        ok = sum(1 for r in results if r and r["status"] == 0)
        by = {}
        for k, name in ((0, "factor"), (1, "solve"), (2, "diag")):
            l = np.array([r["latency_ms"] for i, r in enumerate(results)
                          if r and r["status"] == 0 and kinds[i] == k])
            nfail = sum(1 for i, r in enumerate(results) if r and r["status"] != 0 and kinds[i] == k)
            if l.size or nfail:
                by[name] = {"count": int(l.size), "failed": nfail}
            if l.size:
                by[name].update(p50_ms=float(np.percentile(l, 50)),
                                p99_ms=float(np.percentile(l, 99)))
        logdets = {int(mats[i]): r["logdet"] for i, r in enumerate(results)
                   if r and r["status"] == 0 and kinds[i] == 0}
        return {"requests": nreq, "completed_ok": ok, "makespan_s": makespan,
                "throughput_req_s": ok / makespan,
                "fp64_equiv_tflops": flops / makespan / 1e12,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "by_kind": by, "evicted": stats["evicted"], "failed": stats["failed"],
                "arena_fallbacks": stats["arena_fallbacks"]}, logdets

    # latency below saturation: the same mix at a few lower offered rates
    # (fewer requests each), chosen precision only
    sweep = []
    if args.serve_sweep:
        saved = (args.rate, nreq)
        for rate in [float(x) for x in args.serve_sweep.split(",")]:
            nreq = args.serve_sweep_requests
            arrivals = np.cumsum(np.random.default_rng(7).exponential(1.0 / rate, size=nreq))
            r, _ = one_run(args.precision)
            sweep.append({"rate_req_s": rate, "requests": nreq, "throughput_req_s": r["throughput_req_s"],
                          "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"], "by_kind": r["by_kind"],
                          "completed_ok": r["completed_ok"], "arena_fallbacks": r["arena_fallbacks"]})
        args.rate, nreq = saved
        arrivals = np.cumsum(rng_arrivals.exponential(1.0 / args.rate, size=nreq))
    split, ld_s = one_run(args.precision)
    plain, ld_p = one_run("fp64")
    common = [k for k in ld_s if k in ld_p]
    err = max((abs(ld_s[k] - ld_p[k]) / abs(ld_p[k]) for k in common), default=None)
    line = {"metric": "serve p50/p99 latency and throughput (Poisson %.0f req/s)" % args.rate,
            "value": split["p99_ms"], "unit": "ms (p99)", "n_gpus": 1, "steps": 1, "warmup": 0,
            "ms_per_step": split["makespan_s"] * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16-slices/f64" if args.precision == "split" else "f64",
            "data": "synthetic",
            "config": {"workload": "serve", "rate_req_s": args.rate, "requests": nreq,
                       "mix": {"factor+logdet": 0.7, "solve (1-16 RHS)": 0.2, "rgfdiag": 0.1},
                       "ns_choices": [42, 128, 256, 512, 1024, 1500], "nt_range": [3, 100],
                       "nd_range": [0, 6], "matrix_pool": len(pool), "slots": args.serve_slots,
                       "hbm_budget_gb": args.serve_budget_gb},
            args.precision: split, "fp64": plain,
            "below_saturation": sweep,
            "logdet_rel_err_split_vs_fp64": err}
    print(json.dumps(line), flush=True)


def run_gemm(args):
    """One shape of the device GEMM entry point (rgf_dgemm_device):
    C := -A op(A|B) + C on device buffers, --gemm-reps calls after --warmup,
    timed with CUDA events on the stream the library launches on.  --syrk
    makes the product A A^T (the Schur-update shape of the factorization).
    This is the command the GEMM kernel profiles are taken with; every call
    also creates and frees the split engine, as the entry point does."""
    import torch
    import rgf_gb300
    m, k = args.m, args.k
    n = m if args.syrk else args.n
    dev = torch.device("cuda", 0)
    g = torch.Generator(device="cpu").manual_seed(1)
    A = torch.randn(k, m, dtype=torch.float64, generator=g).to(dev)      # column-major m x k
    B = A if args.syrk else torch.randn(k, n, dtype=torch.float64, generator=g).to(dev)
    C = torch.randn(n, m, dtype=torch.float64, generator=g).to(dev)
    stream = torch.cuda.current_stream(dev)

    def call():
        rgf_gb300.dgemm_device(args.precision, "N", "T", m, n, k, -1.0, A.data_ptr(), m,
                               B.data_ptr(), n, 1.0, C.data_ptr(), m,
                               stream=stream.cuda_stream, slices=args.slices)

    for _ in range(args.warmup):
        call()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.gemm_reps):
        call()
    e1.record(stream)
    e1.synchronize()
    us = e0.elapsed_time(e1) * 1e3 / args.gemm_reps
    flops = 2.0 * m * n * k
    print(json.dumps({"workload": "gemm", "m": m, "n": n, "k": k, "precision": args.precision,
                      "slices": args.slices or None, "syrk": args.syrk, "us_per_call": us,
                      "fp64_equiv_tflops": flops / (us * 1e-6) / 1e12,
                      "finite": bool(torch.isfinite(C).all().item())}), flush=True)


def cfg_of(w):
    return {"ns": w["ns"], "nt": w["nt"], "nd": w["nd"], "seed": w["seed"],
            "spde_grid": w["spde"], "parallelism": "replicas"}


def run_rgf(args, w):
    import torch
    import rgf_gb300
    from rgf_gb300.flops import algorithmic_flops

    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.cuda.current_device()
    ia, ja, a = make_inputs(w)
    ns, nt, nd = w["ns"], w["nt"], w["nd"]
    n = ns * nt + nd
    flops = algorithmic_flops(ns, nt, nd)["total"]
    # pinned host copies for the end-to-end leg
    ia_p = torch.from_numpy(ia.view(np.int64)).pin_memory().numpy().view(np.uint64)
    ja_p = torch.from_numpy(ja.view(np.int64)).pin_memory().numpy().view(np.uint64)
    a_p = torch.from_numpy(a).pin_memory().numpy()
    diag_host = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    del ia, ja, a

    s = rgf_gb300.RGF(ia_p, ja_p, a_p, ns, nt, nd, precision=args.precision,
                      slices=args.slices, device=dev, fp64_diag=not args.no_fp64_diag)
    stream = torch.cuda.ExternalStream(s.stream())

    def step():
        s.factorize()
        s.logDet()
        s.diag_device_ptr()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    k0 = s.info()["kernels_launched"]
    clocks = Clocks(dev)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms_total = e0.elapsed_time(e1)
    launches = s.info()["kernels_launched"] - k0
    logdet = s.logDet()
    # per-stage times of one more step (graph replays, events on the handle's
    # stream): factorize + logDet, then the selected inversion (with the
    # diagonal-block inverses it starts with)
    q = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    q[0].record(stream)
    s.factorize(); s.logDet()
    q[1].record(stream)
    s.diag_device_ptr()
    q[2].record(stream)
    q[2].synchronize()
    stages = {"factorize_logdet_ms": q[0].elapsed_time(q[1]),
              "selinv_ms": q[1].elapsed_time(q[2])}
    # per-class kernel times: one more (untimed) step with CUDA events around
    # every GEMM launch, each product run alone (serialised, warm)
    s.kernel_timer(2 if os.environ.get("RGF_GB300_TIMER_DETAIL") else 1)
    s.kernel_timer_read(reset=True)
    step()
    torch.cuda.synchronize()
    timer = s.kernel_timer_read(reset=True)
    s.kernel_timer(False)
    ms_total = max_over_ranks(ms_total, dist, "cuda")
    ms_step = ms_total / args.steps
    value = replica_throughput(flops, ws, ms_step)

    # end-to-end through the public API: host CSC -> device, diag -> host, a
    # new handle per step (as a caller that builds a solver per evaluation).
    # The CSC upload is asynchronous (the Python default): it overlaps the
    # first factorization.  The device-memory cache (rgf_set_device_cache)
    # hands a destroyed handle's buffers to the next; the first iteration
    # (untimed, reported as cold_ms) fills it.
    e2e_ms = []
    e2e_parts = None
    e2e_cold = None
    cache_bytes = 0 if args.no_device_cache else 64 << 30
    rgf_gb300.set_device_cache(cache_bytes)
    for i in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h = rgf_gb300.RGF(ia_p, ja_p, a_p, ns, nt, nd, precision=args.precision,
                          slices=args.slices, device=dev, fp64_diag=not args.no_fp64_diag)
        t1 = time.perf_counter()
        h.factorize()
        t2 = time.perf_counter()
        h.logDet()
        h.RGFdiag(diag_host)
        t3 = time.perf_counter()
        h.close()
        t4 = time.perf_counter()
        dt = (t4 - t0) * 1e3
        if i == 0:
            e2e_cold = dt
        else:
            e2e_ms.append(dt)
            e2e_parts = {"create_ms": (t1 - t0) * 1e3,
                         "factorize_with_h2d_ms": (t2 - t1) * 1e3,
                         "logdet_rgfdiag_d2h_ms": (t3 - t2) * 1e3, "destroy_ms": (t4 - t3) * 1e3}
    rgf_gb300.set_device_cache(0)
    e2e_med = statistics.median(e2e_ms) if e2e_ms else float("nan")
    if dist and e2e_ms:
        e2e_med = max_over_ranks(max(e2e_ms), dist, "cuda")
    h2d = ia_p.nbytes + ja_p.nbytes + a_p.nbytes
    d2h = diag_host.nbytes + 8

    # 8-RHS solve on the resident factor (refined in FP64 in split precision):
    # time per call (host arrays in and out) and the worst normalized residual
    d_main = s.RGFdiag()  # the timed steps' diagonal, to host (oracle comparison)
    solve_info = None
    bsol = xsol = None
    if not args.no_solve:
        from rgf_gb300 import gen as _gen
        bsol = _gen.random_rhs(n, 8, w["seed"])
        xsol = np.empty_like(bsol)
        s.solve(xsol, bsol, 8)
        t0 = time.perf_counter()
        s.solve(xsol, bsol, 8)
        sms = (time.perf_counter() - t0) * 1e3
        res = max(s.residualNormNormalized(np.ascontiguousarray(xsol[:, q]),
                                           np.ascontiguousarray(bsol[:, q])) for q in range(8))
        solve_info = {"nrhs": 8, "ms": sms, "max_residual_normalized": res,
                      "refined": args.precision == "split"}

    # roofline of the dominant kernel class (timed live over the timed region)
    peak64 = rgf_gb300.measure_fp64_peak()
    peaks, src = load_peaks()
    fp, sp = timer["fp64"], timer["split"]
    kernels = {
        "gemm_fp64_kernel": {"ms_per_step": fp["ms"],
                             "launches_per_step": fp["launches"],
                             "fp64_equiv_tflops": fp["flops"] / max(fp["ms"], 1e-9) / 1e9},
        "split_gemm (slice + tcgen05)": {
            "ms_per_step": sp["ms"], "launches_per_step": sp["launches"],
            "fp64_equiv_tflops": sp["flops"] / max(sp["ms"], 1e-9) / 1e9,
            "tensor_tflops": sp["tensor_flops"] / max(sp["ms"], 1e-9) / 1e9},
    }
    if sp["ms"] > fp["ms"]:
        ach = sp["tensor_flops"] / (sp["ms"] * 1e-3) / 1e12
        roofline = {"bound": "tensor", "kernel": "split_gemm_kernel (tcgen05 bf16 slices)",
                    "achieved": ach, "peak": peaks["bf16_sustained"], "unit": "TFLOP/s",
                    "frac": ach / peaks["bf16_sustained"],
                    # dram read + write of one 2000x2000x2000 launch (ncu --set full,
                    # python bench.py --workload gemm --m 2000 --k 2000 --syrk); operands
                    # are read about once, the slices stay in L2
                    "traffic": 81.6e6, "traffic_unit": "bytes per 2000^3 launch",
                    "peak_source": f"bf16 sustained, {src}",
                    "achieved_counts": "executed bf16 slice-product flops (pairs x 2MNK) / "
                                       "kernel time incl. slicing",
                    "kernel_share_of_step": sp["ms"] / ms_step}
    else:
        ach = fp["flops"] / (fp["ms"] * 1e-3) / 1e12 if fp["ms"] else None
        roofline = {"bound": "tensor", "kernel": "gemm_fp64_kernel (DMMA m8n8k4)",
                    "achieved": ach, "peak": peak64, "unit": "TFLOP/s",
                    "frac": ach / peak64 if ach else None, "traffic": None,
                    "peak_source": "FP64 DMMA m8n8k4 loop measured in this run (the peaks file "
                                   "has no FP64 figure)",
                    "kernel_share_of_step": fp["ms"] / ms_step}
    roofline["kernels"] = kernels

    # the same matrix in plain FP64, and in split precision with native-FP64
    # diagonal blocks, for comparison (speed-up and accuracy); each handle
    # runs two untimed steps (direct launch, graph capture), then one timed
    mf_bytes = s.info()["mf_size"] * 8
    s.close()

    def variant(precision, fp64_diag=1):
        f = rgf_gb300.RGF(ia_p, ja_p, a_p, ns, nt, nd, precision=precision, slices=args.slices,
                          device=dev, fp64_diag=fp64_diag)
        for _ in range(2):
            f.factorize(); f.logDet(); f.diag_device_ptr()
        fs = torch.cuda.ExternalStream(f.stream())
        torch.cuda.synchronize()
        p0 = torch.cuda.Event(enable_timing=True); p1 = torch.cuda.Event(enable_timing=True)
        p0.record(fs)
        f.factorize(); ld = f.logDet(); f.diag_device_ptr()
        p1.record(fs); p1.synchronize()
        pms = p0.elapsed_time(p1)
        d = f.RGFdiag()
        f.close()
        return pms, ld, d

    plain = native_diag = None
    ld64 = d64 = ldn = dn = None
    if args.precision == "split" and not args.no_fp64_ref:
        pms, ld64, d64 = variant("fp64")
        plain = {"value": flops / (pms * 1e-3) / 1e12, "ms_per_step": pms, "steps": 1, "warmup": 2,
                 "speedup_of_split": pms / ms_step,
                 "split_vs_fp64": {"logdet_rel": abs(logdet - ld64) / abs(ld64),
                                   "diag_max_rel": float(np.max(np.abs(d_main - d64) / np.abs(d64)))}}
        if not args.no_fp64_diag:
            nms, ldn, dn = variant("split", fp64_diag="native")
            native_diag = {"value": flops / (nms * 1e-3) / 1e12, "ms_per_step": nms, "steps": 1,
                           "warmup": 2, "diag_products": "native FP64 (DMMA)",
                           "vs_fp64": {"logdet_rel": abs(ldn - ld64) / abs(ld64),
                                       "diag_max_rel": float(np.max(np.abs(dn - d64) / np.abs(d64)))}}

    # the oracle on the whole workload: CPU baseline and parity of every GPU result
    cpu = None
    oracle_err = None
    if rank == 0 and not args.no_cpu:
        if args.cpu_prefix:
            tf, cores, sample, dt = cpu_port_sample(w, target_s=args.ref_seconds)
            cpu = {"value": tf, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                   "sample": sample, "seconds": dt}
        else:
            cpu, ref = cpu_oracle_full(w, ia_p, ja_p, a_p, bsol)
            oracle_err = {args.precision: rel_errors(logdet, d_main, ref),
                          "gates": {"fp64": {"logdet_rel": 1e-12, "diag_max_rel": 1e-10},
                                    "split": {"logdet_rel": 1e-9, "diag_max_rel": 1e-8}}}
            if plain is not None:
                oracle_err["fp64"] = rel_errors(ld64, d64, ref)
            if native_diag is not None:
                oracle_err["split_native_fp64_diag"] = rel_errors(ldn, dn, ref)
            if bsol is not None and ref["x"] is not None:
                oracle_err["solve_8rhs"] = {
                    "x_max_rel": float(np.max(np.abs(xsol - ref["x"])) / np.max(np.abs(ref["x"]))),
                    "max_residual_normalized": solve_info["max_residual_normalized"]}
    if args.precision == "fp64":
        diag_label = "FP64 (DMMA)"
    elif args.no_fp64_diag:
        diag_label = "split-%d (bulk slice count)" % (args.slices or 5)
    else:
        diag_label = "split-7 (55-bit operands: FP64-accurate emulation on the tensor cores)"
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.precision == "fp64" else "bf16-slices/f64",
                "data": "synthetic",
                "config": {"workload": args.workload, **cfg_of(w), "precision": args.precision,
                           "slices": args.slices or 5, "slice_bits": 8 * (args.slices or 5) - 1,
                           "diag_products": diag_label,
                           "l2": "inputs larger than L2 (CSC %.1f GB, factor %.1f GB)" % (
                               h2d / 1e9, mf_bytes / 1e9)},
                "e2e": ({"value": flops * ws / (e2e_med * 1e-3) / 1e12, "unit": "TFLOP/s",
                         "ms_per_step": e2e_med, "h2d_bytes_per_step": h2d,
                         "d2h_bytes_per_step": d2h, "parts": e2e_parts,
                         "upload": "asynchronous: the CSC copy overlaps the first factorization",
                         "device_cache_bytes": cache_bytes,
                         "cold_ms": e2e_cold} if e2e_ms else None),
                "roofline": roofline, "cpu_baseline": cpu, "gpu_launches": launches,
                "stages": stages, "plain_fp64": plain, "split_native_fp64_diag": native_diag,
                "solve": solve_info, "oracle_err": oracle_err,
                "clocks": clk, "logdet": logdet,
                "timed_region": "each stage replayed as one CUDA graph; kernel classes timed "
                                "on one extra step with events around every GEMM, each run "
                                "alone (serialised)"}
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["rgf", "reference"], default="rgf")
    p.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch", "serve", "gemm"],
                   default="ns2000_nt100_nd6")
    p.add_argument("--rate", type=float, default=2000.0)
    p.add_argument("--serve-requests", type=int, default=400)
    p.add_argument("--serve-pool", type=int, default=24)
    p.add_argument("--serve-slots", type=int, default=8)
    p.add_argument("--no-solve", action="store_true", help="skip the 8-RHS solve measurement")
    p.add_argument("--serve-warm", type=int, default=8,
                   help="factors made resident before the request stream starts")
    p.add_argument("--serve-budget-gb", type=float, default=160.0)
    p.add_argument("--serve-sweep", default="5,10,15",
                   help="serve workload: offered rates (req/s) below saturation to report "
                        "p50/p99 at, comma-separated ('' to skip)")
    p.add_argument("--serve-sweep-requests", type=int, default=120)
    p.add_argument("--batch-count", type=int, default=256)
    p.add_argument("--no-per-instance", action="store_true",
                   help="batch workload: skip the instance-after-instance comparison run")
    p.add_argument("--autotune", action="store_true",
                   help="batch workload: time the default knobs, autotune every (ns, nd) "
                        "class, then time again (reported as the line's value)")
    p.add_argument("--precision", choices=["fp64", "split"], default="split")
    p.add_argument("--no-fp64-ref", action="store_true",
                   help="skip the plain-FP64 comparison run (1 warm-up + 1 step)")
    p.add_argument("--slices", type=int, default=0)
    p.add_argument("--no-fp64-diag", action="store_true",
                   help="split precision: also run the diagonal blocks' inner updates as split products")
    p.add_argument("--e2e-steps", type=int, default=1)
    p.add_argument("--no-device-cache", action="store_true",
                   help="e2e leg without the device-memory cache (every handle allocates)")
    p.add_argument("--ref-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-prefix", action="store_true",
                   help="time the oracle on a prefix of the block columns (about "
                        "--ref-seconds) instead of the whole workload; no oracle errors")
    # --workload gemm: one product shape through rgf_dgemm_device
    p.add_argument("--m", type=int, default=2000)
    p.add_argument("--n", type=int, default=2000)
    p.add_argument("--k", type=int, default=2000)
    p.add_argument("--syrk", action="store_true", help="gemm workload: B = A (product A A^T)")
    p.add_argument("--gemm-reps", type=int, default=10)
    args = p.parse_args()
    if args.workload == "gemm":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the gemm workload times one "
                              "product of this library's kernels; the reference has none"}))
        else:
            run_gemm(args)
        return
    if args.workload == "serve":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no request "
                              "loop (one synchronous instance per RGF object)"}))
        else:
            run_serve(args)
        return
    if args.workload == "batch":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the batched workload has no "
                              "reference counterpart (one instance per RGF object)"}))
        else:
            run_batch(args)
        return
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, w)
    else:
        run_rgf(args, w)


if __name__ == "__main__":
    main()
