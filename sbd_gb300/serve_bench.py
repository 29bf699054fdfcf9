"""Serving and batching benchmark: request mixes through the request loop.

    python -m sbd_gb300.serve_bench --config 4 --requests 512 --rates 20,200,inf
    python -m sbd_gb300.serve_bench --config 2 --requests 4096 --rates inf

Workloads (synthetic, from sbd_gb300.generators):
  config 4  serving mix: norb in {24,32,40,48}, n = round(norb/3), alpha and
            beta string counts log-uniform in [200, 4000], 1-3 roots,
            tol 1e-7, Poisson arrivals at each rate (inf = all at once);
  config 2  batch: norb 12, 4+4 electrons, counts log-uniform in [50, 495],
            4 roots, tol 1e-8, all submitted at once.

Measured, on one GPU:
  - the plain path: FP64, one solve at a time through TPBProblem (upload,
    tables, diagonal, Davidson, free), per-solve wall time;
  - the request loop in FP64 and in the mixed form at each arrival rate:
    solves/s (requests / time from the first submission to the last result),
    p50/p99 of the per-request latency (submission to result), and max |dE|
    of every energy against the FP64 energies of the same request.

At arrival rates below the loop's capacity solves/s is the arrival rate; the
rate "inf" gives the capacity.  Requests are generated before the timing, in a
spawn process pool.  Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import queue
import threading
import time

import numpy as np


def _gen(args):
    cfg, i = args
    from . import generators as G
    if cfg == 4:
        p, k = G.config4_request(i)
    else:
        p, k = G.config2_problem(i), 4
    return (p.norb, p.astr, p.bstr, p.ints.h1, p.ints.eri, p.ints.ecore, k)


def generate(cfg: int, n: int, jobs: int):
    with mp.get_context("spawn").Pool(jobs) as pool:
        return pool.map(_gen, [(cfg, i) for i in range(n)], chunksize=4)


def pct(x, q):
    return float(np.percentile(np.asarray(x), q)) if len(x) else None


def solver_opts(cfg: int) -> dict:
    if cfg == 4:
        return {"eps": 1e-7, "max_nb": 20, "init": 1}
    return {"eps": 1e-8, "max_nb": 24, "init": 1}


def run_serial(reqs, cfg: int):
    """The plain path: FP64, one solve at a time, a fresh problem per request."""
    import torch

    from .engine import FP64, Engine, TPBProblem
    eng = Engine(0)
    o = solver_opts(cfg)
    lat, E = [], []
    for (norb, a, b, h1, eri, ecore, k) in reqs:
        t = time.perf_counter()
        p = TPBProblem(eng, norb, a, b, h1, eri, ecore)
        r = p.davidson(nroots=k, precision=FP64, want_vectors=False, **o)
        p.close()
        lat.append(time.perf_counter() - t)
        E.append(r.energies.copy())
    torch.cuda.synchronize()
    eng.close()
    return lat, E


def run_serving(reqs, cfg: int, precision: int, rate: float, workers: int, seed: int, refine_every: int = 0):
    from .serving import Server
    o = dict(solver_opts(cfg), refine_every=refine_every)
    n = len(reqs)
    rng = np.random.default_rng(seed)
    arrivals = np.zeros(n) if math.isinf(rate) else np.cumsum(rng.exponential(1.0 / rate, n))
    results = [None] * n
    q: queue.Queue = queue.Queue()
    with Server(0, workers) as srv:
        def collect():
            for _ in range(n):
                i, t = q.get()
                results[i] = srv.wait(t)

        th = threading.Thread(target=collect)
        th.start()
        t0 = time.perf_counter()
        for i, (norb, a, b, h1, eri, ecore, k) in enumerate(reqs):
            delay = t0 + arrivals[i] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            q.put((i, srv.submit(norb, a, b, h1, eri, ecore, nroots=k, precision=precision, **o)))
        th.join()
        wall = time.perf_counter() - t0
        st = srv.stats()
    return results, wall, st


def run_batch(reqs, cfg: int, chunk: int, precision: int = 0):
    """The batched solver: upload and tables per problem, then one solver call per
    chunk of problems (all problems of the chunk advanced in lock step, one
    graph launch per Davidson iteration).
    Returns (energies, wall seconds of the whole batch, solver seconds, reports)."""
    import torch

    from .engine import Engine, TPBProblem, batch_davidson
    o = solver_opts(cfg)
    eng = Engine(0)
    t0 = time.perf_counter()
    E, reps, t_launch = [], [], 0.0
    for c0 in range(0, len(reqs), chunk):
        part = reqs[c0:c0 + chunk]
        tps = [TPBProblem(eng, norb, a, b, h1, eri, ecore) for (norb, a, b, h1, eri, ecore, k) in part]
        for t in tps:
            t.build_tables()
            t.diag_terms()
        k = part[0][6]
        tl = time.perf_counter()
        res = batch_davidson(eng, tps, nroots=k, max_nb=o["max_nb"], eps=o["eps"], precision=precision)
        t_launch += time.perf_counter() - tl
        E += [r.energies.copy() for r in res]
        reps += [r.report for r in res]
        for t in tps:
            t.close()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    eng.close()
    return E, wall, t_launch, reps


def summarize(results, wall, st, ref_E, precision, rate):
    lat = [r["total_seconds"] for r in results]
    failed = [r for r in results if r["status"] != 0]
    dE, compared, nonfinite = 0.0, 0, 0
    for r, e in zip(results, ref_E):
        if r["status"] == 0 and e is not None:
            d = np.abs(np.asarray(r["energies"], dtype=np.float64) - np.asarray(e, dtype=np.float64))
            if not np.all(np.isfinite(d)):
                nonfinite += 1  # counted, never silently dropped by max()
                continue
            dE = max(dE, float(np.max(d)))
            compared += 1
    return {"precision": "mixed" if precision else "fp64", "rate": "inf" if math.isinf(rate) else rate,
            "requests": len(results), "wall_s": wall, "solves_per_s": len(results) / wall,
            "p50_s": pct(lat, 50), "p99_s": pct(lat, 99), "max_abs_dE": dE, "dE_compared": compared,
            "dE_nonfinite": nonfinite,
            "failed": len(failed), "first_error": failed[0]["message"] if failed else None,
            "not_converged": sum(1 for r in results if not r["converged"]),
            "peak_running": st["peak_running"], "peak_reserved_GB": st["peak_reserved_bytes"] / 1e9,
            "launches": st["launches"], "batched_requests": st["batched"]}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=4, choices=[2, 4])
    ap.add_argument("--requests", type=int, default=None)
    ap.add_argument("--rates", default=None, help="comma list of req/s; inf = all at once")
    ap.add_argument("--max-arrival-seconds", type=float, default=30.0,
                    help="fewer requests at low rates so that arrivals span at most this long")
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--serial", type=int, default=None, help="requests timed on the plain path (default: all)")
    ap.add_argument("--precisions", default="fp64,mixed")
    ap.add_argument("--jobs", type=int, default=min(16, os.cpu_count() or 1))
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--records", default=None, help="write per-request results (JSON lines) to this file")
    ap.add_argument("--batch", type=int, default=0,
                    help="also time the batched solver with this many problems per call (0: skip)")
    ap.add_argument("--batch-precisions", default="fp64,mixed")
    ap.add_argument("--refine-every", type=int, default=0,
                    help="mixed form of the request loop: FP64 refinement every k steps, 0 = two-phase")
    a = ap.parse_args(argv)
    n = a.requests or (512 if a.config == 4 else 4096)
    rates = [float(x) for x in (a.rates or ("20,200,inf" if a.config == 4 else "inf")).split(",")]
    t = time.time()
    reqs = generate(a.config, n, a.jobs)  # before any CUDA work in this process
    out = {"config": a.config, "requests": n, "workers": a.workers, "generate_s": time.time() - t,
           "ndet_median": float(np.median([x[1].size * x[2].size for x in reqs])),
           "ndet_max": int(max(x[1].size * x[2].size for x in reqs))}
    from . import build
    build.build()
    # warm-up: module load, pool growth
    run_serving(reqs[:8], a.config, 0, math.inf, a.workers, a.seed)
    ns = n if a.serial is None else min(a.serial, n)
    lat, E_serial = run_serial(reqs[:ns], a.config)
    out["serial_fp64"] = {"requests": ns, "solves_per_s": ns / sum(lat), "p50_s": pct(lat, 50),
                          "p99_s": pct(lat, 99)}
    ref_E = list(E_serial) + [None] * (n - ns)
    runs = []
    precs = [0 if p == "fp64" else 1 for p in a.precisions.split(",") if p]
    for prec in precs:
        for rate in rates:
            m = n if math.isinf(rate) else max(16, min(n, int(rate * a.max_arrival_seconds)))
            res, wall, st = run_serving(reqs[:m], a.config, prec, rate, a.workers, a.seed, a.refine_every)
            if prec == 0 and math.isinf(rate) and m == n:
                # FP64 energies of the requests the plain path did not time
                ref_E = [ref_E[i] if ref_E[i] is not None else res[i]["energies"] for i in range(n)]
            runs.append(summarize(res, wall, st, ref_E[:m], prec, rate))
            if a.records:
                with open(a.records, "a") as f:
                    for i, r in enumerate(res):
                        e = ref_E[i]
                        f.write(json.dumps({
                            "precision": prec, "rate": "inf" if math.isinf(rate) else rate, "index": i,
                            "norb": int(reqs[i][0]), "ndet": r["ndet"], "nroots": int(reqs[i][6]),
                            "status": r["status"], "converged": r["converged"], "iterations": r["iterations"],
                            "sigma_calls": r["sigma_calls"], "resid": r["resid"], "energies": r["energies"].tolist(),
                            "dE": None if e is None else float(np.max(np.abs(r["energies"] - e))),
                            "run_s": r["run_seconds"], "total_s": r["total_seconds"]}) + "\n")
    if a.records:
        with open(a.records, "a") as f:
            for i in range(ns):
                f.write(json.dumps({"precision": "serial_fp64", "index": i, "seconds": lat[i]}) + "\n")
    out["serving"] = runs
    if a.batch > 0:
        for prec in [0 if p == "fp64" else 1 for p in a.batch_precisions.split(",") if p]:
            Eb, wall_b, t_launch, reps = run_batch(reqs, a.config, a.batch, prec)
            dE = max(float(np.max(np.abs(e - r))) for e, r in zip(Eb, ref_E) if r is not None)
            out["batched" if prec == 0 else "batched_mixed"] = {
                "requests": n, "problems_per_call": a.batch, "wall_s": wall_b,
                "solves_per_s": n / wall_b, "solver_s": t_launch,
                "solves_per_s_solver_only": n / t_launch, "max_abs_dE": dE,
                "not_converged": sum(1 for r in reps if not r["converged"]),
                "sigma_products_mean": float(np.mean([r["sigma_calls"] for r in reps])),
                "fp64_sigma_products_mean": float(np.mean([r["sigma_fp64"] for r in reps])),
                "vs_plain_fp64": (n / wall_b) / out["serial_fp64"]["solves_per_s"]}
    best = {p: max((r["solves_per_s"] for r in runs if r["precision"] == p and r["rate"] == "inf"), default=None)
            for p in ("fp64", "mixed")}
    out["capacity_solves_per_s"] = best
    if best.get("mixed"):
        out["mixed_serving_vs_plain_fp64"] = best["mixed"] / out["serial_fp64"]["solves_per_s"]
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
