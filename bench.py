"""Benchmark: Davidson solves/s on the 36M-determinant configuration, one GB300.

Workload (the configuration the metric is quoted on): norb 36, 12+12
electrons, 6000 alpha x 6000 beta strings drawn independently (N = 36,000,000
determinants, 288 MB per FP64 vector), 2 roots, subspace 24, residual
tolerance 1e-8, plain FP64.  One step = one full Davidson solve (tables and
diagonal resident, starting from the lowest diagonal entries).

  value : solves/s with the problem resident in HBM (device-timed, CUDA events
          on the solver stream, max over ranks)
  e2e   : solves/s through the C ABI with host buffers: upload strings and
          integrals, build tables and diagonal, solve, copy both Ritz vectors
          back -- every step
  roofline : the sigma operator (transpose + alpha sweep + beta sweep), whose
          per-product device time is recorded with CUDA events on its launch
          stream during the timed region; algorithmic bytes per product are
          24*N + 8*nnz_off (read C and hii, write sigma, one 8-byte C read per
          off-diagonal element).  roofline.fp64 gives the same product against
          the measured FP64 FMA rate (one FMA per nonzero), which is what
          bounds these kernels on this GPU
  cpu_baseline : the CPU oracle port of the reference's TRADMODE sigma (OpenMP,
          all host cores) timed on a bounded sample of alpha rows and scaled to
          the solve's sigma count
  serving : a bounded sample of the config-4 request mix through the request
          loop (FP64 and mixed), against the plain FP64 path one solve at a time
  batched : a bounded sample of the config-2 batch (256 problems by default)
          solved in lock step by the batched solver (FP64 and mixed), against
          the plain FP64 path one solve at a time

Multi-GPU: each rank solves its own replica (the path does not shard across
GPUs in this build): scaling "weak", value = total solves / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Davidson solves/s at |ΔE|≤1e-6 Ha vs plain FP64 GPU; p50/p99 latency; HBM GB/s"
UNIT = "solves/s"
WORKLOAD = ("config1: norb 36, 12+12 electrons, 6000x6000 strings (N=36,000,000), 2 roots, "
            "subspace 24, tol 1e-8, plain FP64")
NROOTS, MAX_NB, EPS = 2, 24, 1e-8


def peaks() -> tuple[float, str]:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                         timeout=5).stdout.strip()
                    if out:
                        self.samples.append([x.strip() for x in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)

        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self) -> dict:
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        sm = []
        mx = None
        reasons = set()
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx = float(s[1])
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                               s[3:7]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("SBDGB_BENCH_GLOO") is None else "gloo")
        return dist, dist.get_rank(), ws
    return None, 0, 1


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measure_fp64_rates(device: int) -> dict:
    """FP64 FMA-pipe and FP64 tensor-path rates of the device in TFLOP/s, from
    the benchmark's own probe library (sbd_gb300/bench_csrc/rates.cu)."""
    import ctypes as C
    from sbd_gb300 import build
    L = C.CDLL(build.RATES_LIB)
    L.sbdgb_measure_fp64_rates.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    a, b = C.c_double(), C.c_double()
    rc = L.sbdgb_measure_fp64_rates(device, C.byref(a), C.byref(b))
    if rc != 0:
        raise RuntimeError(f"FP64 rate probe failed ({rc})")
    return {"dfma_tflops": a.value, "dmma_tflops": b.value}


def measure_fp64_overlap(device: int) -> dict:
    """Times (ms) of an FP64 FMA loop, an FP64 MMA loop and one loop with the
    work of both (bench_csrc/rates.cu): near the longer of the two when the FMA
    pipe and the FP64 tensor path run concurrently, near their sum when they
    share the FP64 units."""
    import ctypes as C
    from sbd_gb300 import build
    L = C.CDLL(build.RATES_LIB)
    fp = C.POINTER(C.c_float)
    L.sbdgb_measure_fp64_overlap.argtypes = [C.c_int, fp, fp, fp]
    a, b, c = C.c_float(), C.c_float(), C.c_float()
    rc = L.sbdgb_measure_fp64_overlap(device, C.byref(a), C.byref(b), C.byref(c))
    if rc != 0:
        raise RuntimeError(f"FP64 overlap probe failed ({rc})")
    return {"fma_ms": a.value, "mma_ms": b.value, "both_ms": c.value}


def make_problem():
    from sbd_gb300.generators import config1
    return config1()


# sigma products per config-1 solve: the GPU FP64 solve's count on this
# problem (2 roots, subspace 24, tol 1e-8; bench line "sigma_products_per_solve").
# The reference arm runs without a GPU and takes it from here.
NSIGMA_CONFIG1 = 139


class ReferenceCPU:
    """The reference's CPU path for the config-1 solve, timed on the host cores.

    The oracle port restates the reference's TRADMODE mult (chemistry/tpb/
    mult.h:440-558) and the vector algebra of its Davidson step (davidson.h:
    778-923), OpenMP on `threads` threads.  One solve is modelled as nsigma
    sigma products, each followed by one Davidson step's vector algebra at the
    mean subspace position (the work per step grows linearly with it).  A
    slice is a contiguous range of alpha rows: the sigma rows of that range
    plus the step algebra on its share of the elements.  Slices [i*na/K,
    (i+1)*na/K) for i < K cover one full sigma product and one full step, so
    K timed slices measure that exactly; the diagonal (once per solve) and the
    3x3-24x24 eigensolves are not counted.
    """

    def __init__(self, prob, threads: int, nsigma: float, max_nb: int = MAX_NB):
        import oracle.oracle as orc
        from oracle.oracle import Oracle
        os.environ["OMP_NUM_THREADS"] = str(threads)
        orc.lib().orc_set_threads(threads)  # a launcher may have started OpenMP with one thread
        self.lib = orc.lib()
        self.threads, self.nsigma, self.max_nb = threads, float(nsigma), max_nb
        self.na, self.nb = prob.astr.size, prob.bstr.size
        self.o = Oracle.from_problem(prob)
        rng = np.random.default_rng(5)
        self.C = rng.uniform(-1.0, 1.0, prob.ndet)
        self.S = np.zeros(prob.ndet)
        self.hii = self.o.hii()
        self.ib = max_nb // 2  # mean subspace position of a step, (max_nb - 1) / 2 rounded up
        self._alg = None

    def slice_rows(self, i: int, k: int) -> tuple[int, int]:
        return self.na * i // k, self.na * (i + 1) // k

    def run_slice(self, r0: int, r1: int) -> dict:
        n = (r1 - r0) * self.nb
        if self._alg is None or self._alg[0].size < (self.ib + 2) * n:
            rng = np.random.default_rng(6)
            self._alg = (rng.uniform(-1, 1, (self.ib + 2) * n), rng.uniform(-1, 1, (self.ib + 1) * n),
                         np.zeros(n), np.zeros(n))
        Ca, HCa, W, R = self._alg
        t0 = time.perf_counter()
        self.o.mult(self.C, out=self.S, rows=(r0, r1), hii=self.hii)
        t1 = time.perf_counter()
        self.lib.orc_algebra_step(Ca[:(self.ib + 2) * n], HCa[:(self.ib + 1) * n], W[:n], R[:n],
                                  self.hii[r0 * self.nb:r1 * self.nb], n, self.ib)
        t2 = time.perf_counter()
        return {"sigma_s": t1 - t0, "algebra_s": t2 - t1, "total_s": t2 - t0}

    def describe(self, k: int, sigma_s: float, algebra_s: float) -> str:
        return (f"oracle port (restated reference TRADMODE mult + Davidson step algebra, OpenMP {self.threads} "
                f"threads), config 1 in {k} slices of alpha rows covering one full sigma product: "
                f"{sigma_s:.1f} s sigma + {algebra_s:.2f} s step algebra (subspace position {self.ib} of "
                f"{self.max_nb}) per step, x {self.nsigma:.0f} steps per solve (the GPU FP64 solve's sigma "
                f"count on this problem); diagonal and small eigensolves not counted")


def cpu_baseline(prob, nsigma: float, threads: int, k: int = 20) -> dict:
    """The CPU baseline beside the GPU number: one full sigma + step algebra
    of the reference's CPU path (ReferenceCPU), scaled to a solve."""
    ref = ReferenceCPU(prob, threads, nsigma)
    sig = alg = 0.0
    for i in range(k):
        t = ref.run_slice(*ref.slice_rows(i, k))
        sig += t["sigma_s"]
        alg += t["algebra_s"]
    return {"value": 1.0 / (nsigma * (sig + alg)), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": ref.describe(k, sig, alg), "sigma_seconds": sig, "algebra_seconds": alg}


def run_reference(args):
    """--impl reference: the reference's CPU algorithm (oracle port) on the host
    cores.  Each step is one slice of the config-1 solve (ReferenceCPU): the K
    timed steps together are one full sigma product and one Davidson step's
    vector algebra, i.e. 1/nsigma of a solve, so ms_per_step is the measured
    time of a step and value = 1 / (nsigma x the timed region)."""
    dist, rank, ws = dist_init()
    if rank != 0:
        return 0
    import oracle.oracle as orc
    orc.build()
    threads = os.cpu_count() or 1
    prob = make_problem()
    ref = ReferenceCPU(prob, threads, NSIGMA_CONFIG1)
    K = max(1, args.steps)
    for i in range(args.warmup):
        ref.run_slice(*ref.slice_rows(i % K, K))
    sig = alg = 0.0
    t0 = time.perf_counter()
    for i in range(K):
        t = ref.run_slice(*ref.slice_rows(i, K))
        sig += t["sigma_s"]
        alg += t["algebra_s"]
    wall = time.perf_counter() - t0
    value = 1.0 / (NSIGMA_CONFIG1 * wall)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * wall / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_block(prob, ws),
            "step": (f"one of {K} slices of alpha rows of the config-1 solve's sigma product plus its share of a "
                     f"Davidson step's vector algebra; the timed region is 1/{NSIGMA_CONFIG1} of a solve "
                     "(value extrapolates it to solves/s)"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": ref.describe(K, sig, alg)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line))
    return 0


def config_block(prob, ws: int = 1) -> dict:
    """The line's config: the same keys and values in both arms."""
    return {"workload": WORKLOAD, "parallelism": f"replicas x{ws}",
            "l2": "inputs larger than L2 (288 MB per vector, 13.8 GB subspace)", "ndet": int(prob.ndet)}


def capture_stdout(fn):
    """fn()'s result and what it wrote to file descriptor 1 (the engine's
    per-iteration lines), kept out of the probe's JSON output."""
    import tempfile
    sys.stdout.flush()
    with tempfile.TemporaryFile(mode="w+") as tmp:
        saved = os.dup(1)
        os.dup2(tmp.fileno(), 1)
        try:
            r = fn()
        finally:
            sys.stdout.flush()
            os.dup2(saved, 1)
            os.close(saved)
        tmp.seek(0)
        return r, tmp.read()


def run_sigma_probe(a) -> int:
    """--sigma-probe CONFIG: times sigma (and optionally one Davidson solve per
    precision) on one synthetic configuration and prints one JSON line:
    problem sizes and nonzero counts, table/diagonal build times, the FP64 and
    mixed sigma times (CUDA events on the launch stream, after two untimed
    products) with their model bandwidth (24N + 8 nnz bytes FP64, 16N + 4 nnz
    mixed), the mixed product of 2-4 vectors at once (time per vector) and the
    autotuner's tile choice.  Config 4 takes one request of the seeded mix
    (--request).  This is the command the ncu summaries under profiles/ run."""
    import torch

    from sbd_gb300 import build
    from sbd_gb300 import generators as G
    from sbd_gb300.engine import MIXED, Engine, TPBProblem

    a.config = a.sigma_probe
    build.build()
    t = time.time()
    eps, max_nb = 1e-8, 24
    if a.config == 4:
        prob, a.nroots = G.config4_request(a.request)
        eps, max_nb = 1e-7, 20
    elif a.strings:  # the configuration's generator with fewer strings per spin (a smaller case to profile)
        norb, nel, seed = {0: (16, 5, 0), 1: (36, 12, 1), 3: (58, 16, 3)}[a.config]
        prob = G.make_problem(norb, nel, nel, a.strings, a.strings, seed=seed)
    else:
        prob = {0: G.config0, 1: G.config1, 3: G.config3}[a.config]()
    tgen = time.time() - t
    eng = Engine(0)
    t = time.time()
    p = TPBProblem.from_problem(eng, prob)
    p.build_tables()
    torch.cuda.synchronize()
    ttab = time.time() - t
    t = time.time()
    p.diag_terms()
    tdiag = time.time() - t
    (sa, da), (sb, db) = p.table_counts(0), p.table_counts(1)
    N = prob.ndet
    na, nb = prob.astr.size, prob.bstr.size
    nnz = nb * (sa + da) + na * (sb + db) + sa * sb
    out = {"config": a.config, "N": N, "na": na, "nb": nb, "singles_a": sa, "doubles_a": da, "singles_b": sb,
           "doubles_b": db, "nnz_off": nnz, "nnz_per_row": nnz / N, "t_gen": tgen, "t_tables": ttab, "t_diag": tdiag}
    st = torch.cuda.current_stream()
    C = torch.rand(N, dtype=torch.float64, device="cuda") * 2 - 1
    S = torch.empty_like(C)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(a.reps):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / a.reps

    ms = timed(lambda: p.sigma_device(C.data_ptr(), S.data_ptr(), stream=st.cuda_stream))
    out["sigma_fp64_ms"] = ms
    out["sigma_fp64_GBs_model"] = (24 * N + 8 * nnz) / (ms * 1e-3) / 1e9
    out["sigma_fp64_Gnnz_s"] = nnz / (ms * 1e-3) / 1e9
    out["tuning_fp64"] = p.tuning(0)
    if a.mixed:
        C32 = C.float()
        S32 = torch.empty_like(C32)
        msm = timed(lambda: p.sigma_mixed_device(C32.data_ptr(), S32.data_ptr(), stream=st.cuda_stream))
        out["sigma_mixed_ms"] = msm
        out["sigma_mixed_GBs_model"] = (16 * N + 4 * nnz) / (msm * 1e-3) / 1e9
        out["sigma_mixed_relerr"] = float((S32.double() - S).abs().max() / S.abs().max())
        out["tuning_mixed"] = p.tuning(MIXED)
        # double-float product (the second phase of the mixed solver)
        Cd = torch.stack([C.float(), (C - C.float().double()).float()], dim=1).reshape(-1).contiguous()
        Sd = torch.empty_like(Cd)
        msd = timed(lambda: p.sigma_df_device(Cd.data_ptr(), Sd.data_ptr(), stream=st.cuda_stream))
        out["sigma_df_ms"] = msd
        sd = Sd.double().reshape(-1, 2).sum(dim=1)
        out["sigma_df_relerr"] = float((sd - S).abs().max() / S.abs().max())
        out["tuning_df"] = p.tuning(2)
        del Cd, Sd, sd
        # several FP32 vectors per product: time per vector
        for nv in (2, 3, 4):
            X = torch.rand(nv, N, dtype=torch.float32, device="cuda") * 2 - 1
            Y = torch.empty_like(X)
            ms_b = timed(lambda: p.sigma_mixed_block_device(X.data_ptr(), Y.data_ptr(), nv, stream=st.cuda_stream))
            out[f"sigma_mixed_block{nv}_ms_per_vector"] = ms_b / nv
    if a.davidson:
        for prec, name in ((0, "fp64"), (MIXED, "mixed")):
            # an untimed solve first: it tunes the solver's sigma shapes
            p.davidson(nroots=a.nroots, max_nb=max_nb, eps=eps, init=1, precision=prec, want_vectors=False)
            torch.cuda.synchronize()
            eng.enable_timing(True)
            eng.sigma_timing()
            t = time.time()
            r, log = capture_stdout(lambda: p.davidson(nroots=a.nroots, max_nb=max_nb, eps=eps, init=1,
                                                       precision=prec, want_vectors=False, verbose=True))
            torch.cuda.synchronize()
            wall = time.time() - t
            ncalls, sig_ms = eng.sigma_timing()
            eng.enable_timing(False)
            lines = [x for x in log.splitlines() if "iteration" in x]
            phases = {"fp32": sum("(FP32 phase)" in x for x in lines),
                      "double_float": sum("(double-float phase)" in x for x in lines)}
            phases["fp64"] = len(lines) - phases["fp32"] - phases["double_float"]
            out[f"dav_{name}"] = {"E": r.energies.tolist(), "wall_s": wall, "sigma_ms_total": sig_ms,
                                  "sigma_products_timed": ncalls, "iterations_by_phase": phases, **r.report}
    print(json.dumps(out))
    p.close()
    eng.close()
    return 0


def config3_block(eng, peak: float, peak_kind: str, reps: int = 10) -> dict:
    """sigma on config 3 (norb 58, 16+16 electrons, 12000 x 12000 strings,
    N = 1.44e8, 1.15 GB per FP64 vector: larger than L2 every product) in FP64
    and in the mixed form's FP32 product, CUDA events on the launch stream
    after two untimed products, against the HBM roofline: algorithmic bytes
    24 N + 8 nnz_off (FP64: read C and hii, write sigma, one C read per
    nonzero) and 12 N + 4 nnz_off (FP32: the unshifted product reads hii in
    FP32); then one Davidson solve per precision (1 root, tol 1e-7)."""
    import torch

    from sbd_gb300.engine import MIXED, TPBProblem
    from sbd_gb300.generators import config3
    prob = config3()
    p = TPBProblem.from_problem(eng, prob)
    p.build_tables()
    p.diag_terms()
    (sa, da), (sb, db) = p.table_counts(0), p.table_counts(1)
    N, na, nb = prob.ndet, prob.astr.size, prob.bstr.size
    nnz = nb * (sa + da) + na * (sb + db) + sa * sb
    st = torch.cuda.Stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    C = torch.rand(N, dtype=torch.float64, device="cuda") * 2 - 1
    S = torch.empty_like(C)
    ms64 = timed(lambda: p.sigma_device(C.data_ptr(), S.data_ptr(), stream=st.cuda_stream))
    C32 = C.float()
    S32 = torch.empty_like(C32)
    ms32 = timed(lambda: p.sigma_mixed_device(C32.data_ptr(), S32.data_ptr(), stream=st.cuda_stream))
    rel32 = float((S32.double() - S).abs().max() / S.abs().max())
    del C, S, C32, S32
    b64, b32 = 24.0 * N + 8.0 * nnz, 12.0 * N + 4.0 * nnz
    out = {"workload": "config3: norb 58, 16+16 electrons, 12000x12000 strings (N=144,000,000)",
           "nnz_per_row": nnz / N,
           "fp64": {"ms": ms64, "tiles": p.tuning(0),
                    "roofline": {"bound": "hbm", "achieved": b64 / (ms64 * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                                 "frac": b64 / (ms64 * 1e-3) / 1e9 / peak, "algorithmic_bytes": b64,
                                 "peak_kind": f"{peak_kind} hbm_gbs"}},
           "mixed_fp32": {"ms": ms32, "tiles": p.tuning(MIXED), "max_rel_err_vs_fp64": rel32,
                          "roofline": {"bound": "hbm", "achieved": b32 / (ms32 * 1e-3) / 1e9, "peak": peak,
                                       "unit": "GB/s", "frac": b32 / (ms32 * 1e-3) / 1e9 / peak,
                                       "algorithmic_bytes": b32, "peak_kind": f"{peak_kind} hbm_gbs"}},
           "mixed_vs_fp64_sigma": ms64 / ms32}
    E = {}
    for prec, name in ((0, "fp64"), (MIXED, "mixed")):
        for _ in range(2):  # the second solve is timed (the first tunes the solver's sigma shapes)
            torch.cuda.synchronize()
            t = time.perf_counter()
            r = p.davidson(nroots=1, max_nb=20, eps=1e-7, init=1, precision=prec, want_vectors=False)
            torch.cuda.synchronize()
        E[name] = r.energies
        out[f"solve_{name}"] = {"seconds": time.perf_counter() - t, "iterations": r.report["iterations"],
                                "sigma_products": r.report["sigma_calls"], "converged": r.report["converged"]}
    out["solve_max_abs_dE"] = float(np.max(np.abs(E["mixed"] - E["fp64"])))
    p.close()
    return out


def run_gpu(args):
    dist, rank, ws = dist_init()
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from sbd_gb300 import build as b
    b.build()
    from sbd_gb300.engine import Engine, TPBProblem
    prob = make_problem()
    eng = Engine(local)
    p = TPBProblem.from_problem(eng, prob)
    p.build_tables()
    p.diag_terms()
    (sa, da), (sb, db) = p.table_counts(0), p.table_counts(1)
    N = prob.ndet
    na, nb = prob.astr.size, prob.bstr.size
    nnz_off = nb * (sa + da) + na * (sb + db) + sa * sb
    bytes_sigma = 24.0 * N + 8.0 * nnz_off
    kw = dict(nroots=NROOTS, max_nb=MAX_NB, eps=EPS, init=1, want_vectors=False)
    if args.tiles:  # the solver's sigma shapes fixed instead of timed (a profiler distorts the timing)
        sa, sb, sp = (int(x) for x in args.tiles.split(","))
        p.set_tuning(3, sa, sb)
        p.set_split(3, sp)

    # warm-up solves (untimed)
    for _ in range(args.warmup):
        r = p.davidson(**kw)
    torch.cuda.synchronize()
    energies = r.energies.copy()

    # timed region: K resident solves
    stream = torch.cuda.Stream()
    eng.set_stream(stream.cuda_stream)
    clocks = ClockSampler(local)
    clocks.start()
    eng.enable_timing(True)
    eng.sigma_timing()
    launches0 = eng.launches
    barrier(dist)
    torch.cuda.synchronize()
    lat = []
    nsig = []
    t0 = time.perf_counter()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record(stream)
    for i in range(args.steps):
        r = p.davidson(**kw)
        ev[i + 1].record(stream)
        nsig.append(r.report["sigma_calls"])
    torch.cuda.synchronize()
    barrier(dist)
    wall = time.perf_counter() - t0
    lat = [ev[i].elapsed_time(ev[i + 1]) * 1e-3 for i in range(args.steps)]
    launches = eng.launches - launches0
    ncalls, sigma_ms = eng.sigma_timing()
    eng.enable_timing(False)
    clk = clocks.stop()
    # device time of the K solves (CUDA events on the solver stream), max over ranks
    t_rank = ev[0].elapsed_time(ev[-1]) * 1e-3
    t_max = max_over_ranks(dist, t_rank)
    value = ws * args.steps / t_max
    sigma_ms_per = sigma_ms / max(ncalls, 1)
    achieved = bytes_sigma / (sigma_ms_per * 1e-3) / 1e9
    peak, peak_kind = peaks()
    # the sigma kernels are bound by the FP64 FMA pipe: one FMA per off-diagonal
    # element and per diagonal element, against the measured FP64 FMA rate
    rates = measure_fp64_rates(local)
    fp64_achieved = 2.0 * (nnz_off + N) / (sigma_ms_per * 1e-3) / 1e12
    tiles = p.tuning(3)  # the solver's products: FP64 in the block ordering

    # mixed-precision form on the same problem (reported beside the FP64 headline)
    mixed = None
    if not args.no_mixed:
        from sbd_gb300.engine import MIXED
        mlat, mE = [], None
        for i in range(1 + args.mixed_steps):
            rm = p.davidson(precision=MIXED, refine_every=0, **kw)
            if i > 0:
                mlat.append(rm.report["seconds"])
            mE = rm.energies
        mixed = {"solves_per_s": len(mlat) / max(sum(mlat), 1e-30),
                 "max_abs_dE_vs_fp64": float(np.max(np.abs(mE - energies))),
                 "converged": rm.report["converged"], "sigma_products_per_solve": rm.report["sigma_calls"],
                 "fp64_sigma_products_per_solve": rm.report["sigma_fp64"],
                 "speedup_vs_fp64": (len(mlat) / max(sum(mlat), 1e-30)) / (args.steps / max(t_rank, 1e-30))}

    # end to end through the C ABI with host buffers
    e2e_lat = []
    h2d = prob.astr.nbytes + prob.bstr.nbytes + prob.ints.h1.nbytes + prob.ints.eri.nbytes
    d2h = NROOTS * N * 8 + NROOTS * 8
    p.close()
    for _ in range(max(1, args.e2e_steps if args.e2e_steps is not None else args.steps)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        q = TPBProblem.from_problem(eng, prob)
        rr = q.davidson(nroots=NROOTS, max_nb=MAX_NB, eps=EPS, init=1, want_vectors=True)
        q.close()
        e2e_lat.append(time.perf_counter() - t)
    e2e_t = max_over_ranks(dist, float(np.sum(e2e_lat)))
    e2e_value = ws * len(e2e_lat) / e2e_t

    # config 3 (the streaming case, 0.5 nonzeros per row): sigma against the
    # HBM roofline in both precisions, and one solve per precision
    config3 = None
    if rank == 0 and not args.no_config3:
        config3 = config3_block(eng, peak, peak_kind)

    traffic = None
    prof_path = os.path.join(ROOT, "profiles", "sigma_traffic.json")
    if os.path.exists(prof_path):
        try:
            with open(prof_path) as f:
                traffic = float(json.load(f)["bytes_per_sigma_config1"])
        except Exception:
            traffic = None

    # serving: a bounded sample of the config-4 request mix through the request
    # loop (all submitted at once), against the plain FP64 path one solve at a time
    serving = None
    if rank == 0 and args.serve_requests > 0:
        from sbd_gb300 import serve_bench as sb
        reqs = sb.generate(4, args.serve_requests, min(16, os.cpu_count() or 1))
        slat, sE = sb.run_serial(reqs, 4)
        serving = {"workload": f"config4: first {len(reqs)} requests of the seeded mix (norb 24-48, "
                               "200-4000 strings per spin, 1-3 roots, tol 1e-7), all submitted at once",
                   "plain_fp64_one_at_a_time": {"solves_per_s": len(reqs) / sum(slat),
                                                "p50_s": float(np.percentile(slat, 50)),
                                                "p99_s": float(np.percentile(slat, 99))}}
        for prec, name in ((0, "fp64"), (1, "mixed")):
            res, wall_s, st = sb.run_serving(reqs, 4, prec, float("inf"), args.serve_workers, 7)
            summ = sb.summarize(res, wall_s, st, sE, prec, float("inf"))
            serving[f"loop_{name}"] = {k: summ[k] for k in ("solves_per_s", "p50_s", "p99_s", "max_abs_dE",
                                                             "failed", "not_converged", "peak_running")}
            serving[f"loop_{name}"]["vs_plain_fp64"] = summ["solves_per_s"] / serving["plain_fp64_one_at_a_time"][
                "solves_per_s"]

    # batching: a bounded sample of the config-2 batch (norb 12, 4+4, 4 roots,
    # tol 1e-8) solved in lock step by the batched solver, against the plain
    # FP64 path one solve at a time on its first problems
    batched = None
    if rank == 0 and args.batch_problems > 0:
        from sbd_gb300 import serve_bench as sb
        reqs = sb.generate(2, args.batch_problems, min(16, os.cpu_count() or 1))
        nser = min(args.batch_serial, len(reqs))
        slat, sE = sb.run_serial(reqs[:nser], 2)
        batched = {"workload": f"config2: first {len(reqs)} problems of the seeded batch (norb 12, 4+4 electrons, "
                               "50-495 strings per spin, 4 roots, tol 1e-8), one batched solver call",
                   "plain_fp64_one_at_a_time": {"problems": nser, "solves_per_s": nser / sum(slat),
                                                "p50_s": float(np.percentile(slat, 50)),
                                                "p99_s": float(np.percentile(slat, 99))}}
        for prec, name in ((0, "batched_fp64"), (1, "batched_mixed")):
            Eb, wall_b, t_solver, reps = sb.run_batch(reqs, 2, len(reqs), prec)
            batched[name] = {"problems": len(reqs), "solves_per_s": len(reqs) / wall_b,
                             "solver_seconds": t_solver, "wall_seconds": wall_b,
                             "iterations_mean": float(np.mean([r["iterations"] for r in reps])),
                             "sigma_products_mean": float(np.mean([r["sigma_calls"] for r in reps])),
                             "fp64_sigma_products_mean": float(np.mean([r["sigma_fp64"] for r in reps])),
                             "not_converged": sum(1 for r in reps if not r["converged"]),
                             "max_abs_dE_vs_plain": max(float(np.max(np.abs(e - r))) for e, r in zip(Eb, sE))}
            batched[name]["vs_plain_fp64"] = (batched[name]["solves_per_s"] /
                                              batched["plain_fp64_one_at_a_time"]["solves_per_s"])

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            cpu = cpu_baseline(prob, float(np.mean(nsig)), os.cpu_count() or 1)
        except Exception as e:  # the baseline is reported, not required
            cpu = {"error": str(e)}

    if rank == 0:
        lat_sorted = sorted(lat)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_block(prob, ws),
            "problem": {"nnz_offdiag": int(nnz_off), "nnz_per_row": nnz_off / N},
            "energies": [float(x) for x in energies],
            "latency_s": {"p50": float(np.percentile(lat_sorted, 50)), "p99": float(np.percentile(lat_sorted, 99))},
            "sigma_products_per_solve": float(np.mean(nsig)),
            "sigma_ms": sigma_ms_per,
            "sigma_tiles": tiles,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": ("sigma operator (fused k_sigma_alpha)" if tiles.get("beta_shape") == "fused"
                                    else "sigma operator (k_transpose + k_sigma_alpha + k_sigma_beta)"),
                         "algorithmic_bytes": bytes_sigma, "peak_kind": f"{peak_kind} hbm_gbs",
                         "fp64": {"unit": "TFLOP/s", "achieved": fp64_achieved, "peak": rates["dfma_tflops"],
                                  "frac": fp64_achieved / rates["dfma_tflops"],
                                  "peak_kind": "measured FP64 FMA pipe (bench_csrc/rates.cu)",
                                  "fp64_tensor_peak": rates["dmma_tflops"],
                                  "flops": "2 x (nnz_off + N) per sigma"}},
            "mixed_precision": mixed,
            "config3_sigma": config3,
            "serving": serving,
            "batched": batched,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "clocks": clk,
            "wall_s": wall,
        }
        print(json.dumps(line))
    eng.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=None, help="end-to-end solves (default: --steps)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-config3", action="store_true", help="skip the config-3 sigma roofline block")
    ap.add_argument("--tiles", default=None,
                    help="shape_a,shape_b,split of the solver's FP64 sigma instead of the autotuner's choice")
    ap.add_argument("--mixed-steps", type=int, default=2)
    ap.add_argument("--serve-requests", type=int, default=48, help="config-4 requests for the serving block (0: skip)")
    ap.add_argument("--serve-workers", type=int, default=16)
    ap.add_argument("--batch-problems", type=int, default=256,
                    help="config-2 problems for the batched block (0: skip)")
    ap.add_argument("--batch-serial", type=int, default=32,
                    help="of which solved one at a time on the plain FP64 path")
    ap.add_argument("--sigma-probe", type=int, default=None, choices=[0, 1, 3, 4],
                    help="time sigma on one configuration instead of the solve benchmark")
    ap.add_argument("--request", type=int, default=94, help="--sigma-probe 4: the request of the seeded mix")
    ap.add_argument("--reps", type=int, default=5, help="--sigma-probe: timed products")
    ap.add_argument("--davidson", type=int, default=0, help="--sigma-probe: also one solve per precision")
    ap.add_argument("--mixed", type=int, default=1, help="--sigma-probe: also the mixed sigma")
    ap.add_argument("--nroots", type=int, default=2, help="--sigma-probe: roots of the solve")
    ap.add_argument("--strings", type=int, default=0,
                    help="--sigma-probe 0/1/3: strings per spin instead of the configuration's (a smaller case)")
    ap.add_argument("--fp64-rates", action="store_true",
                    help="print the measured FP64 FMA and MMA rates and their overlap, then exit")
    args = ap.parse_args()
    if args.fp64_rates:
        from sbd_gb300 import build as b
        b.build()
        print(json.dumps({**measure_fp64_rates(0), **measure_fp64_overlap(0)}))
        return 0
    if args.sigma_probe is not None:
        return run_sigma_probe(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
