"""Times sigma and Davidson on one of the synthetic benchmark configurations.

    python -m sbd_gb300.probe --config 1 --reps 5 [--davidson 1] [--mixed 1]
    python -m sbd_gb300.probe --config 4 --request 94 --davidson 1   (one config-4 request)

Prints one JSON line: problem sizes and nonzero counts, table/diagonal build
times, the FP64 and mixed sigma times (CUDA events on the launch stream, after
two untimed products) with their model bandwidth (24N + 8 nnz bytes FP64,
16N + 4 nnz mixed), the mixed product of 2-4 vectors at once (time per
vector), the autotuner's tile choice, and optionally one Davidson solve in
each precision.
"""
from __future__ import annotations

import argparse
import json
import time


def main(argv=None) -> int:
    import torch

    from . import build
    from . import generators as G
    from .engine import MIXED, Engine, TPBProblem

    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=1, choices=[0, 1, 3, 4])
    ap.add_argument("--request", type=int, default=94, help="config 4: the request of the seeded mix")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--davidson", type=int, default=0)
    ap.add_argument("--mixed", type=int, default=1)
    ap.add_argument("--nroots", type=int, default=2)
    a = ap.parse_args(argv)
    build.build()
    t = time.time()
    eps, max_nb = 1e-8, 24
    if a.config == 4:
        prob, a.nroots = G.config4_request(a.request)
        eps, max_nb = 1e-7, 20
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
        # several FP32 vectors per product: time per vector
        for nv in (2, 3, 4):
            X = torch.rand(nv, N, dtype=torch.float32, device="cuda") * 2 - 1
            Y = torch.empty_like(X)
            ms_b = timed(lambda: p.sigma_mixed_block_device(X.data_ptr(), Y.data_ptr(), nv, stream=st.cuda_stream))
            out[f"sigma_mixed_block{nv}_ms_per_vector"] = ms_b / nv
    if a.davidson:
        for prec, name in ((0, "fp64"), (MIXED, "mixed")):
            torch.cuda.synchronize()
            t = time.time()
            r = p.davidson(nroots=a.nroots, max_nb=max_nb, eps=eps, init=1, precision=prec, want_vectors=False)
            torch.cuda.synchronize()
            out[f"dav_{name}"] = {"E": r.energies.tolist(), "wall_s": time.time() - t, **r.report}
    print(json.dumps(out))
    p.close()
    eng.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
