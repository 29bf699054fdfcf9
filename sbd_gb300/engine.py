"""Python front end of the CUDA engine, bound through the C ABI (include/sbdgb.h).

There is no CPU fallback: if libsbdgb.so is missing or no GPU is visible the
constructors raise.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsbdgb.so")

SBDGB_OK = 0
CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy
STATUS = {0: "OK", 1: "E_INPUT", 2: "E_UNSUPPORTED", 3: "E_CUDA", 4: "E_NOMEM", 5: "E_STATE", 6: "E_TIMEOUT"}
FP64, MIXED = 0, 1

SYMBOLS = [
    "sbdgb_abi_version", "sbdgb_ctx_create", "sbdgb_ctx_destroy", "sbdgb_last_error", "sbdgb_ctx_bytes_in_use",
    "sbdgb_ctx_launch_count", "sbdgb_ctx_set_stream", "sbdgb_ctx_enable_timing", "sbdgb_ctx_sigma_timing", "sbdgb_check_comm_sizes", "sbdgb_problem_create", "sbdgb_problem_destroy",
    "sbdgb_problem_footprint", "sbdgb_build_tables", "sbdgb_table_counts", "sbdgb_export_tables",
    "sbdgb_diag_terms", "sbdgb_sigma", "sbdgb_sigma_mixed", "sbdgb_sigma_df", "sbdgb_sigma_mixed_block", "sbdgb_sigma_noalloc", "sbdgb_occupation_density", "sbdgb_string_weights", "sbdgb_string_cut_counts", "sbdgb_rdm", "sbdgb_problem_tuning", "sbdgb_problem_tuning_times", "sbdgb_problem_set_tuning", "sbdgb_problem_split", "sbdgb_problem_set_split", "sbdgb_mult_host", "sbdgb_davidson_default_opts",
    "sbdgb_davidson", "sbdgb_lanczos", "sbdgb_batch_davidson", "sbdgb_server_create", "sbdgb_server_submit", "sbdgb_server_poll", "sbdgb_server_wait",
    "sbdgb_server_stats", "sbdgb_server_last_error", "sbdgb_server_destroy",
]


class SbdgbError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class DavidsonOpts(C.Structure):
    _fields_ = [("max_it", C.c_int), ("max_nb", C.c_int), ("eps", C.c_double), ("max_time", C.c_double),
                ("nroots", C.c_int), ("init", C.c_int), ("precision", C.c_int), ("refine_every", C.c_int),
                ("verbose", C.c_int)]


class Report(C.Structure):
    _fields_ = [("iterations", C.c_int), ("sigma_calls", C.c_int), ("sigma_fp64", C.c_int), ("restarts", C.c_int),
                ("converged", C.c_int), ("seconds", C.c_double), ("resid", C.c_double * 16)]

    def as_dict(self, nroots: int) -> dict:
        return {"iterations": self.iterations, "sigma_calls": self.sigma_calls, "sigma_fp64": self.sigma_fp64,
                "restarts": self.restarts, "converged": bool(self.converged), "seconds": self.seconds,
                "resid": [self.resid[i] for i in range(min(nroots, 16))]}


class Request(C.Structure):
    _fields_ = [("norb", C.c_int), ("astr", C.c_void_p), ("na", C.c_size_t), ("bstr", C.c_void_p),
                ("nb", C.c_size_t), ("h1", C.c_void_p), ("eri_packed", C.c_void_p), ("ecore", C.c_double),
                ("opts", DavidsonOpts), ("vectors_out", C.c_void_p)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("nroots", C.c_int), ("energies", C.c_double * 8), ("resid", C.c_double * 8),
                ("queue_seconds", C.c_double), ("run_seconds", C.c_double), ("total_seconds", C.c_double),
                ("iterations", C.c_int), ("sigma_calls", C.c_int), ("converged", C.c_int), ("worker", C.c_int),
                ("reserved_bytes", C.c_size_t), ("ndet", C.c_uint64), ("message", C.c_char * 200)]


class ServeStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("launches", C.c_uint64), ("budget_bytes", C.c_size_t), ("reserved_bytes", C.c_size_t),
                ("peak_reserved_bytes", C.c_size_t), ("workers", C.c_int), ("running", C.c_int),
                ("peak_running", C.c_int), ("queued", C.c_int), ("batched", C.c_uint64)]


_lib = None
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def load(path: str = LIB_PATH):
    """Loads libsbdgb.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} not found: build it with `python -m sbd_gb300.build` "
                          "(the engine has no CPU fallback)")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.sbdgb_abi_version.restype = C.c_int
    L.sbdgb_ctx_create.argtypes = [C.POINTER(vp), C.c_int, C.c_size_t]
    L.sbdgb_ctx_destroy.argtypes = [vp]
    L.sbdgb_ctx_destroy.restype = None
    L.sbdgb_last_error.argtypes = [vp]
    L.sbdgb_last_error.restype = C.c_char_p
    L.sbdgb_ctx_bytes_in_use.argtypes = [vp]
    L.sbdgb_ctx_bytes_in_use.restype = C.c_size_t
    L.sbdgb_ctx_launch_count.argtypes = [vp]
    L.sbdgb_ctx_launch_count.restype = C.c_uint64
    L.sbdgb_check_comm_sizes.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    L.sbdgb_ctx_set_stream.argtypes = [vp, vp]
    L.sbdgb_ctx_enable_timing.argtypes = [vp, C.c_int]
    L.sbdgb_ctx_sigma_timing.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_double)]
    L.sbdgb_problem_create.argtypes = [vp, C.c_int, _u64p, C.c_size_t, _u64p, C.c_size_t, _f64p, _f64p,
                                       C.c_double, C.POINTER(vp)]
    L.sbdgb_problem_destroy.argtypes = [vp]
    L.sbdgb_problem_destroy.restype = None
    L.sbdgb_problem_footprint.argtypes = [C.c_int, C.c_size_t, C.c_size_t, C.c_int, C.c_int, C.c_int,
                                          C.POINTER(C.c_size_t)]
    L.sbdgb_build_tables.argtypes = [vp]
    L.sbdgb_table_counts.argtypes = [vp, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    L.sbdgb_export_tables.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, vp]
    L.sbdgb_diag_terms.argtypes = [vp, vp]
    L.sbdgb_sigma.argtypes = [vp, vp, vp, C.c_int, vp]
    L.sbdgb_sigma_mixed.argtypes = [vp, vp, vp, vp]
    L.sbdgb_sigma_mixed_block.argtypes = [vp, vp, vp, C.c_int, vp]
    L.sbdgb_sigma_df.argtypes = [vp, vp, vp, C.c_int, vp]
    L.sbdgb_sigma_noalloc.argtypes = [vp, vp, vp, C.c_int, vp]
    L.sbdgb_occupation_density.argtypes = [vp, vp, _f64p, vp]
    L.sbdgb_string_weights.argtypes = [vp, vp, _f64p, _f64p, vp]
    L.sbdgb_rdm.argtypes = [vp, vp, _f64p, vp, vp]
    L.sbdgb_string_cut_counts.argtypes = [vp, vp, C.c_double, _u64p, _u64p, C.POINTER(C.c_double), vp]
    L.sbdgb_mult_host.argtypes = [vp, vp, _f64p, _f64p]
    L.sbdgb_problem_tuning.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int]
    L.sbdgb_problem_tuning_times.argtypes = [vp, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                             C.POINTER(C.c_float)]
    L.sbdgb_problem_split.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_float)]
    L.sbdgb_problem_set_split.argtypes = [vp, C.c_int, C.c_int]
    L.sbdgb_problem_set_tuning.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    L.sbdgb_davidson_default_opts.argtypes = [C.POINTER(DavidsonOpts)]
    L.sbdgb_davidson_default_opts.restype = None
    L.sbdgb_davidson.argtypes = [vp, C.POINTER(DavidsonOpts), _f64p, vp, C.POINTER(Report)]
    L.sbdgb_lanczos.argtypes = [vp, C.POINTER(DavidsonOpts), _f64p, vp, C.POINTER(Report)]
    L.sbdgb_batch_davidson.argtypes = [vp, C.POINTER(vp), C.c_int, C.POINTER(DavidsonOpts), _f64p, vp, vp]
    L.sbdgb_server_create.argtypes = [C.c_int, C.c_int, C.c_size_t, C.POINTER(vp)]
    L.sbdgb_server_submit.argtypes = [vp, C.POINTER(Request), C.POINTER(C.c_uint64)]
    L.sbdgb_server_poll.argtypes = [vp, C.c_uint64, C.POINTER(C.c_int)]
    L.sbdgb_server_wait.argtypes = [vp, C.c_uint64, C.c_double, C.POINTER(Result)]
    L.sbdgb_server_stats.argtypes = [vp, C.POINTER(ServeStats)]
    L.sbdgb_server_last_error.argtypes = [vp]
    L.sbdgb_server_last_error.restype = C.c_char_p
    L.sbdgb_server_destroy.argtypes = [vp]
    L.sbdgb_server_destroy.restype = None
    _lib = L
    return L


class Engine:
    """One device context (sbdgb_ctx)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.sbdgb_ctx_create(C.byref(h), device, hbm_budget)
        if rc != SBDGB_OK:
            raise SbdgbError(rc, f"cannot create a context on device {device}")
        self.h = h
        self.device = device
        self._problems = weakref.WeakSet()

    def close(self):
        """Destroys the context after every problem still open on it."""
        if getattr(self, "h", None):
            for p in list(getattr(self, "_problems", ())):
                p.close()
            self.lib.sbdgb_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def check(self, rc: int):
        if rc != SBDGB_OK:
            raise SbdgbError(rc, self.lib.sbdgb_last_error(self.h).decode())

    @property
    def bytes_in_use(self) -> int:
        return int(self.lib.sbdgb_ctx_bytes_in_use(self.h))

    @property
    def launches(self) -> int:
        return int(self.lib.sbdgb_ctx_launch_count(self.h))

    def set_stream(self, stream: int | None):
        """Runs later calls on the caller's cudaStream_t (None: the context's own stream)."""
        self.check(self.lib.sbdgb_ctx_set_stream(self.h, stream or None))

    def enable_timing(self, on: bool = True):
        self.check(self.lib.sbdgb_ctx_enable_timing(self.h, int(on)))

    def sigma_timing(self) -> tuple[int, float]:
        """(sigma products, summed device milliseconds) since the last call."""
        n, ms = C.c_uint64(0), C.c_double(0.0)
        self.check(self.lib.sbdgb_ctx_sigma_timing(self.h, C.byref(n), C.byref(ms)))
        return int(n.value), float(ms.value)

    def check_comm_sizes(self, h: int, b: int, t: int):
        self.check(self.lib.sbdgb_check_comm_sizes(self.h, h, b, t))


def batch_davidson(engine: Engine, problems: list, nroots: int = 1, max_nb: int = 20, eps: float = 1e-8,
                   max_it: int = 100, want_vectors: bool = False, precision: int = FP64) -> list:
    """Solves every TPBProblem of the list (all on `engine`) with the batched solver:
    all problems advanced in lock step, one captured graph launch per Davidson
    iteration.  precision MIXED runs an FP32 phase first and then the FP64 phase
    (same tolerance, same energies).  Returns one DavidsonResult per problem."""
    n = len(problems)
    o = DavidsonOpts()
    load().sbdgb_davidson_default_opts(C.byref(o))
    o.nroots, o.max_nb, o.eps, o.max_it, o.init, o.precision = nroots, max_nb, eps, max_it, 1, precision
    hs = (C.c_void_p * max(n, 1))(*[p.h.value for p in problems])
    E = np.zeros(max(n * nroots, 1))
    reps = (Report * max(n, 1))()
    xs = [np.zeros((nroots, p.N)) for p in problems] if want_vectors else None
    xp = (C.c_void_p * max(n, 1))(*[x.ctypes.data for x in xs]) if want_vectors else None
    engine.check(engine.lib.sbdgb_batch_davidson(engine.h, hs, n, C.byref(o), E, reps, xp))
    return [DavidsonResult(E[i * nroots:(i + 1) * nroots].copy(), xs[i] if xs else None, reps[i].as_dict(nroots))
            for i in range(n)]


def footprint(norb: int, na: int, nb: int, max_nb: int, nroots: int, precision: int = FP64) -> int:
    out = C.c_size_t(0)
    rc = load().sbdgb_problem_footprint(norb, na, nb, max_nb, nroots, precision, C.byref(out))
    if rc != SBDGB_OK:
        raise SbdgbError(rc, "footprint")
    return int(out.value)


@dataclass
class DavidsonResult:
    energies: np.ndarray
    vectors: np.ndarray | None
    report: dict


class TPBProblem:
    """One uploaded problem (sbdgb_problem)."""

    def __init__(self, engine: Engine, norb: int, astr, bstr, h1, eri, ecore: float = 0.0):
        self.engine = engine
        self.lib = engine.lib
        self.norb = int(norb)
        self.astr = np.ascontiguousarray(astr, dtype=np.uint64)
        self.bstr = np.ascontiguousarray(bstr, dtype=np.uint64)
        self.na, self.nb = int(self.astr.size), int(self.bstr.size)
        self.N = self.na * self.nb
        h = C.c_void_p()
        h1 = np.ascontiguousarray(h1, dtype=np.float64).ravel()
        eri = np.ascontiguousarray(eri, dtype=np.float64)
        rc = self.lib.sbdgb_problem_create(engine.h, self.norb, self.astr, self.na, self.bstr, self.nb, h1, eri,
                                           float(ecore), C.byref(h))
        engine.check(rc)
        self.h = h
        engine._problems.add(self)

    @classmethod
    def from_problem(cls, engine: Engine, p) -> "TPBProblem":
        return cls(engine, p.norb, p.astr, p.bstr, p.ints.h1, p.ints.eri, p.ints.ecore)

    def close(self):
        if getattr(self, "h", None):
            if getattr(self.engine, "h", None):
                self.lib.sbdgb_problem_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def build_tables(self):
        self.engine.check(self.lib.sbdgb_build_tables(self.h))

    def table_counts(self, spin: int) -> tuple[int, int]:
        ns, nd = C.c_uint64(0), C.c_uint64(0)
        self.engine.check(self.lib.sbdgb_table_counts(self.h, spin, C.byref(ns), C.byref(nd)))
        return int(ns.value), int(nd.value)

    def export_tables(self, spin: int) -> dict:
        """Tables of one spin in the reference helper layout (offsets, kets, CrAn)."""
        ns, nd = self.table_counts(spin)
        n = self.na if spin == 0 else self.nb
        off_s = np.zeros(n + 1, dtype=np.uint64)
        off_d = np.zeros(n + 1, dtype=np.uint64)
        ket_s = np.zeros(max(ns, 1), dtype=np.uint64)
        ket_d = np.zeros(max(nd, 1), dtype=np.uint64)
        cran_s = np.zeros(max(2 * ns, 1), dtype=np.int32)
        cran_d = np.zeros(max(4 * nd, 1), dtype=np.int32)
        self.engine.check(self.lib.sbdgb_export_tables(self.h, spin, off_s.ctypes.data, ket_s.ctypes.data,
                                                       cran_s.ctypes.data, off_d.ctypes.data, ket_d.ctypes.data,
                                                       cran_d.ctypes.data))
        return {"off_s": off_s, "ket_s": ket_s[:ns], "cran_s": cran_s[:2 * ns],
                "off_d": off_d, "ket_d": ket_d[:nd], "cran_d": cran_d[:4 * nd]}

    def diag_terms(self) -> np.ndarray:
        out = np.zeros(self.N)
        self.engine.check(self.lib.sbdgb_diag_terms(self.h, out.ctypes.data))
        return out

    def mult(self, Wk: np.ndarray, Wb: np.ndarray | None = None, hii: np.ndarray | None = None) -> np.ndarray:
        """Reference semantics: Wb += H Wk (host vectors)."""
        wk = np.ascontiguousarray(Wk, dtype=np.float64).ravel()
        wb = np.zeros(self.N) if Wb is None else Wb
        if wb.dtype != np.float64 or not wb.flags["C_CONTIGUOUS"]:
            raise ValueError("Wb must be a contiguous float64 array")
        hp = None
        if hii is not None:
            hii = np.ascontiguousarray(hii, dtype=np.float64)
            hp = hii.ctypes.data
        self.engine.check(self.lib.sbdgb_mult_host(self.h, hp, wk, wb))
        return wb

    def tuning(self, precision: int = FP64) -> dict:
        """Sigma tile shapes chosen by the autotuner and the candidates' timings (ms)."""
        a, b = C.c_int(-1), C.c_int(-1)
        ma, mb = (C.c_float * 4)(), (C.c_float * 4)()
        self.engine.check(self.lib.sbdgb_problem_tuning(self.h, precision, C.byref(a), C.byref(b), ma, mb, 4))
        mf, ms, mt = (C.c_float * 4)(), (C.c_float * 2)(), (C.c_float * 2)()
        self.engine.check(self.lib.sbdgb_problem_tuning_times(self.h, precision, mf, ms, mt))
        shapes = ["8x128", "8x256", "8x512", "16x256", "fused", "sparse", "stream"]
        alpha = shapes[a.value] if a.value >= 0 else None
        if b.value >= 5:
            alpha = ["8 rows", "16 rows"][a.value]
        return {"alpha_shape": alpha, "beta_shape": shapes[b.value] if b.value >= 0 else None,
                "alpha_ms": [round(x, 4) for x in ma], "beta_ms": [round(x, 4) for x in mb],
                "fused_ms": [round(x, 4) for x in mf], "sparse_ms": [round(x, 4) for x in ms],
                "stream_ms": [round(x, 4) for x in mt],
                "alpha_beta": self.split(precision)}

    def set_tuning(self, precision: int, shape_a: int, shape_b: int):
        """Forces the sigma tile shapes (shape_b 4 = the fused single kernel, 5 = the
        sparse-row kernel with shape_a 0/1 = 8/16 rows per tile)."""
        self.engine.check(self.lib.sbdgb_problem_set_tuning(self.h, precision, shape_a, shape_b))

    def split(self, precision: int = FP64) -> dict:
        """Whether sigma's alpha x beta single pairs run in their own kernel (1),
        inside the tuned shapes (0) or are undecided (-1), with the autotuner's
        time (ms) of one product without and with that kernel."""
        sp = C.c_int(-1)
        ms = (C.c_float * 2)()
        self.engine.check(self.lib.sbdgb_problem_split(self.h, precision, C.byref(sp), ms))
        return {"split": sp.value, "ms_inline": ms[0], "ms_split": ms[1]}

    def set_split(self, precision: int, split: int):
        """Forces the alpha x beta pairs into their own kernel (1) or into the tuned shapes (0)."""
        self.engine.check(self.lib.sbdgb_problem_set_split(self.h, precision, split))

    def sigma(self, C_in: np.ndarray) -> np.ndarray:
        return self.mult(C_in)

    @staticmethod
    def _stream_arg(stream):
        # None: the context's stream; 0 (the legacy default stream handle) maps to
        # cudaStreamLegacy so that it is not mistaken for "none given"
        if stream is None:
            return None
        return stream if stream != 0 else CUDA_STREAM_LEGACY

    def sigma_device(self, c_ptr: int, s_ptr: int, accumulate: bool = False, stream: int | None = None):
        self.engine.check(self.lib.sbdgb_sigma(self.h, c_ptr, s_ptr, int(accumulate), self._stream_arg(stream)))

    def sigma_mixed_device(self, c_ptr: int, s_ptr: int, stream: int | None = None):
        self.engine.check(self.lib.sbdgb_sigma_mixed(self.h, c_ptr, s_ptr, self._stream_arg(stream)))

    def sigma_df_device(self, c_ptr: int, s_ptr: int, accumulate: bool = False, stream: int | None = None):
        """Double-float sigma on device vectors of N (hi, lo) FP32 pairs."""
        self.engine.check(self.lib.sbdgb_sigma_df(self.h, c_ptr, s_ptr, int(accumulate), self._stream_arg(stream)))

    def sigma_mixed_block_device(self, c_ptr: int, s_ptr: int, nvec: int, stream: int | None = None):
        self.engine.check(self.lib.sbdgb_sigma_mixed_block(self.h, c_ptr, s_ptr, nvec, self._stream_arg(stream)))

    def lanczos(self, max_it: int = 20, num_block: int = 40, eps: float = 1e-12, init: int = 0,
                want_vector: bool = True, W0: np.ndarray | None = None, max_time: float = 0.0,
                verbose: bool = False) -> DavidsonResult:
        """The reference's --method 2 solver (restarted Lanczos, one root)."""
        o = DavidsonOpts()
        self.lib.sbdgb_davidson_default_opts(C.byref(o))
        o.nroots, o.max_nb, o.eps, o.max_it, o.max_time, o.verbose = 1, num_block, eps, max_it, max_time, int(verbose)
        o.init = 2 if W0 is not None else init
        E = np.zeros(1)
        X = None
        if want_vector or W0 is not None:
            X = np.zeros(self.N) if W0 is None else np.ascontiguousarray(W0, dtype=np.float64).copy()
        rep = Report()
        self.engine.check(self.lib.sbdgb_lanczos(self.h, C.byref(o), E, X.ctypes.data if X is not None else None,
                                                 C.byref(rep)))
        return DavidsonResult(E, X, rep.as_dict(1))

    def _vec(self, W):
        if isinstance(W, int):
            return W, None
        w = np.ascontiguousarray(W, dtype=np.float64).ravel()
        if w.size != self.N:
            raise ValueError("vector size mismatch")
        return w.ctypes.data, w

    def string_weights(self, W) -> tuple[np.ndarray, np.ndarray]:
        """Alpha and beta string weights sum |W|^2 (the carry-over ranking)."""
        ptr, keep = self._vec(W)
        wa, wb = np.zeros(self.na), np.zeros(self.nb)
        self.engine.check(self.lib.sbdgb_string_weights(self.h, ptr, wa, wb, None))
        return wa, wb

    def string_cut_counts(self, W, cutoff: float) -> tuple[np.ndarray, np.ndarray, float]:
        """Per string, the number of determinants with |W|^2 > cutoff; and their total weight."""
        ptr, keep = self._vec(W)
        ca, cb = np.zeros(self.na, dtype=np.uint64), np.zeros(self.nb, dtype=np.uint64)
        tot = C.c_double(0.0)
        self.engine.check(self.lib.sbdgb_string_cut_counts(self.h, ptr, float(cutoff), ca, cb, C.byref(tot), None))
        return ca, cb, tot.value

    def rdm(self, W, two_body: bool = True) -> tuple[np.ndarray, np.ndarray | None]:
        """One-particle (2, L*L) and two-particle (4, L^4) RDMs in the reference's layout."""
        ptr, keep = self._vec(W)
        L = self.norb
        one = np.zeros((2, L * L))
        two = np.zeros((4, L ** 4)) if two_body else None
        self.engine.check(self.lib.sbdgb_rdm(self.h, ptr, one, two.ctypes.data if two is not None else None, None))
        return one, two

    def occupation_density(self, W) -> np.ndarray:
        """Occupation density [2*norb] of W (a host array or a device pointer)."""
        out = np.zeros(2 * self.norb)
        if isinstance(W, int):
            self.engine.check(self.lib.sbdgb_occupation_density(self.h, W, out, None))
            return out
        w = np.ascontiguousarray(W, dtype=np.float64).ravel()
        if w.size != self.N:
            raise ValueError("vector size mismatch")
        self.engine.check(self.lib.sbdgb_occupation_density(self.h, w.ctypes.data, out, None))
        return out

    def davidson(self, nroots: int = 1, max_nb: int = 20, eps: float = 1e-8, max_it: int = 100,
                 init: int = 0, precision: int = FP64, refine_every: int = 0, max_time: float = 0.0,
                 want_vectors: bool = True, X0: np.ndarray | None = None, verbose: bool = False) -> DavidsonResult:
        o = DavidsonOpts()
        self.lib.sbdgb_davidson_default_opts(C.byref(o))
        o.nroots, o.max_nb, o.eps, o.max_it = nroots, max_nb, eps, max_it
        o.init, o.precision, o.refine_every, o.max_time, o.verbose = init, precision, refine_every, max_time, int(verbose)
        E = np.zeros(nroots)
        X = None
        if want_vectors or X0 is not None:
            X = np.zeros((nroots, self.N)) if X0 is None else np.ascontiguousarray(X0, dtype=np.float64).copy()
        rep = Report()
        self.engine.check(self.lib.sbdgb_davidson(self.h, C.byref(o), E, X.ctypes.data if X is not None else None,
                                                  C.byref(rep)))
        return DavidsonResult(E, X, rep.as_dict(nroots))
