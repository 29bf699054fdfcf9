"""Request loop of the engine: many Davidson solves on one GPU at once.

A thin front end of the server in csrc/serve.cu (sbdgb_server_* in
include/sbdgb.h).  Worker threads on the C++ side each own a CUDA stream, so
the solves of requests that arrive while others run overlap on the device;
admission is by HBM footprint.  Each request is the reference app's single
diagonalisation (apps/chemistry_tpb_selected_basis_diagonalization/main.cc,
sbd::tpb::diag in chemistry/tpb/sbdiag.h) on its own strings and integrals.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from .engine import FP64, SBDGB_OK, STATUS, DavidsonOpts, Request, Result, SbdgbError, ServeStats, load

E_TIMEOUT = 6


class Server:
    """sbdgb_server: `workers` solver threads on `device`, HBM budget in bytes (0 = 90% of free)."""

    def __init__(self, device: int = 0, workers: int = 8, hbm_budget: int = 0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.sbdgb_server_create(device, workers, hbm_budget, C.byref(h))
        if rc != SBDGB_OK:
            raise SbdgbError(rc, f"cannot create a server on device {device}")
        self.h = h
        self._keep: dict[int, tuple] = {}  # per ticket: the arrays the server still writes into
        self._mu = threading.Lock()

    def close(self):
        if getattr(self, "h", None):
            self.lib.sbdgb_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    def _error(self) -> str:
        return self.lib.sbdgb_server_last_error(self.h).decode()

    def submit(self, norb: int, astr, bstr, h1, eri, ecore: float = 0.0, nroots: int = 1, eps: float = 1e-8,
               max_nb: int = 20, max_it: int = 100, init: int = 1, precision: int = FP64, refine_every: int = 0,
               want_vectors: bool = False) -> int:
        """Queues one solve and returns its ticket (the inputs are copied)."""
        a = np.ascontiguousarray(astr, dtype=np.uint64)
        b = np.ascontiguousarray(bstr, dtype=np.uint64)
        h1 = np.ascontiguousarray(h1, dtype=np.float64).ravel()
        eri = np.ascontiguousarray(eri, dtype=np.float64)
        o = DavidsonOpts()
        self.lib.sbdgb_davidson_default_opts(C.byref(o))
        o.nroots, o.eps, o.max_nb, o.max_it = nroots, eps, max_nb, max_it
        o.init, o.precision, o.refine_every = init, precision, refine_every
        X = np.zeros((nroots, a.size * b.size)) if want_vectors else None
        q = Request(norb=int(norb), astr=a.ctypes.data, na=a.size, bstr=b.ctypes.data, nb=b.size,
                    h1=h1.ctypes.data, eri_packed=eri.ctypes.data, ecore=float(ecore), opts=o,
                    vectors_out=X.ctypes.data if X is not None else None)
        t = C.c_uint64(0)
        rc = self.lib.sbdgb_server_submit(self.h, C.byref(q), C.byref(t))
        if rc != SBDGB_OK:
            raise SbdgbError(rc, self._error())
        with self._mu:
            self._keep[t.value] = (X,)
        return int(t.value)

    def submit_problem(self, prob, **kw) -> int:
        """Queues a generators.Problem."""
        return self.submit(prob.norb, prob.astr, prob.bstr, prob.ints.h1, prob.ints.eri, prob.ints.ecore, **kw)

    def poll(self, ticket: int) -> bool:
        done = C.c_int(0)
        rc = self.lib.sbdgb_server_poll(self.h, ticket, C.byref(done))
        if rc != SBDGB_OK:
            raise SbdgbError(rc, "unknown ticket")
        return bool(done.value)

    def wait(self, ticket: int, timeout: float | None = None) -> dict:
        """The ticket's result; raises TimeoutError if it is not ready within `timeout` seconds."""
        r = Result()
        rc = self.lib.sbdgb_server_wait(self.h, ticket, -1.0 if timeout is None else float(timeout), C.byref(r))
        if rc == E_TIMEOUT:
            raise TimeoutError(f"ticket {ticket} not done after {timeout} s")
        if rc != SBDGB_OK:
            raise SbdgbError(rc, self._error())
        with self._mu:
            (X,) = self._keep.pop(ticket, (None,))
        k = r.nroots
        return {"ticket": ticket, "status": r.status, "status_name": STATUS.get(r.status, str(r.status)),
                "message": r.message.decode(errors="replace"), "energies": np.array(r.energies[:k]),
                "resid": list(r.resid[:k]), "queue_seconds": r.queue_seconds, "run_seconds": r.run_seconds,
                "total_seconds": r.total_seconds, "iterations": r.iterations, "sigma_calls": r.sigma_calls,
                "converged": bool(r.converged), "worker": r.worker, "reserved_bytes": int(r.reserved_bytes),
                "ndet": int(r.ndet), "vectors": X}

    def stats(self) -> dict:
        s = ServeStats()
        rc = self.lib.sbdgb_server_stats(self.h, C.byref(s))
        if rc != SBDGB_OK:
            raise SbdgbError(rc, "stats")
        return {f: getattr(s, f) for f, _ in ServeStats._fields_}
