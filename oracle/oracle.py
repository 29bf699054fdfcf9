"""ctypes front end of the CPU oracle (oracle/sbd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py to check or time against the reference's
algorithm.  The product package never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "sbdref")

_lib = None

_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_szp = np.ctypeslib.ndpointer(dtype=np.uintp, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def build() -> str:
    """Compiles the oracle port (gcc + OpenMP) into oracle/_build."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def build_reference(reference_root: str | None = None) -> str | None:
    """Compiles the reference harness into oracle/_ref when the reference tree
    exists.  The tree is `reference_root`, else $SBD_REFERENCE_ROOT, else the
    default that oracle/Makefile names; without a tree nothing is built."""
    root = reference_root or os.environ.get("SBD_REFERENCE_ROOT")
    cmd = ["make", "-s", "-C", HERE, "ref"] + ([f"REFERENCE_ROOT={root}"] if root else [])
    probe = subprocess.run(["make", "-s", "-C", HERE, "reference-root"] + cmd[5:], capture_output=True, text=True)
    tree = probe.stdout.strip()
    if probe.returncode != 0 or not os.path.isdir(os.path.join(tree, "include", "sbd")):
        return None
    subprocess.run(cmd, check=True)
    return REF_BIN


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_ints_create.restype = C.c_void_p
        L.orc_ints_create.argtypes = [C.c_int, C.c_double, _f64p, _f64p]
        L.orc_ints_destroy.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads.restype = None
        L.orc_excitations.restype = C.c_int
        L.orc_excitations.argtypes = [_u64p, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_int,
                                      _szp, _szp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_hii.argtypes = [C.c_void_p, _u64p, C.c_size_t, _u64p, C.c_size_t, C.c_int, C.c_int, _f64p,
                              C.c_size_t, C.c_size_t]
        tab = [_szp, _u64p, _i32p] * 4
        L.orc_mult.argtypes = ([C.c_void_p, _u64p, C.c_size_t, _u64p, C.c_size_t, C.c_int, C.c_int] + tab
                               + [_f64p, _f64p, _f64p, C.c_size_t, C.c_size_t])
        L.orc_hamiltonian_offdiag.restype = C.c_size_t
        L.orc_hamiltonian_offdiag.argtypes = ([C.c_void_p, _u64p, C.c_size_t, _u64p, C.c_size_t, C.c_int, C.c_int]
                                              + tab + [C.c_void_p, C.c_void_p, C.c_void_p])
        L.orc_davidson.restype = C.c_int
        L.orc_davidson.argtypes = ([C.c_void_p, _u64p, C.c_size_t, _u64p, C.c_size_t, C.c_int, C.c_int] + tab
                                   + [_f64p, _f64p, C.c_int, C.c_int, C.c_double,
                                      C.POINTER(C.c_double), C.POINTER(C.c_double)])
        L.orc_density.argtypes = [_u64p, C.c_size_t, _u64p, C.c_size_t, C.c_int, C.c_int, C.c_int, _f64p, _f64p]
        L.orc_correlation.argtypes = ([_u64p, C.c_size_t, _u64p, C.c_size_t, C.c_int, C.c_int, C.c_int] + tab
                                      + [_f64p, _f64p, _f64p])
        L.orc_inner.restype = C.c_double
        L.orc_inner.argtypes = [_f64p, _f64p, C.c_size_t]
        L.orc_algebra_step.restype = None
        L.orc_algebra_step.argtypes = [_f64p, _f64p, _f64p, _f64p, _f64p, C.c_size_t, C.c_int]
        L.orc_symeig.argtypes = [C.c_int, _f64p, C.c_int, _f64p]
        _lib = L
    return _lib


class SpinTables:
    """CSR excitation lists of one spin, in the reference helper layout."""

    def __init__(self, off_s, ket_s, cran_s, off_d, ket_d, cran_d):
        self.off_s, self.ket_s, self.cran_s = off_s, ket_s, cran_s
        self.off_d, self.ket_d, self.cran_d = off_d, ket_d, cran_d

    def args(self):
        return [self.off_s, self.ket_s, self.cran_s, self.off_d, self.ket_d, self.cran_d]


def excitations(words: np.ndarray, norb: int, bit_length: int, spin: int) -> SpinTables:
    L = lib()
    words = np.ascontiguousarray(words, dtype=np.uint64)
    n, nw = words.shape
    off_s = np.zeros(n + 1, dtype=np.uintp)
    off_d = np.zeros(n + 1, dtype=np.uintp)
    L.orc_excitations(words.ravel(), n, nw, bit_length, norb, spin, off_s, off_d, None, None, None, None)
    ns, nd = int(off_s[-1]), int(off_d[-1])
    ket_s = np.zeros(max(ns, 1), dtype=np.uint64)
    cran_s = np.zeros(max(2 * ns, 1), dtype=np.int32)
    ket_d = np.zeros(max(nd, 1), dtype=np.uint64)
    cran_d = np.zeros(max(4 * nd, 1), dtype=np.int32)
    rc = L.orc_excitations(words.ravel(), n, nw, bit_length, norb, spin, off_s, off_d,
                           ket_s.ctypes.data, cran_s.ctypes.data, ket_d.ctypes.data, cran_d.ctypes.data)
    if rc != 0:
        raise ValueError("strings with different popcounts in one list")
    return SpinTables(off_s, ket_s[:ns] if ns else ket_s, cran_s, off_d, ket_d[:nd] if nd else ket_d, cran_d)


class Oracle:
    """The reference algorithm on one problem (strings are uint64, L <= 64)."""

    def __init__(self, norb, h1, eri, ecore, astr, bstr, bit_length: int = 20):
        from sbd_gb300.strings import to_words
        self.norb = int(norb)
        self.bit_length = int(bit_length)
        self.astr = np.asarray(astr, dtype=np.uint64)
        self.bstr = np.asarray(bstr, dtype=np.uint64)
        self.aw = np.ascontiguousarray(to_words(self.astr, self.norb, self.bit_length))
        self.bw = np.ascontiguousarray(to_words(self.bstr, self.norb, self.bit_length))
        self.words = self.aw.shape[1]
        self.na, self.nb = self.astr.size, self.bstr.size
        self.N = self.na * self.nb
        self._h1 = np.ascontiguousarray(h1, dtype=np.float64).ravel()
        self._eri = np.ascontiguousarray(eri, dtype=np.float64)
        self.ints = lib().orc_ints_create(self.norb, float(ecore), self._h1, self._eri)
        self.ta = excitations(self.aw, self.norb, self.bit_length, 0)
        self.tb = excitations(self.bw, self.norb, self.bit_length, 1)
        self._hii = None

    @classmethod
    def from_problem(cls, p, bit_length: int = 20):
        return cls(p.norb, p.ints.h1, p.ints.eri, p.ints.ecore, p.astr, p.bstr, bit_length)

    def __del__(self):
        if getattr(self, "ints", None) and _lib is not None:
            _lib.orc_ints_destroy(self.ints)
            self.ints = None

    def _head(self):
        return [self.ints, self.aw.ravel(), self.na, self.bw.ravel(), self.nb, self.words, self.bit_length]

    def _tabs(self):
        return self.ta.args() + self.tb.args()

    def hii(self, rows=None) -> np.ndarray:
        """Diagonal; with rows=(r0, r1) only those bra alpha rows are filled."""
        if rows is not None:
            h = np.zeros(self.N)
            lib().orc_hii(self.ints, self.aw.ravel(), self.na, self.bw.ravel(), self.nb, self.words,
                          self.bit_length, h, rows[0], rows[1])
            return h
        if self._hii is None:
            h = np.zeros(self.N)
            lib().orc_hii(self.ints, self.aw.ravel(), self.na, self.bw.ravel(), self.nb, self.words,
                          self.bit_length, h, 0, self.na)
            self._hii = h
        return self._hii

    def mult(self, C_in: np.ndarray, out: np.ndarray | None = None, rows=None, hii=None) -> np.ndarray:
        """sigma += H C (the reference accumulates into its output); rows=(r0, r1)
        restricts the bra alpha rows."""
        c = np.ascontiguousarray(C_in, dtype=np.float64).ravel()
        s = np.zeros(self.N) if out is None else out
        r0, r1 = (0, self.na) if rows is None else rows
        h = self.hii() if hii is None else hii
        lib().orc_mult(*self._head(), *self._tabs(), h, c, s, r0, r1)
        return s

    def sigma(self, C_in: np.ndarray) -> np.ndarray:
        return self.mult(C_in)

    def hamiltonian(self):
        """Sparse H (scipy CSR) including the diagonal."""
        import scipy.sparse as sp
        nnz = lib().orc_hamiltonian_offdiag(*self._head(), *self._tabs(), None, None, None)
        rows = np.zeros(max(nnz, 1), dtype=np.int64)
        cols = np.zeros(max(nnz, 1), dtype=np.int64)
        vals = np.zeros(max(nnz, 1))
        lib().orc_hamiltonian_offdiag(*self._head(), *self._tabs(), rows.ctypes.data, cols.ctypes.data,
                                      vals.ctypes.data)
        H = sp.coo_matrix((vals[:nnz], (rows[:nnz], cols[:nnz])), shape=(self.N, self.N)).tocsr()
        H = H + sp.diags(self.hii())
        return H

    def lowest(self, k: int = 1, tol: float = 1e-12) -> np.ndarray:
        """The k lowest eigenvalues of the assembled H (dense for small N)."""
        H = self.hamiltonian()
        if self.N <= 4000:
            w = np.linalg.eigvalsh(H.toarray())
            return w[:k]
        import scipy.sparse.linalg as sla
        w = sla.eigsh(H, k=k, which="SA", tol=tol, return_eigenvectors=False)
        return np.sort(w)

    def davidson(self, max_it=100, max_nb=10, eps=1e-8, W0=None):
        W = np.zeros(self.N) if W0 is None else np.array(W0, dtype=np.float64)
        if W0 is None:
            W[0] = 1.0  # BasisInitVector init 0 (chemistry/tpb/davidson.h:174-177)
        e = C.c_double(0.0)
        r = C.c_double(0.0)
        ns = lib().orc_davidson(*self._head(), *self._tabs(), self.hii(), W, max_it, max_nb, eps,
                                C.byref(e), C.byref(r))
        return e.value, W, ns, r.value

    def density(self, W: np.ndarray) -> np.ndarray:
        """Occupation density [2L] (OccupationDensity, chemistry/tpb/occupation.h:11-95)."""
        out = np.zeros(2 * self.norb)
        lib().orc_density(self.aw.ravel(), self.na, self.bw.ravel(), self.nb, self.words, self.bit_length,
                          self.norb, np.ascontiguousarray(W, dtype=np.float64), out)
        return out

    def correlation(self, W: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """One-particle (2, L*L) and two-particle (4, L^4) RDMs of W in the reference's
        layout (Correlation, chemistry/tpb/correlation.h:379-640)."""
        L = self.norb
        one = np.zeros((2, L * L))
        two = np.zeros((4, L ** 4))
        lib().orc_correlation(self.aw.ravel(), self.na, self.bw.ravel(), self.nb, self.words, self.bit_length,
                              L, *self._tabs(), np.ascontiguousarray(W, dtype=np.float64), one, two)
        return one, two

    def lanczos(self, max_it=20, num_block=40, eps=1e-12, W0=None):
        """Matrix-free Lanczos of chemistry/tpb/lanczos.h:169-320 (restart from the
        Ritz vector, no reorthogonalisation; stop when the lowest Ritz value moves
        by less than eps or the off-diagonal falls below eps).  Returns (E0, W)."""
        N = self.N
        W = np.zeros(N) if W0 is None else np.array(W0, dtype=np.float64)
        if W0 is None:
            W[0] = 1.0
        E = np.zeros(1)
        for _ in range(max_it):
            A = np.zeros((num_block, num_block))
            Cs = [W.copy()]
            HC = np.zeros(N)
            n, stop, E_old = 0, False, 1.0e8
            for ib in range(num_block):
                n += 1
                self.mult(Cs[ib], HC)
                A[ib, ib] = lib().orc_inner(np.ascontiguousarray(Cs[ib]), HC, N)
                E, U = np.linalg.eigh(A[:n, :n])
                if abs(E[0] - E_old) < eps:
                    stop = True
                    break
                E_old = E[0]
                if ib + 1 == num_block:
                    break
                HC -= A[ib, ib] * Cs[ib]
                nxt = HC.copy()
                b = np.sqrt(lib().orc_inner(nxt, nxt, N))
                nxt /= b
                A[ib, ib + 1] = A[ib + 1, ib] = b
                Cs.append(nxt)
                if abs(b) < eps:
                    break
                HC = -b * Cs[ib]
            E, U = np.linalg.eigh(A[:n, :n])
            W = sum(U[j, 0] * Cs[j] for j in range(n))
            if stop:
                break
        return float(E[0]), W

    def carry_over(self, W: np.ndarray, carryover_type: int, ratio: float = 0.0, threshold: float = 0.01) -> dict:
        """The carry-over branch of sbd::tpb::diag (chemistry/tpb/sbdiag.h:749-796):
        CarryOverAdet/Bdet (rdmat.h:62-135, 189-261) and SinglesExtendHalfdets
        (extend.h:13-318), restated with plain loops."""
        M = np.asarray(W, dtype=np.float64).reshape(self.na, self.nb)
        L = self.norb

        def weights(rows):  # D[i] = sum_j |W|^2, accumulated in order
            out = []
            for r in rows:
                acc = 0.0
                for x in r:
                    acc += x * x
                out.append(acc)
            return out

        def ranked(D):
            return sorted(range(len(D)), key=lambda i: (-D[i], i))

        def by_threshold(strs, D):
            order, acc, kept = ranked(D), 0.0, []
            for i in order:
                kept.append(int(strs[i]))
                if acc + D[i] > 1.0 - threshold:
                    break
                acc += D[i]
            return kept

        def by_count(strs, D, n):
            order = ranked(D)[:n]
            acc = 0.0
            for i in order:
                acc += D[i]
            return [int(strs[i]) for i in order], 1.0 - acc

        def extend(strs):
            out = set()
            for v in strs:
                out.add(v)
                for i in range(L):
                    if v >> i & 1:
                        for a in range(L):
                            if not v >> a & 1:
                                out.add(v ^ (1 << i) ^ (1 << a))
            return sorted(out)

        res = {}
        if carryover_type in (1, 2):
            Da, Db = weights(M), weights(M.T)
            if ratio == 0.0:
                a, b = by_threshold(self.astr, Da), by_threshold(self.bstr, Db)
            else:
                a, res["truncated_a"] = by_count(self.astr, Da, int(ratio * self.na))
                b, res["truncated_b"] = by_count(self.bstr, Db, int(ratio * self.nb))
            if carryover_type == 2:
                a, b = extend(a), extend(b)
        else:
            W2 = M * M
            sel = W2 > threshold
            res["total_weight"] = float(sum(W2[sel].tolist()))
            a = extend([int(self.astr[i]) for i in range(self.na) if sel[i].any()])
            b = extend([int(self.bstr[j]) for j in range(self.nb) if sel[:, j].any()])
        res["alpha"] = np.array(a, dtype=np.uint64)
        res["beta"] = np.array(b, dtype=np.uint64)
        return res

    def energy(self, W: np.ndarray) -> float:
        """<W|H|W> as the reference reports it after the solve (sbdiag.h:488-526)."""
        HW = self.mult(W)
        return lib().orc_inner(np.ascontiguousarray(W), HW, self.N)


def parse_sbdref(path: str) -> dict:
    """Reads the tagged binary records written by oracle/_ref/sbdref."""
    out: dict = {}
    codes = {"Q": np.uint64, "i": np.int32, "d": np.float64}
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        n = int.from_bytes(data[pos:pos + 4], "little")
        pos += 4
        name = data[pos:pos + n].decode()
        pos += n
        code = chr(data[pos])
        pos += 1
        cnt = int.from_bytes(data[pos:pos + 8], "little")
        pos += 8
        dt = np.dtype(codes[code])
        arr = np.frombuffer(data[pos:pos + cnt * dt.itemsize], dtype=dt).copy()
        pos += cnt * dt.itemsize
        if name in out:
            prev = out[name]
            out[name] = np.concatenate([np.atleast_1d(prev), arr])
        else:
            out[name] = arr
    return out
