"""Seeded synthetic problems with the shapes of the benchmark configurations.

RNG: numpy ``Generator(PCG64(seed))``; integrals and each string list get
their own child streams from ``SeedSequence(seed)`` so that changing one list
size does not change the integrals.

Integrals (every configuration):
  * h1 symmetric, diagonal ``linspace(-2, 1, L)`` (ascending), off-diagonal
    N(0, 0.05);
  * ERI ``(ij|kl) = sum_{l<32} B^l_ij B^l_kl`` with B^l symmetric, entries
    N(0, 0.1) plus 0.3 on the diagonal -- positive semi-definite and 8-fold
    symmetric;
  * core energy 0.
Strings: ``n`` occupied orbitals drawn without replacement with weights
``w_p = exp(-p / tau)``, ``tau = L / 4``; duplicates dropped until the
requested count is reached; sorted ascending.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from itertools import combinations

import numpy as np

from .fcidump import Integrals


@dataclass
class Problem:
    """One TPB selected-CI problem: integrals plus sorted alpha/beta strings."""

    ints: Integrals
    astr: np.ndarray
    bstr: np.ndarray
    nalpha: int
    nbeta: int
    meta: dict = field(default_factory=dict)

    @property
    def norb(self) -> int:
        return self.ints.norb

    @property
    def ndet(self) -> int:
        return int(self.astr.size) * int(self.bstr.size)


def eri_from_factors(Bp: np.ndarray) -> np.ndarray:
    """8-fold packed ERI from pair factors: (P|Q) = sum_l Bp[l, P] * Bp[l, Q].

    Summed element-wise in a fixed order (no BLAS), so the result is the same
    bit pattern on every platform.
    """
    Bp = np.asarray(Bp, dtype=np.float64)
    npair = Bp.shape[1]
    P, Q = np.tril_indices(npair)
    eri = np.zeros(P.size)
    for l in range(Bp.shape[0]):
        eri += Bp[l, P] * Bp[l, Q]
    out = np.empty_like(eri)
    out[P * (P + 1) // 2 + Q] = eri
    return out


def make_factors(norb: int, rng: np.random.Generator, nchol: int = 32) -> np.ndarray:
    """Bp[l, P] = B^l_ij over packed pairs P = (i >= j); B^l symmetric, N(0, 0.1) + 0.3 I."""
    L = norb
    ii, jj = np.tril_indices(L)  # packed pair order (i >= j)
    Bp = np.empty((nchol, ii.size))
    for c in range(nchol):
        B = rng.normal(0.0, 0.1, size=(L, L))
        B = np.triu(B) + np.triu(B, 1).T
        B[np.diag_indices(L)] += 0.3
        Bp[c] = B[ii, jj]
    return Bp


def make_h1(norb: int, rng: np.random.Generator) -> np.ndarray:
    L = norb
    h1 = rng.normal(0.0, 0.05, size=(L, L))
    h1 = np.triu(h1, 1)
    h1 = h1 + h1.T
    h1[np.diag_indices(L)] = np.linspace(-2.0, 1.0, L)
    return h1


def make_integrals(norb: int, nelec: int, rng: np.random.Generator, nchol: int = 32) -> Integrals:
    h1 = make_h1(norb, rng)
    Bp = make_factors(norb, rng, nchol)
    ints = Integrals(norb=norb, nelec=nelec, ecore=0.0, h1=h1, eri=eri_from_factors(Bp))
    ints.factors = Bp
    return ints


def draw_strings(norb: int, nocc: int, count: int, rng: np.random.Generator) -> np.ndarray:
    """``count`` distinct popcount-``nocc`` strings, sorted ascending (uint64)."""
    total = math.comb(norb, nocc)
    if count > total:
        raise ValueError(f"only {total} strings with {nocc} of {norb} orbitals exist")
    w = np.exp(-np.arange(norb) / (norb / 4.0))
    if count * 2 >= total:
        # dense regime: weight every combination and sample without replacement
        combos = np.array(list(combinations(range(norb), nocc)), dtype=np.int64)
        cw = np.prod(w[combos], axis=1)
        pick = rng.choice(total, size=count, replace=False, p=cw / cw.sum())
        vals = np.zeros(count, dtype=np.uint64)
        for c in range(nocc):
            vals |= np.uint64(1) << combos[pick, c].astype(np.uint64)
        return np.sort(vals)
    p = w / w.sum()
    seen: set[int] = set()
    out = []
    while len(out) < count:
        batch = max(64, 2 * (count - len(out)))
        for _ in range(batch):
            occ = rng.choice(norb, size=nocc, replace=False, p=p)
            v = 0
            for o in occ:
                v |= 1 << int(o)
            if v not in seen:
                seen.add(v)
                out.append(v)
                if len(out) == count:
                    break
    return np.sort(np.array(out, dtype=np.uint64))


def make_problem(norb: int, nalpha: int, nbeta: int, n_astr: int, n_bstr: int | None = None,
                 seed: int = 0, closed_shell: bool = False, nchol: int = 32) -> Problem:
    """Synthetic problem.  ``closed_shell`` reuses the alpha list for beta."""
    ss = np.random.SeedSequence(seed)
    s_int, s_a, s_b = ss.spawn(3)
    ints = make_integrals(norb, nalpha + nbeta, np.random.Generator(np.random.PCG64(s_int)), nchol)
    astr = draw_strings(norb, nalpha, n_astr, np.random.Generator(np.random.PCG64(s_a)))
    if closed_shell:
        bstr = astr.copy()
    else:
        nb = n_astr if n_bstr is None else n_bstr
        bstr = draw_strings(norb, nbeta, nb, np.random.Generator(np.random.PCG64(s_b)))
    meta = {"seed": seed, "rng": "numpy PCG64 via SeedSequence.spawn(3)", "nchol": nchol,
            "closed_shell": closed_shell}
    return Problem(ints, astr, bstr, nalpha, nbeta, meta)


# --- the benchmark configurations ------------------------------------------

def config0(seed: int = 0) -> Problem:
    """norb 16, 5+5 electrons, 800 closed-shell strings (N = 640,000)."""
    return make_problem(16, 5, 5, 800, seed=seed, closed_shell=True)


def config1(seed: int = 1) -> Problem:
    """norb 36, 12+12 electrons, 6000 alpha and 6000 beta strings (N = 36M)."""
    return make_problem(36, 12, 12, 6000, 6000, seed=seed)


def config2_problem(index: int, seed: int = 2) -> Problem:
    """One of the 4096 batched tiny problems: norb 12, 4+4, counts log-uniform in [50, 495]."""
    rng = np.random.Generator(np.random.PCG64(np.random.SeedSequence([seed, index])))
    na = int(round(math.exp(rng.uniform(math.log(50), math.log(495)))))
    nb = int(round(math.exp(rng.uniform(math.log(50), math.log(495)))))
    return make_problem(12, 4, 4, na, nb, seed=int(rng.integers(1 << 62)))


def config3(seed: int = 3) -> Problem:
    """norb 58, 16+16 electrons, 12000 x 12000 strings (N = 144M)."""
    return make_problem(58, 16, 16, 12000, 12000, seed=seed)


def config4_request(index: int, seed: int = 4) -> tuple[Problem, int]:
    """One serving request: norb in {24,32,40,48}, n = round(L/3), counts log-uniform
    in [200, 4000], 1-3 roots.  Returns (problem, nroots)."""
    rng = np.random.Generator(np.random.PCG64(np.random.SeedSequence([seed, index])))
    L = int(rng.choice([24, 32, 40, 48]))
    n = int(round(L / 3))
    na = int(round(math.exp(rng.uniform(math.log(200), math.log(4000)))))
    nb = int(round(math.exp(rng.uniform(math.log(200), math.log(4000)))))
    nroots = int(rng.integers(1, 4))
    return make_problem(L, n, n, na, nb, seed=int(rng.integers(1 << 62))), nroots
