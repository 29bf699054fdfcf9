"""FCIDUMP reading/writing and integral setup.

Restates the reference's loader and integral layout:

* ``load_fcidump`` follows ``sbd::LoadFCIDump`` (framework/fcidump.h:29-95):
  blank lines and lines starting with ``!`` are skipped; header text is
  accumulated (with ``&FCI`` removed) until a line containing ``&END`` (that
  line itself is dropped); the header is split on ``,`` into ``KEY=VALUE``
  tokens; every later line is ``value i j k l``.
* ``setup_integrals`` follows ``sbd::SetupIntegrals`` for the restricted
  (default) build (chemistry/basic/makeintegrals.h:123-174): ``i=j=k=l=0`` is
  the core energy, ``k=l=0`` a one-body element written to (i,j) and (j,i), and
  anything else a two-body element stored once in the 8-fold packed array
  (chemistry/basic/integrals.h:94-102).  Later lines overwrite earlier ones.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Integrals:
    """Spatial-orbital integrals in the reference's storage order.

    ``h1`` is the (L, L) one-body matrix, ``eri`` the 8-fold packed two-body
    array of length B(B+1)/2 with B = L(L+1)/2, ``ecore`` the constant.
    """

    norb: int
    nelec: int
    ecore: float
    h1: np.ndarray
    eri: np.ndarray
    ms2: int = 0

    @property
    def n_pair(self) -> int:
        return self.norb * (self.norb + 1) // 2


def pair_index(i, j):
    """Packed index of the unordered pair (i, j) (integrals.h:97-98)."""
    i = np.asarray(i, dtype=np.int64)
    j = np.asarray(j, dtype=np.int64)
    a = np.maximum(i, j)
    b = np.minimum(i, j)
    return a * (a + 1) // 2 + b


def eri_index(i, j, k, l):
    """8-fold packed index of (ij|kl) in spatial orbitals (integrals.h:94-102)."""
    ij = pair_index(i, j)
    kl = pair_index(k, l)
    a = np.maximum(ij, kl)
    b = np.minimum(ij, kl)
    return a * (a + 1) // 2 + b


def load_fcidump(path: str) -> tuple[dict, np.ndarray]:
    """Returns (header dict, (n, 5) array of value, i, j, k, l rows in file order)."""
    header_text = []
    body = []
    in_header = True
    with open(path, "r") as f:
        for line in f:
            line = line.rstrip("\n")
            if not line or line[0] == "!":
                continue
            if in_header:
                if "&END" in line:
                    in_header = False
                    continue
                pos = line.find("&FCI")
                if pos >= 0:
                    line = line[:pos] + line[pos + 4:]
                header_text.append(line)
            else:
                body.append(line)
    header = {}
    for tok in "".join(header_text).split(","):
        if "=" in tok:
            key, value = tok.split("=", 1)
            header[key.strip(" \t")] = value.strip(" \t")
    if body:
        rows = np.array(" ".join(body).split(), dtype=np.float64)
        if rows.size % 5 != 0:
            raise ValueError(f"{path}: integral lines must have 5 fields")
        rows = rows.reshape(-1, 5)
    else:
        rows = np.zeros((0, 5))
    return header, rows


def setup_integrals(header: dict, rows: np.ndarray) -> Integrals:
    if "NORB" not in header:
        raise ValueError("FCIDUMP header has no NORB")
    L = int(header["NORB"])
    nelec = int(header.get("NELEC", "0"))
    ms2 = int(header.get("MS2", "0"))
    npair = L * (L + 1) // 2
    h1 = np.zeros((L, L), dtype=np.float64)
    eri = np.zeros(npair * (npair + 1) // 2, dtype=np.float64)
    ecore = 0.0
    if rows.shape[0] == 0:
        return Integrals(L, nelec, ecore, h1, eri, ms2)
    v = rows[:, 0]
    idx = rows[:, 1:].astype(np.int64)
    i, j, k, l = idx[:, 0], idx[:, 1], idx[:, 2], idx[:, 3]
    if np.any(idx < 0) or np.any(idx > L):
        raise ValueError("FCIDUMP orbital index out of range")
    core = (i == 0) & (j == 0) & (k == 0) & (l == 0)
    one = (~core) & (k == 0) & (l == 0)
    two = ~(core | one)
    if np.any(core):
        ecore = float(v[np.nonzero(core)[0][-1]])
    if np.any(one):
        oi, oj = i[one], j[one]
        if np.any(oi == 0) or np.any(oj == 0):
            # the reference would index one-body storage out of range here
            raise ValueError("FCIDUMP one-body line with a zero orbital index")
        ov = v[one]
        # the reference writes (i,j) then (j,i) for each line in file order
        for a, b, x in zip(oi - 1, oj - 1, ov):
            h1[a, b] = x
            h1[b, a] = x
    if np.any(two):
        ti, tj, tk, tl = i[two], j[two], k[two], l[two]
        if np.any(ti == 0) or np.any(tj == 0) or np.any(tk == 0) or np.any(tl == 0):
            raise ValueError("FCIDUMP two-body line with a zero orbital index")
        p = eri_index(ti - 1, tj - 1, tk - 1, tl - 1)
        tv = v[two]
        # last occurrence wins
        rev_p = p[::-1]
        uniq, first_in_rev = np.unique(rev_p, return_index=True)
        eri[uniq] = tv[::-1][first_in_rev]
    return Integrals(L, nelec, ecore, h1, eri, ms2)


def read_integrals(path: str) -> Integrals:
    header, rows = load_fcidump(path)
    return setup_integrals(header, rows)


def write_fcidump(path: str, ints: Integrals, tol: float = 0.0) -> None:
    """Writes the integrals in the reference's FCIDUMP text form.

    Every unique (ij|kl) with |value| > tol is written once (1-based indices),
    then the upper triangle of h1 as ``v i j 0 0`` and the core energy as
    ``v 0 0 0 0``.  Values use 17 significant digits so the file round-trips.
    """
    L = ints.norb
    lines = [
        f" &FCI NORB={L},NELEC={ints.nelec},MS2={ints.ms2},",
        "  ORBSYM=" + ",".join(["1"] * L) + ",",
        "  ISYM=1,",
        " &END",
    ]
    out = ["\n".join(lines)]
    ii, jj = np.tril_indices(L)
    pi = pair_index(ii, jj)
    order = np.argsort(pi)
    ii, jj = ii[order], jj[order]
    npair = L * (L + 1) // 2
    P, Q = np.tril_indices(npair)
    vals = ints.eri[P * (P + 1) // 2 + Q]
    keep = np.abs(vals) > tol
    P, Q, vals = P[keep], Q[keep], vals[keep]
    body = np.column_stack([vals, ii[P] + 1, jj[P] + 1, ii[Q] + 1, jj[Q] + 1])
    chunks = []
    for row in body:
        chunks.append(f"{row[0]:.17g} {int(row[1])} {int(row[2])} {int(row[3])} {int(row[4])}")
    for a in range(L):
        for b in range(a + 1):
            x = ints.h1[a, b]
            if abs(x) > tol or a == b:
                chunks.append(f"{x:.17g} {a + 1} {b + 1} 0 0")
    chunks.append(f"{ints.ecore:.17g} 0 0 0 0")
    with open(path, "w") as f:
        f.write(out[0] + "\n")
        f.write("\n".join(chunks) + "\n")
