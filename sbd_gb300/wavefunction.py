"""Wavefunction files in the reference's format (the SQD loop's hand-over between
iterations).

SaveWavefunction (chemistry/tpb/restart.h:21-67) at communicator size 1
writes one file, the name followed by the six-digit rank tag "000000":

    size_t na, size_t nb, size_t det_length,
    na strings x det_length words, nb strings x det_length words,
    na*nb doubles (W[ia*nb + ib])

with a string stored in the reference's word layout (orbital p in word
p / bit_length, bit p % bit_length; framework/bit_manipulation.h:195-233).

LoadWavefunction (restart.h:415-660) maps a saved vector onto the current
string lists: the coefficient of a saved (alpha, beta) pair lands on the
determinant with the same two strings, pairs whose strings are no longer in
the lists are dropped, and the result is normalised.
"""
from __future__ import annotations

import numpy as np

from .strings import from_words, to_words

RANK_TAG = "000000"


def save_wavefunction(name: str, astr, bstr, norb: int, W, bit_length: int = 20) -> str:
    """Writes W over the sorted lists astr x bstr; returns the file written."""
    a = np.asarray(astr, dtype=np.uint64)
    b = np.asarray(bstr, dtype=np.uint64)
    W = np.ascontiguousarray(W, dtype=np.float64).ravel()
    if W.size != a.size * b.size:
        raise ValueError("W does not match the string lists")
    aw, bw = to_words(a, norb, bit_length), to_words(b, norb, bit_length)
    path = name + RANK_TAG
    with open(path, "wb") as f:
        np.array([a.size, b.size, aw.shape[1]], dtype=np.uint64).tofile(f)
        aw.astype(np.uint64).tofile(f)
        bw.astype(np.uint64).tofile(f)
        W.tofile(f)
    return path


def read_wavefunction(name: str, bit_length: int = 20) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """The saved strings (uint64) and vector of one file."""
    with open(name + RANK_TAG, "rb") as f:
        na, nb, dl = (int(x) for x in np.fromfile(f, dtype=np.uint64, count=3))
        aw = np.fromfile(f, dtype=np.uint64, count=na * dl).reshape(na, dl)
        bw = np.fromfile(f, dtype=np.uint64, count=nb * dl).reshape(nb, dl)
        W = np.fromfile(f, dtype=np.float64, count=na * nb)
    if W.size != na * nb:
        raise ValueError("truncated wavefunction file")
    return from_words(aw, bit_length), from_words(bw, bit_length), W


def load_wavefunction(name: str, astr, bstr, bit_length: int = 20) -> np.ndarray:
    """The saved vector mapped onto the lists astr x bstr and normalised."""
    la, lb, lw = read_wavefunction(name, bit_length)
    a = np.asarray(astr, dtype=np.uint64)
    b = np.asarray(bstr, dtype=np.uint64)
    ia = np.searchsorted(a, la)
    ib = np.searchsorted(b, lb)
    ka = (ia < a.size) & (a[np.minimum(ia, a.size - 1)] == la)
    kb = (ib < b.size) & (b[np.minimum(ib, b.size - 1)] == lb)
    W = np.zeros(a.size * b.size)
    sa, sb = np.nonzero(ka)[0], np.nonzero(kb)[0]
    if sa.size and sb.size:
        dst = (ia[sa][:, None] * b.size + ib[sb][None, :]).ravel()
        src = (sa[:, None] * lb.size + sb[None, :]).ravel()
        np.add.at(W, dst, lw[src])
    n = np.sqrt(np.dot(W, W))
    if n > 0:
        W /= n
    return W
