"""Occupation bit strings: text format, ordering and packing.

The reference stores a spin string as ``ceil(L / bit_length)`` words with
``bit_length`` orbital bits per word (framework/bit_manipulation.h:195-233) and
sorts the list "from the back" (most significant word first) with duplicates
removed (bit_manipulation.h:386-439, chemistry/basic/makedeterminants.h:167-191).
That order is numeric order of the L-bit integer, so this package keeps one
uint64 per string (L <= 64) and sorts numerically: the position of a string in
the sorted array is the reference's determinant index.
"""
from __future__ import annotations

import numpy as np

MAX_ORB = 64


def from_string(s: str, norb: int) -> int:
    """Text -> integer, character s[L-1-i] is orbital i (bit_manipulation.h:219-233)."""
    if len(s) < norb:
        raise ValueError(f"bit string '{s}' shorter than norb={norb}")
    v = 0
    for i in range(norb):
        if s[norb - 1 - i] == "1":
            v |= 1 << i
    return v


def make_string(v: int, norb: int) -> str:
    """Integer -> text, orbital L-1 first (bit_manipulation.h:195-211)."""
    return "".join("1" if (int(v) >> (i - 1)) & 1 else "0" for i in range(norb, 0, -1))


def load_strings(path: str, norb: int) -> np.ndarray:
    """Reads a string file and returns the sorted, duplicate-free uint64 array."""
    if norb > MAX_ORB:
        raise ValueError(f"norb={norb} exceeds {MAX_ORB} orbitals per spin string")
    vals = []
    with open(path, "r") as f:
        for line in f:
            line = line.rstrip("\n")
            vals.append(from_string(line, norb))
    return sort_unique(np.array(vals, dtype=np.uint64))


def write_strings(path: str, strs: np.ndarray, norb: int) -> None:
    with open(path, "w") as f:
        for v in np.asarray(strs, dtype=np.uint64):
            f.write(make_string(int(v), norb) + "\n")


def sort_unique(strs: np.ndarray) -> np.ndarray:
    return np.unique(np.asarray(strs, dtype=np.uint64))


def to_words(strs: np.ndarray, norb: int, bit_length: int = 20) -> np.ndarray:
    """uint64 strings -> reference word layout, shape (n, ceil(L/bit_length))."""
    strs = np.asarray(strs, dtype=np.uint64)
    words = (norb + bit_length - 1) // bit_length
    out = np.zeros((strs.shape[0], words), dtype=np.uint64)
    mask = np.uint64((1 << bit_length) - 1) if bit_length < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
    for w in range(words):
        out[:, w] = (strs >> np.uint64(w * bit_length)) & mask
    return out


def from_words(words: np.ndarray, bit_length: int = 20) -> np.ndarray:
    words = np.asarray(words, dtype=np.uint64)
    if words.ndim == 1:
        words = words[:, None]
    out = np.zeros(words.shape[0], dtype=np.uint64)
    for w in range(words.shape[1]):
        out |= words[:, w] << np.uint64(w * bit_length)
    return out


def popcounts(strs: np.ndarray) -> np.ndarray:
    x = np.asarray(strs, dtype=np.uint64)
    c = np.zeros(x.shape, dtype=np.int64)
    for s in range(64):
        c += ((x >> np.uint64(s)) & np.uint64(1)).astype(np.int64)
    return c
