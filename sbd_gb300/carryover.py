"""Carry-over string selection and singles extension between SQD iterations.

After a solve, sbd::tpb::diag (chemistry/tpb/sbdiag.h:749-796) selects the
strings to carry into the next iteration's basis:

  type 1  the dominant strings by weight, where the weight of a string is its
          diagonal half-determinant density sum |W|^2 (rdmat.h:13-60,
          137-187): with ratio == 0 the heaviest strings whose cumulative
          weight first exceeds 1 - threshold (CarryOverAdet, rdmat.h:62-99),
          otherwise the ratio*n heaviest (rdmat.h:101-135), in order of
          decreasing weight;
  type 2  type 1 followed by SinglesExtendHalfdets on the selected strings
          (extend.h:186-318): the selection and all its single excitations,
          sorted, duplicates removed;
  type 3  the strings of the determinants with |W|^2 > threshold, extended by
          their single excitations (extend.h:13-183), sorted.

The weights and the per-string counts come from the device
(sbdgb_string_weights / sbdgb_string_cut_counts); the ranking and the
extension are host work on n strings.  Ties in weight are ranked by string
index (the reference's std::sort leaves their order unspecified).  The
extension assumes equal alpha and beta electron counts, as the reference's
does.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def rank_by_weight(weights: np.ndarray) -> np.ndarray:
    return np.argsort(-np.asarray(weights, dtype=np.float64), kind="stable")


def select_threshold(strs: np.ndarray, weights: np.ndarray, threshold: float) -> np.ndarray:
    """Heaviest strings up to and including the one whose cumulative weight exceeds 1 - threshold."""
    order = rank_by_weight(weights)
    S = np.cumsum(np.asarray(weights, dtype=np.float64)[order])
    imax = min(int(np.searchsorted(S, 1.0 - threshold, side="right")) + 1, order.size)
    return np.asarray(strs, dtype=np.uint64)[order[:imax]]


def select_count(strs: np.ndarray, weights: np.ndarray, kept: int) -> tuple[np.ndarray, float]:
    """The `kept` heaviest strings and the weight left out (1 - their sum)."""
    order = rank_by_weight(weights)[:kept]
    w = np.asarray(weights, dtype=np.float64)[order]
    s = 0.0
    for x in w:  # sequential sum, as the reference accumulates
        s += x
    return np.asarray(strs, dtype=np.uint64)[order], 1.0 - s


def single_excitations(strs: np.ndarray, norb: int) -> np.ndarray:
    """Every string one occupied->empty move away from a string of the list."""
    out = []
    for v in np.asarray(strs, dtype=np.uint64).tolist():
        occ = [i for i in range(norb) if v >> i & 1]
        emp = [a for a in range(norb) if not v >> a & 1]
        out.extend(v ^ (1 << i) ^ (1 << a) for i in occ for a in emp)
    return np.array(out, dtype=np.uint64)


def extend_singles(strs: np.ndarray, norb: int) -> np.ndarray:
    """The strings and all their single excitations, sorted and unique."""
    s = np.asarray(strs, dtype=np.uint64)
    return np.unique(np.concatenate([s, single_excitations(s, norb)]))


@dataclass
class CarryOver:
    alpha: np.ndarray
    beta: np.ndarray
    truncated_a: float | None = None
    truncated_b: float | None = None
    total_weight: float | None = None


def carry_over(problem, W, carryover_type: int, ratio: float = 0.0, threshold: float = 0.01) -> CarryOver:
    """The carry-over strings of sbd::tpb::diag for a solved problem.

    problem: an engine.TPBProblem; W: its ground vector (host array or device pointer)."""
    norb = problem.norb
    if carryover_type in (1, 2):
        wa, wb = problem.string_weights(W)
        if ratio == 0.0:
            res = CarryOver(select_threshold(problem.astr, wa, threshold), select_threshold(problem.bstr, wb, threshold))
        else:
            a, ta = select_count(problem.astr, wa, int(ratio * problem.na))
            b, tb = select_count(problem.bstr, wb, int(ratio * problem.nb))
            res = CarryOver(a, b, ta, tb)
        if carryover_type == 2:
            res.alpha, res.beta = extend_singles(res.alpha, norb), extend_singles(res.beta, norb)
        return res
    if carryover_type == 3:
        ca, cb, total = problem.string_cut_counts(W, threshold)
        return CarryOver(extend_singles(problem.astr[ca > 0], norb), extend_singles(problem.bstr[cb > 0], norb),
                         total_weight=total)
    raise ValueError("carryover_type must be 1, 2 or 3")
