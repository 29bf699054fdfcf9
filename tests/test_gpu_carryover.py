"""Carry-over through the engine: device string weights and cut counts, host
ranking and extension, against the reference's own selections."""
import numpy as np
import pytest

from golden_io import load
from sbd_gb300.carryover import carry_over
from sbd_gb300.engine import TPBProblem

pytestmark = pytest.mark.gpu
CASES = ["fci_L8", "open_L10", "cfg0_shape_L16"]
RUNS = {"co1t": (1, 0.0, 0.05), "co1r": (1, 0.5, 0.01), "co2": (2, 0.0, 0.2), "co3": (3, 0.0, 1e-4)}


@pytest.mark.parametrize("name", CASES)
def test_carry_over_matches_reference(engine, name):
    c = load(name)
    p = TPBProblem(engine, c.norb, c.astr, c.bstr, c.h1, c.eri, c.ecore)
    p.build_tables()
    p.diag_terms()
    W = c.d["W"]
    M = W.reshape(c.astr.size, c.bstr.size)
    wa, wb = p.string_weights(W)
    assert np.abs(wa - (M * M).sum(1)).max() <= 1e-15 and np.abs(wb - (M * M).sum(0)).max() <= 1e-15
    for tag, (typ, ratio, thr) in RUNS.items():
        r = carry_over(p, W, typ, ratio, thr)
        assert np.array_equal(r.alpha, c.d[f"{tag}_a"]), tag
        assert np.array_equal(r.beta, c.d[f"{tag}_b"]), tag
        if typ == 3:
            assert abs(r.total_weight - float(c.d["co3_total_weight"])) <= 1e-13
        if tag == "co1r":
            assert abs(r.truncated_a - float(c.d["co1r_truncated_a"])) <= 1e-13
    p.close()
