"""Carry-over selection and singles extension (sbd::tpb::diag's carry-over
branch) against the strings the reference itself selected."""
import numpy as np
import pytest

from golden_io import load

CASES = ["fci_L8", "open_L10", "cfg0_shape_L16"]
RUNS = {"co1t": (1, 0.0, 0.05), "co1r": (1, 0.5, 0.01), "co2": (2, 0.0, 0.2), "co3": (3, 0.0, 1e-4)}


def _check(c, tag, a, b, extra):
    assert np.array_equal(a.astype(np.uint64), c.d[f"{tag}_a"])
    assert np.array_equal(b.astype(np.uint64), c.d[f"{tag}_b"])
    for key, val in extra.items():
        if val is not None and f"{tag}_{key}" in c.d.files:
            assert abs(val - float(c.d[f"{tag}_{key}"])) <= 1e-14


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("tag", list(RUNS))
def test_oracle_carry_over(name, tag):
    from oracle.oracle import Oracle
    c = load(name)
    o = Oracle(c.norb, c.h1, c.eri, c.ecore, c.astr, c.bstr)
    typ, ratio, thr = RUNS[tag]
    r = o.carry_over(c.d["W"], typ, ratio, thr)
    _check(c, tag, r["alpha"], r["beta"], {k: r.get(k) for k in ("truncated_a", "truncated_b", "total_weight")})


@pytest.mark.parametrize("name", CASES)
def test_host_selection_with_exact_weights(name):
    """The product's host-side ranking and extension, fed weights computed here."""
    from sbd_gb300 import carryover as co
    c = load(name)
    M = c.d["W"].reshape(c.astr.size, c.bstr.size)
    wa, wb = (M * M).sum(1), (M * M).sum(0)
    _check(c, "co1t", co.select_threshold(c.astr, wa, 0.05), co.select_threshold(c.bstr, wb, 0.05), {})
    a, ta = co.select_count(c.astr, wa, int(0.5 * c.astr.size))
    b, tb = co.select_count(c.bstr, wb, int(0.5 * c.bstr.size))
    assert np.array_equal(a, c.d["co1r_a"]) and np.array_equal(b, c.d["co1r_b"])
    assert abs(ta - float(c.d["co1r_truncated_a"])) < 1e-12 and abs(tb - float(c.d["co1r_truncated_b"])) < 1e-12
    a2 = co.extend_singles(co.select_threshold(c.astr, wa, 0.2), c.norb)
    b2 = co.extend_singles(co.select_threshold(c.bstr, wb, 0.2), c.norb)
    assert np.array_equal(a2, c.d["co2_a"]) and np.array_equal(b2, c.d["co2_b"])
