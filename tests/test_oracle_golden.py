"""The CPU oracle reproduces the reference's own outputs (golden fixtures).

This pins the oracle: tables bit-exact, hii and sigma to 1e-12 (max-norm
relative), the reference Davidson energy to 1e-8 Ha, and the assembled
Hamiltonian's spectrum.
"""
import numpy as np
import pytest

from golden_io import load, max_rel, names
from oracle.oracle import Oracle

CASES = names()


@pytest.fixture(scope="module", params=CASES)
def case_oracle(request):
    c = load(request.param)
    return c, Oracle(c.norb, c.h1, c.eri, c.ecore, c.astr, c.bstr)


def test_fixture_set_present():
    assert len(CASES) >= 7


def test_tables_bit_exact(case_oracle):
    c, o = case_oracle
    for spin, t in (("a", o.ta), ("b", o.tb)):
        g = c.tables(spin)
        assert np.array_equal(g["off_s"].astype(np.int64), t.off_s.astype(np.int64))
        assert np.array_equal(g["off_d"].astype(np.int64), t.off_d.astype(np.int64))
        ns, nd = int(g["off_s"][-1]), int(g["off_d"][-1])
        assert np.array_equal(g["ket_s"].astype(np.int64), t.ket_s[:ns].astype(np.int64))
        assert np.array_equal(g["ket_d"].astype(np.int64), t.ket_d[:nd].astype(np.int64))
        assert np.array_equal(g["cran_s"], t.cran_s[:2 * ns])
        assert np.array_equal(g["cran_d"], t.cran_d[:4 * nd])


def test_hii(case_oracle):
    c, o = case_oracle
    assert max_rel(o.hii(), c.hii) <= 1e-12


def test_sigma(case_oracle):
    c, o = case_oracle
    assert max_rel(o.mult(c.C), c.sigma) <= 1e-12


def test_davidson_energy(case_oracle):
    c, o = case_oracle
    E, W, nsig, res = o.davidson(max_it=200, max_nb=12, eps=1e-10)
    assert abs(E - c.energy) < 1e-8
    assert abs(o.energy(W) - c.energy) < 1e-8


def test_assembled_spectrum(case_oracle):
    c, o = case_oracle
    w = o.lowest(len(c.lowest))
    assert np.allclose(w, c.lowest, atol=1e-8, rtol=0)
