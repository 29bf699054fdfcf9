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


def test_occupation_density(case_oracle):
    c, o = case_oracle
    d = o.density(c.C)
    assert max_rel(d, c.density_c) <= 1e-12
    # alpha and beta occupations sum to the electron counts times |C|^2
    w2 = float(np.dot(c.C, c.C))
    na_e = bin(int(c.astr[0])).count("1")
    nb_e = bin(int(c.bstr[0])).count("1")
    assert abs(d[0::2].sum() - na_e * w2) <= 1e-10 * w2 * na_e
    assert abs(d[1::2].sum() - nb_e * w2) <= 1e-10 * w2 * nb_e


def test_rdms(case_oracle):
    c, o = case_oracle
    if c.rdm1 is None:
        pytest.skip("RDM fixtures are stored for norb <= 12")
    one, two = o.correlation(c.C)
    scale1 = np.abs(c.rdm1).max()
    scale2 = np.abs(c.rdm2).max()
    assert np.abs(one - c.rdm1).max() <= 1e-12 * scale1
    assert np.abs(two - c.rdm2).max() <= 1e-12 * scale2
    # the diagonal of the one-particle RDM is the occupation density
    L = c.norb
    dens = np.empty(2 * L)
    dens[0::2] = np.diag(one[0].reshape(L, L))
    dens[1::2] = np.diag(one[1].reshape(L, L))
    assert max_rel(dens, c.density_c) <= 1e-12


def test_lanczos_energy(case_oracle):
    c, o = case_oracle
    E, W = o.lanczos(max_it=20, num_block=40, eps=1e-12)
    assert abs(E - c.lanczos_energy) < 1e-8
    if c.irreducible:
        assert abs(E - c.lowest[0]) < 1e-8
