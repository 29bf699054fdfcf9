"""Wavefunction files: byte-identical to the reference's SaveWavefunction, and
mapped onto new string lists exactly as its LoadWavefunction does."""
import numpy as np
import pytest

from golden_io import load
from sbd_gb300.wavefunction import RANK_TAG, load_wavefunction, read_wavefunction, save_wavefunction

CASES = ["fci_L8", "open_L10"]


@pytest.mark.parametrize("name", CASES)
def test_save_is_byte_identical(tmp_path, name):
    c = load(name)
    ref = c.d["wf_saved"].tobytes()
    (tmp_path / ("ref" + RANK_TAG)).write_bytes(ref)
    a, b, W = read_wavefunction(str(tmp_path / "ref"))
    assert np.array_equal(a, c.astr) and np.array_equal(b, c.bstr)
    assert abs(np.dot(W, W) - 1.0) < 1e-12
    path = save_wavefunction(str(tmp_path / "ours"), c.astr, c.bstr, c.norb, W)
    assert open(path, "rb").read() == ref


@pytest.mark.parametrize("name", CASES)
def test_saved_vector_is_the_ground_state(tmp_path, name):
    from oracle.oracle import Oracle
    c = load(name)
    (tmp_path / ("ref" + RANK_TAG)).write_bytes(c.d["wf_saved"].tobytes())
    _, _, W = read_wavefunction(str(tmp_path / "ref"))
    o = Oracle(c.norb, c.h1, c.eri, c.ecore, c.astr, c.bstr)
    assert abs(o.energy(W) - c.energy) < 1e-8


@pytest.mark.parametrize("name", CASES)
def test_load_maps_onto_new_lists(tmp_path, name):
    c = load(name)
    (tmp_path / ("ref" + RANK_TAG)).write_bytes(c.d["wf_saved"].tobytes())
    W = load_wavefunction(str(tmp_path / "ref"), c.d["load_astr"], c.d["load_bstr"])
    assert np.abs(W - c.d["loaded_W"]).max() <= 1e-15


def test_round_trip_and_missing_strings(tmp_path):
    rng = np.random.default_rng(3)
    a = np.array(sorted({int(x) for x in rng.integers(1, 1 << 30, 40)}), dtype=np.uint64)
    b = np.array(sorted({int(x) for x in rng.integers(1, 1 << 30, 30)}), dtype=np.uint64)
    W = rng.normal(size=a.size * b.size)
    W /= np.linalg.norm(W)
    save_wavefunction(str(tmp_path / "w"), a, b, 30, W)
    assert np.allclose(load_wavefunction(str(tmp_path / "w"), a, b), W, rtol=0, atol=1e-15)
    # strings absent from the file get zero weight; the rest is renormalised
    a2 = np.sort(np.concatenate([a[::2], np.array([(1 << 30) + 5], dtype=np.uint64)]))
    W2 = load_wavefunction(str(tmp_path / "w"), a2, b)
    M = W.reshape(a.size, b.size)[::2]
    assert abs(np.linalg.norm(W2) - 1.0) < 1e-12
    assert np.allclose(W2.reshape(a2.size, b.size)[:-1], M / np.linalg.norm(M), atol=1e-15)
    assert np.all(W2.reshape(a2.size, b.size)[-1] == 0.0)
