"""The C++ mirror's wavefunction files (include/sbdgb/tpb.hpp) against the
reference's own SaveWavefunction bytes and LoadWavefunction mapping."""
import os
import subprocess

import numpy as np
import pytest

from golden_io import load
from sbd_gb300.wavefunction import RANK_TAG, read_wavefunction

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("wfio") / "wavefunction_io")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "wavefunction_io.cpp"), "-o", out], check=True)
    return out


def _list(path, v):
    with open(path, "w") as f:
        f.write("\n".join(str(int(x)) for x in v) + "\n")


@pytest.mark.parametrize("name", ["fci_L8", "open_L10"])
def test_cpp_save_and_load(exe, tmp_path, name):
    c = load(name)
    ref = c.d["wf_saved"].tobytes()
    (tmp_path / ("ref" + RANK_TAG)).write_bytes(ref)
    a, b, W = read_wavefunction(str(tmp_path / "ref"))
    _list(tmp_path / "a.txt", a)
    _list(tmp_path / "b.txt", b)
    W.tofile(tmp_path / "w.bin")
    subprocess.run([exe, "save", str(tmp_path / "ours"), str(c.norb), str(tmp_path / "a.txt"),
                    str(tmp_path / "b.txt"), str(tmp_path / "w.bin")], check=True)
    assert (tmp_path / ("ours" + RANK_TAG)).read_bytes() == ref
    _list(tmp_path / "la.txt", c.d["load_astr"])
    _list(tmp_path / "lb.txt", c.d["load_bstr"])
    subprocess.run([exe, "load", str(tmp_path / "ref"), str(tmp_path / "la.txt"), str(tmp_path / "lb.txt"),
                    str(tmp_path / "out.bin")], check=True)
    got = np.fromfile(tmp_path / "out.bin", dtype=np.float64)
    assert np.abs(got - c.d["loaded_W"]).max() <= 1e-15
