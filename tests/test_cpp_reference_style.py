"""A caller written against the reference's namespace sbd (its argument lists
and types: det_vector, TaskHelpers, oneInt/twoInt, MPI communicators),
compiled against include/sbdgb/sbd_compat.hpp with only a namespace alias,
using the project's single-rank MPI stand-in (oracle/ref/mpi.h).  The CPU test
checks that it compiles and links; the GPU tests run it on the reference's H2O
and N2 inputs against the energies the reference publishes."""
import os
import re
import subprocess

import numpy as np
import pytest

from golden_io import molecule
from sbd_gb300 import build
from sbd_gb300.fcidump import Integrals, write_fcidump
from sbd_gb300.strings import write_strings

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def compile_program(out: str) -> str:
    lib = build.build()
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "oracle", "ref"),
                    os.path.join(ROOT, "tests", "cpp", "tpb_reference_style.cpp"), "-L" + os.path.dirname(lib),
                    "-lsbdgb", "-Wl,-rpath," + os.path.dirname(lib), "-o", out], check=True)
    return out


def test_reference_style_caller_compiles(tmp_path):
    exe = compile_program(str(tmp_path / "tpb_reference_style"))
    assert os.access(exe, os.X_OK)


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    return compile_program(str(tmp_path_factory.mktemp("cppref") / "tpb_reference_style"))


def _inputs(tmp_path, mol, label):
    m = molecule(mol)
    ints = Integrals(norb=m.norb, nelec=m.nelec, ecore=m.ecore, h1=m.h1, eri=m.eri)
    write_fcidump(str(tmp_path / "fcidump.txt"), ints)
    write_strings(str(tmp_path / "a.txt"), m.strings[label][::-1], m.norb)  # unsorted on disk
    return m


FLAGS = ["--block", "16", "--iteration", "60", "--tolerance", "1e-9"]


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["diag", "diagfile", "inner"])
@pytest.mark.parametrize("mol,label", [("h2o", "1em3"), ("n2", "1em3")])
def test_reference_style_caller_energy(exe, tmp_path, mode, mol, label):
    m = _inputs(tmp_path, mol, label)
    r = subprocess.run([exe, "--mode", mode, "--fcidump", str(tmp_path / "fcidump.txt"), "--adetfile",
                        str(tmp_path / "a.txt"), *FLAGS], capture_output=True, text=True, check=True)
    key = "Davidson energy" if mode == "inner" else "Energy"
    e = float(re.search(key + r" = ([-0-9.eE+]+)", r.stdout).group(1))
    assert abs(e - m.energy[label]) <= 1e-8, r.stdout
    if mode == "diag":
        n = float(re.search(r"electrons = ([-0-9.eE+]+)", r.stdout).group(1))
        assert abs(n - m.nelec) < 1e-8
    if mode == "inner":
        d = float(re.search(r"MultBase relative difference = ([-0-9.eE+]+)", r.stdout).group(1))
        assert d <= 1e-14
