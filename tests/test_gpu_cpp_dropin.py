"""The C++ mirror (include/sbdgb/tpb.hpp) used like the reference app: FCIDUMP
and string files in, diag, <W|H|W> out -- compiled with g++ against the C ABI."""
import os
import re
import subprocess

import numpy as np
import pytest

from golden_io import load
from sbd_gb300 import build
from sbd_gb300.fcidump import Integrals, write_fcidump
from sbd_gb300.strings import write_strings

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    lib = build.build()
    out = str(tmp_path_factory.mktemp("cpp") / "tpb_drop_in")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "tpb_drop_in.cpp"), "-L" + os.path.dirname(lib), "-lsbdgb",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", out], check=True)
    return out


@pytest.mark.parametrize("name", ["open_L10", "wide_L36"])
def test_cpp_drop_in_matches_reference_energy(exe, tmp_path, name):
    c = load(name)
    ints = Integrals(norb=c.norb, nelec=0, ecore=c.ecore, h1=c.h1, eri=c.eri)
    write_fcidump(str(tmp_path / "fcidump.txt"), ints)
    write_strings(str(tmp_path / "a.txt"), c.astr, c.norb)
    write_strings(str(tmp_path / "b.txt"), c.bstr, c.norb)
    r = subprocess.run([exe, "--fcidump", str(tmp_path / "fcidump.txt"), "--adetfile", str(tmp_path / "a.txt"),
                        "--bdetfile", str(tmp_path / "b.txt"), "--block", "12", "--iteration", "200",
                        "--tolerance", "1e-10"], capture_output=True, text=True, check=True)
    e = float(re.search(r"Energy = ([-0-9.eE+]+)", r.stdout).group(1))
    assert abs(e - c.energy) < 1e-8

    na_e, nb_e = bin(int(c.astr[0])).count("1"), bin(int(c.bstr[0])).count("1")
    dens = [float(x) for x in re.search(r"Density sums = (\S+) (\S+)", r.stdout).groups()]
    assert abs(dens[0] - na_e) < 1e-8 and abs(dens[1] - nb_e) < 1e-8


@pytest.mark.parametrize("name", ["fci_L8", "wide_L58"])
def test_cpp_drop_in_lanczos_method(exe, tmp_path, name):
    """--method 2 runs the Lanczos solver, like the reference app."""
    c = load(name)
    ints = Integrals(norb=c.norb, nelec=0, ecore=c.ecore, h1=c.h1, eri=c.eri)
    write_fcidump(str(tmp_path / "fcidump.txt"), ints)
    write_strings(str(tmp_path / "a.txt"), c.astr, c.norb)
    write_strings(str(tmp_path / "b.txt"), c.bstr, c.norb)
    r = subprocess.run([exe, "--fcidump", str(tmp_path / "fcidump.txt"), "--adetfile", str(tmp_path / "a.txt"),
                        "--bdetfile", str(tmp_path / "b.txt"), "--method", "2", "--block", "40", "--iteration", "20",
                        "--tolerance", "1e-12"], capture_output=True, text=True, check=True)
    e = float(re.search(r"Solver energy = ([-0-9.eE+]+)", r.stdout).group(1))
    assert abs(e - c.lanczos_energy) < 1e-8


@pytest.fixture(scope="module")
def exe_full(tmp_path_factory):
    lib = build.build()
    out = str(tmp_path_factory.mktemp("cppfull") / "tpb_diag_full")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "tpb_diag_full.cpp"), "-L" + os.path.dirname(lib), "-lsbdgb",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", out], check=True)
    return out


@pytest.mark.parametrize("name", ["fci_L8", "open_L10"])
def test_cpp_full_diag_carry_over_rdm_and_files(exe_full, tmp_path, name):
    """The reference-shaped diag: carry-over type 2 strings as the reference
    selected them, RDM traces = electron counts, and a saved wavefunction that
    restarts the next solve at the same energy."""
    c = load(name)
    ints = Integrals(norb=c.norb, nelec=0, ecore=c.ecore, h1=c.h1, eri=c.eri)
    write_fcidump(str(tmp_path / "fcidump.txt"), ints)
    write_strings(str(tmp_path / "a.txt"), c.astr, c.norb)
    write_strings(str(tmp_path / "b.txt"), c.bstr, c.norb)
    args = [exe_full, "--fcidump", str(tmp_path / "fcidump.txt"), "--adetfile", str(tmp_path / "a.txt"),
            "--bdetfile", str(tmp_path / "b.txt"), "--block", "12", "--iteration", "200", "--tolerance", "1e-10",
            "--rdm", "1", "--carryover_type", "2", "--carryover_threshold", "0.2"]
    r = subprocess.run(args + ["--savename", str(tmp_path / "wf")], capture_output=True, text=True, check=True)
    e = float(re.search(r"Energy = ([-0-9.eE+]+)", r.stdout).group(1))
    assert abs(e - c.energy) < 1e-8
    co_a = [int(x) for x in re.search(r"CarryOver alpha =(.*)", r.stdout).group(1).split()]
    co_b = [int(x) for x in re.search(r"CarryOver beta =(.*)", r.stdout).group(1).split()]
    assert co_a == [int(x) for x in c.d["co2_a"]] and co_b == [int(x) for x in c.d["co2_b"]]
    na_e, nb_e = bin(int(c.astr[0])).count("1"), bin(int(c.bstr[0])).count("1")
    tr = [float(x) for x in re.search(r"RDM1 traces = (\S+) (\S+)", r.stdout).groups()]
    assert abs(tr[0] - na_e) < 1e-8 and abs(tr[1] - nb_e) < 1e-8
    assert os.path.exists(str(tmp_path / "wf000000"))
    r2 = subprocess.run(args + ["--loadname", str(tmp_path / "wf")], capture_output=True, text=True, check=True)
    e2 = float(re.search(r"Energy = ([-0-9.eE+]+)", r2.stdout).group(1))
    assert abs(e2 - c.energy) < 1e-8


def test_cpp_batch_davidson_matches_reference_energies(tmp_path):
    """BatchDavidson of the C++ mirror: several fixture problems in one call,
    FP64 and mixed, each at the reference's energy."""
    lib = build.build()
    exe = str(tmp_path / "batch_solve")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "batch_solve.cpp"), "-L" + os.path.dirname(lib), "-lsbdgb",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True)
    names = ["fci_L8", "open_L10", "wide_L36"]
    args = []
    for name in names:
        c = load(name)
        ints = Integrals(norb=c.norb, nelec=0, ecore=c.ecore, h1=c.h1, eri=c.eri)
        write_fcidump(str(tmp_path / f"{name}.fcidump"), ints)
        write_strings(str(tmp_path / f"{name}.a"), c.astr, c.norb)
        write_strings(str(tmp_path / f"{name}.b"), c.bstr, c.norb)
        args += [str(tmp_path / f"{name}.fcidump"), str(tmp_path / f"{name}.a"), str(tmp_path / f"{name}.b")]
    r = subprocess.run([exe] + args, capture_output=True, text=True, check=True)
    got = re.findall(r"problem (\d+) fp64 (\S+) mixed (\S+)", r.stdout)
    assert len(got) == len(names)
    for (i, e64, emx), name in zip(got, names):
        ref = load(name).energy
        assert abs(float(e64) - ref) < 1e-8 and abs(float(emx) - ref) < 1e-8, (name, e64, emx, ref)
