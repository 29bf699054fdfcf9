"""Loading of the golden fixtures produced by tests/golden/make_golden.py."""
from __future__ import annotations

import glob
import os

import numpy as np

from sbd_gb300.generators import eri_from_factors

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names() -> list[str]:
    """The synthetic reference-harness cases (molecules.npz holds the molecular sets)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if os.path.basename(p) != "molecules.npz")


class Case:
    def __init__(self, name: str):
        d = np.load(os.path.join(GOLDEN, name + ".npz"))
        self.name = name
        self.d = d
        self.norb = int(d["norb"])
        self.ecore = float(d["ecore"])
        self.h1 = d["h1"]
        self.eri = eri_from_factors(d["factors"])
        self.astr = d["astr"].astype(np.uint64)
        self.bstr = d["bstr"].astype(np.uint64)
        self.C = d["C"]
        self.hii = d["hii"]
        self.sigma = d["sigma"]
        self.energy = float(d["energy"])
        self.lowest = d["lowest"]
        self.irreducible = bool(d["irreducible"])
        self.density_c = d["density_c"]
        self.lanczos_energy = float(d["lanczos_energy"])
        self.rdm1 = d["rdm1"] if "rdm1" in d.files else None
        self.rdm2 = d["rdm2"] if "rdm2" in d.files else None

    def tables(self, spin: str) -> dict:
        t = "a" if spin in ("a", 0, "alpha") else "b"
        return {k: self.d[f"{t}_{k}"] for k in ("off_s", "ket_s", "cran_s", "off_d", "ket_d", "cran_d")}


def load(name: str) -> Case:
    return Case(name)


def max_rel(x: np.ndarray, ref: np.ndarray) -> float:
    den = max(float(np.abs(ref).max()), 1e-300)
    return float(np.abs(np.asarray(x) - np.asarray(ref)).max()) / den


class Molecule:
    """One molecule of tests/golden/molecules.npz (written by make_molecules.py
    from the reference's data/ directory): integrals, and per string list the
    strings (alpha = beta) and the energy the reference publishes for it."""

    def __init__(self, d, name: str):
        self.name = name
        self.norb = int(d[f"{name}/norb"])
        self.nelec = int(d[f"{name}/nelec"])
        self.ecore = float(d[f"{name}/ecore"])
        self.h1 = d[f"{name}/h1"]
        self.eri = d[f"{name}/eri"]
        self.labels = [str(x) for x in d[f"{name}/labels"]]
        self.strings = {lb: d[f"{name}/{lb}/strings"].astype(np.uint64) for lb in self.labels}
        self.energy = {lb: float(d[f"{name}/{lb}/energy"]) for lb in self.labels}
        self.source = {lb: str(d[f"{name}/{lb}/source"]) for lb in self.labels}


def molecule(name: str) -> Molecule:
    with np.load(os.path.join(GOLDEN, "molecules.npz")) as d:
        return Molecule(d, name)
