"""Writes tests/golden/molecules.npz from the reference's own molecular datasets.

The reference ships FCIDUMP integrals and selected alpha-string lists for
H2O cc-pVDZ, N2 6-31G and C2H2 cc-pVDZ, with the ground-state energies its TPB
Davidson reaches on each list (data/h2o/README.md:6-9, data/n2/README.md:6-14,
data/c2h2/README.md:6-7).  The solve is closed shell: the beta list is the
alpha list (the reference app reads one string file for both spins when no
beta file is given).

This script reads those files through the project's own FCIDUMP and string
readers (sbd_gb300/fcidump.py, sbd_gb300/strings.py) and stores, per
molecule, h1 (L x L), the 8-fold packed ERI, the core energy, the electron
count, and per string list the sorted uint64 strings and the published
energy.  The GPU machine has no reference tree, so the tests read only this
fixture.

    python tests/golden/make_molecules.py [reference_root]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from sbd_gb300 import fcidump, strings  # noqa: E402

# molecule -> (fcidump, [(label, string file, published energy, source)])
SETS = {
    "h2o": ("data/h2o/fcidump.txt", [
        ("1em3", "data/h2o/h2o-1em3-alpha.txt", -76.23594663, "data/h2o/README.md:6"),
        ("1em4", "data/h2o/h2o-1em4-alpha.txt", -76.24295848, "data/h2o/README.md:7"),
        ("1em5", "data/h2o/h2o-1em5-alpha.txt", -76.24373504, "data/h2o/README.md:8"),
        ("1em6", "data/h2o/h2o-1em6-alpha.txt", -76.24377593, "data/h2o/README.md:9"),
    ]),
    "n2": ("data/n2/fcidump.txt", [
        ("1em3", "data/n2/1em3-alpha.txt", -109.04162110, "data/n2/README.md:6"),
        ("3em4", "data/n2/3em4-alpha.txt", -109.04697304, "data/n2/README.md:7"),
        ("1em4", "data/n2/1em4-alpha.txt", -109.04835269, "data/n2/README.md:8"),
        ("1em5", "data/n2/1em5-alpha.txt", -109.04871934, "data/n2/README.md:10"),
        ("1em6", "data/n2/1em6-alpha.txt", -109.04874139, "data/n2/README.md:12"),
        ("1em7", "data/n2/1em7-alpha.txt", -109.04874198, "data/n2/README.md:14"),
    ]),
    "c2h2": ("data/c2h2/fcidump.txt", [
        ("30k", "data/c2h2/alpha-30k.txt", -77.10918904, "data/c2h2/README.md:6"),
        ("100k", "data/c2h2/alpha-100k.txt", -77.11337996, "data/c2h2/README.md:7"),
    ]),
}


def main(ref_root: str) -> str:
    out = {}
    for mol, (fcd, lists) in SETS.items():
        ints = fcidump.read_integrals(os.path.join(ref_root, fcd))
        out[f"{mol}/norb"] = np.int64(ints.norb)
        out[f"{mol}/nelec"] = np.int64(ints.nelec)
        out[f"{mol}/ecore"] = np.float64(ints.ecore)
        out[f"{mol}/h1"] = ints.h1
        out[f"{mol}/eri"] = ints.eri
        labels = []
        for label, path, energy, source in lists:
            s = strings.load_strings(os.path.join(ref_root, path), ints.norb)
            out[f"{mol}/{label}/strings"] = s
            out[f"{mol}/{label}/energy"] = np.float64(energy)
            out[f"{mol}/{label}/source"] = np.array(source)
            labels.append(label)
        out[f"{mol}/labels"] = np.array(labels)
    path = os.path.join(HERE, "molecules.npz")
    np.savez_compressed(path, **out)
    return path


if __name__ == "__main__":
    print(main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
