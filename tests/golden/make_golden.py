"""Generates the golden fixtures of tests/golden/ from the reference itself.

Each case is a seeded synthetic problem.  It is written out in the
reference's own formats (FCIDUMP, string files), run through oracle/_ref/sbdref
-- the reference's header-only TPB CPU path compiled from its sources by
oracle/Makefile -- and the reference's results are stored:
  * the sorted strings and both spins' excitation tables (helper layout);
  * hii, sigma = H*C for a seeded C, and the ground energy of the reference's
    own Davidson;
  * the three lowest eigenvalues of the explicitly assembled H, whose
    matrix-vector product is checked here against the reference's sigma;
  * the occupation density of C (OccupationDensity), for norb <= 12 the one-
    and two-particle RDMs of C (Correlation), and the ground energy of the
    reference's matrix-free Lanczos (the --method 2 solver);
  * for norb <= 10 the bytes of the reference's SaveWavefunction file of its
    Davidson vector, and that file mapped by LoadWavefunction onto sub-lists
    of the strings (every third alpha and every fourth beta string dropped);
  * for norb <= 16 with equal alpha and beta electron counts, the reference's
    Davidson vector W and the carry-over strings sbd::tpb::diag selects from
    it (types 1 by threshold and by ratio, 2 and 3; sbdiag.h:749-796).
Integrals are stored as h1 plus pair factors (the ERI is rebuilt with
sbd_gb300.generators.eri_from_factors, an order-fixed elementwise sum).

Run from the repository root in a container that has the reference tree:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import REF_BIN, Oracle, build_reference, parse_sbdref  # noqa: E402
from sbd_gb300.fcidump import Integrals, write_fcidump  # noqa: E402
from sbd_gb300.generators import draw_strings, eri_from_factors, make_factors, make_h1  # noqa: E402
from sbd_gb300.strings import from_words, write_strings  # noqa: E402

# name: (norb, n_alpha_elec, n_beta_elec, n_alpha_strings, n_beta_strings (None = same list), nchol, seed)
CASES = {
    "fci_L8": (8, 3, 3, 56, None, 16, 11),
    "open_L10": (10, 3, 3, 60, 50, 16, 5),
    "spin_L12": (12, 4, 3, 70, 90, 16, 7),
    "cfg0_shape_L16": (16, 5, 5, 120, None, 32, 13),
    "wide_L36": (36, 12, 12, 60, 70, 8, 17),
    "wide_L58": (58, 16, 16, 50, 44, 4, 19),
    "full_word_L64": (64, 8, 8, 48, 52, 4, 23),
}


def walk_strings(norb, nocc, count, rng):
    """Strings reached by random single/double excitations from the lowest-orbital
    string (virtuals drawn uniformly, so the top orbital occurs): a connected list,
    like the strings a selected-CI loop keeps around a reference."""
    start = (1 << nocc) - 1
    seen = {start}
    out = [start]
    while len(out) < count:
        base = out[int(rng.integers(len(out)))]
        occ = [i for i in range(norb) if base >> i & 1]
        vir = [i for i in range(norb) if not base >> i & 1]
        k = 1 if rng.random() < 0.4 else 2
        rem = rng.choice(occ, size=k, replace=False)
        add = rng.choice(vir, size=k, replace=False)
        v = base
        for r in rem:
            v &= ~(1 << int(r))
        for a in add:
            v |= 1 << int(a)
        if v not in seen:
            seen.add(v)
            out.append(v)
    return np.sort(np.array(out, dtype=np.uint64))


def dense_strings(norb, nocc, count, rng):
    """Weighted draws for small norb; excitation walks for wide strings so that
    the lists stay connected."""
    if norb <= 16:
        return draw_strings(norb, nocc, count, rng)
    return walk_strings(norb, nocc, count, rng)


def make_case(norb, na_e, nb_e, n_as, n_bs, nchol, seed):
    ss = np.random.SeedSequence(seed)
    s_int, s_a, s_b, s_c = ss.spawn(4)
    rng_i = np.random.Generator(np.random.PCG64(s_int))
    h1 = make_h1(norb, rng_i)
    Bp = make_factors(norb, rng_i, nchol)
    eri = eri_from_factors(Bp)
    ints = Integrals(norb=norb, nelec=na_e + nb_e, ecore=0.25, h1=h1, eri=eri)
    astr = dense_strings(norb, na_e, n_as, np.random.Generator(np.random.PCG64(s_a)))
    if n_bs is None:
        bstr = astr.copy()
    else:
        bstr = dense_strings(norb, nb_e, n_bs, np.random.Generator(np.random.PCG64(s_b)))
    C = np.random.Generator(np.random.PCG64(s_c)).uniform(-1.0, 1.0, astr.size * bstr.size)
    return ints, Bp, astr, bstr, C


def run_case(name, spec, outdir):
    norb, na_e, nb_e, n_as, n_bs, nchol, seed = spec
    ints, Bp, astr, bstr, C = make_case(*spec)
    with tempfile.TemporaryDirectory() as d:
        write_fcidump(f"{d}/fcidump.txt", ints)
        write_strings(f"{d}/a.txt", astr, norb)
        write_strings(f"{d}/b.txt", bstr, norb)
        C.tofile(f"{d}/c.bin")
        args = [REF_BIN, "--fcidump", f"{d}/fcidump.txt", "--adet", f"{d}/a.txt", "--bdet", f"{d}/b.txt",
                "--out", f"{d}/o.bin", "--cvec", f"{d}/c.bin", "--davidson", "1", "--block", "12",
                "--iteration", "200", "--tolerance", "1e-10", "--density", "1", "--lanczos", "1",
                "--lanczos_block", "40", "--lanczos_iteration", "20", "--lanczos_tolerance", "1e-12"]
        if norb <= 12:
            args += ["--rdm", "1"]
        if norb <= 10:
            args += ["--save", f"{d}/wf"]
        subprocess.run(args, check=True, capture_output=True, env=dict(os.environ, OMP_NUM_THREADS="4"))
        r = parse_sbdref(f"{d}/o.bin")
        co = None
        if norb <= 16 and na_e == nb_e:
            co = {"W": r["W"]}
            runs = {"co1t": ["--carryover", "1", "--carryover_threshold", "0.05"],
                    "co1r": ["--carryover", "1", "--carryover_ratio", "0.5"],
                    "co2": ["--carryover", "2", "--carryover_threshold", "0.2"],
                    "co3": ["--carryover", "3", "--carryover_threshold", "1e-4"]}
            base = args[:args.index("--density")]
            for tag, extra in runs.items():
                cargs = [x if x != f"{d}/o.bin" else f"{d}/c_{tag}.bin" for x in base] + extra
                subprocess.run(cargs, check=True, capture_output=True, env=dict(os.environ, OMP_NUM_THREADS="4"))
                cr = parse_sbdref(f"{d}/c_{tag}.bin")
                assert np.array_equal(cr["W"], r["W"]), (name, tag, "Davidson vector differs between runs")
                words = (norb + 19) // 20
                co[f"{tag}_a"] = from_words(cr["co_adet_words"].reshape(-1, words))
                co[f"{tag}_b"] = from_words(cr["co_bdet_words"].reshape(-1, words))
                for key in ("truncated_a", "truncated_b", "total_weight"):
                    if key in cr:
                        co[f"{tag}_{key}"] = np.float64(cr[key][0])
        wf = None
        if norb <= 10:
            wf = {"wf_saved": np.fromfile(f"{d}/wf000000", dtype=np.uint8)}
            la = np.delete(astr, np.arange(0, astr.size, 3))
            lb = np.delete(bstr, np.arange(0, bstr.size, 4))
            write_strings(f"{d}/la.txt", la, norb)
            write_strings(f"{d}/lb.txt", lb, norb)
            largs = [REF_BIN, "--fcidump", f"{d}/fcidump.txt", "--adet", f"{d}/la.txt", "--bdet", f"{d}/lb.txt",
                     "--out", f"{d}/l.bin", "--tables", "0", "--hii", "0", "--load", f"{d}/wf"]
            subprocess.run(largs, check=True, capture_output=True, env=dict(os.environ, OMP_NUM_THREADS="4"))
            lr = parse_sbdref(f"{d}/l.bin")
            wf.update({"load_astr": la, "load_bstr": lb, "loaded_W": lr["loaded_W"]})
    types = {int(r[f"task{k}.type"][0]): k for k in range(3)}
    ka, kb = types[2], types[1]
    out = {
        "norb": np.int64(norb), "ecore": np.float64(ints.ecore), "h1": ints.h1, "factors": Bp,
        "astr": astr, "bstr": bstr, "C": C, "hii": r["hii"], "sigma": r["sigma"],
        "energy": np.float64(r["energy"][0]), "density_c": r["density_c"],
        "lanczos_energy": np.float64(r["lanczos_energy"][0]),
    }
    if wf is not None:
        out.update(wf)
    if co is not None:
        out.update(co)
    if norb <= 12:
        out["rdm1"] = np.stack([r["rdm1_0"], r["rdm1_1"]])
        out["rdm2"] = np.stack([r[f"rdm2_{k}"] for k in range(4)])
    for tag, k, sp in (("a", ka, "Alpha"), ("b", kb, "Beta")):
        out[f"{tag}_off_s"] = r[f"task{k}.SinglesFrom{sp}Offset"]
        out[f"{tag}_ket_s"] = r[f"task{k}.SinglesFrom{sp}"]
        out[f"{tag}_cran_s"] = r[f"task{k}.Singles{sp}CrAn"]
        out[f"{tag}_off_d"] = r[f"task{k}.DoublesFrom{sp}Offset"]
        out[f"{tag}_ket_d"] = r[f"task{k}.DoublesFrom{sp}"]
        out[f"{tag}_cran_d"] = r[f"task{k}.Doubles{sp}CrAn"]
    # the type-0 task repeats the singles lists; they must agree with types 2 and 1
    k0 = types[0]
    assert np.array_equal(r[f"task{k0}.SinglesFromAlpha"], out["a_ket_s"])
    assert np.array_equal(r[f"task{k0}.SinglesFromBeta"], out["b_ket_s"])
    # the assembled H reproduces the reference sigma, so its spectrum is pinned to it
    orc = Oracle(norb, ints.h1, ints.eri, ints.ecore, astr, bstr)
    H = orc.hamiltonian()
    s_h = H @ C
    rel = np.abs(s_h - r["sigma"]).max() / np.abs(r["sigma"]).max()
    assert rel < 1e-12, (name, rel)
    nlow = min(4, astr.size * bstr.size)
    w = np.linalg.eigvalsh(H.toarray()) if H.shape[0] <= 5000 else orc.lowest(nlow)
    out["lowest"] = np.asarray(w[:nlow])
    # the reference Davidson starts on determinant 0, so on a reducible H it
    # finds the lowest root of that determinant's block, which must still be
    # an eigenvalue of H
    from scipy.sparse.csgraph import connected_components
    ncomp, _ = connected_components(abs(H) > 0, directed=False)
    out["irreducible"] = np.bool_(ncomp == 1)
    assert np.min(np.abs(w - out["energy"])) < 1e-8, (name, out["energy"])
    if ncomp == 1:
        assert abs(out["lowest"][0] - out["energy"]) < 1e-8, (name, out["lowest"][0], out["energy"])
    np.savez_compressed(os.path.join(outdir, f"{name}.npz"), **out)
    print(f"{name}: N={astr.size * bstr.size} singles a/b={out['a_ket_s'].size}/{out['b_ket_s'].size} "
          f"doubles a/b={out['a_ket_d'].size}/{out['b_ket_d'].size} E0={out['energy']:.12f} lowest={out['lowest']} "
          f"irreducible={bool(out['irreducible'])}")


def main():
    if not os.path.exists(REF_BIN):
        if build_reference() is None:
            sys.exit("reference tree not available: cannot regenerate fixtures")
    outdir = os.path.dirname(os.path.abspath(__file__))
    names = sys.argv[1:] or list(CASES)
    for n in names:
        run_case(n, CASES[n], outdir)


if __name__ == "__main__":
    main()
