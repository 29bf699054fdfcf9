"""The batched solver (sbdgb_batch_davidson): all problems in lock step, one
captured graph per iteration; same energies as the regular solver and the
assembled Hamiltonian, in FP64 and in the mixed form (FP32 phase, then FP64)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problems(n, seed):
    from sbd_gb300.generators import config2_problem, make_problem
    out = [config2_problem(i, seed=seed) for i in range(n)]
    out += [make_problem(10, 3, 3, 40, 30, seed=seed + 1), make_problem(8, 3, 3, 1, 5, seed=seed + 2),
            make_problem(16, 5, 5, 60, 70, seed=seed + 3)]
    return out


@pytest.mark.parametrize("nroots,precision", [(1, 0), (3, 0), (4, 0), (1, 1), (4, 1)])
def test_batch_matches_single_solves(engine, nroots, precision):
    from sbd_gb300.engine import TPBProblem, batch_davidson
    probs = _problems(6, 11)
    tps = [TPBProblem.from_problem(engine, p) for p in probs]
    for t in tps:
        t.build_tables()
        t.diag_terms()
    try:
        res = batch_davidson(engine, tps, nroots=nroots, max_nb=24, eps=1e-9, want_vectors=True,
                             precision=precision)
        for t, r in zip(tps, res):
            k = min(nroots, t.N)
            single = t.davidson(nroots=k, max_nb=24, eps=1e-9, init=1, want_vectors=False)
            assert r.report["converged"], (t.N, r.report)
            assert np.abs(r.energies[:k] - single.energies).max() < 1e-8
            # Ritz vectors: normalised, Rayleigh quotient = energy
            x = r.vectors[0]
            assert abs(np.dot(x, x) - 1.0) < 1e-8
            assert abs(np.dot(x, t.mult(x)) - r.energies[0]) < 1e-7
    finally:
        for t in tps:
            t.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_against_dense_spectrum(engine, precision):
    from oracle.oracle import Oracle
    from sbd_gb300.engine import TPBProblem, batch_davidson
    from sbd_gb300.generators import make_problem
    probs = [make_problem(10, 3, 3, 50, 45, seed=s) for s in range(4)]
    tps = [TPBProblem.from_problem(engine, p) for p in probs]
    try:
        res = batch_davidson(engine, tps, nroots=2, max_nb=16, eps=1e-10, precision=precision)
        for p, r in zip(probs, res):
            w = np.linalg.eigvalsh(Oracle.from_problem(p).hamiltonian().toarray())
            assert np.abs(r.energies - w[:2]).max() < 1e-8
    finally:
        for t in tps:
            t.close()


def test_mixed_batch_moves_sigma_products_to_fp32(engine):
    """On the norb-12 batch the FP32 phase takes most sigma products: the FP64
    products are fewer than the plain form needs, and energies agree."""
    from sbd_gb300.engine import TPBProblem, batch_davidson
    from sbd_gb300.generators import config2_problem
    probs = [config2_problem(i) for i in range(6)]
    tps = [TPBProblem.from_problem(engine, p) for p in probs]
    try:
        r64 = batch_davidson(engine, tps, nroots=4, max_nb=24, eps=1e-8)
        rmx = batch_davidson(engine, tps, nroots=4, max_nb=24, eps=1e-8, precision=1)
        for a, b in zip(r64, rmx):
            assert a.report["converged"] and b.report["converged"]
            assert np.abs(a.energies - b.energies).max() < 1e-8
            assert b.report["sigma_fp64"] < a.report["sigma_fp64"]
            assert b.report["sigma_calls"] > b.report["sigma_fp64"]
    finally:
        for t in tps:
            t.close()
