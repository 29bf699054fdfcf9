"""The batched solver (sbdgb_batch_davidson): one thread block per problem,
whole Davidson on the device, same energies as the regular solver and the
assembled Hamiltonian."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problems(n, seed):
    from sbd_gb300.generators import config2_problem, make_problem
    out = [config2_problem(i, seed=seed) for i in range(n)]
    out += [make_problem(10, 3, 3, 40, 30, seed=seed + 1), make_problem(8, 3, 3, 1, 5, seed=seed + 2),
            make_problem(16, 5, 5, 60, 70, seed=seed + 3)]
    return out


@pytest.mark.parametrize("nroots", [1, 3, 4])
def test_batch_matches_single_solves(engine, nroots):
    from sbd_gb300.engine import TPBProblem, batch_davidson
    probs = _problems(6, 11)
    tps = [TPBProblem.from_problem(engine, p) for p in probs]
    for t in tps:
        t.build_tables()
        t.diag_terms()
    try:
        res = batch_davidson(engine, tps, nroots=nroots, max_nb=24, eps=1e-9, want_vectors=True)
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


def test_batch_against_dense_spectrum(engine):
    from oracle.oracle import Oracle
    from sbd_gb300.engine import TPBProblem, batch_davidson
    from sbd_gb300.generators import make_problem
    probs = [make_problem(10, 3, 3, 50, 45, seed=s) for s in range(4)]
    tps = [TPBProblem.from_problem(engine, p) for p in probs]
    try:
        res = batch_davidson(engine, tps, nroots=2, max_nb=16, eps=1e-10)
        for p, r in zip(probs, res):
            w = np.linalg.eigvalsh(Oracle.from_problem(p).hamiltonian().toarray())
            assert np.abs(r.energies - w[:2]).max() < 1e-8
    finally:
        for t in tps:
            t.close()
