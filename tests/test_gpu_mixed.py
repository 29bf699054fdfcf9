"""Mixed precision (FP32 vectors and products, FP64 accumulation, FP64
refinement) against the plain FP64 path, through the C ABI."""
import numpy as np
import pytest

from golden_io import load, max_rel
from sbd_gb300.engine import MIXED, TPBProblem
from sbd_gb300.generators import make_problem

pytestmark = pytest.mark.gpu


def test_mixed_sigma_close_to_fp64(engine):
    torch = pytest.importorskip("torch")
    prob = make_problem(16, 5, 5, 300, 280, seed=31)
    p = TPBProblem.from_problem(engine, prob)
    p.build_tables()
    p.diag_terms()
    C = np.random.default_rng(2).uniform(-1, 1, prob.ndet)
    ref = p.mult(C)
    c32 = torch.tensor(C, dtype=torch.float32, device="cuda")
    s32 = torch.zeros_like(c32)
    p.sigma_mixed_device(c32.data_ptr(), s32.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    # FP32 storage of C and of the table values bounds the agreement near 1e-6
    assert max_rel(s32.cpu().double().numpy(), ref) < 5e-6


@pytest.mark.parametrize("refine_every", [4, 0])
@pytest.mark.parametrize("name,k", [("cfg0_shape_L16", 1), ("spin_L12", 3), ("wide_L36", 2)])
def test_mixed_davidson_matches_fp64(engine, name, k, refine_every):
    """refine_every 4: FP64 anchors and an FP32 subspace; 0: the two-phase form
    (FP32 Davidson, then FP64 from its lowest Ritz vectors)."""
    c = load(name)
    p = TPBProblem(engine, c.norb, c.astr, c.bstr, c.h1, c.eri, c.ecore)
    r64 = p.davidson(nroots=k, max_nb=16, eps=1e-9, init=1)
    rmx = p.davidson(nroots=k, max_nb=16, eps=1e-9, init=1, precision=MIXED, refine_every=refine_every)
    assert r64.report["converged"] and rmx.report["converged"]
    assert np.max(np.abs(rmx.energies - r64.energies)) < 1e-9
    assert np.allclose(rmx.energies, c.lowest[:k], atol=1e-8, rtol=0)
    assert rmx.report["sigma_fp64"] < rmx.report["sigma_calls"]
    if refine_every == 0:  # FP32 and double-float phases, then the FP64 check of the k Ritz vectors
        assert rmx.report["sigma_fp64"] <= 3 * k
    # same eigenvectors up to sign
    for q in range(k):
        ov = abs(float(rmx.vectors[q] @ r64.vectors[q]))
        assert ov > 1 - 1e-8


def test_mixed_davidson_config0_shape(engine):
    prob = make_problem(16, 5, 5, 800, seed=0, closed_shell=True)
    p = TPBProblem.from_problem(engine, prob)
    r64 = p.davidson(nroots=1, max_nb=20, eps=1e-8, init=1, want_vectors=False)
    rmx = p.davidson(nroots=1, max_nb=20, eps=1e-8, init=1, precision=MIXED, want_vectors=False)
    assert r64.report["converged"] and rmx.report["converged"]
    assert abs(rmx.energies[0] - r64.energies[0]) < 1e-6


@pytest.mark.parametrize("refine_every", [4, 0])
def test_mixed_davidson_two_roots_norb16(engine, refine_every):
    """Both mixed forms at a size with restarts (N = 40,000, 2 roots), against FP64."""
    prob = make_problem(16, 5, 5, 200, seed=3)
    p = TPBProblem.from_problem(engine, prob)
    r64 = p.davidson(nroots=2, max_nb=12, eps=1e-8, init=1, want_vectors=False)
    rmx = p.davidson(nroots=2, max_nb=12, eps=1e-8, init=1, precision=MIXED, refine_every=refine_every,
                     want_vectors=False)
    assert r64.report["converged"] and rmx.report["converged"]
    assert np.max(np.abs(rmx.energies - r64.energies)) < 1e-8
    if refine_every == 0:
        assert rmx.report["sigma_fp64"] < r64.report["sigma_fp64"]


def test_two_phase_caller_start_vectors_and_many_roots(engine):
    """The two-phase form with init 2 (caller vectors seed the FP32 phase) and
    with eight roots, against the FP64 solver."""
    prob = make_problem(12, 4, 4, 120, 110, seed=17)
    p = TPBProblem.from_problem(engine, prob)
    r64 = p.davidson(nroots=8, max_nb=24, eps=1e-8, init=1, want_vectors=True)
    assert r64.report["converged"]
    r8 = p.davidson(nroots=8, max_nb=24, eps=1e-8, init=1, precision=MIXED, refine_every=0, want_vectors=False)
    assert r8.report["converged"]
    assert np.max(np.abs(r8.energies - r64.energies)) < 1e-8
    # start from slightly perturbed FP64 vectors: converges to the same pair
    X0 = r64.vectors[:2] + 1e-3 * np.random.default_rng(0).standard_normal((2, prob.ndet))
    r2 = p.davidson(nroots=2, max_nb=16, eps=1e-8, init=2, precision=MIXED, refine_every=0, X0=X0)
    assert r2.report["converged"]
    assert np.max(np.abs(r2.energies - r64.energies[:2])) < 1e-8


@pytest.mark.parametrize("na,nb,k", [(1, 5, 3), (2, 2, 3)])
def test_two_phase_more_than_half_the_space_in_roots(engine, na, nb, k):
    from oracle.oracle import Oracle
    prob = make_problem(8, 3, 3, na, nb, seed=70 + na + nb)
    p = TPBProblem.from_problem(engine, prob)
    w = np.linalg.eigvalsh(Oracle.from_problem(prob).hamiltonian().toarray())
    r = p.davidson(nroots=k, max_nb=24, eps=1e-9, init=1, precision=MIXED, refine_every=0, want_vectors=False)
    assert np.allclose(r.energies, w[:k], atol=1e-8)
