"""Full-size checks of the CUDA engine (benchmark shapes), through the C ABI.

At the 640,000-determinant config-0 shape sigma is compared element-wise with
the CPU oracle; at every size the size-independent properties of H hold:
symmetry, linearity, determinism."""
import numpy as np
import pytest

from golden_io import max_rel
from oracle.oracle import Oracle
from sbd_gb300.engine import SbdgbError, TPBProblem
from sbd_gb300.generators import config0, make_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg0(engine):
    prob = config0()
    p = TPBProblem.from_problem(engine, prob)
    p.build_tables()
    p.diag_terms()
    yield prob, p
    p.close()


def test_config0_against_oracle(cfg0):
    prob, p = cfg0
    o = Oracle.from_problem(prob)
    for spin, t in ((0, o.ta), (1, o.tb)):
        g = p.export_tables(spin)
        assert np.array_equal(g["off_s"].astype(np.int64), t.off_s.astype(np.int64))
        assert np.array_equal(g["ket_d"].astype(np.int64), t.ket_d.astype(np.int64))
        assert np.array_equal(g["cran_d"], t.cran_d)
    assert max_rel(p.diag_terms(), o.hii()) <= 1e-12
    C = np.random.default_rng(7).uniform(-1, 1, prob.ndet)
    assert max_rel(p.mult(C), o.mult(C)) <= 1e-12
    assert max_rel(p.occupation_density(C), o.density(C)) <= 1e-12


def test_symmetry_linearity_determinism(cfg0):
    prob, p = cfg0
    rng = np.random.default_rng(3)
    x = rng.standard_normal(prob.ndet)
    y = rng.standard_normal(prob.ndet)
    hx, hy = p.mult(x), p.mult(y)
    assert abs(x @ hy - y @ hx) <= 1e-11 * abs(x @ hy)
    hxy = p.mult(2.0 * x - 0.5 * y)
    assert max_rel(hxy, 2.0 * hx - 0.5 * hy) <= 1e-12
    assert np.array_equal(p.mult(x), hx)


def test_davidson_two_roots_against_assembled_h(engine):
    prob = make_problem(16, 5, 5, 200, seed=21, closed_shell=True)
    o = Oracle.from_problem(prob)
    ref = o.lowest(2)
    p = TPBProblem.from_problem(engine, prob)
    r = p.davidson(nroots=2, max_nb=24, eps=1e-8, init=1)
    assert r.report["converged"]
    assert np.allclose(r.energies, ref, atol=1e-8, rtol=0)


def test_input_errors(engine):
    prob = make_problem(10, 3, 3, 30, seed=1)
    with pytest.raises(SbdgbError) as e:
        TPBProblem(engine, 10, prob.astr[::-1].copy(), prob.bstr, prob.ints.h1, prob.ints.eri)
    assert e.value.status == 1
    bad = prob.astr.copy()
    bad[0] |= np.uint64(1) << np.uint64(9)  # popcount differs
    bad = np.unique(bad)
    with pytest.raises(SbdgbError):
        TPBProblem(engine, 10, bad, prob.bstr, prob.ints.h1, prob.ints.eri)
    with pytest.raises(SbdgbError) as e:
        engine.check_comm_sizes(2, 1, 1)
    assert e.value.status == 2
    engine.check_comm_sizes(1, 1, 1)


def test_device_pointer_sigma(engine):
    torch = pytest.importorskip("torch")
    prob = make_problem(12, 4, 4, 60, 70, seed=9)
    p = TPBProblem.from_problem(engine, prob)
    p.build_tables()
    p.diag_terms()
    C = np.random.default_rng(0).uniform(-1, 1, prob.ndet)
    ref = p.mult(C)
    c_dev = torch.tensor(C, dtype=torch.float64, device="cuda")
    s_dev = torch.zeros_like(c_dev)
    stream = torch.cuda.current_stream()
    p.sigma_device(c_dev.data_ptr(), s_dev.data_ptr(), accumulate=False, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    assert max_rel(s_dev.cpu().numpy(), ref) <= 1e-14


def test_rdms_against_oracle_norb16(engine):
    """RDMs at norb 16 (beyond the fixtures) against the oracle's restatement."""
    prob = make_problem(16, 5, 5, 150, 120, seed=21)
    p = TPBProblem.from_problem(engine, prob)
    p.build_tables()
    o = Oracle.from_problem(prob)
    W = np.random.default_rng(4).uniform(-1, 1, prob.ndet)
    one, two = p.rdm(W)
    ro, rt = o.correlation(W)
    assert np.abs(one - ro).max() <= 1e-12 * np.abs(ro).max()
    assert np.abs(two - rt).max() <= 1e-12 * np.abs(rt).max()
    p.close()


@pytest.mark.parametrize("na,nb", [(1, 1), (1, 7), (9, 1), (2, 2)])
def test_degenerate_lists_against_dense(engine, na, nb):
    """Lists of one or two strings (no same-spin excitations on one side, N as small
    as 1): sigma equals the assembled H, and every solver finds its lowest eigenvalue."""
    from sbd_gb300.engine import MIXED
    prob = make_problem(8, 3, 3, na, nb, seed=40 + na + nb)
    p = TPBProblem.from_problem(engine, prob)
    p.build_tables()
    p.diag_terms()
    o = Oracle.from_problem(prob)
    H = o.hamiltonian().toarray()
    C = np.random.default_rng(1).uniform(-1, 1, prob.ndet)
    assert max_rel(p.mult(C), H @ C) <= 1e-12
    w = np.linalg.eigvalsh(H)
    k = min(2, prob.ndet)
    r = p.davidson(nroots=k, eps=1e-10, max_nb=8, init=1)
    assert np.allclose(r.energies, w[:k], atol=1e-8)
    rm = p.davidson(nroots=1, eps=1e-9, max_nb=8, init=1, precision=MIXED)
    assert abs(rm.energies[0] - w[0]) < 1e-6
    rl = p.lanczos(max_it=20, num_block=min(10, max(2, prob.ndet)), eps=1e-12, init=1)
    assert abs(rl.energies[0] - w[0]) < 1e-8
    p.close()


@pytest.mark.parametrize("na,nb,k", [(1, 5, 4), (2, 2, 3), (3, 3, 8)])
def test_more_than_half_the_space_in_roots(engine, na, nb, k):
    """2 * nroots > N: the subspace is capped at N and the solver still returns the
    lowest eigenvalues (regular and batched solvers)."""
    from sbd_gb300.engine import batch_davidson
    prob = make_problem(8, 3, 3, na, nb, seed=60 + na + nb)
    p = TPBProblem.from_problem(engine, prob)
    try:
        p.build_tables()
        p.diag_terms()
        w = np.linalg.eigvalsh(Oracle.from_problem(prob).hamiltonian().toarray())
        r = p.davidson(nroots=k, eps=1e-9, max_nb=24, init=1)
        assert np.allclose(r.energies, w[:k], atol=1e-8)
        rb = batch_davidson(engine, [p], nroots=k, max_nb=24, eps=1e-9)[0]
        assert np.allclose(rb.energies, w[:k], atol=1e-8)
    finally:
        p.close()


def test_more_roots_than_determinants_is_an_error(engine):
    prob = make_problem(8, 3, 3, 1, 2, seed=3)
    p = TPBProblem.from_problem(engine, prob)
    p.build_tables()
    p.diag_terms()
    with pytest.raises(SbdgbError) as e:
        p.davidson(nroots=3)
    assert e.value.status == 1
    p.close()


def test_eight_roots_restart_basis_over_sixteen_columns(engine):
    """Eight roots with a small subspace: once some roots converge the restart
    keeps 2k Ritz vectors plus previous directions (up to 24 columns)."""
    prob = make_problem(12, 4, 4, 150, 140, seed=23)
    p = TPBProblem.from_problem(engine, prob)
    try:
        w = Oracle.from_problem(prob).lowest(8)
        r = p.davidson(nroots=8, max_nb=26, eps=1e-9, init=1, want_vectors=False)
        assert r.report["converged"] and r.report["restarts"] > 0
        assert np.allclose(r.energies, w, atol=1e-8)
    finally:
        p.close()


def test_measured_fp64_rates():
    """The bench's FP64 rate probe (its own library, not the engine's) runs and
    gives plausible FP64 rates (TFLOP/s)."""
    from bench import measure_fp64_rates
    r = measure_fp64_rates(0)
    assert 0.05 < r["dfma_tflops"] < 200.0 and 0.05 < r["dmma_tflops"] < 200.0


@pytest.mark.parametrize("nb", [280, 282, 283])
@pytest.mark.parametrize("variant", [0, 1])
def test_row_kernel_against_oracle(engine, nb, variant):
    """The row kernel (shape_b 6; norb 40, 10+10 electrons, 300 x nb strings:
    at most 17 beta pairs per column).  Variant 0 is the persistent,
    double-buffered form where it applies (FP32: nb a multiple of 4, 280;
    FP64 and double-float: nb even, 280 and 282) and the one-row-per-CTA form
    otherwise (283, one element per thread); variant 1 is the 1024-thread
    one-row-per-CTA form.  FP64 and double-float at 1e-12 against the oracle,
    overwrite and accumulate; FP32 at its bound."""
    torch = pytest.importorskip("torch")
    prob = make_problem(40, 10, 10, 300, nb, seed=43)
    p = TPBProblem.from_problem(engine, prob)
    p.build_tables()
    p.diag_terms()
    for prec in (0, 1, 2):
        p.set_tuning(prec, variant, 6)
    o = Oracle.from_problem(prob)
    rng = np.random.default_rng(7 * variant + nb)
    C = rng.uniform(-1, 1, prob.ndet)
    ref = o.mult(C)
    assert max_rel(p.mult(C), ref) <= 1e-12
    base = rng.uniform(-1, 1, prob.ndet)
    st = torch.cuda.current_stream().cuda_stream
    c = torch.tensor(C, device="cuda")
    s = torch.tensor(base, device="cuda")
    p.sigma_device(c.data_ptr(), s.data_ptr(), accumulate=True, stream=st)
    torch.cuda.synchronize()
    assert max_rel(s.cpu().numpy(), base + ref) <= 1e-12
    c32 = c.float()
    s32 = torch.empty_like(c32)
    p.sigma_mixed_device(c32.data_ptr(), s32.data_ptr(), stream=st)
    torch.cuda.synchronize()
    assert max_rel(s32.double().cpu().numpy(), ref) <= 5e-6
    hi = C.astype(np.float32)
    lo = (C - hi.astype(np.float64)).astype(np.float32)
    X = torch.tensor(np.stack([hi, lo], axis=-1).ravel(), device="cuda")
    Y = torch.zeros_like(X)
    p.sigma_df_device(X.data_ptr(), Y.data_ptr(), stream=st)
    torch.cuda.synchronize()
    assert max_rel(Y.double().cpu().numpy().reshape(-1, 2).sum(axis=1), ref) <= 1e-12
    p.close()


@pytest.mark.parametrize("nb", [280, 283])
@pytest.mark.parametrize("variant", [0, 1])
def test_sparse_kernel_against_oracle(engine, nb, variant):
    """The sparse-row streaming kernel (16-byte accesses when the beta count is a
    multiple of the vector width, 280; one element per thread otherwise, 283),
    in both row-tile sizes: overwrite and accumulate forms against the oracle,
    and the mixed form against it at the FP32 bound."""
    torch = pytest.importorskip("torch")
    prob = make_problem(16, 5, 5, 300, nb, seed=41)
    p = TPBProblem.from_problem(engine, prob)
    p.build_tables()
    p.diag_terms()
    p.set_tuning(0, variant, 5)
    p.set_tuning(1, variant, 5)
    o = Oracle.from_problem(prob)
    rng = np.random.default_rng(variant + nb)
    C = rng.uniform(-1, 1, prob.ndet)
    ref = o.mult(C)
    assert max_rel(p.mult(C), ref) <= 1e-12
    base = rng.uniform(-1, 1, prob.ndet)
    c = torch.tensor(C, device="cuda")
    s = torch.tensor(base, device="cuda")
    p.sigma_device(c.data_ptr(), s.data_ptr(), accumulate=True, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert max_rel(s.cpu().numpy(), base + ref) <= 1e-12
    c32 = c.float()
    s32 = torch.empty_like(c32)
    p.sigma_mixed_device(c32.data_ptr(), s32.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert max_rel(s32.double().cpu().numpy(), ref) <= 5e-6
    p.close()
