"""CUDA engine vs the reference's own outputs (golden fixtures), through the C ABI.

Bars: tables bit-exact; hii and sigma within 1e-12 max-norm relative; ground
energy within 1e-8 Ha of the reference Davidson; excited roots within 1e-8 Ha
of the assembled-Hamiltonian spectrum.
"""
import numpy as np
import pytest

from golden_io import load, max_rel, names
from sbd_gb300.engine import TPBProblem

pytestmark = pytest.mark.gpu
CASES = names()


@pytest.fixture(scope="module", params=CASES)
def gcase(request, engine):
    c = load(request.param)
    p = TPBProblem(engine, c.norb, c.astr, c.bstr, c.h1, c.eri, c.ecore)
    p.build_tables()
    yield c, p
    p.close()


def test_tables_bit_exact(gcase):
    c, p = gcase
    for spin, tag in ((0, "a"), (1, "b")):
        g = c.tables(tag)
        t = p.export_tables(spin)
        for k in ("off_s", "off_d", "ket_s", "ket_d"):
            assert np.array_equal(g[k].astype(np.int64), t[k].astype(np.int64)), (spin, k)
        assert np.array_equal(g["cran_s"], t["cran_s"])
        assert np.array_equal(g["cran_d"], t["cran_d"])


def test_hii(gcase):
    c, p = gcase
    assert max_rel(p.diag_terms(), c.hii) <= 1e-12


def test_sigma(gcase):
    c, p = gcase
    p.diag_terms()
    assert max_rel(p.mult(c.C), c.sigma) <= 1e-12


def test_sigma_accumulates_like_the_reference(gcase):
    c, p = gcase
    base = np.linspace(-1.0, 1.0, c.C.size)
    out = p.mult(c.C, base.copy())
    assert max_rel(out - base, c.sigma) <= 1e-12


def test_sigma_with_caller_diagonal(gcase):
    c, p = gcase
    zero = np.zeros(c.C.size)
    s_off = p.mult(c.C, hii=zero)
    assert max_rel(s_off + c.hii * c.C, c.sigma) <= 1e-12


def test_ground_energy_matches_reference_davidson(gcase):
    c, p = gcase
    r = p.davidson(nroots=1, max_nb=12, eps=1e-10, max_it=200, init=0)
    assert r.report["converged"]
    assert abs(r.energies[0] - c.energy) < 1e-8
    x = r.vectors[0]
    assert abs(np.linalg.norm(x) - 1.0) < 1e-10
    # <x|H|x> through the sigma path equals the Ritz value
    assert abs(x @ p.mult(x) - r.energies[0]) < 1e-8


def test_lowest_roots_match_assembled_spectrum(gcase):
    c, p = gcase
    if not c.irreducible:
        pytest.skip("reducible Hamiltonian")
    k = len(c.lowest)
    r = p.davidson(nroots=k, max_nb=4 * k + 8, eps=1e-9, max_it=200, init=1)
    assert r.report["converged"]
    assert np.allclose(r.energies, c.lowest, atol=1e-8, rtol=0)
    X = r.vectors
    G = X @ X.T
    assert np.allclose(G, np.eye(k), atol=1e-8)


def test_occupation_density(gcase):
    c, p = gcase
    p.diag_terms()
    assert max_rel(p.occupation_density(c.C), c.density_c) <= 1e-12


def test_lanczos_matches_reference_lanczos(gcase):
    """The reference's --method 2 solver from its init-0 vector, same Krylov size and tolerance."""
    c, p = gcase
    p.diag_terms()
    r = p.lanczos(max_it=20, num_block=40, eps=1e-12, init=0)
    assert abs(r.energies[0] - c.lanczos_energy) < 1e-8
    # the Ritz vector is normalised and its Rayleigh quotient is the energy
    W = r.vectors
    assert abs(np.dot(W, W) - 1.0) < 1e-8
    assert abs(np.dot(W, p.mult(W)) - r.energies[0]) < 1e-7


def test_rdms_match_reference(gcase):
    """One- and two-particle RDMs of C against the reference's Correlation (norb <= 12 fixtures)."""
    c, p = gcase
    if c.rdm1 is None:
        pytest.skip("RDM fixtures are stored for norb <= 12")
    one, two = p.rdm(c.C)
    assert np.abs(one - c.rdm1).max() <= 1e-12 * np.abs(c.rdm1).max()
    assert np.abs(two - c.rdm2).max() <= 1e-12 * np.abs(c.rdm2).max()
    one_only, none = p.rdm(c.C, two_body=False)
    assert none is None and np.abs(one_only - c.rdm1).max() <= 1e-12 * np.abs(c.rdm1).max()


@pytest.mark.parametrize("shapes", [(0, 0), (1, 2), (3, 3), (0, 4), (2, 4), (3, 4), (0, 5), (1, 5), (0, 6), (1, 6)])
def test_sigma_every_tile_shape(gcase, shapes):
    """Every tile shape, the fused single kernel (shape_b 4) and the two
    streaming kernels for sparse rows (shape_b 5, 6) give the reference sigma,
    in both precisions."""
    c, p = gcase
    p.diag_terms()
    p.set_tuning(0, *shapes)
    assert max_rel(p.sigma(c.C), c.sigma) <= 1e-12
    import torch
    p.set_tuning(1, *shapes)
    C32 = torch.tensor(c.C, dtype=torch.float32, device="cuda")
    S32 = torch.empty_like(C32)
    p.sigma_mixed_device(C32.data_ptr(), S32.data_ptr(), stream=0)
    torch.cuda.synchronize()
    assert max_rel(S32.double().cpu().numpy(), c.sigma) <= 1e-5


@pytest.mark.parametrize("shapes", [(0, 0), (1, 2), (3, 3), (0, 4), (3, 4), (0, 5), (1, 6)])
@pytest.mark.parametrize("nvec", [2, 3, 4, 5])
def test_mixed_block_sigma_equals_single(gcase, shapes, nvec):
    """The multi-vector FP32 product gives each vector's single-vector product: bit
    for bit when both sum the alpha-beta terms in the same order (norb > 32), to
    FP32 rounding otherwise (with 32-bit words the single-vector kernel takes the
    beta singles outside, the multi-vector one inside)."""
    import torch
    c, p = gcase
    p.diag_terms()
    p.set_tuning(1, *shapes)
    N = c.C.size
    rng = np.random.default_rng(nvec)
    X = torch.tensor(rng.uniform(-1, 1, (nvec, N)), dtype=torch.float32, device="cuda")
    Y = torch.empty_like(X)
    p.sigma_mixed_block_device(X.data_ptr(), Y.data_ptr(), nvec, stream=0)
    for j in range(nvec):
        y = torch.empty(N, dtype=torch.float32, device="cuda")
        p.sigma_mixed_device(X[j].data_ptr(), y.data_ptr(), stream=0)
        torch.cuda.synchronize()
        if c.norb > 32 or shapes[1] >= 5:
            assert torch.equal(Y[j], y), (j, shapes)
        else:
            assert max_rel(Y[j].double().cpu().numpy(), y.double().cpu().numpy()) <= 2e-6, (j, shapes)


def _df(x):
    """A float64 array as interleaved double-float pairs (hi, lo)."""
    hi = x.astype(np.float32)
    lo = (x - hi.astype(np.float64)).astype(np.float32)
    return np.stack([hi, lo], axis=-1).ravel()


@pytest.mark.parametrize("shapes", [None, (1, 1), (3, 4), (0, 5), (1, 6)])
def test_double_float_sigma_matches_reference(gcase, shapes):
    """The double-float sigma (48-bit values, FP32-pipe arithmetic) against the
    reference sigma at 1e-12, in the autotuned shape and forced ones, in the
    overwrite and accumulate forms."""
    import torch
    c, p = gcase
    p.diag_terms()
    if shapes is not None:
        p.set_tuning(2, *shapes)
    X = torch.tensor(_df(c.C), device="cuda")
    Y = torch.zeros_like(X)
    st = torch.cuda.current_stream().cuda_stream
    p.sigma_df_device(X.data_ptr(), Y.data_ptr(), stream=st)
    y = Y.double().cpu().numpy().reshape(-1, 2).sum(axis=1)
    assert max_rel(y, c.sigma) <= 1e-12
    base = np.random.default_rng(4).uniform(-1, 1, c.C.size)
    Y = torch.tensor(_df(base), device="cuda")
    p.sigma_df_device(X.data_ptr(), Y.data_ptr(), accumulate=True, stream=st)
    y = Y.double().cpu().numpy().reshape(-1, 2).sum(axis=1)
    assert max_rel(y, base + c.sigma) <= 1e-12


@pytest.mark.parametrize("shapes", [(1, 1), (3, 4), (1, 5), (0, 6)])
def test_sigma_alpha_beta_kernel(gcase, shapes):
    """The alpha x beta single pairs in their own kernel (k_sigma_ab: the C rows
    and (P|Q) rows of each alpha row's singles staged in shared memory) next to
    each kind of the other kernels (two sweeps, fused, sparse-row), in FP64
    (1e-12), double-float (1e-12) and FP32 (1e-5), overwrite and accumulate."""
    import torch
    c, p = gcase
    p.diag_terms()
    st = torch.cuda.current_stream().cuda_stream
    for prec in (0, 1, 2):
        p.set_tuning(prec, *shapes)
        p.set_split(prec, 1)
    try:
        for prec in (0, 1, 2):
            assert p.split(prec)["split"] == 1
        assert max_rel(p.mult(c.C), c.sigma) <= 1e-12
        base = np.linspace(-1.0, 1.0, c.C.size)
        assert max_rel(p.mult(c.C, base.copy()) - base, c.sigma) <= 1e-12
        C32 = torch.tensor(c.C, dtype=torch.float32, device="cuda")
        S32 = torch.empty_like(C32)
        p.sigma_mixed_device(C32.data_ptr(), S32.data_ptr(), stream=st)
        torch.cuda.synchronize()
        assert max_rel(S32.double().cpu().numpy(), c.sigma) <= 1e-5
        X = torch.tensor(_df(c.C), device="cuda")
        Y = torch.zeros_like(X)
        p.sigma_df_device(X.data_ptr(), Y.data_ptr(), stream=st)
        torch.cuda.synchronize()
        assert max_rel(Y.double().cpu().numpy().reshape(-1, 2).sum(axis=1), c.sigma) <= 1e-12
    finally:
        for prec in (0, 1, 2):
            p.set_split(prec, 0)


def test_solvers_with_alpha_beta_kernel(gcase):
    """The solvers' products in the block ordering with the alpha x beta kernel
    (forced on for FP64, FP32 and double-float) reach the reference energy: the
    plain FP64 Davidson and the mixed form."""
    from sbd_gb300.engine import MIXED
    c, p = gcase
    p.diag_terms()
    for prec in (3, 4, 5):
        p.set_tuning(prec, 1, 1)
        p.set_split(prec, 1)
    try:
        r = p.davidson(nroots=1, max_nb=12, eps=1e-10, max_it=200, init=0)
        assert r.report["converged"] and abs(r.energies[0] - c.energy) < 1e-8
        rm = p.davidson(nroots=1, max_nb=12, eps=1e-10, max_it=200, init=0, precision=MIXED)
        assert rm.report["converged"] and abs(rm.energies[0] - c.energy) < 1e-8
        assert p.split(3)["split"] == 1
    finally:
        for prec in (3, 4, 5):
            p.set_split(prec, 0)
