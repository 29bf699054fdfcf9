"""The allocation-free sigma entry point (sbdgb_sigma_noalloc) through the C ABI.

Callers that cannot allocate device memory while they run (a host application
whose pool allocator owns the device, a fixed memory plan) use this entry
point: its transposed-vector scratch is a file-scope device array, so the call
itself makes no allocation.  The test compares it with the regular sbdgb_sigma
on two calls in a row and checks that the context's device memory does not
grow.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from golden_io import max_rel

pytestmark = pytest.mark.gpu


def _entry(lib):
    f = lib.sbdgb_sigma_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_sigma_matches_regular_sigma():
    torch = pytest.importorskip("torch")
    from sbd_gb300.engine import Engine, TPBProblem
    from sbd_gb300.generators import make_problem

    eng = Engine(0)
    prob = make_problem(16, 5, 5, 300, 280, seed=77)
    p = TPBProblem.from_problem(eng, prob)
    p.build_tables()
    p.diag_terms()
    f = _entry(eng.lib)
    rng = np.random.default_rng(11)
    C1 = torch.tensor(rng.uniform(-1, 1, prob.ndet), dtype=torch.float64, device="cuda")
    C2 = torch.tensor(rng.uniform(-1, 1, prob.ndet), dtype=torch.float64, device="cuda")
    outs = []
    before = eng.bytes_in_use
    torch.cuda.synchronize()
    for cvec in (C1, C2):  # two calls in a row share the scratch
        s = torch.full_like(cvec, float("nan"))
        rc = f(p.h, cvec.data_ptr(), s.data_ptr(), 0, None)
        assert rc == 0, eng.lib.sbdgb_last_error(eng.h)
        outs.append(s)
    torch.cuda.synchronize()
    assert eng.bytes_in_use == before  # nothing allocated by the two calls
    for cvec, s in zip((C1, C2), outs):
        ref = torch.zeros_like(cvec)
        p.sigma_device(cvec.data_ptr(), ref.data_ptr(), accumulate=False, stream=0)
        torch.cuda.synchronize()
        assert max_rel(s.cpu().numpy(), ref.cpu().numpy()) <= 1e-12
    # accumulate form: Wb += H Wk
    acc = torch.ones_like(C1)
    assert f(p.h, C1.data_ptr(), acc.data_ptr(), 1, None) == 0
    torch.cuda.synchronize()
    assert max_rel(acc.cpu().numpy() - 1.0, outs[0].cpu().numpy()) <= 1e-12
    p.close()
    eng.close()


@pytest.mark.parametrize("shapes,split", [((1, 1), 0), ((1, 4), 0), ((0, 5), 0), ((1, 1), 1), ((1, 4), 1)])
def test_noalloc_sigma_in_every_kind_of_shape(shapes, split):
    """The allocation-free sigma follows the problem's tuned shapes: two sweeps
    on the transposed copy (the scratch in use), the fused kernel and the
    sparse-row kernel (no transposed copy), with and without the alpha x beta
    kernel; each against the regular sigma in the same shapes."""
    torch = pytest.importorskip("torch")
    from sbd_gb300.engine import Engine, TPBProblem
    from sbd_gb300.generators import make_problem

    eng = Engine(0)
    prob = make_problem(12, 4, 4, 200, 190, seed=78)
    p = TPBProblem.from_problem(eng, prob)
    p.build_tables()
    p.diag_terms()
    p.set_tuning(0, *shapes)
    p.set_split(0, split)
    f = _entry(eng.lib)
    rng = np.random.default_rng(12)
    C1 = torch.tensor(rng.uniform(-1, 1, prob.ndet), dtype=torch.float64, device="cuda")
    before = eng.bytes_in_use
    s = torch.full_like(C1, float("nan"))
    assert f(p.h, C1.data_ptr(), s.data_ptr(), 0, None) == 0, eng.lib.sbdgb_last_error(eng.h)
    torch.cuda.synchronize()
    assert eng.bytes_in_use == before
    ref = torch.zeros_like(C1)
    p.sigma_device(C1.data_ptr(), ref.data_ptr(), accumulate=False, stream=0)
    torch.cuda.synchronize()
    assert max_rel(s.cpu().numpy(), ref.cpu().numpy()) <= 1e-12
    p.close()
    eng.close()


def test_noalloc_sigma_captures_into_a_cuda_graph():
    """A call made under stream capture (global mode: an allocation, a
    synchronisation or any other call that capture forbids would fail it)
    records into a graph; replaying the graph gives the regular sigma, twice."""
    torch = pytest.importorskip("torch")
    from sbd_gb300.engine import Engine, TPBProblem
    from sbd_gb300.generators import make_problem

    eng = Engine(0)
    prob = make_problem(16, 5, 5, 300, 280, seed=79)
    p = TPBProblem.from_problem(eng, prob)
    p.build_tables()
    p.diag_terms()
    f = _entry(eng.lib)
    rng = np.random.default_rng(13)
    C1 = torch.tensor(rng.uniform(-1, 1, prob.ndet), dtype=torch.float64, device="cuda")
    s = torch.zeros_like(C1)
    assert f(p.h, C1.data_ptr(), s.data_ptr(), 0, None) == 0  # first call on the device: outside capture
    ref = torch.zeros_like(C1)
    p.sigma_device(C1.data_ptr(), ref.data_ptr(), accumulate=False, stream=0)  # allocates its own scratch
    torch.cuda.synchronize()
    before = eng.bytes_in_use
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rc = f(p.h, C1.data_ptr(), s.data_ptr(), 0, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, eng.lib.sbdgb_last_error(eng.h)
    assert eng.bytes_in_use == before
    for _ in range(2):
        s.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        assert max_rel(s.cpu().numpy(), ref.cpu().numpy()) <= 1e-12
    assert eng.bytes_in_use == before
    del g
    p.close()
    eng.close()


def test_noalloc_sigma_rejects_large_problems():
    torch = pytest.importorskip("torch")
    from sbd_gb300.engine import Engine, TPBProblem
    from sbd_gb300.generators import make_problem

    eng = Engine(0)
    big = make_problem(24, 4, 4, 1600, 1600, seed=6)  # 2,560,000 determinants > 2,097,152
    p = TPBProblem.from_problem(eng, big)
    p.build_tables()
    p.diag_terms()
    f = _entry(eng.lib)
    c = torch.zeros(big.ndet, dtype=torch.float64, device="cuda")
    s = torch.zeros_like(c)
    rc = f(p.h, c.data_ptr(), s.data_ptr(), 0, None)  # rejected on the host before any launch
    assert rc == 2
    assert b"at most" in eng.lib.sbdgb_last_error(eng.h)
    p.close()
    eng.close()
