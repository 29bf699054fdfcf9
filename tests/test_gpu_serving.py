"""The request loop (sbdgb_server_*): results alone and in the mix, admission
by HBM footprint, timeouts, failures and shutdown."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (norb, electrons per spin, alpha strings, beta strings, roots)
SPECS = [(12, 4, 4, 120, 90, 1), (14, 5, 5, 300, 200, 2), (12, 4, 4, 495, 495, 3), (16, 5, 5, 400, 350, 1),
         (10, 3, 3, 100, 120, 2), (14, 4, 4, 250, 300, 1), (12, 4, 4, 60, 400, 2), (16, 6, 6, 500, 450, 1)]


def _mix():
    from sbd_gb300.generators import make_problem
    return [(make_problem(L, n, n, na, nb, seed=300 + i), k) for i, (L, n, _, na, nb, k) in enumerate(SPECS)]


@pytest.fixture(scope="module")
def alone():
    """Each problem solved by itself through sbdgb_davidson (FP64)."""
    from sbd_gb300.engine import Engine, TPBProblem
    eng = Engine(0)
    out = []
    for p, k in _mix():
        t = TPBProblem.from_problem(eng, p)
        r = t.davidson(nroots=k, eps=1e-9, max_nb=20, init=1, want_vectors=True)
        out.append(r)
        t.close()
    eng.close()
    return out


def test_fp64_results_same_alone_and_in_mix(alone):
    from sbd_gb300.serving import Server
    mix = _mix()
    with Server(0, workers=4) as srv:
        tickets = [srv.submit_problem(p, nroots=k, eps=1e-9, max_nb=20, init=1, want_vectors=True) for p, k in mix]
        res = [srv.wait(t, timeout=300) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(mix) and st["failed"] == 0
    assert st["peak_running"] >= 2  # solves overlapped
    for (p, k), r, a in zip(mix, res, alone):
        assert r["status"] == 0, r["message"]
        assert r["converged"]
        assert np.max(np.abs(r["energies"] - a.energies)) <= 1e-10
        for j in range(k):  # same eigenvectors up to sign
            ov = abs(float(np.dot(r["vectors"][j], a.vectors[j])))
            assert ov >= 1 - 1e-8


@pytest.mark.parametrize("refine_every", [4, 0])
def test_mixed_results_in_mix_match_fp64_alone(alone, refine_every):
    """Both mixed forms in the request loop; every request fits its footprint
    (a request whose workspaces outgrow its reservation fails with E_NOMEM)."""
    from sbd_gb300.engine import MIXED
    from sbd_gb300.serving import Server
    mix = _mix()
    with Server(0, workers=3) as srv:
        tickets = [srv.submit_problem(p, nroots=k, eps=1e-8, max_nb=20, init=1, precision=MIXED,
                                      refine_every=refine_every) for p, k in mix]
        res = [srv.wait(t, timeout=300) for t in tickets]
    for r, a in zip(res, alone):
        assert r["status"] == 0, r["message"]
        assert np.max(np.abs(r["energies"] - a.energies)) <= 1e-6


def test_admission_respects_the_budget():
    from sbd_gb300.engine import SbdgbError
    from sbd_gb300.generators import make_problem
    from sbd_gb300.serving import Server
    budget = 256 << 20
    mix = _mix()
    with Server(0, workers=4, hbm_budget=budget) as srv:
        tickets = [srv.submit_problem(p, nroots=k, eps=1e-8, max_nb=20, init=1) for p, k in mix]
        res = [srv.wait(t, timeout=300) for t in tickets]
        st = srv.stats()
        assert all(r["status"] == 0 for r in res), [r["message"] for r in res]
        assert 0 < st["peak_reserved_bytes"] <= budget
        assert st["reserved_bytes"] == 0 and st["running"] == 0
        big = make_problem(24, 8, 8, 3000, 3000, seed=5)  # 9M determinants: far over 256 MiB
        with pytest.raises(SbdgbError) as e:
            srv.submit_problem(big, nroots=1)
        assert e.value.status == 4  # SBDGB_E_NOMEM, rejected at submission


def test_wait_timeout_failed_request_and_shutdown():
    from sbd_gb300.generators import make_problem
    from sbd_gb300.serving import Server
    first = make_problem(16, 6, 6, 800, 800, seed=8)
    small = make_problem(10, 3, 3, 60, 60, seed=9)
    srv = Server(0, workers=1)
    t1 = srv.submit_problem(first, nroots=2, eps=1e-8)
    t2 = srv.submit_problem(small, nroots=1, eps=1e-8)
    with pytest.raises(TimeoutError):
        srv.wait(t2, timeout=0.0)  # queued behind t1 on the single worker
    assert srv.wait(t1)["status"] == 0
    assert srv.wait(t2, timeout=120)["status"] == 0
    # malformed strings fail inside the worker; the server keeps running
    bad = srv.submit(small.norb, small.astr[::-1].copy(), small.bstr, small.ints.h1, small.ints.eri)
    r = srv.wait(bad, timeout=60)
    assert r["status"] == 1 and "sorted" in r["message"]
    assert srv.wait(srv.submit_problem(small), timeout=60)["status"] == 0
    # shutdown with requests still queued: the running one finishes, the queued ones are dropped
    for _ in range(3):
        srv.submit_problem(first, nroots=1, eps=1e-8)
    srv.close()


def test_small_requests_are_batched(alone):
    """With one worker busy, the small requests queued behind it start together
    as one batched solve; each result equals the lone solve."""
    from sbd_gb300.generators import make_problem
    from sbd_gb300.serving import Server
    blocker = make_problem(16, 6, 6, 900, 900, seed=11)  # 810,000 determinants: solved alone
    mix = _mix()
    with Server(0, workers=1) as srv:
        t0 = srv.submit_problem(blocker, nroots=1, eps=1e-8)
        ts = [srv.submit_problem(p, nroots=1, eps=1e-9, max_nb=20, init=1) for p, _ in mix]
        assert srv.wait(t0, timeout=300)["status"] == 0
        res = [srv.wait(t, timeout=300) for t in ts]
        st = srv.stats()
    assert st["batched"] >= 2
    for (p, k), r, a in zip(mix, res, alone):
        assert r["status"] == 0, r["message"]
        assert abs(r["energies"][0] - a.energies[0]) <= 1e-10


def test_concurrent_solves_of_different_sizes_all_converge():
    """Requests above the batching threshold run concurrently on separate
    workers, each with its own row length, so their kernels ask for different
    amounts of dynamic shared memory at the same time (the alpha x beta kernel,
    the Rayleigh-Ritz kernel).  Every request converges to its lone result."""
    from sbd_gb300.engine import Engine, TPBProblem
    from sbd_gb300.generators import make_problem
    from sbd_gb300.serving import Server
    specs = [(16, 5, 620, 560), (16, 5, 700, 650), (16, 5, 560, 900), (18, 6, 820, 480), (16, 5, 900, 500),
             (18, 6, 600, 700), (16, 5, 760, 610), (18, 6, 950, 420)]
    mix = [make_problem(L, n, n, na, nb, seed=700 + i) for i, (L, n, na, nb) in enumerate(specs)]
    assert min(p.ndet for p in mix) > 300000  # above the batching threshold: one solve per worker
    eng = Engine(0)
    lone = []
    for p in mix:
        t = TPBProblem.from_problem(eng, p)
        lone.append(t.davidson(nroots=1, eps=1e-8, max_nb=20, init=1, want_vectors=False).energies)
        t.close()
    eng.close()
    with Server(0, workers=8) as srv:
        tickets = [srv.submit_problem(p, nroots=1, eps=1e-8, max_nb=20, init=1) for p in mix]
        res = [srv.wait(t, timeout=600) for t in tickets]
        st = srv.stats()
    assert st["failed"] == 0 and st["peak_running"] >= 2
    for r, e in zip(res, lone):
        assert r["status"] == 0 and r["converged"], r["message"]
        assert abs(r["energies"][0] - e[0]) <= 1e-8
