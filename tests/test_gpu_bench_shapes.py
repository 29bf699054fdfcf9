"""sigma at the benchmark shapes against the oracle, on sampled alpha rows.

Config 1 (norb 36, 12+12 electrons, 6000 x 6000 strings, N = 3.6e7, 78
nonzeros per row) and config 3 (norb 58, 16+16 electrons, 12000 x 12000
strings, N = 1.44e8, 0.5 nonzeros per row) are the bench's workloads.  The
full sigma is computed on the GPU through the C ABI; the oracle (the
reference's TRADMODE mult, chemistry/tpb/mult.h:440-558) computes the first,
a middle and the last alpha rows, which cross the heaviest and lightest row
tiles, every beta column chunk, and the 32-bit element offsets at the far end
of the vector.

Bars: FP64 sigma 1e-12 max-norm relative per row block; the mixed form (FP32
C, FP32 table values, FP64 accumulation) 5e-6, the bound FP32 storage of C
and of the table values sets.
"""
import numpy as np
import pytest

from golden_io import max_rel
from oracle.oracle import Oracle
from sbd_gb300 import generators as G
from sbd_gb300.engine import TPBProblem

pytestmark = pytest.mark.gpu

ROWS = 16


@pytest.mark.parametrize("config", [1, 3])
def test_sigma_rows_at_bench_shape(engine, config):
    torch = pytest.importorskip("torch")
    prob = G.config1() if config == 1 else G.config3()
    na, nb = prob.astr.size, prob.bstr.size
    p = TPBProblem.from_problem(engine, prob)
    p.build_tables()
    hii = p.diag_terms().reshape(na, nb)
    rng = np.random.default_rng(100 + config)
    C = rng.uniform(-1.0, 1.0, prob.ndet)
    got = p.mult(C).reshape(na, nb)
    c32 = torch.tensor(C, dtype=torch.float32, device="cuda")
    s32 = torch.zeros_like(c32)
    p.sigma_mixed_device(c32.data_ptr(), s32.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got32 = s32.cpu().double().numpy().reshape(na, nb)
    del c32, s32
    p.close()
    o = Oracle.from_problem(prob)
    for r0 in (0, na // 2 - ROWS // 2, na - ROWS):
        r1 = r0 + ROWS
        h = o.hii(rows=(r0, r1))
        assert max_rel(hii[r0:r1], h.reshape(na, nb)[r0:r1]) <= 1e-12
        ref = o.mult(C, rows=(r0, r1), hii=h).reshape(na, nb)[r0:r1]
        assert max_rel(got[r0:r1], ref) <= 1e-12, (config, r0)
        assert max_rel(got32[r0:r1], ref) <= 5e-6, (config, r0)
