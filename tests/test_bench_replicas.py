"""bench.py with several ranks (one replica per GPU in this build), on the CPU:
two gloo ranks started by torch.distributed.run.  The reference arm runs on
rank 0 only and prints one JSON line; the other rank exits 0 without work.
The max-over-ranks timing helper is checked on two spawned gloo ranks."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_two_ranks_prints_once():
    env = dict(os.environ, SBDGB_BENCH_GLOO="1", SBDGB_REF_ROWS="1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
                        os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["cores"] >= 1 and d["e2e"]["h2d_bytes_per_step"] == 0


def _rank(rank, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), SBDGB_BENCH_GLOO="1")
    sys.path.insert(0, ROOT)
    import bench
    dist, r, ws = bench.dist_init()
    t = bench.max_over_ranks(dist, 1.0 + rank)
    bench.barrier(dist)
    q.put((r, ws, t))
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=120)
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[0] for g in got] == [0, 1]
    assert all(g[1] == 2 and g[2] == 2.0 for g in got)
    assert all(p.exitcode == 0 for p in ps)
