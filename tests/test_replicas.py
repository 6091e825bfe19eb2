"""The bench's multi-process path (replicas only: one process per GPU, no
collective on the data path) on CPU with gloo, world size 2: the barrier and
the max over ranks the whole-job timing uses, and the reference arm under
torchrun, where rank 0 alone works and prints and the other rank exits 0."""

import json
import os
import socket
import subprocess
import sys

REPO = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, REPO)
    import bench
    d = bench.Dist("gloo")
    d.barrier()
    q.put((rank, d.max(1.5 + rank), d.world, d.rank))
    d.barrier()
    d.close()


def test_dist_max_over_ranks_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p_ in ps:
        p_.start()
    for p_ in ps:
        p_.join(120)
        assert p_.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.5, 2, 0), (1, 2.5, 2, 1)]


def test_reference_arm_under_torchrun_rank0_only():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(REPO, "bench.py"),
           "--impl", "reference", "--workload", "meander200k", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    out = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["cores"] == 1
