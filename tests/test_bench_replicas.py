"""bench.py's multi-GPU path is replicas only (a solve fits one GPU; requests are
partitioned, with no data-path collective).  Its host logic on the CPU, world
size 2 over gloo: every rank takes the slowest rank's time, the whole-job value
is world x requests per rank / that time, and the host reference arm runs on
rank 0 alone."""
import multiprocessing as mp
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    world, r, _, dist = bench.dist_setup("gloo")
    t = bench.max_over_ranks(1.0 + r, dist)  # rank 1 is the slower replica
    q.put((r, world, t, bench.replicas_value(world, 32, t)))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_replica, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
    assert all(p.exitcode == 0 for p in ps)
    assert [r for r, *_ in res] == [0, 1]
    for _, world, t, v in res:
        assert world == 2 and t == 2.0 and v == 32.0


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == ""
