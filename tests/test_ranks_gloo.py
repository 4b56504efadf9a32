"""The N-replica host logic of bench.py on CPU: two gloo ranks pass the
barriers and agree on the maximum over ranks, which is how the timed region's
duration is taken when one process runs per GPU."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r = bench.Ranks(backend="gloo")
    r.barrier()
    m = r.max(float(10 * rank + 1))
    r.barrier()
    r.close()
    q.put((rank, r.world, m))


def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 11.0), (1, 2, 11.0)]


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        r = bench.Ranks(backend="gloo")
        assert r.world == 1 and r.dist is None
        r.barrier()
        assert r.max(3.5) == 3.5
    finally:
        os.environ.update(env)


def test_reference_arm_other_ranks_exit_without_work():
    """Under torchrun the reference arm runs on rank 0 alone; rank 1 exits 0
    and prints nothing."""
    import subprocess
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "3"],
                         capture_output=True, text=True, env=env, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    assert res.stdout.strip() == ""
