"""The --gpus N replica path of bench.py on CPU: two gloo ranks meet at the
barrier around the timed region, gather each other's numbers, and rank 0
reports all ranks' work over the slowest rank's time."""
import importlib.util
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    argv = sys.argv
    sys.argv = ["bench.py"]
    try:
        spec.loader.exec_module(mod)
    finally:
        sys.argv = argv
    return mod


def _rank(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    b = _bench()
    r = b.Ranks()
    r.barrier()
    objs = r.gather({"rank": rank, "sec": 1.0 + rank})  # rank 1 is the slow one
    r.barrier()
    r.close()
    q.put((rank, objs, b.replica_rate(objs, 100)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_gather_and_take_the_slowest():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(k, 2, port, q)) for k in range(2)]
    for p in ps:
        p.start()
    out = dict((r, (objs, rate)) for r, objs, rate in (q.get(timeout=120) for _ in ps))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        objs, rate = out[r]
        assert [o["rank"] for o in objs] == [0, 1]
        # 2 replicas x 100 units over the slower rank's 2 s
        assert abs(rate - 100.0) < 1e-12


def test_single_process_needs_no_group():
    b = _bench()
    r = b.Ranks()
    assert r.world == 1 and r.gather({"sec": 2.0}) == [{"sec": 2.0}]
    r.barrier()
    r.close()
    assert b.replica_rate([{"sec": 2.0}], 50) == 25.0
