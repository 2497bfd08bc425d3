"""The multi-GPU path is replicas only: every rank runs the whole workload and
nothing is exchanged on the data path.  These CPU tests run two gloo ranks and
check the measurement glue: the barrier, the maximum elapsed time over ranks
and the whole-job rate."""
import multiprocessing as mp
import os
import socket
import time


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "gridaphybrid.jl_gb300"))
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from gridaphybrid_gb300 import replicas
    r, n, local = replicas.init(backend="gloo")
    replicas.barrier()
    t0 = time.perf_counter()
    time.sleep(0.05 if rank == 0 else 0.25)  # rank 1 is the slow replica
    elapsed = time.perf_counter() - t0
    replicas.barrier()
    rate, tmax = replicas.aggregate_rate(100.0, elapsed)
    q.put((r, n, local, elapsed, tmax, rate))
    replicas.finalize()


def test_two_gloo_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, n0, l0, e0, t0, rate0), (r1, n1, l1, e1, t1, rate1) = out
    assert (r0, r1) == (0, 1) and n0 == n1 == 2 and (l0, l1) == (0, 1)
    assert t0 == t1 == max(e0, e1)          # every rank sees the same maximum
    assert e1 > e0 and t0 >= 0.25
    assert abs(rate0 - 2 * 100.0 / t0) < 1e-9 and rate0 == rate1


def test_single_process_is_a_no_op(monkeypatch):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "gridaphybrid.jl_gb300"))
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from gridaphybrid_gb300 import replicas
    assert replicas.init() == (0, 1, 0)
    replicas.barrier()
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.aggregate_rate(10.0, 2.0) == (5.0, 2.0)
