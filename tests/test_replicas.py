"""The multi-GPU path (independent replicas) exercised on CPU with gloo.

Two ranks join a gloo process group as torchrun would set them up, each runs
its own replica of a small problem (the oracle stands in for the GPU here --
the point is the rank logic, not the kernels), and the whole-job rate is
aggregated exactly as bench.py does it: work of all ranks over the slowest
rank's time.  No collective touches the data: each replica's result must
match a replica run alone.
"""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, fake_seconds, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from fv3d_gb300 import problems, replicas
    from oracle import pyoracle
    try:
        w, r, local = replicas.init("gloo")
        pr = problems.sedov(32, tend=1.0e30)
        o = pyoracle.Oracle(pr.params)
        o.set_prim(*pr.prim)
        replicas.barrier()
        t, n = o.advance(1.0e30, max_steps=3)
        rate, slowest = replicas.aggregate_rate(pr.cells * n, w, fake_seconds[r])
        q.put((r, w, local, rate, slowest, np.stack(o.get_prim())))
        replicas.shutdown()
    except Exception as e:  # surfaced by the parent
        q.put((rank, "error", repr(e), None, None, None))


@pytest.mark.timeout(300)
def test_two_replicas_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    fake = [1.5, 2.5]  # seconds per rank; the slower one sets the rate
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, fake, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=240) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
    assert all(o[1] != "error" for o in out), out
    out.sort(key=lambda o: o[0])
    cells_steps = 32 * 32 * 3
    for r, w, local, rate, slowest, state in out:
        assert (w, local) == (world, r)
        assert slowest == max(fake)
        assert rate == pytest.approx(cells_steps * world / max(fake))
    # replicas are independent: both equal a single run
    from fv3d_gb300 import problems
    from oracle import pyoracle
    pr = problems.sedov(32, tend=1.0e30)
    o = pyoracle.Oracle(pr.params)
    o.set_prim(*pr.prim)
    o.advance(1.0e30, max_steps=3)
    alone = np.stack(o.get_prim())
    for o_ in out:
        np.testing.assert_array_equal(o_[5], alone)


def test_single_process_is_world_one(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from fv3d_gb300 import replicas
    assert replicas.init("gloo") == (1, 0, 0)
    rate, slowest = replicas.aggregate_rate(100, 1, 2.0)
    assert (rate, slowest) == (50.0, 2.0)
