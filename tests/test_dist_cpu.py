"""Multi-process host logic of bench.py on CPU with two gloo ranks (the replicas path for
N > 1): the rendezvous from the torchrun environment, the barrier around the timed region,
and the max-over-ranks reduction that turns per-rank times into the job's time.  The
reference arm runs on rank 0 only; the other ranks return without work or output."""
import contextlib
import io
import os
import socket
import types

import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    w, r, local, pg = bench.dist_setup()
    bench.barrier(pg)
    v = bench.allmax(pg, 1.5 + r)
    out = ""
    if r != 0:
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            bench.run_reference(types.SimpleNamespace(gpus=world, steps=1, warmup=0), w, r, pg)
        out = buf.getvalue()
    bench.barrier(pg)
    q.put((r, w, local, v, out))
    pg.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(60)
    assert [p.exitcode for p in procs] == [0, 0]
    assert res == [(0, 2, 0, 2.5, ""), (1, 2, 1, 2.5, "")]
