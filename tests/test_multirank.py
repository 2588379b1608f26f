"""The benchmark's multi-process path on the CPU (gloo, world size 2).

bench.py runs one replica per GPU (independent meshes, no data-path
collective); its only cross-rank step is the max over ranks of the timed
values.  Two spawned processes check the rank discovery from the launcher's
environment, that reduction, and that the reference arm does no work on
ranks other than 0."""
import json
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r = bench._dist()
    v = bench._barrier_max(10.0 * (rank + 1), ws)

    class Args:                       # the reference arm returns at once off rank 0
        steps, warmup, gpus = 1, 0, world
    ran = "skipped"
    if r != 0:
        bench.run_reference(Args())
        ran = "returned"
    dist.destroy_process_group()
    out.put(json.dumps({"rank": r, "ws": ws, "max": v, "ref": ran}))


def test_two_ranks_reduce_max_and_reference_arm_idles():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [json.loads(q.get(timeout=120)) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort(key=lambda d: d["rank"])
    assert [d["rank"] for d in res] == [0, 1]
    assert all(d["ws"] == 2 for d in res)
    assert all(d["max"] == 20.0 for d in res)
    assert res[1]["ref"] == "returned"
