"""The N > 1 path of the bench on the CPU: two ranks over torch.distributed's gloo
backend (127.0.0.1), run as the driver launches them (RANK, WORLD_SIZE,
MASTER_ADDR, MASTER_PORT in the environment).  Circuits are independent, so each
rank takes its own seeded slice (seed + rank) and solves it with no collective on
the data path; the only collectives are the barrier around the timed region and
the max over ranks of its time, and the whole job's rate is every rank's units
over that slowest time.  Here the oracle solves each rank's slice (no GPU)."""
import os
import socket
import sys
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, B, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    from oracle import oracle as orc
    r, w, local = bench.dist_env()
    assert (r, w, local) == (rank, world, rank)
    dist.init_process_group("gloo", rank=r, world_size=w)
    el, nn, vals = bench.generator("bjt_ce")(B, 7 + r)  # the bench's slice: seed + rank
    pk = orc.Packed(el, nn, vals[0])
    dist.barrier()
    t0 = time.perf_counter()
    ok = 0
    for c in range(B):
        pk.values[:] = vals[c]
        ok += orc.op(pk, orc.options(reltol=1e-6))[0] == 0
    if r == 1:
        time.sleep(0.2)  # one rank slower: the job's time is its
    mine = time.perf_counter() - t0
    t = torch.tensor([mine], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total = torch.tensor([float(ok)], dtype=torch.float64)
    dist.all_reduce(total, op=dist.ReduceOp.SUM)
    fp = torch.tensor([float(vals.sum())], dtype=torch.float64)
    fps = [torch.zeros(1, dtype=torch.float64) for _ in range(w)]
    dist.all_gather(fps, fp)
    dist.barrier()
    np.save(os.path.join(out_dir, "rank%d.npy" % r),
            np.array([mine, float(t.item()), float(total.item()), ok] + [float(f.item()) for f in fps]))
    dist.destroy_process_group()


def test_two_ranks_share_the_work_and_time_the_slowest(tmp_path):
    world, B = 2, 64
    mp.spawn(rank_main, args=(world, free_port(), B, str(tmp_path)), nprocs=world, join=True)
    res = [np.load(os.path.join(tmp_path, "rank%d.npy" % r)) for r in range(world)]
    mine = [x[0] for x in res]
    # every rank saw the same max, the slowest rank's own time
    assert res[0][1] == res[1][1] == max(mine) and max(mine) >= 0.2
    # all circuits of both slices solved, and the slices are different circuits
    assert res[0][2] == res[1][2] == world * B and res[0][3] == res[1][3] == B
    assert res[0][4] != res[0][5] and list(res[0][4:]) == list(res[1][4:])
    # the whole job's rate as the bench reports it: every rank's units over the slowest time
    value = world * B / res[0][1]
    assert value <= world * B / min(mine)


def rank_dies(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import datetime
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=5))
    if rank == 1:
        os._exit(3)  # leaves between steps, with nothing in flight
    t0 = time.perf_counter()
    try:
        dist.barrier()
        outcome = "returned"
    except RuntimeError as e:
        outcome = "error: " + str(e).splitlines()[0][:200]
    with open(os.path.join(out_dir, "rank0.txt"), "w") as f:
        f.write("%s\n%.3f\n" % (outcome, time.perf_counter() - t0))


def test_a_rank_that_leaves_ends_the_others_collective_with_an_error(tmp_path):
    """A rank that exits between steps: the surviving rank's next collective ends
    with an error within the process group's timeout instead of waiting for ever."""
    ctx = mp.get_context("spawn")
    port = free_port()
    procs = [ctx.Process(target=rank_dies, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    for p in procs:
        if p.is_alive():
            p.kill()
            pytest.fail("a rank did not finish")
    assert procs[1].exitcode == 3
    outcome, secs = open(os.path.join(tmp_path, "rank0.txt")).read().split("\n")[:2]
    assert outcome.startswith("error"), outcome
    assert float(secs) < 60
