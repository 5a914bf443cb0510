"""bench.py's multi-rank host logic with two gloo ranks on the CPU: the
slowest rank's time is the job's, the value is the whole job's frames/s,
every rank fuses its own scene, and the reference arm runs on rank 0 alone."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    slowest = bench.max_over_ranks(10.0 + 5.0 * rank, w, device="cpu")
    both = bench.max_over_ranks(3.0, w, device="cpu")
    value = bench.job_throughput(w, 95, slowest / 1e3)
    seeds = [None] * w
    dist.all_gather_object(seeds, bench.rank_seed(r))

    class Args:
        steps, warmup, prefill = 2, 1, 1

    buf = io.StringIO()
    if r != 0:
        with redirect_stdout(buf):
            bench.run_reference(Args, r, w)  # other ranks return at once, printing nothing
    dist.barrier()
    dist.destroy_process_group()
    out.put((r, w, local, slowest, both, value, seeds, buf.getvalue()))


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, local, slowest, both, value, seeds, printed) in enumerate(res):
        assert (rank, world, local) == (r, 2, r)
        assert slowest == 15.0 and both == 3.0  # the max over ranks, identical on both
        assert value == pytest.approx(2 * 95 / 0.015)
        assert seeds[0] != seeds[1]
        assert printed == ""


def test_cpu_aggregate_runs_one_sample_per_process():
    """The multi-core CPU aggregate: each spawned process runs the bounded
    single-core sample from the same resident volume; frames/s are summed."""
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    from merge_fusion_gb300 import scenes
    frames, poses = scenes.render_room_torch(3, seed=0, device="cpu")
    frames = frames.numpy().view(np.uint16)
    resident = (np.zeros(0, np.uint32), np.zeros((0, 2), np.float32))
    total, res = bench.cpu_aggregate(frames, poses, 1, 1, 0.01, resident, 2)
    assert len(res) == 2 and all(r[2] == 1 for r in res)
    assert abs(total - sum(r[0] for r in res)) < 1e-9 and total > 0
    info = bench.host_cpu()
    assert info["nproc"] >= 1 and info["cpu_model"]
