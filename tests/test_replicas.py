"""Several GPUs are replicas: each process runs its own jobs of the `-j/-n`
split and the processes meet only to agree on the slowest time and to add up
counts.  Here two gloo processes on the CPU stand for two GPUs: each takes
its jobs of a 4-job split of order 26 (compression 2), searches their word
ranges with the oracle, and the results are combined the way bench.py
combines replicas.  The union must be the single-job search."""
import os
import socket
import tempfile

import pytest

torch = pytest.importorskip("torch")

import golaypair_gb300 as gp  # noqa: E402
from golaypair_gb300 import replicas  # noqa: E402

ORDER, COMPRESS, PAF, NJOBS = 26, 2, 0, 4


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, outdir):
    import ctypes

    import torch.distributed as dist

    from conftest import GenStats, load_oracle

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert replicas.dist_env() == (world, rank, rank)
    orc = load_oracle()
    m = (1 << 64) - 1
    mine, neck, lines = [], 0, []
    for j in replicas.jobs_of_rank(rank, world, NJOBS):
        for k, (lo, hi) in enumerate(gp.job_ranges(ORDER, COMPRESS, PAF, j, NJOBS)):
            mine.append((lo, hi))
            pa, pb = os.path.join(outdir, f"a{rank}_{j}_{k}"), os.path.join(outdir, f"b{rank}_{j}_{k}")
            st = GenStats()
            assert orc.gpo_generate_window(ORDER, COMPRESS, PAF, pa.encode(), pb.encode(), lo >> 64, lo & m,
                                           hi >> 64, hi & m, ctypes.byref(st)) == 0
            neck += st.necklaces
            for path in (pa, pb):
                with open(path) as f:
                    lines += [("a" if path == pa else "b", ln) for ln in f.read().splitlines()]
    total = replicas.sum_over_ranks(float(neck))
    slowest = replicas.max_over_ranks(float(rank + 1))
    gathered = [None] * world
    dist.all_gather_object(gathered, (mine, lines))
    if rank == 0:
        with open(os.path.join(outdir, "result"), "w") as f:
            f.write(repr((total, slowest, gathered)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_cover_the_single_job(tmp_path, oracle_lib):
    import ctypes

    from conftest import GenStats
    world = 2
    torch.multiprocessing.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    total, slowest, gathered = eval((tmp_path / "result").read_text())
    assert slowest == world  # the max over ranks of rank + 1
    ranges = sorted(r for mine, _ in gathered for r in mine)
    for (lo1, hi1), (lo2, _) in zip(ranges, ranges[1:]):
        assert lo1 < hi1 <= lo2  # disjoint
    # the whole search in one job
    st = GenStats()
    a, b = str(tmp_path / "wa"), str(tmp_path / "wb")
    assert oracle_lib.gpo_generate(ORDER, COMPRESS, PAF, a.encode(), b.encode(), 0, 1, ctypes.byref(st)) == 0
    assert int(total) == st.necklaces
    whole = sorted([("a", ln) for ln in open(a).read().splitlines()] +
                   [("b", ln) for ln in open(b).read().splitlines()])
    assert sorted(x for _, lines in gathered for x in lines) == whole


def _lossy_worker(rank, world, port, outdir):
    import datetime

    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    if rank == 1:
        return  # this replica is lost before the step's collective
    try:
        replicas.max_over_ranks(1.0)
        outcome = "no error"
    except Exception as e:  # the loss surfaces on the host as an error
        outcome = "detected: " + type(e).__name__
    with open(os.path.join(outdir, "lossy"), "w") as f:
        f.write(outcome)


def test_lost_replica_is_detected_on_the_host(tmp_path):
    """A replica that leaves between steps: the others learn of it on the
    host when they next meet (an error from the collective, bounded by the
    process group's timeout), not by a hang."""
    import time
    t0 = time.time()
    torch.multiprocessing.spawn(_lossy_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    assert (tmp_path / "lossy").read_text().startswith("detected")
    assert time.time() - t0 < 60
