"""The replica path of bench.py on CPU: two gloo ranks, each with frames of its own, a barrier
and the max-over-ranks time that the whole-job rate is divided by; the reference arm's other
ranks exit without work."""
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, _ = bench.dist_init()
    barrier, max_over_ranks = bench.rank_sync(w, "cpu")
    barrier()
    q.put((r, w, max_over_ranks(10.0 + 5.0 * r), bench.frame_indices(r, 8)))
    barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, *_ in res] == [0, 1] and all(w == 2 for _, w, _, _ in res)
    assert all(t == 15.0 for _, _, t, _ in res)  # both ranks divide by the slower rank's time
    f0, f1 = res[0][3], res[1][3]
    assert len(f0) == len(f1) == 8 and not set(f0) & set(f1)  # weak scaling: distinct frames


def test_one_rank_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench
    barrier, max_over_ranks = bench.rank_sync(1, "cpu")
    barrier()
    assert max_over_ranks(3.5) == 3.5
    assert bench.frame_indices(0, 3) == [0, 1, 2]


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
