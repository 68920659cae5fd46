"""The multi-GPU arm of bench.py runs independent replicas (one hierarchy
per rank, no inter-GPU traffic on the solve path). Its host logic on CPU
with two gloo ranks over 127.0.0.1: each rank takes its own seed and
builds its own hierarchy (host-side plans), and the job time is the MAX
over ranks. And the reference arm's non-zero ranks exit 0 without work."""
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    from pamr_amrd_gb300 import workloads as W
    from pamr_amrd_gb300.solver import Solver
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    case = W.poisson2d_uneven(seed=rank, n=33, levels=3, min_boxes=2, max_boxes=4, min_side=5, max_side=17)
    s = Solver(case, host_only=True)   # this replica's own hierarchy and plans
    levels = s.num_levels()
    s.close()
    t = bench.max_over_ranks(10.0 * (rank + 1), dist, torch, "cpu")
    dist.barrier()
    out.put((rank, case.name, levels, t))
    dist.destroy_process_group()


def test_two_gloo_replicas_reduce_to_the_slowest():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    assert res[0][1] != res[1][1]                    # different seeds, different hierarchies
    assert res[0][3] == res[1][3] == 20.0            # MAX over ranks


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, timeout=120, env=env, cwd=ROOT)
    assert r.returncode == 0 and r.stdout.strip() == ""
