"""Multi-GPU as replicas: the host logic of `bench.py --gpus N` (max of the
step time over ranks) and of the sharded sweep (independent units split
round robin, gathered on rank 0), run as two gloo processes on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from hamiltonian_diagonalization_gb300 import sweep
        # the job is charged the slowest replica's time
        slowest = bench.max_over_ranks(10.0 + rank, "cpu")
        units = sweep.work_units([0, 2, 4, 6, 8], 64, 32)
        mine = sweep.shard(units, rank, world)
        done = {f"{t},{j0 + j}": rank for (t, j0, c) in mine for j in range(c)}
        parts = sweep.gather_to_rank0(done)
        if rank == 0:
            merged = {}
            for p in parts:
                assert not (set(merged) & set(p))      # no unit solved twice
                merged.update(p)
            out.put((slowest, len(units), len(merged), sorted(set(merged.values()))))
        else:
            assert parts is None
    finally:
        dist.destroy_process_group()


def test_replica_host_logic_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    slowest, nunits, nsolves, ranks = out.get(timeout=10)
    assert slowest == 11.0
    assert nunits == 10 and nsolves == 320 and ranks == [0, 1]


def test_sharding_covers_every_unit_once():
    from hamiltonian_diagonalization_gb300 import sweep
    units = sweep.work_units([0, 2, 4], 50, 16)
    assert [u[2] for u in units if u[0] == 0] == [16, 16, 16, 2]
    for world in (1, 2, 3, 8):
        got = [u for r in range(world) for u in sweep.shard(units, r, world)]
        assert sorted(got) == sorted(units)


@pytest.mark.parametrize("npts,stride", [(64, 4), (5, 4), (9, 4), (12, 3), (1, 4)])
def test_continuation_plan_covers_points_once(npts, stride):
    import numpy as np

    from hamiltonian_diagonalization_gb300 import sweep
    v1s = np.linspace(0.5, 3.0, npts)
    anchors, rest, near = sweep.continuation_plan(v1s, stride)
    assert sorted(anchors.tolist() + rest.tolist()) == list(range(npts))
    assert anchors[0] == 0 and np.all(np.diff(anchors) == stride)
    step = v1s[1] - v1s[0] if npts > 1 else 0.0
    for i, a in zip(rest, near):
        d = np.abs(v1s[anchors] - v1s[i])
        assert d[a] == d.min() and d[a] <= (stride - 1) * step + 1e-12
