"""Shard arithmetic of the multi-rank path, on CPU (gloo, world size 2).

The weight solves shard by evaluation rows with no data-path collective.  This test checks
the host-side row partition that bench.py uses under torchrun (bench.node_set /
bench.shard_rows: rank r owns rows [r*R, (r+1)*R) of one global node set) and the max-over-
ranks timing reduction.  Each rank computes its shard with the CPU oracle -- not with
librbffd, which needs a GPU -- and the gathered shards must equal the single-rank operator.
The library's own row-range interface (rbffd_problem.row_begin/row_end) is checked on the
GPU by test_gpu_parity.py::test_row_range_shards."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, root, out_dir):
    import sys

    sys.path.insert(0, root)
    import bench
    from oracle import oracle as orc

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    nx = 24
    X, _ = bench.node_set(nx, world)  # nx columns x (nx * world) rows, rows ordered x-fastest
    rb, re = bench.shard_rows(rank, world, nx * nx)
    p, n, deg, ops = bench.WORKLOAD["p"], bench.WORKLOAD["n"], bench.WORKLOAD["deg"], bench.WORKLOAD["ops"]
    r = orc.generate(X, X[rb:re], p, n, deg, ops, nthreads=1)
    W = torch.from_numpy(np.ascontiguousarray(r["W"]))
    C = torch.from_numpy(r["cols"].astype(np.int64))
    Ws = [torch.empty_like(W) for _ in range(world)]
    Cs = [torch.empty_like(C) for _ in range(world)]
    dist.all_gather(Ws, W)
    dist.all_gather(Cs, C)
    t = bench.max_over_ranks(float(rank + 1), dist)
    if rank == 0:
        np.save(os.path.join(out_dir, "W.npy"), torch.cat(Ws, 1).numpy())
        np.save(os.path.join(out_dir, "C.npy"), torch.cat(Cs, 0).numpy())
        np.save(os.path.join(out_dir, "t.npy"), np.array([t]))
    dist.barrier()
    dist.destroy_process_group()


def test_row_shards_gather_to_full_operator(tmp_path, orc):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), root, str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    import sys

    sys.path.insert(0, root)
    import bench

    X, _ = bench.node_set(24, world)
    p, n, deg, ops = bench.WORKLOAD["p"], bench.WORKLOAD["n"], bench.WORKLOAD["deg"], bench.WORKLOAD["ops"]
    full = orc.generate(X, X, p, n, deg, ops)
    W = np.load(tmp_path / "W.npy")
    C = np.load(tmp_path / "C.npy")
    assert (C == full["cols"]).all()
    assert np.array_equal(W, full["W"])  # same arithmetic per row: bit-identical
    assert float(np.load(tmp_path / "t.npy")[0]) == 2.0  # max over ranks


def test_shard_rows_partition():
    import bench

    for world in (1, 2, 4, 8):
        spans = [bench.shard_rows(r, world, 1000) for r in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == 1000 * world
        assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
