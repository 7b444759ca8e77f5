"""World-size-2 gloo run of the benchmark's replica path on CPU: rank-local workloads, the
max-over-ranks timing, the whole-job throughput, and the reference arm running on rank 0 only.
(The path has no data exchange between ranks: realizations are independent replicas.)"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, outdir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import __graft_entry__ as ge
    import bench
    d, r, ws = bench._dist()
    assert d is not None and r == rank and ws == world and d.get_backend() == "gloo"
    pkg = ge.load_package()
    N, logK, dh, Qs, obs = bench.make_workload(pkg, 2, seed0=1000 * r, grid=(6, 5, 4), mins=(0, 0, 0),
                                               maxs=(10, 8, 3))
    # each rank's timed region differs; the job is as slow as its slowest rank
    t = bench._max_over_ranks(d, 0.5 + r)

    class Args:
        steps, warmup = 1, 0
    ref = bench.run_reference(Args, d, r, ws) if r != 0 else "skipped"
    np.savez(os.path.join(outdir, "rank%d.npz" % r), logK=logK, N=N, t=t, nobs=len(obs[0]),
             ref_none=(ref is None), value=bench.replica_throughput(2, 3, ws, t))
    d.barrier()
    dist.destroy_process_group()


def test_replicas_world_size_2(tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    r0 = np.load(tmp_path / "rank0.npz")
    r1 = np.load(tmp_path / "rank1.npz")
    assert int(r0["N"]) == int(r1["N"]) == 120
    assert r0["logK"].shape == r1["logK"].shape == (240,)
    assert not np.allclose(r0["logK"], r1["logK"])      # each rank solves its own realizations
    assert float(r0["t"]) == float(r1["t"]) == 1.5      # max over ranks, seen by every rank
    assert bool(r1["ref_none"])                         # reference arm: rank 1 does no work
    assert float(r0["value"]) == pytest.approx(2 * 3 * 2 / 1.5)
