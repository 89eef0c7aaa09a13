"""Multi-GPU form of the benchmark: independent replicas, one per rank, no
collective on the data path; the job's time is the slowest rank's and its
work the sum over ranks.  Checked here with two gloo ranks on the CPU, each
stepping its replica through the CPU restatement of the time step."""
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


def _rank_main(rank, world, port, out_dir):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "sci-solver_level-set_gb300"), os.path.join(root, "oracle"), root):
        sys.path.insert(0, p)
    import bench
    import lsoracle
    import synth

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = synth.workload("c2", n=8)
    ol = lsoracle.OracleLayout(3, w["xyz"], w["elems"], w["npart"], w["nparts"])
    prm = ol.params(update_kind=lsoracle.UPDATE["advect"], dt=w["dt"], bandwidth=w["bandwidth"], nthreads=1)
    hist, _, _, st = ol.solve(prm, w["phi0"], w["vel"], 2)
    ms = 10.0 + rank  # a stand-in per-rank time: rank 1 is the slow one
    ms_job, updates_job = bench.job_totals(ms, st["nb_vertex_updates"], dist)
    np.savez(os.path.join(out_dir, "rank%d.npz" % rank), phi=hist[-1], updates=st["nb_vertex_updates"],
             ms_job=ms_job, updates_job=updates_job)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replica_ranks(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    r = [np.load(str(tmp_path / ("rank%d.npz" % k))) for k in range(world)]
    # replicas: identical work and results on every rank
    assert np.array_equal(r[0]["phi"], r[1]["phi"])
    assert int(r[0]["updates"]) == int(r[1]["updates"]) > 0
    for k in range(world):
        assert float(r[k]["ms_job"]) == 11.0  # max over ranks
        assert float(r[k]["updates_job"]) == 2 * int(r[0]["updates"])  # sum over ranks
