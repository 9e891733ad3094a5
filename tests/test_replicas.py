"""Replicas: the photon path shards by photon index (one Philox stream per photon, disjoint
index ranges per rank) and needs no collective on the data path; the only exchange is a
sum of the raw accumulators, done once at the end (as the reference's dead MPI path would,
cpp/3d/MC3D.hpp:1777-1790).  Checked with two gloo ranks on the CPU oracle, and on the GPU
with photon offsets."""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle
from golden.make_golden import cases

N = 6000


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch
    p = cases()["phantom3d"][0]
    share = N // world
    r = oracle.run(p, rng=oracle.RNG_PHILOX, nthreads=1, nphoton=share, photon_offset=rank * share,
                   seed=4242, normalize=False)
    acc = torch.tensor(np.concatenate([r.ER, r.EBR, [float(r.steps)]]))
    dist.all_reduce(acc, op=dist.ReduceOp.SUM)
    if rank == 0:
        q.put(acc.numpy())
    dist.destroy_process_group()


def test_two_gloo_replicas_sum_to_one_run(built):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    got = q.get(timeout=120)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    p = cases()["phantom3d"][0]
    full = oracle.run(p, rng=oracle.RNG_PHILOX, nthreads=1, nphoton=N, seed=4242, normalize=False)
    want = np.concatenate([full.ER, full.EBR, [float(full.steps)]])
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-15)


@pytest.mark.gpu
def test_gpu_photon_offsets_are_disjoint_slices_of_one_stream(built):
    import valomc_gb300 as V
    p = cases()["phantom3d"][0]
    a = V.run(p, nphoton=20000, seed=9, photon_offset=0, normalize=False, precision=V.VMC_FP64)
    b = V.run(p, nphoton=20000, seed=9, photon_offset=20000, normalize=False, precision=V.VMC_FP64)
    c = V.run(p, nphoton=40000, seed=9, photon_offset=0, normalize=False, precision=V.VMC_FP64)
    np.testing.assert_allclose(a.ER + b.ER, c.ER, rtol=1e-9, atol=1e-300)
    assert a.stats["steps"] + b.stats["steps"] == c.stats["steps"]
