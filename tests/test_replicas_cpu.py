"""Multi-GPU replicas, host side, on the CPU: the frame partition, reassembly in
frame order, and a world_size-2 gloo run of replicas.run_sharded -- the split
a strong-scaling job takes -- in which each rank reconstructs the frame list
it is given (the FP64 oracle stands in for the per-GPU engine) and rank 0
collects the images: they must equal a single-process reconstruction of all
frames, and each rank must have been given exactly its shard."""
import os
import socket

import numpy as np
import pytest

from risa_gb300 import replicas

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("n,world,planes", [(12, 2, 2), (12, 3, 1), (7, 4, 1), (8, 3, 2), (4, 8, 2)])
def test_shard_partition(n, world, planes):
    shards = [replicas.shard_indices(n, r, world, planes) for r in range(world)]
    allidx = np.concatenate(shards)
    assert sorted(allidx.tolist()) == list(range(n))  # every frame once
    for s in shards:
        assert (s % planes == np.arange(len(s)) % planes).all()  # still plane-interleaved
        assert (np.diff(s) > 0).all()
    imgs = [np.stack([np.full((2, 2), i, np.float32) for i in s]) if len(s) else np.zeros((0, 2, 2), np.float32)
            for s in shards]
    out = replicas.reassemble(imgs, n, world, planes)
    assert (out[:, 0, 0] == np.arange(n)).all()


def test_shard_rejects_bad_arguments():
    with pytest.raises(ValueError):
        replicas.shard_indices(5, 0, 2, 2)  # not a multiple of the plane count
    with pytest.raises(ValueError):
        replicas.shard_indices(4, 2, 2, 1)


def _case():
    from risa_gb300 import phantom
    from tests.helpers import SMALL, ns

    d = dict(SMALL, n_planes=2, source_diameter=[430.0, 430.0], delta_x=[0.0, 0.0],
             delta_z=[1417.0, 1430.0], source_angle=[360.0, 360.0], n_par_proj=48, n_par_det=64, n_pixels=48)
    sc = phantom.make_scan(4, 2, 500, 432, 215.0, 240.0, seed=21, defect_fraction=0.01, distinct=4)
    return ns(d), sc


def _oracle_fbp(g, sc, idx):
    import oracle

    op = oracle.make_params(quirk=oracle.QUIRK_NONE, filter_type="sheppLogan", defects=True, masking=True)
    ref, dark = oracle.attenuation_init(sc.ref, sc.dark, 2, 0.67, 1.5, True, oracle.QUIRK_NONE)
    rec = oracle.f2p_records(g, oracle.QUIRK_NONE)
    return oracle.fbp(g, op, rec, ref, dark, sc.raw[idx], sc.planes[idx], n_threads=1)


def _rank(rank, world, port, outdir):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        g, sc = _case()
        n = sc.raw.shape[0]
        given = []

        def worker(idx):
            given.append(np.asarray(idx))
            return _oracle_fbp(g, sc, idx)

        images = replicas.run_sharded(n, 2, worker)
        np.save(os.path.join(outdir, f"given{rank}.npy"), given[0])
        slowest = replicas.max_over_ranks(1.5 + rank)
        if rank == 0:
            np.save(os.path.join(outdir, "gathered.npy"), images)
            np.save(os.path.join(outdir, "slowest.npy"), np.array([slowest]))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_match_one_process(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    g, sc = _case()
    expect = _oracle_fbp(g, sc, np.arange(sc.raw.shape[0]))
    got = np.load(tmp_path / "gathered.npy")
    np.testing.assert_array_equal(got, expect)
    n = sc.raw.shape[0]
    for r in range(world):
        np.testing.assert_array_equal(np.load(tmp_path / f"given{r}.npy"), replicas.shard_indices(n, r, world, 2))
    assert float(np.load(tmp_path / "slowest.npy")[0]) == 2.5
