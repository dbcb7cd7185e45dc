"""Frozen-phonon configurations split across ranks and the averaged images
(qstem_gb300/phonons.py), with two CPU ranks over gloo: the multi-GPU path's
host side, which needs no GPU."""
import os
import socket

import numpy as np
import pytest

from qstem_gb300 import config, phonons


def test_rank_configurations_partition_the_set():
    for world in (1, 2, 3, 4):
        got = sorted(j for r in range(world) for j in phonons.rank_configurations(30, r, world))
        assert got == list(range(30))
    with pytest.raises(ValueError):
        phonons.rank_configurations(4, 2, 2)


def test_displacements_are_seeded_and_per_element():
    atoms, *_ = config.replicate(config.srtio3_cell(), 2, 2, 2)
    a = phonons.displaced(atoms, 3, 1000, {8: 0.09, 38: 0.08, 22: 0.08})
    b = phonons.displaced(atoms, 3, 1000, {8: 0.09, 38: 0.08, 22: 0.08})
    c = phonons.displaced(atoms, 4, 1000, {8: 0.09, 38: 0.08, 22: 0.08})
    assert np.array_equal(a, b) and not np.array_equal(a["x"], c["x"])
    d = phonons.displaced(atoms, 3, 1000, {8: 0.09})
    assert np.array_equal(d["x"][atoms["Znum"] == 38], atoms["x"][atoms["Znum"] == 38])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, nconf, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        acc = phonons.ImageSum(torch.zeros((2, 3, 4, 4)))
        for j in phonons.rank_configurations(nconf, rank, world):
            acc.add(torch.full((2, 3, 4, 4), float(j)) + torch.arange(16.0).reshape(4, 4))
        mean = acc.mean()
        np.save(out % rank, mean.numpy())
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_average_like_one():
    import tempfile

    import torch.multiprocessing as mp
    nconf = 7
    d = tempfile.mkdtemp()
    out = os.path.join(d, "mean_%d.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), nconf, out), nprocs=2, join=True, start_method="spawn")
    want = np.mean([np.full((2, 3, 4, 4), float(j)) + np.arange(16.0).reshape(4, 4) for j in range(nconf)], axis=0)
    for r in range(2):
        got = np.load(out % r)
        assert np.allclose(got, want, rtol=1e-6, atol=1e-6)


def test_single_process_mean_without_distributed():
    import torch
    acc = phonons.ImageSum(torch.zeros(3))
    for v in (1.0, 2.0, 6.0):
        acc.add(torch.full((3,), v))
    assert torch.allclose(acc.mean(), torch.full((3,), 3.0))
    with pytest.raises(ValueError):
        phonons.ImageSum(torch.zeros(1)).mean()
