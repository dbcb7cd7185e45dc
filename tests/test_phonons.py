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


def test_rank_positions_tile_the_raster():
    """Every raster position on exactly one rank, in whole scan rows, in
    raster order within a rank."""
    from qstem_gb300 import config
    p = config.make_params(nx=64, resolutionX=0.1, v0=200, slices=4, sliceThickness=2.0, ax=20.0, by=20.0, c=8.0,
                           scan=(2.0, 8.0, 7, 2.0, 8.0, 5), detectors=[(40, 100, "A")])
    full = config.scan_offsets(p)
    for world in (1, 2, 3, 4, 7, 9):
        parts = [phonons.rank_positions(p, r, world) for r in range(world)]
        for k in range(4):
            assert np.array_equal(np.concatenate([q[k] for q in parts]), full[k])
        for q in parts:
            assert len(q[0]) % p.scanYN == 0
    with pytest.raises(ValueError):
        phonons.rank_positions(p, 2, 2)


def _scan_rank_main(rank, world, port, out):
    import torch.distributed as dist
    from oracle import oracle
    from oracle_ctx import OracleContext
    from conftest import Golden
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        oracle.build()
        g = Golden("sto64")
        det = phonons.scan_images(OracleContext(), g.params, g["T"], rank, world, probe=g["probe"])
        np.save(out % rank, det.numpy())
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(180)
def test_scan_split_across_two_gloo_ranks():
    """One configuration's scan split into row tiles on two ranks (the
    oracle stands in for each rank's GPU) and all-reduced: every rank ends
    with the reference's detector images of the whole raster."""
    import tempfile

    import torch.multiprocessing as mp
    from conftest import Golden
    d = tempfile.mkdtemp()
    out = os.path.join(d, "det_%d.npy")
    mp.start_processes(_scan_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    want = Golden("sto64")["det"]
    for r in range(2):
        got = np.load(out % r)
        assert got.shape == want.shape
        assert np.linalg.norm(got - want) <= 1e-6 * np.linalg.norm(want)
