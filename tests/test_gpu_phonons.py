"""The frozen-phonon average on the GPU (qstem_gb300.phonons.average_images)
equals the mean of the configurations run one by one."""
import numpy as np
import pytest

from conftest import Golden, rel_l2
from qstem_gb300 import lib, phonons

pytestmark = pytest.mark.gpu


def test_average_equals_mean_of_single_configurations():
    import torch
    g = Golden("sto64")
    p, atoms = g.params, g["atoms"]
    ctx = lib.Context(0)
    try:
        sigma = {8: 0.09, 38: 0.08, 22: 0.08}
        mean = phonons.average_images(ctx, p, atoms, 3, 77, sigma).cpu().numpy()
        singles = []
        for j in range(3):
            T = ctx.slices(p, phonons.displaced(atoms, j, 77, sigma))
            det, _, _ = ctx.multislice(p, T)
            singles.append(det)
        assert rel_l2(mean, np.mean(singles, axis=0)) <= 1e-6
        assert rel_l2(singles[0], singles[1]) > 1e-4  # the configurations differ
    finally:
        ctx.close()


def test_scan_tiles_sum_to_the_whole_scan():
    """The row tiles of every rank of a 3-rank split, each run through the
    library (one after another on this GPU, no collective), sum to the
    whole scan's detector images bit for bit, and match the reference's."""
    import torch
    g = Golden("sto64")
    p = g.params
    ctx = lib.Context(0)
    try:
        T = torch.from_numpy(np.ascontiguousarray(g["T"])).cuda()
        probe = torch.from_numpy(np.ascontiguousarray(g["probe"])).cuda()
        whole, _, _ = ctx.multislice(p, g["T"], g["probe"])
        tiles = [phonons.scan_images(ctx, p, T, r, 3, probe=probe).cpu().numpy() for r in range(3)]
        assert np.array_equal(np.sum(tiles, axis=0), whole)
        assert rel_l2(whole, g["det"]) <= 1e-4
    finally:
        ctx.close()
