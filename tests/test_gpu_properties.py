"""Size-independent properties of the GPU multislice at full workload sizes,
where the oracle would take too long: conservation of |psi|^2, translation
equivariance of the scan, batch independence and determinism."""
import numpy as np
import pytest

from conftest import rel_l2
from qstem_gb300 import config, lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = lib.Context(0)
    yield c
    c.close()


def cfg3(npix=4, slices=40, ncell=(10, 10, 20)):
    """The 512^2 batched-STEM geometry (SrTiO3 10x10x20, 40 slices)."""
    atoms, ax, by, c = config.replicate(config.srtio3_cell(), *ncell)
    a = 3.905
    p = config.make_params(nx=512, resolutionX=39.05 / 512, v0=200, slices=slices, sliceThickness=1.9525, ax=ax,
                           by=by, c=c, scan=(19.525, 23.43, npix, 19.525, 23.43, npix),
                           detectors=[(0, 10, "BF"), (10, 25, "LAADF"), (25, 70, "MAADF"), (70, 200, "HAADF")],
                           alpha=20)
    return p, atoms


def test_vacuum_conserves_intensity(ctx):
    """Empty specimen: the probe lies inside the 2/3 band, so every slice
    keeps sum|psi|^2 = N and the exit intensity equals the probe's."""
    p, _ = cfg3(npix=2, slices=40)
    empty = np.zeros(0, dtype=config.abi.ATOM_DTYPE)
    T = ctx.slices(p, empty)
    _, _, ew = ctx.multislice(p, T, want_det=False, want_exit_waves=True)
    N = p.nx * p.ny
    for w in ew:
        assert abs(np.sum(w.astype(np.float64) ** 2) / N - 1) < 1e-4


def test_full_size_determinism_and_batch_independence(ctx):
    import torch
    p, atoms = cfg3(npix=8)
    T = torch.from_numpy(ctx.slices(p, atoms)).cuda()
    nt = p.thickness_count()
    det1 = torch.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), device="cuda")
    det2 = torch.zeros_like(det1)
    ctx.multislice(p, T, det=det1)
    ctx.multislice(p, T, det=det2)
    assert torch.equal(det1, det2)  # no atomics on the multislice path
    # position 5 alone gives the same pixel as in the full batch
    px, py, dx, dy = config.scan_offsets(p)
    sel = [np.array([v[5]]) for v in (px, py, dx, dy)]
    det3 = torch.zeros_like(det1)
    ctx.multislice(p, T, positions=sel, det=det3)
    i, j = dx[5], dy[5]
    assert torch.equal(det3[:, :, i, j], det1[:, :, i, j])


def test_translation_equivariance(ctx):
    """With 50 pixels per SrTiO3 unit cell, windows one cell apart see the
    same periodic potential, so their diffraction patterns agree (up to the
    float rounding of the atom coordinates)."""
    ncell = (14, 14, 4)
    atoms, ax, by, c = config.replicate(config.srtio3_cell(), *ncell)
    res = 3.905 / 50
    p = config.make_params(nx=512, resolutionX=res, v0=200, slices=8, sliceThickness=1.9525, ax=ax, by=by, c=c,
                           scan=(3.905 * 7, 3.905 * 8, 1, 3.905 * 7, 3.905 * 8, 1), detectors=[], alpha=20)
    assert p.potNx - p.nx == 50
    T = ctx.slices(p, atoms)
    pos = (np.array([0, 50, 0, 50]), np.array([0, 0, 50, 50]), np.zeros(4), np.zeros(4))
    _, dp, _ = ctx.multislice(p, T, positions=pos, want_det=False, want_diffpats=True)
    for k in (1, 2, 3):
        assert rel_l2(dp[k], dp[0]) < 1e-4


def test_detector_sum_rules(ctx):
    """BF+LAADF+MAADF+HAADF annuli partition 0..200 mrad; their sum equals the
    total intensity inside 200 mrad of the final diffraction pattern."""
    p, atoms = cfg3(npix=2, slices=10, ncell=(10, 10, 5))
    T = ctx.slices(p, atoms)
    det, dps, _ = ctx.multislice(p, T, want_diffpats=True)
    final = det[-1]  # [ndet][x][y]
    scaleDiff = 1.0 / np.sqrt(p.nx * p.ny)
    N = p.nx * p.ny
    scale = float(np.float32(p.electronScale)) / (N * N)
    for pos in range(4):
        I = dps[pos].astype(np.float64) / scaleDiff
        # the four annuli overlap only on their shared boundaries (measure zero on this grid)
        total_det = sum(final[d].ravel()[pos] for d in range(4))
        assert total_det <= I.sum() * scale * (1 + 1e-5)
        assert total_det > 0
