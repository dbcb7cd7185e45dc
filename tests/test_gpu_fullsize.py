"""The measured workloads at their full sizes.

The batched STEM workload (SrTiO3 10x10x20, 512^2, 40 slices, 64x64
positions, 4 detectors): the slice stack against the oracle's, the detector
images of five positions (corners and centre of the raster) against the
oracle's run of those positions, and chunking invariance (the scan in
batches of 512 positions equals the one-batch scan bit for bit).  The TEM
workload (Si [110] 10x7x26, 1024^2, 50 slices, band limit): the exit wave of
one configuration against the oracle's.

Tolerances: stack 1e-5, detector values and exit waves 1e-4 (relative)."""
import numpy as np
import pytest

from conftest import rel_l2
from qstem_gb300 import config, lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from oracle import oracle
    oracle.build()
    c = lib.Context(0)
    yield c
    c.close()


def test_batched_stem_workload(ctx):
    import torch
    import bench
    from oracle import oracle
    p, atoms = bench.workload_params(64)
    T = torch.empty((p.slices, p.potNx, p.potNy, 2), dtype=torch.float32, device="cuda")
    ctx.slices(p, atoms, out=T)
    Th = T.cpu().numpy()
    To = oracle.transmission(p, oracle.potential(p, atoms))
    assert rel_l2(Th, To) <= 1e-5
    probe = torch.from_numpy(ctx.probe(p)).cuda()
    nt = p.thickness_count()
    det = torch.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), dtype=torch.float32, device="cuda")
    ctx.multislice(p, T, probe, det=det)
    whole = det.cpu().numpy()
    # the same scan in batches of 512 positions
    px, py, dx, dy = config.scan_offsets(p)
    parts = np.zeros_like(whole)
    for c0 in range(0, len(px), 512):
        d = torch.zeros_like(det)
        ctx.multislice(p, T, probe, positions=(px[c0:c0 + 512], py[c0:c0 + 512], dx[c0:c0 + 512],
                                               dy[c0:c0 + 512]), det=d)
        parts += d.cpu().numpy()
    assert np.array_equal(parts, whole)
    # five positions through the oracle
    pr = probe.cpu().numpy()
    for ix, iy in [(0, 0), (0, p.scanYN - 1), (p.scanXN - 1, 0), (p.scanXN - 1, p.scanYN - 1),
                   (p.scanXN // 2, p.scanYN // 2)]:
        i = ix * p.scanYN + iy
        _, do, _ = oracle.run_position(p, To, int(px[i]), int(py[i]), pr)
        got = whole[:, :, ix, iy]
        assert got.shape == do.shape
        assert np.max(np.abs(got - do) / np.maximum(np.abs(do), 1e-30)) <= 1e-4, (ix, iy, got, do)


def test_tem_workload_exit_wave(ctx):
    import bench
    from oracle import oracle
    p, configs, ctf, defoci = bench.tem_workload()
    atoms = configs[0]
    _, _, ew = ctx.tem(p, [atoms], want_exit_waves=True)
    To = oracle.transmission(p, oracle.potential(p, atoms))
    plane = np.zeros((p.nx, p.ny, 2), np.float32)
    plane[..., 0] = 1.0
    wo, _, _ = oracle.run_position(p, To, 0, 0, plane)
    assert rel_l2(ew[0], wo) <= 1e-4
