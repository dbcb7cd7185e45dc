"""The wave-resident slice loop of 256^2 waves (QS_RESIDENT: one launch; each
wave held by a cluster of four CTAs in distributed shared memory for all of
its slices) against the two-pass loop (a row and a column pass per slice
through HBM) and against the oracle.

Both loops make the same float operations on every element of the wave, so
patterns and exit waves agree to 1e-6 (the detector sums add their partial
sums in another order); against the oracle the multislice contract's 1e-4
holds."""
import numpy as np
import pytest

from conftest import rel_l2
from qstem_gb300 import config, lib

pytestmark = pytest.mark.gpu

TOL_MS = 1e-4
TOL_SAME = 1e-6
DETS = [(0, 10, "BF"), (10, 25, "LA"), (25, 70, "MA"), (70, 200, "HAADF")]


@pytest.fixture(scope="module")
def ctx():
    from oracle import oracle
    oracle.build()
    c = lib.Context(0)
    yield c
    c.close()


def sto256(slices=8, scan_px=3, out_every=3, ncell=(5, 5, 4), alpha=20.0, res=(0.0763, 0.0763)):
    cell = config.srtio3_cell()
    atoms, ax, by, c = config.replicate(cell, *ncell)
    a = 3.905
    x0, y0 = a * (ncell[0] // 2), a * (ncell[1] // 2)
    p = config.make_params(nx=256, resolutionX=res[0], resolutionY=res[1], v0=200.0, slices=slices,
                           sliceThickness=1.9525, ax=ax, by=by, c=c, scan=(x0, x0 + a, scan_px, y0, y0 + a, scan_px),
                           detectors=DETS, alpha=alpha, outputInterval=out_every)
    return p, atoms


@pytest.fixture(scope="module")
def case(ctx):
    from oracle import oracle
    p, atoms = sto256()
    T = ctx.slices(p, atoms)
    return p, atoms, T, oracle.transmission(p, oracle.potential(p, atoms))


def test_resident_vs_two_pass_and_oracle(ctx, case):
    """Detector images of every thickness slot, final patterns and exit
    waves of a 3x3 scan."""
    from oracle import oracle
    p, _, T, To = case
    out = ctx.multislice(p, T, want_diffpats=True, want_exit_waves=True, resident=True)
    two = ctx.multislice(p, T, want_diffpats=True, want_exit_waves=True)
    for r, t in zip(out, two):
        assert float(np.abs(t).max()) > 0
        assert rel_l2(r, t) <= TOL_SAME
    ref = oracle.stem(p, To, diffpats=True, exit_waves=True)
    det, dps, ews = ctx.multislice(p, To, want_diffpats=True, want_exit_waves=True, resident=True)
    for r, o in zip((det, dps, ews), ref):
        assert rel_l2(r, o) <= TOL_MS


def test_resident_series_patterns(ctx, case):
    """QS_SERIES patterns (collectIntensity's diff_<t>.img): one per slot,
    from one resident launch."""
    p, _, T, _ = case
    _, dps, _ = ctx.multislice(p, T, want_det=False, want_diffpats=True, series=True, resident=True)
    _, dpt, _ = ctx.multislice(p, T, want_det=False, want_diffpats=True, series=True)
    assert dps.shape[0] == p.thickness_count()
    for k in range(dps.shape[0]):
        assert rel_l2(dps[k], dpt[k]) <= TOL_SAME, k


def test_resident_slabs_and_sequences(ctx, case):
    """Two slabs through one reused stack and a stacking sequence: the step
    table of the resident launch walks the same slices as the two passes."""
    p, _, T, _ = case
    q = p.copy()
    q.cellDiv = 2
    r = ctx.multislice(q, T, want_diffpats=True, resident=True)
    t = ctx.multislice(q, T, want_diffpats=True)
    assert rel_l2(r[0], t[0]) <= TOL_SAME and rel_l2(r[1], t[1]) <= TOL_SAME
    s = p.copy()
    s.mulsRepeat1, s.mulsRepeat2 = 2, 2
    r = ctx.multislice(s, T, want_diffpats=True, resident=True)
    t = ctx.multislice(s, T, want_diffpats=True)
    assert rel_l2(r[0], t[0]) <= TOL_SAME and rel_l2(r[1], t[1]) <= TOL_SAME


def test_resident_device_buffers_and_graph(ctx, case):
    """Device buffers, an explicit batch of window offsets and the graph
    replay of the resident launch."""
    torch = pytest.importorskip("torch")
    p, _, T, _ = case
    Td = torch.from_numpy(np.ascontiguousarray(T)).cuda()
    n = 40
    rng = np.random.default_rng(5)
    ix = rng.integers(0, p.potNx - p.nx + 1, n).astype(np.int32)
    iy = rng.integers(0, p.potNy - p.ny + 1, n).astype(np.int32)
    pos = (ix, iy, np.zeros(n, np.int32), np.arange(n, dtype=np.int32) % p.scanYN)
    dp = torch.zeros((n, p.nx, p.ny), dtype=torch.float32, device="cuda")
    ctx.multislice(p, Td, positions=pos, want_det=False, diffpats=dp)
    want = dp.cpu().numpy().copy()
    for _ in range(3):
        dp.zero_()
        ctx.multislice(p, Td, positions=pos, want_det=False, diffpats=dp, graph=True, resident=True)
        assert rel_l2(dp.cpu().numpy(), want) <= TOL_SAME


def test_non_square_pixels(ctx):
    """Different x and y sampling: the band keeps fewer columns than rows."""
    from oracle import oracle
    p, atoms = sto256(slices=4, scan_px=2, out_every=2, res=(0.0763, 0.0691))
    To = oracle.transmission(p, oracle.potential(p, atoms))
    det, dps, ews = ctx.multislice(p, To, want_diffpats=True, want_exit_waves=True, resident=True)
    ref = oracle.stem(p, To, diffpats=True, exit_waves=True)
    for r, o in zip((det, dps, ews), ref):
        assert rel_l2(r, o) <= TOL_MS
