"""QS_GRAPH: the slice loop replayed as a CUDA graph gives bit-identical
results to the launched loop, and a replay sees new contents of the same
buffers (a new slice stack, new scan positions)."""
import numpy as np
import pytest

from conftest import Golden
from qstem_gb300 import config, lib, phonons

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import torch
    g = Golden("sto64")
    p = g.params
    ctx = lib.Context(0)
    T = torch.from_numpy(np.ascontiguousarray(g["T"])).cuda()
    probe = torch.from_numpy(np.ascontiguousarray(g["probe"])).cuda()
    yield ctx, g, p, T, probe
    ctx.close()


_BUFS = {}


def _run(ctx, p, T, probe, graph, positions=None, series=False):
    """One scan into output buffers kept per shape (a graph is keyed by
    buffer addresses, so the same buffers are passed every time)."""
    import torch
    nt = p.thickness_count()
    npos = p.scanXN * p.scanYN if positions is None else len(positions[0])
    lead = (nt, npos) if series else (npos,)
    if (series, npos) not in _BUFS:
        _BUFS[(series, npos)] = (
            torch.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), dtype=torch.float32, device="cuda"),
            torch.zeros(lead + (p.nx, p.ny), dtype=torch.float32, device="cuda"),
            torch.zeros(lead + (p.nx, p.ny, 2), dtype=torch.float32, device="cuda"))
    det, dp, ew = _BUFS[(series, npos)]
    for b in (det, dp, ew):
        b.fill_(-1.0)  # the call must write everything it returns
    torch.cuda.synchronize()
    ctx.multislice(p, T, probe, positions=positions, det=det, diffpats=dp, exit_waves=ew, graph=graph, series=series)
    return det.cpu().numpy(), dp.cpu().numpy(), ew.cpu().numpy()


def test_replay_equals_launches(setup):
    ctx, g, p, T, probe = setup
    ref = _run(ctx, p, T, probe, False)
    for _ in range(3):  # eager, capture, replay
        got = _run(ctx, p, T, probe, True)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
    ser_ref = _run(ctx, p, T, probe, False, series=True)
    for _ in range(3):
        got = _run(ctx, p, T, probe, True, series=True)
        for a, b in zip(got, ser_ref):
            assert np.array_equal(a, b)


def test_replay_reads_new_buffer_contents(setup):
    import torch
    ctx, g, p, T, probe = setup
    for _ in range(2):
        _run(ctx, p, T, probe, True)  # the graph exists from here on
    # a new slice stack in the same buffer
    T2 = torch.from_numpy(ctx.slices(p, phonons.displaced(g["atoms"], 0, 5, 0.1))).cuda()
    saved = T.clone()
    T.copy_(T2)
    try:
        got = _run(ctx, p, T, probe, True)
        want = _run(ctx, p, T, probe, False)
        for a, b in zip(got, want):
            assert np.array_equal(a, b)
        assert not np.array_equal(got[0], _run(ctx, p, saved, probe, False)[0])
    finally:
        T.copy_(saved)
    # other positions of the same count
    px, py, dx, dy = config.scan_offsets(p)
    pos = (px[::-1].copy(), py[::-1].copy(), dx, dy)
    for _ in range(2):
        _run(ctx, p, T, probe, True, positions=pos)
    rev = (px.copy(), py.copy(), dx[::-1].copy(), dy[::-1].copy())
    got = _run(ctx, p, T, probe, True, positions=rev)
    want = _run(ctx, p, T, probe, False, positions=rev)
    for a, b in zip(got, want):
        assert np.array_equal(a, b)


def test_replays_are_counted(setup):
    ctx, g, p, T, probe = setup
    for _ in range(2):
        _run(ctx, p, T, probe, True)
    ctx.profile(False)
    n0 = ctx.stats()["launches"]
    _run(ctx, p, T, probe, False)
    n1 = ctx.stats()["launches"]
    _run(ctx, p, T, probe, True)
    n2 = ctx.stats()["launches"]
    assert n2 - n1 == n1 - n0 > 0
