"""qs_multislice_run_noalloc -- the entry point for callers that cannot
allocate device memory while they run -- against the regular
qs_multislice_run, through the C ABI, on two calls in a row.

This file is collected last (test_zz_*) and also passes alone in a fresh
process: the first call on the device performs the scratch-address lookup."""
import ctypes

import numpy as np
import pytest

from conftest import Golden, rel_l2
from qstem_gb300 import abi, config, lib

pytestmark = pytest.mark.gpu

TOL = 1e-4  # relative L2, the multislice tolerance of the other GPU tests


def _run_both(p, T, probe, positions):
    import torch
    L = lib.load()
    ctx = lib.Context(0)
    nt = p.thickness_count()
    npos = len(positions[0])
    det_ref = torch.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), device="cuda")
    dp_ref = torch.zeros((npos, p.nx, p.ny), device="cuda")
    ew_ref = torch.zeros((npos, p.nx, p.ny, 2), device="cuda")
    ctx.multislice(p, T, probe, positions=positions, det=det_ref, diffpats=dp_ref, exit_waves=ew_ref)
    arrs = [np.ascontiguousarray(a, dtype=np.int32) for a in positions]
    b = abi.QsBatch(npos, *[a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) for a in arrs])
    outs = []
    for _ in range(2):  # two calls in a row share the scratch area
        det = torch.full_like(det_ref, 7.0)
        dp = torch.full_like(dp_ref, 7.0)
        ew = torch.zeros_like(ew_ref)
        rc = L.qs_multislice_run_noalloc(None, ctypes.byref(p), ctypes.c_void_p(T.data_ptr()),
                                         ctypes.c_void_p(probe.data_ptr()), ctypes.byref(b),
                                         ctypes.c_void_p(det.data_ptr()), ctypes.c_void_p(dp.data_ptr()),
                                         ctypes.c_void_p(ew.data_ptr()))
        assert rc == 0, L.qs_last_error().decode()
        torch.cuda.synchronize()
        outs.append((det.cpu().numpy(), dp.cpu().numpy(), ew.cpu().numpy()))
    ctx.close()
    ref = (det_ref.cpu().numpy(), dp_ref.cpu().numpy(), ew_ref.cpu().numpy())
    return ref, outs


def test_noalloc_matches_regular_entry_point_small():
    import torch
    g = Golden("sto64")
    p = g.params
    T = torch.from_numpy(np.ascontiguousarray(g["T"])).cuda()
    probe = torch.from_numpy(np.ascontiguousarray(g["probe"])).cuda()
    px, py, dx, dy = config.scan_offsets(p)
    ref, outs = _run_both(p, T, probe, (px, py, dx, dy))
    for det, dp, ew in outs:
        assert rel_l2(det, ref[0]) <= TOL
        assert rel_l2(dp, ref[1]) <= TOL
        assert rel_l2(ew, ref[2]) <= TOL
    assert rel_l2(ref[0], g["det"]) <= TOL


def test_noalloc_512_and_limit():
    import torch
    atoms, ax, by, c = config.replicate(config.srtio3_cell(), 10, 10, 4)
    p = config.make_params(nx=512, resolutionX=39.05 / 512, v0=200, slices=8, sliceThickness=1.9525, ax=ax, by=by,
                           c=c, scan=(19.525, 23.43, 4, 19.525, 23.43, 4),
                           detectors=[(0, 10, "BF"), (10, 25, "LA"), (25, 70, "MA"), (70, 200, "HA")], alpha=20,
                           outputInterval=3)
    ctx = lib.Context(0)
    T = torch.from_numpy(ctx.slices(p, atoms)).cuda()
    probe = torch.from_numpy(ctx.probe(p)).cuda()
    ctx.close()
    px, py, dx, dy = config.scan_offsets(p)
    sel = slice(0, 12)
    ref, outs = _run_both(p, T, probe, (px[sel], py[sel], dx[sel], dy[sel]))
    for det, dp, ew in outs:
        assert rel_l2(det, ref[0]) <= TOL
        assert rel_l2(dp, ref[1]) <= TOL
        assert rel_l2(ew, ref[2]) <= TOL
    # a batch beyond the fixed scratch is refused with a clear message
    L = lib.load()
    n = 64
    arrs = [np.zeros(n, np.int32) for _ in range(4)]
    b = abi.QsBatch(n, *[a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) for a in arrs])
    det = torch.zeros((p.thickness_count(), p.detectorNum, p.scanXN, p.scanYN), device="cuda")
    rc = L.qs_multislice_run_noalloc(None, ctypes.byref(p), ctypes.c_void_p(T.data_ptr()),
                                     ctypes.c_void_p(probe.data_ptr()), ctypes.byref(b),
                                     ctypes.c_void_p(det.data_ptr()), None, None)
    assert rc == abi.QS_ERR_ARG
    assert b"bytes of scratch" in L.qs_last_error()


def test_noalloc_captured_in_a_graph_and_replayed():
    """After its first call, the entry point can be captured into a CUDA
    graph: it copies nothing from host memory (the tables and positions
    travel as kernel arguments), so each replay reads the slice stack's and
    the probe's current contents and rewrites the outputs."""
    import torch
    g = Golden("sto64")
    p = g.params
    T = torch.from_numpy(np.ascontiguousarray(g["T"])).cuda()
    probe = torch.from_numpy(np.ascontiguousarray(g["probe"])).cuda()
    px, py, dx, dy = config.scan_offsets(p)
    ref, _ = _run_both(p, T, probe, (px, py, dx, dy))  # includes the first, uncaptured calls
    L = lib.load()
    arrs = [np.ascontiguousarray(a, dtype=np.int32) for a in (px, py, dx, dy)]
    b = abi.QsBatch(len(px), *[a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) for a in arrs])
    det = torch.zeros(ref[0].shape, device="cuda")
    dp = torch.zeros(ref[1].shape, device="cuda")
    ew = torch.zeros(ref[2].shape, device="cuda")
    graph = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.graph(graph, stream=s):
        rc = L.qs_multislice_run_noalloc(ctypes.c_void_p(s.cuda_stream), ctypes.byref(p),
                                         ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(probe.data_ptr()),
                                         ctypes.byref(b), ctypes.c_void_p(det.data_ptr()),
                                         ctypes.c_void_p(dp.data_ptr()), ctypes.c_void_p(ew.data_ptr()))
    assert rc == 0, L.qs_last_error().decode()
    del arrs  # the replay needs none of the host arrays
    for _ in range(2):
        det.fill_(7.0)
        dp.fill_(7.0)
        graph.replay()
        torch.cuda.synchronize()
        assert rel_l2(det.cpu().numpy(), ref[0]) <= TOL
        assert rel_l2(dp.cpu().numpy(), ref[1]) <= TOL
        assert rel_l2(ew.cpu().numpy(), ref[2]) <= TOL
    # the replay reads the stack's current contents: a vacuum stack (T = 1)
    # leaves the probe's own intensity in the bright field
    T[..., 0] = 1.0
    T[..., 1] = 0.0
    graph.replay()
    torch.cuda.synchronize()
    assert rel_l2(det.cpu().numpy(), ref[0]) > 1e-3
