"""Invalid calls through the C ABI return a QS_ERR_* code and a message
(qs_last_error), never exit or fault, and leave the context usable: the
reference's printf + exit(0) error handling is replaced by status codes."""
import ctypes

import numpy as np
import pytest

from conftest import Golden, rel_l2
from qstem_gb300 import abi, lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    import torch
    g = Golden("sto64")
    ctx = lib.Context(0)
    T = torch.from_numpy(np.ascontiguousarray(g["T"])).cuda()
    yield ctx, g, T
    ctx.close()


def expect(code, fn, *a, **k):
    with pytest.raises(lib.QsError) as e:
        fn(*a, **k)
    assert e.value.code == code, str(e.value)
    assert len(str(e.value)) > len("qstem_gpu error -1: ")
    return str(e.value)


def test_argument_and_support_errors(case):
    ctx, g, T = case
    p = g.params
    # a window outside the potential array
    n = 2
    bad = (np.array([0, p.potNx], np.int32), np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.int32))
    msg = expect(abi.QS_ERR_ARG, ctx.multislice, p, T, positions=bad, want_det=False,
                 diffpats=None, want_diffpats=False)
    assert "outside" in msg
    # a slab index beyond cellDiv
    expect(abi.QS_ERR_ARG, ctx.slices, p, g["atoms"], slab=1)
    # options a driver does not implement
    target = T.new_zeros((p.scanXN * p.scanYN, p.nx, p.ny, 2))[..., 0].contiguous()
    probe = T.new_zeros((p.nx, p.ny, 2))
    r = p.copy()
    r.bandlimittrans = 1
    expect(abi.QS_ERR_UNSUPPORTED, ctx.adjoint, r, T, probe, target)
    s = p.copy()
    s.detectors[0].shiftX = 1.0
    expect(abi.QS_ERR_UNSUPPORTED, ctx.multislice, s, T)
    # a negative slab count
    t = p.copy()
    t.cellDiv = 0
    expect(abi.QS_ERR_ARG, ctx.slices, t, g["atoms"])
    # stacking sequences: negative repeats
    u = p.copy()
    u.mulsRepeat2 = -1
    expect(abi.QS_ERR_ARG, ctx.multislice, u, T)


def test_null_pointers_through_the_raw_abi(case):
    ctx, g, T = case
    L = lib.load()
    p = g.params
    assert L.qs_slices_build(ctx.h, ctypes.byref(p), None, 5, None, 0) == abi.QS_ERR_ARG
    assert L.qs_multislice_run(ctx.h, ctypes.byref(p), None, None, None, None, None, None, 0) == abi.QS_ERR_ARG
    assert L.qs_probe(None, ctypes.byref(p), 0.0, 0.0, None, 0) == abi.QS_ERR_ARG
    assert L.qs_last_error() not in (None, b"")


def test_context_still_works_after_errors(case):
    ctx, g, T = case
    p = g.params
    det, _, _ = ctx.multislice(p, g["T"], g["probe"])
    assert rel_l2(det, g["det"]) <= 1e-4
