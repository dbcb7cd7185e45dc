"""Stacking sequences in the library (qs_multislice_run with mulsRepeat1/2):
the wave's steps against the same steps unrolled into one stack.  A
sequence m1 m2 over cellDiv slabs is m2 passes through the slabs, each
slab's stack m1 times; the detector images of every thickness slot come
from the step collectIntensity's index assigns it last.  Tolerance 1e-4
relative L2 (1e-6 typical) for detector images, patterns and exit waves."""
import numpy as np
import pytest

from conftest import Golden, rel_l2
from oracle_ctx import OracleContext
from qstem_gb300 import lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = lib.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name,m1,m2", [("sto64", 3, 1), ("sto64d2u", 2, 2), ("sto64d2", 1, 3)])
def test_sequence_walk_matches_the_unrolled_steps(ctx, name, m1, m2):
    g = Golden(name)
    p = g.params
    p.mulsRepeat1, p.mulsRepeat2 = m1, m2
    slabs = p.cellDiv > 1 and not p.equalDivs
    T = np.concatenate([ctx.slices(p, g["atoms"], slab=k) for k in range(p.cellDiv)]) if slabs else np.asarray(g["T"])
    probe = np.ascontiguousarray(g["probe"])
    det, dps, ews = ctx.multislice(p, T, probe, want_diffpats=True, want_exit_waves=True, slab_stacks=slabs)
    n = p.scanXN * p.scanYN
    from qstem_gb300 import config
    offs = config.scan_offsets(p)
    rdet, rdp, rew = OracleContext().multislice(p, T, probe, positions=offs, want_diffpats=True,
                                                want_exit_waves=True, slab_stacks=slabs)
    assert det.shape == rdet.shape and len(dps) == n
    assert rel_l2(det, rdet) <= 1e-4
    assert rel_l2(dps, rdp) <= 1e-4 and rel_l2(ews, rew) <= 1e-4
    # the repeats change the result
    q = p.copy()
    q.mulsRepeat1 = q.mulsRepeat2 = 1
    det1, _, _ = ctx.multislice(q, T, probe, slab_stacks=slabs)
    assert rel_l2(det1, det) > 1e-3


def test_tem_through_a_sequence(ctx):
    """qs_tem_run with a stacking sequence: the exit wave of the plane wave
    through the sequence's steps equals the plane wave through the stack
    repeated by hand (m1 = 2 over one slab, m2 = 2)."""
    g = Golden("si64tem")
    p = g.params
    atoms = g["atoms"]
    T = ctx.slices(p, atoms)
    plane = np.zeros((p.nx, p.ny, 2), np.float32)
    plane[..., 0] = 1.0
    q = p.copy()
    q.mulsRepeat1, q.mulsRepeat2 = 2, 2
    _, _, ew = ctx.tem(q, [atoms], want_exit_waves=True)
    r = p.copy()
    r.slices = r.outputInterval = 4 * p.slices
    pos = tuple(np.zeros(1, np.int32) for _ in range(4))
    _, _, ref = ctx.multislice(r, np.concatenate([T] * 4), plane, positions=pos, want_det=False,
                               want_exit_waves=True)
    assert rel_l2(ew[0], ref[0]) <= 1e-5
    _, _, once = ctx.tem(p, [atoms], want_exit_waves=True)
    assert rel_l2(once[0], ref[0]) > 1e-3


@pytest.mark.parametrize("m1,m2", [(2, 3), (1, 2)])
def test_cbed_batch_through_a_sequence(ctx, m1, m2):
    """qs_cbed_batch_run with a stacking sequence (the instance's stack laid
    out in step order) gives the final pattern qs_multislice_run gives for
    the same sequence; an instance without one in the same batch is
    unchanged."""
    g = Golden("si64cbed")
    plain = g.params
    p = plain.copy()
    p.mulsRepeat1, p.mulsRepeat2 = m1, m2
    T = ctx.slices(p, g["atoms"])
    probe = ctx.probe(p, float(np.float32(np.float32(p.scanXStart) - np.float32(p.potOffsetX))),
                      float(np.float32(np.float32(p.scanYStart) - np.float32(p.potOffsetY))))
    pos = tuple(np.zeros(1, np.int32) for _ in range(4))
    _, dps, _ = ctx.multislice(p, T, probe, positions=pos, want_det=False, want_diffpats=True)
    _, ref1, _ = ctx.multislice(plain, T, probe, positions=pos, want_det=False, want_diffpats=True)
    pats, _ = ctx.cbed_batch([(p, g["atoms"]), (plain, g["atoms"])])
    assert rel_l2(pats[0], dps[0]) <= 1e-5
    assert rel_l2(pats[1], ref1[0]) <= 1e-5
    assert rel_l2(pats[0], pats[1]) > 1e-3


@pytest.mark.parametrize("m1,m2,ckpt", [(2, 1, 1), (2, 2, 3)])
def test_adjoint_through_a_sequence(ctx, m1, m2, ckpt):
    """qs_adjoint_run through a stacking sequence equals the adjoint of the
    stack repeated by hand: the same loss, and each stack slice's dL/dV
    the sum over its steps.  Tolerances: loss 1e-6, dL/dV 1e-5 (relative)."""
    import torch
    g = Golden("sto64")
    p = g.params
    p.mulsRepeat1, p.mulsRepeat2 = m1, m2
    from qstem_gb300 import config
    pos = config.scan_offsets(p)
    T = torch.from_numpy(np.ascontiguousarray(g["T"])).cuda()
    probe = torch.from_numpy(np.ascontiguousarray(g["probe"])).cuda()
    reps = m1 * m2
    q = p.copy()
    q.slices, q.mulsRepeat1, q.mulsRepeat2 = p.slices * reps, 1, 1
    Tcat = torch.cat([T] * reps)
    target = torch.rand((len(pos[0]), p.nx, p.ny), device="cuda")
    loss, dV, _ = ctx.adjoint(p, T, probe, target, positions=pos, ckpt=ckpt)
    lref, dref, _ = ctx.adjoint(q, Tcat, probe, target, positions=pos, ckpt=ckpt)
    assert abs(loss - lref) <= 1e-6 * abs(lref)
    dref = dref.cpu().numpy().reshape(reps, p.slices, p.potNx, p.potNy).sum(0)
    assert rel_l2(dV.cpu().numpy(), dref) <= 1e-5
