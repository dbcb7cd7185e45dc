"""The adjoint through a cell divided into slabs (cellDiv > 1) against the
same problem undivided: the slab loop is the wave continuing through the
slabs' stacks, so the loss and dL/dV must equal those of one stack of all
absolute slices (for a reused stack, its dL/dV sums the concatenation's
slices of every use).  Atom gradients through slab stacks against central
finite differences of that loss.  Tolerances: loss 1e-6, dL/dV 1e-5
(relative), atom gradients 1e-2 (knot crossings are re-derived in the
differences)."""
import numpy as np
import pytest

from conftest import Golden, rel_l2
from qstem_gb300 import config, lib, phonons

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = lib.Context(0)
    yield c
    c.close()


def _setup(ctx, name):
    import torch
    g = Golden(name)
    p = g.params
    atoms = g["atoms"]
    pos = config.scan_offsets(p)
    probe = torch.from_numpy(ctx.probe(p)).cuda()
    stacks = [ctx.slices(p, atoms, slab=k) for k in range(p.cellDiv)]
    # the target: the same cell with displaced atoms, through the same slabs
    tatoms = phonons.displaced(atoms, 0, 11, 0.05)
    tst = torch.from_numpy(np.concatenate([ctx.slices(p, tatoms, slab=k) for k in range(p.cellDiv)])).cuda()
    q = p.copy()
    q.cellDiv, q.slices, q.equalDivs = 1, p.slices * p.cellDiv, 0
    _, tgt, _ = ctx.multislice(q, tst, probe, positions=pos, want_det=False,
                               diffpats=torch.zeros((len(pos[0]), p.nx, p.ny), device="cuda"))
    return g, p, q, atoms, pos, probe, stacks, tgt


@pytest.mark.parametrize("ckpt", [1, 3, 0])
def test_reused_stack_equals_the_concatenation(ctx, ckpt):
    import torch
    g, p, q, atoms, pos, probe, stacks, tgt = _setup(ctx, "sto64d2")
    assert p.cellDiv == 2 and p.equalDivs
    S0 = p.slices
    T = torch.from_numpy(stacks[0]).cuda()
    Tcat = torch.cat([T, T])
    loss, dV, _ = ctx.adjoint(p, T, probe, tgt, positions=pos, ckpt=ckpt)
    lref, dref, _ = ctx.adjoint(q, Tcat, probe, tgt, positions=pos, ckpt=ckpt)
    assert abs(loss - lref) <= 1e-6 * abs(lref)
    dV, dref = dV.cpu().numpy(), dref.cpu().numpy()
    assert dV.shape[0] == S0
    assert rel_l2(dV, dref[:S0] + dref[S0:]) <= 1e-5


@pytest.mark.parametrize("ckpt", [1, 2])
def test_slab_stacks_equal_the_concatenation(ctx, ckpt):
    import torch
    g, p, q, atoms, pos, probe, stacks, tgt = _setup(ctx, "sto64d2u")
    assert p.cellDiv == 2 and not p.equalDivs
    Tst = torch.from_numpy(np.concatenate(stacks)).cuda()
    loss, dV, _ = ctx.adjoint(p, Tst, probe, tgt, positions=pos, ckpt=ckpt, slab_stacks=True)
    lref, dref, _ = ctx.adjoint(q, Tst, probe, tgt, positions=pos, ckpt=ckpt)
    assert abs(loss - lref) <= 1e-6 * abs(lref)
    assert dV.shape[0] == p.slices * p.cellDiv
    assert rel_l2(dV.cpu().numpy(), dref.cpu().numpy()) <= 1e-5


def test_atom_gradients_through_slab_stacks(ctx):
    """dL/d(x, y) of the Ti and O atoms with the largest gradients (those on
    both sides of the slab boundary among them) against central differences
    (h = 1e-3 A) of the loss rebuilt from displaced atoms.  The Sr atoms sit
    on pixel-aligned lattice points where the differences cross knots of the
    piecewise-linear LUT on many pixels at once; they differ by ~8 % with or
    without slabs and are covered by the interval-holding comparisons of the
    undivided adjoint."""
    import torch
    g, p, q, atoms, pos, probe, stacks, tgt = _setup(ctx, "sto64d2u")
    Tst = torch.from_numpy(np.concatenate(stacks)).cuda()
    _, dV, _ = ctx.adjoint(p, Tst, probe, tgt, positions=pos, ckpt=1, slab_stacks=True)
    grad = ctx.atoms_grad(p, atoms, dV, slab_stacks=True)

    def loss_of(a):
        T = torch.from_numpy(np.concatenate([ctx.slices(p, a, slab=k) for k in range(p.cellDiv)])).cuda()
        return ctx.adjoint(p, T, probe, tgt, positions=pos, ckpt=1, slab_stacks=True)[0]

    h = 1e-3
    mag = np.abs(grad).sum(1) * (atoms["Znum"] != 38)
    pick = np.argsort(-mag)[:6]
    fd = np.zeros((len(pick), 2))
    for i, j in enumerate(pick):
        for k, ax in enumerate(("x", "y")):
            ap, am = atoms.copy(), atoms.copy()
            ap[ax][j] = np.float32(float(atoms[ax][j]) + h)
            am[ax][j] = np.float32(float(atoms[ax][j]) - h)
            fd[i, k] = (loss_of(ap) - loss_of(am)) / (float(ap[ax][j]) - float(am[ax][j]))
    assert np.abs(grad[pick]).max() > 0
    assert rel_l2(grad[pick], fd) <= 1e-2


def test_autograd_through_slab_stacks(ctx):
    """MultisliceLoss and AtomsLoss with slab stacks: the same loss and
    gradients as the C entry points."""
    import torch
    from qstem_gb300 import autograd
    g, p, q, atoms, pos, probe, stacks, tgt = _setup(ctx, "sto64d2u")
    V = torch.from_numpy(np.concatenate([ctx.slices(p, atoms, potential_only=True, slab=k)[..., 0]
                                         for k in range(p.cellDiv)])).cuda().requires_grad_(True)
    L = autograd.MultisliceLoss.apply(V, ctx, p, probe, tgt, pos, 1, True)
    L.backward()
    Tst = torch.from_numpy(np.concatenate(stacks)).cuda()
    loss, dV, _ = ctx.adjoint(p, Tst, probe, tgt, positions=pos, ckpt=1, slab_stacks=True)
    assert abs(float(L.detach()) - loss) <= 1e-5 * abs(loss)
    assert rel_l2(V.grad.cpu().numpy(), dV.cpu().numpy()) <= 1e-4
    xy = torch.from_numpy(np.stack([atoms["x"], atoms["y"]], 1).astype(np.float64)).requires_grad_(True)
    La = autograd.AtomsLoss.apply(xy, ctx, p, atoms, probe, tgt, pos, 1, True)
    La.backward()
    # the stacks are rebuilt from the atoms: the scatter's float reductions
    # sum in a different order, ~1e-7 of the potential
    assert abs(float(La.detach()) - loss) <= 1e-5 * abs(loss)
    assert rel_l2(xy.grad.numpy(), ctx.atoms_grad(p, atoms, dV, slab_stacks=True)) <= 1e-4
