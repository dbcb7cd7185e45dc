"""The adjoint multislice (qs_adjoint_run, qs_atoms_grad) against the float64
CPU autograd of the same forward model (oracle/torch_ref.py) and central
finite differences.

Tolerances: loss 1e-4 relative; dL/dV and dL/d(x,y) 1e-3 relative L2 (the
contract's gradient bound); central differences with h = 1e-3 A, 1e-3
relative on the gradient vector of the checked atoms."""
import numpy as np
import pytest

from conftest import Golden, rel_l2
from qstem_gb300 import config, lib

pytestmark = pytest.mark.gpu

TOL_LOSS = 1e-4
TOL_GRAD = 1e-3


def displaced(atoms, sigma, seed):
    rng = np.random.default_rng(seed)
    a = atoms.copy()
    a["x"] = (a["x"].astype(np.float64) + rng.standard_normal(len(a)) * sigma).astype(np.float32)
    a["y"] = (a["y"].astype(np.float64) + rng.standard_normal(len(a)) * sigma).astype(np.float32)
    return a


@pytest.fixture(scope="module")
def case():
    import torch
    from oracle import oracle, torch_ref
    oracle.build()
    g = Golden("sto64")
    p = g.params
    atoms = g["atoms"]
    target_atoms = displaced(atoms, 0.05, 20261203 + 300)
    ctx = lib.Context(0)
    px, py, dx, dy = config.scan_offsets(p)
    pos = (px, py, dx, dy)
    probe = torch.from_numpy(ctx.probe(p)).cuda()
    Tt = torch.from_numpy(ctx.slices(p, target_atoms)).cuda()
    _, tgt, _ = ctx.multislice(p, Tt, probe, positions=pos, want_det=False,
                               diffpats=torch.zeros((len(px), p.nx, p.ny), device="cuda"))
    T = torch.from_numpy(ctx.slices(p, atoms)).cuda()
    V = torch.from_numpy(ctx.slices(p, atoms, potential_only=True)[..., 0].copy()).cuda()
    yield dict(ctx=ctx, p=p, atoms=atoms, pos=pos, probe=probe, T=T, V=V, target=tgt, torch_ref=torch_ref)
    ctx.close()


def fp64_reference(c, need_xy=False):
    import torch
    tr = c["torch_ref"]
    p = c["p"]
    probe = c["probe"].cpu().numpy()
    probe = torch.from_numpy(probe[..., 0].astype(np.float64) + 1j * probe[..., 1].astype(np.float64))
    positions = [(int(a), int(b)) for a, b in zip(c["pos"][0], c["pos"][1])]
    target = torch.from_numpy(c["target"].cpu().numpy().astype(np.float64))
    plan = tr.AtomPlan(p, c["atoms"])
    xy = torch.from_numpy(np.stack([c["atoms"]["x"], c["atoms"]["y"]], 1).astype(np.float64)).requires_grad_(need_xy)
    V = plan.V(xy)
    if not need_xy:
        V = V.detach().requires_grad_(True)
    else:
        V.retain_grad()
    L, _ = tr.loss_from_V(p, V, probe, positions, target)
    L.backward()
    return float(L.detach()), V.grad.numpy(), (xy.grad.numpy() if need_xy else None), plan, probe, positions, target


@pytest.mark.parametrize("deterministic", [False, True])
def test_dLdV_matches_fp64_autograd(case, deterministic):
    c = case
    loss, dV, _ = c["ctx"].adjoint(c["p"], c["T"], c["probe"], c["target"], positions=c["pos"], ckpt=3,
                                   deterministic=deterministic)
    L64, dV64, _, _, _, _, _ = fp64_reference(c)
    assert abs(loss - L64) <= TOL_LOSS * L64
    assert rel_l2(dV.cpu().numpy(), dV64) <= TOL_GRAD


def test_checkpoint_interval_does_not_change_the_gradient(case):
    """With the fixed-order sum (QS_DETERMINISTIC) every checkpoint interval
    gives the same bits; the default float-atomic sum of dL/dV over positions
    agrees with it to float rounding (the loss does not depend on it)."""
    c = case
    ref = None
    for ckpt in (1, 3, 8, 0):  # 0: the automatic interval (every state here)
        loss, dV, dps = c["ctx"].adjoint(c["p"], c["T"], c["probe"], c["target"], positions=c["pos"], ckpt=ckpt,
                                         want_diffpats=True, deterministic=True)
        d = dV.cpu().numpy()
        if ref is None:
            ref = (loss, d)
        else:
            assert loss == ref[0]
            assert np.array_equal(d, ref[1])
        la, dVa, _ = c["ctx"].adjoint(c["p"], c["T"], c["probe"], c["target"], positions=c["pos"], ckpt=ckpt)
        assert la == ref[0]
        assert rel_l2(dVa.cpu().numpy(), ref[1]) <= 1e-5
    # the forward patterns of the adjoint run equal qs_multislice_run's
    _, dp2, _ = c["ctx"].multislice(c["p"], c["T"], c["probe"], positions=c["pos"], want_det=False,
                                    diffpats=dps.clone().zero_())
    assert rel_l2(dps.cpu().numpy(), dp2.cpu().numpy()) <= 1e-6


def test_atom_gradients_match_fp64_autograd_and_finite_differences(case):
    import torch
    c = case
    p = c["p"]
    loss, dV, _ = c["ctx"].adjoint(p, c["T"], c["probe"], c["target"], positions=c["pos"], ckpt=3)
    g = c["ctx"].atoms_grad(p, c["atoms"], dV)
    L64, _, gxy64, plan, probe, positions, target = fp64_reference(c, need_xy=True)
    assert rel_l2(g, gxy64) <= TOL_GRAD
    # Central differences, h = 1e-3 A, on the float64 model.  The radial LUT
    # is piecewise linear (knots every dr = dx/2), so V has kinks; with the
    # lookups held in their planned intervals the central difference measures
    # the one-sided (kink-consistent) derivative the adjoint computes.
    tr = c["torch_ref"]
    h = 1e-3
    atoms = c["atoms"]
    rng = np.random.default_rng(7)
    idx = rng.choice(np.flatnonzero(np.abs(g).sum(1) > 0), 6, replace=False)
    fd, fd_knots, an = [], [], []
    base = torch.from_numpy(np.stack([atoms["x"], atoms["y"]], 1).astype(np.float64))
    for i in idx:
        for k, key in enumerate(("x", "y")):
            vals, vals_k = [], []
            for sgn in (1, -1):
                xy = base.clone()
                xy[i, k] += sgn * h
                L, _ = tr.loss_from_V(p, plan.V(xy, frozen=True), probe, positions, target)
                vals.append(float(L))
                # the same with the intervals re-derived (knot crossings honoured)
                a = atoms.copy()
                a[key][i] = np.float32(float(a[key][i]) + sgn * h)
                Lk, _ = tr.loss_from_V(p, tr.AtomPlan(p, a).V(xy), probe, positions, target)
                vals_k.append(float(Lk))
            fd.append((vals[0] - vals[1]) / (2 * h))
            fd_knots.append((vals_k[0] - vals_k[1]) / (2 * h))
            an.append(g[i, k])
    fd, fd_knots, an = np.array(fd), np.array(fd_knots), np.array(an)
    assert rel_l2(an, fd) <= TOL_GRAD, (fd, an)
    # Across knots the central difference averages two slopes: about
    # 2h/dr = 4 % of an atom's pixels sit within h of a knot, which bounds the
    # disagreement at the per-cent level.
    assert rel_l2(an, fd_knots) <= 2e-2, (fd_knots, an)
