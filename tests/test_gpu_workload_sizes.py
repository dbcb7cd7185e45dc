"""The measured workloads at their own sizes, through the C ABI, against the
oracle (the C restatement of the reference, bit-exact with it) and, for the
adjoint, against the float64 autograd model (oracle/torch_ref.py).

  * plain STEM HAADF: SrTiO3 5x5x10, 256^2, 20 slices, 16x16 positions,
    70-200 mrad -- the whole run, atoms to image (qs_stem_run);
  * uneven CBED: one instance at each grid of the workload (256^2, 384^2,
    512^2, 768^2, 1024^2), fcc Au / Si / SrTiO3, ~40 A lateral cells,
    5-25 mrad, transmission band limit on, all in one qs_cbed_batch_run;
    thin (3-5 slices of 2 A) so that the oracle finishes in seconds;
  * differentiable 4D-STEM: SrTiO3 6x6x20, 256^2, 40 slices, potential
    298^2, 25 mrad, checkpoints every 6 slices; a 4x4 subset of the 32x32
    positions (their own window offsets); loss, dL/dV and dL/d(x,y) of a
    set of atoms against float64 autograd.

Tolerances: 1e-4 relative L2 for detector images and patterns (complex FP32
multislice), loss 1e-4, gradients 1e-3 (the gradient contract)."""
import numpy as np
import pytest

import bench
from conftest import rel_l2
from qstem_gb300 import abi, config, lib

pytestmark = pytest.mark.gpu

TOL_MS = 1e-4
TOL_LOSS = 1e-4
TOL_GRAD = 1e-3


@pytest.fixture(scope="module")
def ctx():
    from oracle import oracle
    oracle.build()
    c = lib.Context(0)
    yield c
    c.close()


def test_stem_haadf_256_whole_run(ctx):
    """Configuration 1 exactly: atoms in, HAADF image out, against the
    oracle's run of the same atoms (potential, transmission, 256 positions)."""
    from oracle import oracle
    p, atoms = bench.stem256_workload()
    assert (p.nx, p.slices, p.scanXN, p.scanYN, p.potNx) == (256, 20, 16, 16, 307)
    img = ctx.stem_run(p, atoms)
    To = oracle.transmission(p, oracle.potential(p, atoms))
    ref, _, _ = oracle.stem(p, To)
    assert img.shape == ref.shape and float(ref.sum()) > 0
    assert rel_l2(img, ref) <= TOL_MS


def _cbed_instances():
    """One thin instance per grid of the uneven-CBED workload."""
    cells = {"Au": config.fcc_cell(79, 4.078), "Si": config.diamond_cell(), "SrTiO3": config.srtio3_cell()}
    plan = [(256, "Au", 3, 5.0), (384, "Si", 4, 11.0), (512, "SrTiO3", 5, 17.0), (768, "Au", 4, 23.0),
            (1024, "Si", 3, 25.0)]
    jobs = []
    for n, name, slices, alpha in plan:
        cell = cells[name]
        nl = max(1, int(round(40.0 / cell.a)))
        nz = int(np.ceil(slices * 2.0 / cell.c))
        atoms, ax, by, c = config.replicate(cell, nl, nl, nz)
        p = config.make_params(mode=abi.QS_MODE_CBED, nx=n, resolutionX=float(np.float32(ax)) / n,
                               resolutionY=float(np.float32(by)) / n, v0=200, slices=slices, sliceThickness=2.0,
                               ax=ax, by=by, c=c, scan=None, alpha=alpha, bandlimit=True)
        jobs.append((p, atoms))
    return jobs


def test_cbed_every_workload_grid(ctx):
    """qs_cbed_batch_run with an instance at each grid 256^2 ... 1024^2: the
    band-limited slice stack, the probe at doCBED's position and the
    pattern after the last slice, each against the oracle."""
    from oracle import oracle
    jobs = _cbed_instances()
    dps, rep = ctx.cbed_batch(jobs)
    assert rep["groups"] == len(jobs)
    for (p, atoms), dp in zip(jobs, dps):
        T = oracle.transmission(p, oracle.potential(p, atoms))
        dx = float(np.float32(p.scanXStart) - np.float32(p.potOffsetX))
        dy = float(np.float32(p.scanYStart) - np.float32(p.potOffsetY))
        ref = oracle.run_position(p, T, 0, 0, oracle.probe(p, dx, dy))[2]
        assert dp.shape == (p.nx, p.ny) and float(ref.sum()) > 0
        assert rel_l2(dp, ref) <= TOL_MS, p.nx


def _adjoint_case(ctx):
    import torch
    p, atoms, tgt_atoms = bench.adjoint_workload()
    assert (p.nx, p.slices, p.potNx, p.potNy, p.scanXN) == (256, 40, 298, 298, 32)
    px, py, dx, dy = config.scan_offsets(p)
    sel = np.array([ix * p.scanYN + iy for ix in range(0, 32, 8) for iy in range(0, 32, 8)])
    pos = (px[sel], py[sel], dx[sel], dy[sel])
    probe = torch.from_numpy(ctx.probe(p)).cuda()
    T = torch.empty((p.slices, p.potNx, p.potNy, 2), dtype=torch.float32, device="cuda")
    ctx.slices(p, tgt_atoms, out=T)
    target = torch.zeros((len(sel), p.nx, p.ny), dtype=torch.float32, device="cuda")
    ctx.multislice(p, T, probe, positions=pos, want_det=False, diffpats=target)
    ctx.slices(p, atoms, out=T)
    V = ctx.slices(p, atoms, potential_only=True)[..., 0].copy()
    return p, atoms, pos, probe, T, V, target


def test_adjoint_4dstem_workload_geometry(ctx):
    """The benchmarked adjoint (256^2, 40 slices, potential 298^2, checkpoints
    every 6 slices) on 16 of its positions: loss and dL/dV against float64
    autograd of the same forward model (the GPU's V and probe as inputs),
    and dL/d(x,y) of 24 atoms against the float64 chain rule through
    make3DSlices' interpolation applied to the float64 dL/dV."""
    import torch
    from oracle import torch_ref as tr
    p, atoms, pos, probe, T, V, target = _adjoint_case(ctx)
    loss, dV, _ = ctx.adjoint(p, T, probe, target, positions=pos, ckpt=6)
    dV = dV.cpu().numpy()
    # float64: the loss is a sum over positions, so each position's backward
    # adds into V.grad (the autograd graph of one position at a time)
    pr = probe.cpu().numpy().astype(np.float64)
    pr = torch.from_numpy(pr[..., 0] + 1j * pr[..., 1])
    tg = torch.from_numpy(target.cpu().numpy().astype(np.float64))
    V64 = torch.from_numpy(V.astype(np.float64)).requires_grad_(True)
    L64 = 0.0
    for k in range(len(pos[0])):
        L, _ = tr.loss_from_V(p, V64, pr, [(int(pos[0][k]), int(pos[1][k]))], tg[k:k + 1])
        L.backward()
        L64 += float(L.detach())
    g64 = V64.grad.numpy()
    assert abs(loss - L64) <= TOL_LOSS * L64, (loss, L64)
    assert rel_l2(dV, g64) <= TOL_GRAD
    # atom gradients: a spread of atoms with a nonzero gradient
    g = ctx.atoms_grad(p, atoms, torch.from_numpy(dV).cuda())
    rng = np.random.default_rng(11)
    idx = np.sort(rng.choice(np.flatnonzero(np.abs(g).sum(1) > 0), 24, replace=False))
    sub = atoms[idx]
    plan = tr.AtomPlan(p, sub)
    xy = torch.from_numpy(np.stack([sub["x"], sub["y"]], 1).astype(np.float64)).requires_grad_(True)
    (plan.V(xy) * torch.from_numpy(g64)).sum().backward()
    assert rel_l2(g[idx], xy.grad.numpy()) <= TOL_GRAD
