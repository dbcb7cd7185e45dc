"""torch.autograd bindings of the adjoint multislice.

MultisliceLoss: V (slice potentials, CUDA float32 tensor [slices][potNx][potNy])
    -> L = sum_p sum_k (I_p(k) - target_p(k))^2, with dL/dV from the
    hand-written adjoint (qs_adjoint_run).
AtomsLoss: atom (x, y) positions -> the same loss through the slice builder,
    with dL/d(x, y) from qs_atoms_grad.

The adjoint needs the forward waves anyway (kept every `ckpt` slices), so the
forward call runs the adjoint too and keeps the gradient for backward.
For a cell divided into slabs (cellDiv > 1) the wave runs through every
slab; with slab_stacks each slab has its own stack (V then holds
cellDiv x slices slices), otherwise the one stack serves every slab.
"""
import numpy as np
import torch

from . import abi


class MultisliceLoss(torch.autograd.Function):
    @staticmethod
    def forward(fctx, V, qctx, p, probe, target, positions=None, ckpt=0, slab_stacks=False):
        q = p
        if slab_stacks and p.cellDiv > 1:  # the grating of every slab's stack
            q = p.copy()
            q.slices = p.slices * p.cellDiv
        trans = qctx.phase_grating(q, V.contiguous())
        loss, dV, _ = qctx.adjoint(p, trans, probe, target, positions=positions, ckpt=ckpt, slab_stacks=slab_stacks)
        fctx.save_for_backward(dV)
        return torch.tensor(loss, dtype=torch.float64, device=V.device)

    @staticmethod
    def backward(fctx, gL):
        (dV,) = fctx.saved_tensors
        return (gL.to(dV.dtype) * dV, None, None, None, None, None, None, None)


class AtomsLoss(torch.autograd.Function):
    @staticmethod
    def forward(fctx, xy, qctx, p, atoms, probe, target, positions=None, ckpt=0, slab_stacks=False):
        a = abi.atoms_to_numpy(atoms).copy()
        xyn = xy.detach().cpu().numpy()
        a["x"] = xyn[:, 0].astype(np.float32)
        a["y"] = xyn[:, 1].astype(np.float32)
        nst = p.cellDiv if (slab_stacks and p.cellDiv > 1) else 1
        trans = torch.empty((p.slices * nst, p.potNx, p.potNy, 2), dtype=torch.float32, device=probe.device)
        for k in range(nst):  # make3DSlices of every slab
            qctx.slices(p, a, out=trans[k * p.slices:(k + 1) * p.slices], slab=k)
        loss, dV, _ = qctx.adjoint(p, trans, probe, target, positions=positions, ckpt=ckpt, slab_stacks=slab_stacks)
        g = qctx.atoms_grad(p, a, dV, slab_stacks=slab_stacks)
        fctx.save_for_backward(torch.from_numpy(g).to(xy.device, xy.dtype))
        return torch.tensor(loss, dtype=torch.float64, device=xy.device)

    @staticmethod
    def backward(fctx, gL):
        (g,) = fctx.saved_tensors
        return (gL.to(g.dtype) * g, None, None, None, None, None, None, None, None)
