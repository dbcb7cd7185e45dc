"""Frozen-phonon configurations and scan tiles across ranks, and the
reduction of their detector images.

doSTEM repeats the scan for `avgRuns` thermally displaced configurations
(stem3/stem3.cpp:2722-2961), each with its own make3DSlices; the images of
the configurations are averaged.  The reference displaces atoms with a
time-seeded generator (libs/fileio_fftw3.cpp:496); here configuration j is
drawn from numpy.random.default_rng(seed + j), so any rank can produce any
configuration and a run is reproducible.

With N ranks (one GPU each) configuration j runs on rank j mod N; the only
exchange is one all-reduce (sum) of the per-rank image sums and counts at
the end, which is also all the averaging needs.  A single configuration's
scan can be split the same way: contiguous tiles of scan rows per rank
(rank_positions), each rank holding the whole slice stack, and one
all-reduce of the images (scan_images).
"""
import numpy as np

from . import abi


def rank_configurations(nconf, rank, world):
    """Configurations of `rank` among `world` ranks: j = rank, rank + world, ..."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    return list(range(rank, nconf, world))


def rank_positions(p, rank, world):
    """A contiguous tile of the scan raster for `rank` among `world` ranks:
    raster positions i = ix*scanYN + iy, split into whole scan rows as evenly
    as the rows allow (rank r gets rows [r*R/W, (r+1)*R/W)).  Returns the
    positions as (iPosX, iPosY, detPosX, detPosY) int32 arrays, as
    qs_multislice_run takes them (config.scan_offsets)."""
    from . import config
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    rows = p.scanXN
    r0, r1 = rank * rows // world, (rank + 1) * rows // world
    offs = config.scan_offsets(p)
    return tuple(a[r0 * p.scanYN:r1 * p.scanYN] for a in offs)


def scan_images(ctx, p, trans, rank=0, world=1, group=None, probe=None):
    """One configuration's scan split across ranks (each rank holds the same
    slice stack): this rank's tile of positions through qs_multislice_run,
    then one all-reduce (sum) of the detector images, where every pixel has
    exactly one writer.  trans and probe may be device (torch) or host
    (numpy) arrays; returns the full images [slot][detector][x][y] as a
    float32 torch tensor on the trans device (CPU for numpy input)."""
    import torch
    import torch.distributed as dist
    pos = rank_positions(p, rank, world)
    nt = p.thickness_count()
    on_device = isinstance(trans, torch.Tensor) and trans.is_cuda
    det = torch.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), dtype=torch.float32,
                      device=trans.device if on_device else "cpu")
    if len(pos[0]) and on_device:
        torch.cuda.synchronize()  # the zeroed buffer before the library's stream writes it
        ctx.multislice(p, trans, probe, positions=pos, det=det)
    elif len(pos[0]):
        out, _, _ = ctx.multislice(p, trans, probe, positions=pos)
        det = torch.from_numpy(np.ascontiguousarray(out))
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(det, op=dist.ReduceOp.SUM, group=group)
    return det


def displaced(atoms, j, seed, sigma):
    """Configuration j: Gaussian displacements per Cartesian axis.
    sigma: one value for every atom, a dict {Znum: sigma} (others 0), or a
    per-atom array (e.g. the Einstein model's, qsc.QscRun.einstein_sigma)."""
    rng = np.random.default_rng(seed + j)
    a = abi.atoms_to_numpy(atoms).copy()
    if isinstance(sigma, dict):
        sig = np.array([sigma.get(int(z), 0.0) for z in a["Znum"]], np.float64)
    elif np.ndim(sigma) == 1:
        sig = np.asarray(sigma, np.float64)
        if len(sig) != len(a):
            raise ValueError("one sigma per atom expected")
    else:
        sig = np.full(len(a), float(sigma))
    for k in ("x", "y", "z"):
        a[k] = (a[k].astype(np.float64) + rng.standard_normal(len(a)) * sig).astype(np.float32)
    return a


class ImageSum:
    """Running sum of detector images (torch tensors, any device) and the
    number of configurations in it."""

    def __init__(self, like):
        import torch
        self.sum = torch.zeros_like(like, dtype=torch.float64)
        self.count = 0

    def add(self, images):
        self.sum += images.to(self.sum.dtype)
        self.count += 1

    def mean(self, group=None):
        """The mean over all configurations of all ranks: one all-reduce of
        the sums and counts when torch.distributed is initialised."""
        import torch
        import torch.distributed as dist
        total, count = self.sum, torch.tensor([float(self.count)], dtype=torch.float64, device=self.sum.device)
        if dist.is_available() and dist.is_initialized():
            total = total.clone()
            dist.all_reduce(total, op=dist.ReduceOp.SUM, group=group)
            dist.all_reduce(count, op=dist.ReduceOp.SUM, group=group)
        n = float(count.item())
        if n < 1:
            raise ValueError("no configurations to average")
        return (total / n).to(torch.float32)


def average_images(ctx, p, atoms, nconf, seed, sigma, rank=0, world=1, group=None):
    """doSTEM over `nconf` frozen-phonon configurations split across ranks:
    slice stack + scan per configuration on this rank's GPU (device buffers),
    then the mean detector images of all configurations (torch, on the GPU)."""
    import torch
    nt = p.thickness_count()
    det = torch.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), dtype=torch.float32, device="cuda")
    stack = torch.empty((p.slices, p.potNx, p.potNy, 2), dtype=torch.float32, device="cuda")
    acc = ImageSum(det)
    torch.cuda.synchronize()  # the zeroed buffers are ready before the library's stream uses them
    stream = torch.cuda.ExternalStream(ctx.stream_handle)
    for j in rank_configurations(nconf, rank, world):
        ctx.slices(p, displaced(atoms, j, seed, sigma), out=stack, sync=False)
        ctx.multislice(p, stack, det=det, sync=False)
        with torch.cuda.stream(stream):
            acc.add(det)
    torch.cuda.synchronize()
    return acc.mean(group)
