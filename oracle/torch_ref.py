"""Float64 restatement of the differentiable 4D-STEM forward model (CPU).

TEST INFRASTRUCTURE ONLY: the FP64 reference gradient for the GPU adjoint
(qs_adjoint_run / qs_atoms_grad).  torch autograd in float64 differentiates

    atoms (x, y) -> V            make3DSlices' scatter-sum with the radial
                                 linear LUT interpolation
                                 (stem3/stemlib.cpp:894-1213)
    V -> t = exp(i sigma V)      initSTEMSlices (stem3/stemlib.cpp:2280-2299)
    t -> psi_S(k)                runMulsSTEM's slice loop
                                 (stem3/stemlib.cpp:2405-2483)
    I = |psi_S(k)|^2/sqrt(N)     collectIntensity's diffpat (:2630), fftshifted
    L = sum (I - target)^2

The LUTs and the probe come from the C restatement (oracle/qs_oracle.c), the
propagator and k^2 tables from the reference's float formulas.
"""
import math

import numpy as np
import torch

from oracle import oracle
from qstem_gb300 import config

F32 = np.float32


def sigma(p):
    return float(F32(1.0) + F32(p.v0) / F32(511.0)) * config.wavelength(float(F32(p.v0)))


def propagator(p):
    """conj-free propagator P(kx, ky) with the 2/3 band limit, complex128."""
    nx, ny = p.nx, p.ny
    ax, by = F32(F32(p.resolutionX) * F32(nx)), F32(F32(p.resolutionY) * F32(ny))
    scale = F32(float(F32(p.sliceThickness)) * 3.14159265358979)
    wl = F32(config.wavelength(float(F32(p.v0))))
    i = np.arange(nx)
    kx = np.where(i > nx // 2, (i - nx).astype(F32) / ax, i.astype(F32) / ax).astype(F32)
    j = np.arange(ny)
    ky = np.where(j > ny // 2, (j - ny).astype(F32) / by, j.astype(F32) / by).astype(F32)
    kx2, ky2 = (kx * kx).astype(F32), (ky * ky).astype(F32)
    tx, ty = (scale * (kx2 * wl)).astype(F32), (scale * (ky2 * wl)).astype(F32)
    px = np.cos(tx.astype(np.float64)) - 1j * np.sin(tx.astype(np.float64))
    py = np.cos(ty.astype(np.float64)) - 1j * np.sin(ty.astype(np.float64))
    k2max = F32(min(F32(nx / F32(2.0 * ax)), F32(ny / F32(2.0 * by))))
    k2max = F32(F32(2.0 / 3.0 * k2max) ** 2)
    mask = (kx2[:, None] < k2max) & ((kx2[:, None] + ky2[None, :]) < k2max)
    return torch.from_numpy(np.where(mask, px[:, None] * py[None, :], 0).astype(np.complex128))


def loss_from_V(p, V, probe, positions, target):
    """V: float64 tensor (slices, potNx, potNy); probe complex128 (nx, ny);
    positions: list of (iPosX, iPosY); target float64 (npos, nx, ny)."""
    t = torch.exp(1j * sigma(p) * V)
    P = propagator(p)
    N = p.nx * p.ny
    total = 0.0
    pats = []
    for n, (ix, iy) in enumerate(positions):
        w = probe
        for s in range(p.slices):
            w = w * t[s, ix:ix + p.nx, iy:iy + p.ny]
            W = torch.fft.fft2(w) * P
            if s < p.slices - 1:
                w = torch.fft.ifft2(W)
        I = (W.real ** 2 + W.imag ** 2) / math.sqrt(N)
        Ish = torch.fft.fftshift(I)
        pats.append(Ish)
        total = total + ((Ish - target[n]) ** 2).sum()
    return total, torch.stack(pats)


class AtomPlan:
    """Index arrays of every (atom, pixel, slice) LUT lookup of the scatter-sum,
    following make3DSlices' default branch (the same control flow as
    qso_potential in qs_oracle.c).  Radial indices are frozen at the planned
    positions; the interpolation weight stays differentiable."""

    def __init__(self, p, atoms):
        self.p = p
        Bs = {}
        order = np.argsort(atoms["z"], kind="stable")
        at = atoms[order]
        c = F32(p.sliceThickness) * F32(p.slices)
        dx, dy, dz = F32(p.resolutionX), F32(p.resolutionY), F32(p.sliceThickness)
        self.dr = float(F32(p.resolutionX) / F32(2.0))
        iRadX = int(math.ceil(F32(p.atomRadius) / dx))
        iRadY = int(math.ceil(F32(p.atomRadius) / dy))
        iRadZ = int(math.ceil(F32(p.atomRadius) / dz))
        lut0, nzsub = oracle.lut(p, 8, 0.0)
        Nz, Nr = lut0.shape
        self.Nr, self.Nz = Nr, Nz
        luts = {}
        ent = {k: [] for k in ("atom", "cx", "cy", "slice", "row", "fx", "fy", "q", "lut", "lutq", "r0", "ir0")}
        natom = len(at)
        ia = 0
        while ia < natom:
            while ia < natom and at["Znum"][ia] == 0:
                ia += 1
            if ia >= natom:
                break

            def az(i):
                zz = F32(float(F32(F32(at["z"][i]) + F32(p.czOffset))) - 0.5 * float(F32(p.sliceThickness)) * (1 - p.centerSlices))
                return F32(zz - F32(p.sliceThickness))
            atomZ = az(ia)
            if p.nonPeriodZ:
                if atomZ - F32(p.atomRadius) > c:
                    break
                while True:
                    if atomZ + F32(p.atomRadius) + F32(p.sliceThickness) >= 0:
                        break
                    ia += 1
                    atomZ = az(ia)
                    if not ia < natom - 1:
                        break
            atomX = F32(F32(at["x"][ia]) - F32(p.potOffsetX))
            atomY = F32(F32(at["y"][ia]) - F32(p.potOffsetY))
            iAtomX = int(math.floor(F32(atomX / dx)))
            iAtomY = int(math.floor(F32(atomY / dy)))
            atomZ = F32(atomZ + F32(p.sliceThickness))
            iAtomZ = int(math.floor(float(F32(atomZ / dz)) + 0.5))
            if p.nonPeriod:
                iax0, iax1 = max(iAtomX - iRadX, 0), min(iAtomX + iRadX, p.potNx - 1)
                iay0, iay1 = max(iAtomY - iRadY, 0), min(iAtomY + iRadY, p.potNy - 1)
                if not (iax0 < p.potNx and iax1 >= 0 and iay0 < p.potNy and iay1 >= 0):
                    ia += 1
                    continue
            else:
                iax0, iax1 = iAtomX - iRadX, iAtomX + iRadX - 1
                iay0, iay1 = iAtomY - iRadY, iAtomY + iRadY - 1
            iaz0 = -iAtomZ if iAtomZ - iRadZ < 0 else -iRadZ
            iaz1 = p.slices - iAtomZ - 1 if iAtomZ + iRadZ >= p.slices else iRadZ
            if not (iAtomZ + iaz0 < p.slices and iAtomZ + iaz1 >= 0):
                ia += 1
                continue
            Z = int(at["Znum"][ia])
            q = float(at["q"][ia])
            B = 0.0 if p.tds else float(at["dw"][ia])
            if (Z, 0) not in luts:
                luts[(Z, 0)] = oracle.lut(p, Z, B)[0]
            if q != 0 and (Z, 1) not in luts:
                luts[(Z, 1)] = oracle.lut(p, Z, B, charged=True)[0]
            dOffsZ = float(F32(F32(F32(iAtomZ + iaz0) - F32(atomZ / dz)) * F32(nzsub)))
            iOffs0 = int(dOffsZ + 0.5) * Nr
            ixs = np.arange(iax0, iax1 + 1)
            iys = np.arange(iay0, iay1 + 1)
            IX, IY = np.meshgrid(ixs, iys, indexing="ij")
            fx = (IX.astype(F32) * dx).astype(F32)
            fy = (IY.astype(F32) * dy).astype(F32)
            # the reference forms the offsets in float (x2 = iax*dx - atomX,
            # stem3/stemlib.cpp:931-938)
            r = np.sqrt((fx - atomX).astype(F32).astype(np.float64) ** 2 +
                        (fy - atomY).astype(F32).astype(np.float64) ** 2)
            ir = np.floor(r / self.dr).astype(np.int64)
            ok = ir < Nr - 1
            cx = IX if p.nonPeriod else np.mod(IX, p.potNx)
            cy = IY if p.nonPeriod else np.mod(IY, p.potNy)
            for k, iaz in enumerate(range(iaz0, iaz1 + 1)):
                off = iOffs0 + k * nzsub * Nr
                if off < 0:
                    if not off > -Nr * (Nz - 1):
                        continue
                    row = -off + Nr
                else:
                    if not off < Nr * (Nz - 1):
                        continue
                    row = off
                m = ok
                n = int(m.sum())
                ent["atom"].append(np.full(n, order[ia]))
                ent["cx"].append(cx[m])
                ent["cy"].append(cy[m])
                ent["slice"].append(np.full(n, iAtomZ + iaz))
                ent["row"].append(np.full(n, row) + 0)
                ent["fx"].append(fx[m].astype(np.float64))
                ent["fy"].append(fy[m].astype(np.float64))
                ent["r0"].append(r[m] == 0.0)
                ent["ir0"].append(ir[m])
                ent["q"].append(np.full(n, q))
                ent["lut"].append(np.full(n, list(luts).index((Z, 0))))
                ent["lutq"].append(np.full(n, list(luts).index((Z, 1)) if q != 0 else -1))
            ia += 1
        self.e = {k: np.concatenate(v) if v else np.zeros(0) for k, v in ent.items()}
        self.luts = [torch.from_numpy(luts[k].astype(np.float64).ravel()) for k in luts]
        self.lut_sizes = [luts[k].size for k in luts]
        self.potOffsetX, self.potOffsetY = float(F32(p.potOffsetX)), float(F32(p.potOffsetY))

    def V(self, xy, frozen=False):
        """xy: float64 tensor (natom, 2) of atom x, y (A).  frozen=True keeps
        every lookup in the radial interval of the planned positions (the
        model whose derivative is the one-sided, kink-consistent one)."""
        p, e = self.p, self.e
        a = torch.from_numpy(e["atom"].astype(np.int64))
        ax = xy[a, 0] - self.potOffsetX
        ay = xy[a, 1] - self.potOffsetY
        # An atom exactly on a pixel (r = 0 in the reference's float offsets)
        # sits at the tip of a cone: the term is constant to first order and
        # its central difference vanishes, so it carries no gradient.
        r2 = (torch.from_numpy(e["fx"]) - ax) ** 2 + (torch.from_numpy(e["fy"]) - ay) ** 2
        r0 = torch.from_numpy(e["r0"].astype(bool))
        r = torch.where(r0, torch.zeros_like(r2), torch.sqrt(torch.where(r0, torch.ones_like(r2), r2)))
        rr = r / self.dr
        ir = torch.from_numpy(e["ir0"].astype(np.int64)) if frozen else torch.floor(rr.detach()).long()
        ok = ir < self.Nr - 1
        ddr = rr - ir
        cat = torch.cat(self.luts)
        offs = np.concatenate([[0], np.cumsum(self.lut_sizes)[:-1]]).astype(np.int64)
        base = torch.from_numpy(offs[e["lut"].astype(np.int64)] + e["row"].astype(np.int64)) + ir
        irc = torch.clamp(base, max=cat.numel() - 2)
        val = (1 - ddr) * cat[irc] + ddr * cat[irc + 1]
        hasq = e["lutq"] >= 0
        if hasq.any():
            baseq = torch.from_numpy(offs[np.maximum(e["lutq"], 0).astype(np.int64)] + e["row"].astype(np.int64)) + ir
            baseq = torch.clamp(baseq, max=cat.numel() - 2)
            valq = (1 - ddr) * cat[baseq] + ddr * cat[baseq + 1]
            val = val + torch.from_numpy(np.where(hasq, e["q"], 0.0)) * valq
        val = torch.where(ok, val, torch.zeros_like(val))
        flat = (torch.from_numpy(e["slice"].astype(np.int64)) * p.potNx + torch.from_numpy(e["cx"].astype(np.int64))) \
            * p.potNy + torch.from_numpy(e["cy"].astype(np.int64))
        V = torch.zeros(p.slices * p.potNx * p.potNy, dtype=torch.float64)
        V = V.index_add(0, flat, val)
        return V.reshape(p.slices, p.potNx, p.potNy)
