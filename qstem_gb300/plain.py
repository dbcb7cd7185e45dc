"""The plain GPU multislice: one probe at a time, one kernel per step.

This is the unfused baseline the batched path is measured against: for each
probe position and slice it launches transmit, a cuFFT 2-D forward
transform, the propagator multiply, the detector reduction and a cuFFT
inverse transform with normalisation, as separate torch operations (the
structure of runMulsSTEM, stem3/stemlib.cpp:2403-2486).  It is a measurement
reference only; the library's entry points never call it.
"""
import numpy as np
import torch

from . import config


def tables(p, device):
    """propagate_slow's kx2/ky2 and propagator factors (stem3/stemlib.cpp:2783-2824)."""
    f = np.float32
    nx, ny = p.nx, p.ny
    ax, by = f(f(p.resolutionX) * f(nx)), f(f(p.resolutionY) * f(ny))
    scale = f(float(f(p.sliceThickness)) * 3.14159265358979)
    wl = f(config.wavelength(float(f(p.v0))))
    i = np.arange(nx)
    kx = np.where(i > nx // 2, (i - nx).astype(f) / ax, i.astype(f) / ax).astype(f)
    j = np.arange(ny)
    ky = np.where(j > ny // 2, (j - ny).astype(f) / by, j.astype(f) / by).astype(f)
    kx2, ky2 = (kx * kx).astype(f), (ky * ky).astype(f)
    ax_ = (scale * (kx2 * wl)).astype(f)
    ay_ = (scale * (ky2 * wl)).astype(f)
    px = (np.cos(ax_) - 1j * np.sin(ax_)).astype(np.complex64)
    py = (np.cos(ay_) - 1j * np.sin(ay_)).astype(np.complex64)
    k2max = f(min(f(nx / f(2.0 * ax)), f(ny / f(2.0 * by))))
    k2max = f(2.0 / 3.0 * k2max)
    k2max = f(k2max * k2max)
    k2 = (kx2[:, None] + ky2[None, :]).astype(f)
    mask = (kx2[:, None] < k2max) & (k2 < k2max)
    prop = np.where(mask, py[None, :] * px[:, None], 0).astype(np.complex64)
    dev = torch.device(device)
    return torch.from_numpy(prop).to(dev), torch.from_numpy(k2).to(dev)


def run_positions(p, trans, probe, positions, device="cuda"):
    """trans: (slices, potNx, potNy) complex64 tensor; probe (nx, ny) complex64;
    positions: list of (iPosX, iPosY).  Returns [npos][ndet] detector values of
    the final slice."""
    prop, k2 = tables(p, device)
    N = p.nx * p.ny
    scale = float(np.float32(p.electronScale)) / (N * N)
    masks = [((k2 >= float(np.float32(p.detectors[d].k2Inside))) & (k2 <= float(np.float32(p.detectors[d].k2Outside))))
             for d in range(p.detectorNum)]
    out = torch.zeros((len(positions), p.detectorNum), dtype=torch.float64, device=device)
    for n, (ix, iy) in enumerate(positions):
        w = probe.clone()
        for s in range(p.slices):
            w = w * trans[s, ix:ix + p.nx, iy:iy + p.ny]
            w = torch.fft.fft2(w)
            w = w * prop
            if s == p.slices - 1:
                I = (w.real * w.real + w.imag * w.imag)
                for d, m in enumerate(masks):
                    out[n, d] = (I * m).sum(dtype=torch.float64) * scale
            w = torch.fft.ifft2(w) if s < p.slices - 1 else w
    return out
