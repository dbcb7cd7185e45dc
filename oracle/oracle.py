"""ctypes wrapper of the C restatement (liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline as the checker; never by the shipped library.
"""
import ctypes
import os
import subprocess

import numpy as np

from qstem_gb300 import abi, config

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")
_lib = None


def build(quiet=True, ref_dir=None):
    """Compile liboracle.so and, when the reference checkout is given (ref_dir,
    else the QS_REFERENCE_DIR environment variable) and present, the
    reference's own programs in _ref/ with oracle/Makefile."""
    out = subprocess.run(["make", "-C", HERE, "-j8"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    ref = ref_dir or os.environ.get("QS_REFERENCE_DIR")
    if ref and os.path.isdir(ref):
        # the reference's programs, and its stem3 with the drop-in adapter
        # (this one links the GPU library, built before the oracle)
        for target in ("ref", "adapter"):
            out = subprocess.run(["make", "-C", HERE, "-j8", target, "REF=" + os.path.abspath(ref)],
                                 capture_output=True, text=True)
            if out.returncode != 0 and not quiet:
                print(out.stdout + out.stderr)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER(abi.QsParams)
        fp = ctypes.c_void_p
        L.qso_wavelength.restype = ctypes.c_double
        L.qso_wavelength.argtypes = [ctypes.c_double]
        L.qso_lut.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_int, fp,
                              ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                              ctypes.POINTER(ctypes.c_int)]
        L.qso_lut2d.argtypes = [P, ctypes.c_int, ctypes.c_double, fp, ctypes.POINTER(ctypes.c_int),
                                ctypes.POINTER(ctypes.c_int)]
        L.qso_potential_ft.argtypes = [P, fp, ctypes.c_int, fp, ctypes.c_int, fp, fp, ctypes.c_int, fp]
        L.qso_potential.argtypes = [P, fp, ctypes.c_int, fp]
        L.qso_potential_slab.argtypes = [P, fp, ctypes.c_int, ctypes.c_int, fp]
        L.qso_stem_slabs.argtypes = [P, fp, ctypes.c_int, fp, ctypes.c_int, ctypes.c_int, fp, fp, fp, ctypes.c_int]
        L.qso_transmission.argtypes = [P, fp]
        L.qso_probe.argtypes = [P, ctypes.c_double, ctypes.c_double, fp]
        L.qso_run_position.argtypes = [P, fp, ctypes.c_int, ctypes.c_int, fp, fp, fp]
        L.qso_stem.argtypes = [P, fp, fp, ctypes.c_int, ctypes.c_int, fp, fp, fp, ctypes.c_int]
        L.qso_scan_offsets.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_int)]
        L.qso_thickness_count.argtypes = [P]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def lut(p, Z, B=0.0, charged=False):
    L = lib()
    nz, nr, ns = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    rc = L.qso_lut(ctypes.byref(p), Z, B, int(charged), None, ctypes.byref(nz), ctypes.byref(nr), ctypes.byref(ns))
    assert rc == 0, rc
    out = np.zeros((nz.value, nr.value), np.float32)
    rc = L.qso_lut(ctypes.byref(p), Z, B, int(charged), _ptr(out), None, None, None)
    assert rc == 0, rc
    return out, ns.value


def lut2d(p, Z, B=0.0):
    """getAtomPotential2D: the (nx, ny, 2) complex table."""
    L = lib()
    nx, ny = ctypes.c_int(), ctypes.c_int()
    rc = L.qso_lut2d(ctypes.byref(p), Z, B, None, ctypes.byref(nx), ctypes.byref(ny))
    assert rc == 0, rc
    out = np.zeros((nx.value, ny.value, 2), np.float32)
    rc = L.qso_lut2d(ctypes.byref(p), Z, B, _ptr(out), None, None)
    assert rc == 0, rc
    return out


def potential_ft(p, atoms, k, Zs, f):
    """make3DSlicesFT with the custom table k[nk], f[kind][nk] of elements Zs."""
    out = np.zeros((p.slices, p.potNx, p.potNy, 2), np.float32)
    a = abi.atoms_to_numpy(atoms)
    k = np.ascontiguousarray(k, np.float64)
    Z = np.ascontiguousarray(Zs, np.int32)
    f = np.ascontiguousarray(f, np.float64)
    rc = lib().qso_potential_ft(ctypes.byref(p), _ptr(a), len(a), _ptr(k), len(k), _ptr(Z), _ptr(f), len(Z),
                                _ptr(out))
    assert rc == 0, rc
    return out


def potential(p, atoms, slab=0):
    """make3DSlices (slab `slab` of a cell divided into cellDiv slabs)."""
    out = np.zeros((p.slices, p.potNx, p.potNy, 2), np.float32)
    a = abi.atoms_to_numpy(atoms)
    rc = lib().qso_potential_slab(ctypes.byref(p), _ptr(a), len(a), int(slab), _ptr(out))
    assert rc == 0, rc
    return out


def transmission(p, V):
    out = np.ascontiguousarray(V, dtype=np.float32).copy()
    rc = lib().qso_transmission(ctypes.byref(p), _ptr(out))
    assert rc == 0, rc
    return out


def probe(p, dx=None, dy=None):
    if dx is None:
        dx = p.nx // 2 * float(np.float32(p.resolutionX))
    if dy is None:
        dy = p.ny // 2 * float(np.float32(p.resolutionY))
    out = np.zeros((p.nx, p.ny, 2), np.float32)
    rc = lib().qso_probe(ctypes.byref(p), dx, dy, _ptr(out))
    assert rc == 0, rc
    return out


def stem(p, trans, probe_wave=None, p0=0, p1=None, det=True, diffpats=False, exit_waves=False,
         nthreads=0, slab_stacks=False):
    """The doSTEM position loop for raster positions [p0, p1), through cellDiv
    slabs (trans: one stack reused, or cellDiv stacks with slab_stacks)."""
    npix = p.scanXN * p.scanYN
    p1 = npix if p1 is None else p1
    nt = p.thickness_count()
    d = np.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), np.float32) if det else None
    dp = np.zeros((p1 - p0, p.nx, p.ny), np.float32) if diffpats else None
    ew = np.zeros((p1 - p0, p.nx, p.ny, 2), np.float32) if exit_waves else None
    t = np.ascontiguousarray(trans, dtype=np.float32)
    pw = None if probe_wave is None else np.ascontiguousarray(probe_wave, dtype=np.float32)
    rc = lib().qso_stem_slabs(ctypes.byref(p), _ptr(t), int(bool(slab_stacks)), _ptr(pw), p0, p1, _ptr(d), _ptr(dp),
                              _ptr(ew), nthreads)
    assert rc == 0, rc
    return d, dp, ew


def run_position(p, trans, iPosX, iPosY, wave):
    w = np.ascontiguousarray(wave, dtype=np.float32).copy()
    nt = p.thickness_count()
    det = np.zeros((nt, max(p.detectorNum, 1)), np.float32)
    dp = np.zeros((p.nx, p.ny), np.float32)
    rc = lib().qso_run_position(ctypes.byref(p), _ptr(np.ascontiguousarray(trans, np.float32)),
                                iPosX, iPosY, _ptr(w), _ptr(det), _ptr(dp))
    assert rc == 0, rc
    return w, det[:, :p.detectorNum], dp


def run_reference(qsc_path, outdir, run=True, clock=None):
    """Run the reference's own CPU path on a .qsc through the harness.
    clock: the value the reference's time() returns (its thermal
    displacements and CBED source offsets are seeded with -time(NULL));
    None leaves the real clock."""
    os.makedirs(outdir, exist_ok=True)
    args = [REF_HARNESS, os.path.basename(qsc_path), os.path.abspath(outdir)]
    if run:
        args.append("run")
    env = dict(os.environ)
    env.pop("QS_REF_CLOCK", None)
    if clock is not None:
        env["QS_REF_CLOCK"] = str(int(clock))
    r = subprocess.run(args, cwd=os.path.dirname(os.path.abspath(qsc_path)), stdin=subprocess.DEVNULL,
                       capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("reference harness failed: " + r.stdout[-2000:] + r.stderr[-2000:])
    return outdir


def ctf_transfer(p, ctf, df):
    """Objective-lens transfer H(k) of GUI_Matlab/simImageFromWave.m:57-73 in
    float64, in FFT order on the wave grid (k = (i < n/2 ? i : i - n)/(n dx),
    the script's fftshifted [-n/2, n/2) grid).  ctf: dict of the qs_ctf
    fields; the aperture gets an optional raised-cosine edge of width
    `edge` (the script's hard aperture when edge = 0)."""
    lam = config.wavelength(float(np.float32(p.v0)))
    c = dict(Cs=0.0, astig=0.0, astigPhi=0.0, focalSpread=0.0, alpha=0.0, kmax=0.0, edge=0.0)
    c.update(ctf or {})
    ix = np.arange(p.nx)
    iy = np.arange(p.ny)
    kx = np.where(ix < p.nx // 2, ix, ix - p.nx) / (p.nx * float(np.float32(p.resolutionX)))
    ky = np.where(iy < p.ny // 2, iy, iy - p.ny) / (p.ny * float(np.float32(p.resolutionY)))
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    k2 = KX ** 2 + KY ** 2
    k = np.sqrt(k2)
    if c["kmax"] > 0:
        if c["edge"] <= 0:
            A = (k2 < c["kmax"] ** 2).astype(np.float64)
        else:
            lo, hi = c["kmax"] - 0.5 * c["edge"], c["kmax"] + 0.5 * c["edge"]
            A = np.where(k <= lo, 1.0, np.where(k >= hi, 0.0, 0.5 * (1 + np.cos(np.pi * (k - lo) / c["edge"]))))
    else:
        A = np.ones_like(k2)
    phi = np.arctan2(KY, KX)
    Et = np.exp(-2.0 * (c["focalSpread"] * lam * k2) ** 2)
    Es = np.exp(-(np.pi * c["alpha"] * df + np.pi * c["alpha"] * lam ** 2 * c["Cs"] * k2) ** 2 * k2)
    chi = np.pi * (lam * (df + c["astig"] * np.cos(2 * (phi - c["astigPhi"]))) * k2 + 0.5 * lam ** 3 * c["Cs"] * k2 ** 2)
    return A * Et * Es * np.exp(-1j * chi)


def tem(p, stacks, ctf=None, defoci=()):
    """doTEM over frozen-phonon configurations (stem3/stem3.cpp:2354-2710):
    the untilted plane wave psi = 1 (:2403-2406) through each configuration's
    transmission stack (runMulsSTEM), the mean exit intensity, and the mean
    over configurations of |IFFT(FFT(psi_exit) H_df)|^2 (float64 FFTs)."""
    plane = np.zeros((p.nx, p.ny, 2), np.float32)
    plane[..., 0] = 1.0
    ews = [run_position(p, T, 0, 0, plane)[0] for T in stacks]
    mean = np.mean([w[..., 0].astype(np.float64) ** 2 + w[..., 1].astype(np.float64) ** 2 for w in ews], axis=0)
    imgs = []
    for df in defoci:
        H = ctf_transfer(p, ctf, df)
        acc = np.zeros((p.nx, p.ny))
        for w in ews:
            z = w[..., 0].astype(np.float64) + 1j * w[..., 1].astype(np.float64)
            acc += np.abs(np.fft.ifft2(np.fft.fft2(z) * H)) ** 2
        imgs.append(acc / len(ews))
    return mean, (np.array(imgs) if len(imgs) else None), np.array(ews)
