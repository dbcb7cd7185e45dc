"""ctypes wrapper of the C restatement (liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline as the checker; never by the shipped library.
"""
import ctypes
import os
import subprocess

import numpy as np

from qstem_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")
_lib = None


def build(quiet=True):
    """Compile liboracle.so (and, when the reference tree is present, the
    reference harness) with oracle/Makefile."""
    out = subprocess.run(["make", "-C", HERE, "-j8"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if os.path.isdir(os.environ.get("QS_REFERENCE_DIR", "/root/reference")):
        out = subprocess.run(["make", "-C", HERE, "-j8", "ref"], capture_output=True, text=True)
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
        L.qso_potential.argtypes = [P, fp, ctypes.c_int, fp]
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


def potential(p, atoms):
    out = np.zeros((p.slices, p.potNx, p.potNy, 2), np.float32)
    a = abi.atoms_to_numpy(atoms)
    rc = lib().qso_potential(ctypes.byref(p), _ptr(a), len(a), _ptr(out))
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
         nthreads=0):
    """The doSTEM position loop for raster positions [p0, p1)."""
    npix = p.scanXN * p.scanYN
    p1 = npix if p1 is None else p1
    nt = p.thickness_count()
    d = np.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), np.float32) if det else None
    dp = np.zeros((p1 - p0, p.nx, p.ny), np.float32) if diffpats else None
    ew = np.zeros((p1 - p0, p.nx, p.ny, 2), np.float32) if exit_waves else None
    t = np.ascontiguousarray(trans, dtype=np.float32)
    pw = None if probe_wave is None else np.ascontiguousarray(probe_wave, dtype=np.float32)
    rc = lib().qso_stem(ctypes.byref(p), _ptr(t), _ptr(pw), p0, p1, _ptr(d), _ptr(dp), _ptr(ew), nthreads)
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


def run_reference(qsc_path, outdir, run=True):
    """Run the reference's own CPU path on a .qsc through the harness."""
    os.makedirs(outdir, exist_ok=True)
    args = [REF_HARNESS, os.path.basename(qsc_path), os.path.abspath(outdir)]
    if run:
        args.append("run")
    r = subprocess.run(args, cwd=os.path.dirname(os.path.abspath(qsc_path)), stdin=subprocess.DEVNULL,
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference harness failed: " + r.stdout[-2000:] + r.stderr[-2000:])
    return outdir
