"""ctypes binding of libqstem_gpu.so and a thin Python host API over it.

The functions mirror the reference's call surface (stem3/stemlib.h):
make3DSlices+initSTEMSlices -> Context.slices, probe -> Context.probe,
the doSTEM/runMulsSTEM position loop -> Context.multislice,
collectIntensity -> Context.collect, getAtomPotential3D -> Context.lut.
Buffers may be numpy arrays (host, copied through the library's staging
buffers) or CUDA torch tensors (device pointers, no copies).
There is no CPU fallback: when the library cannot be loaded every call
raises.
"""
import ctypes
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libqstem_gpu.so")

EXPORTS = ["qs_ctx_create", "qs_ctx_destroy", "qs_last_error", "qs_abi_version", "qs_ctx_stream",
           "qs_params_finalize", "qs_thickness_count", "qs_lut_build", "qs_slices_build", "qs_probe",
           "qs_multislice_run", "qs_collect", "qs_stem_run", "qs_ctx_profile", "qs_ctx_stats",
           "qs_multislice_run_noalloc", "qs_phase_grating", "qs_adjoint_run", "qs_atoms_grad", "qs_tem_run",
           "qs_cbed_batch_run", "qs_slab_build", "qs_tem_run_tilted", "qs_slices_build_custom"]

_lib = None


class QsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("qstem_gpu error %d: %s" % (code, msg))
        self.code = code


def load(path=LIB_PATH):
    """Load the library (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build as _b
        _b.build()
    L = ctypes.CDLL(path)
    P = ctypes.POINTER(abi.QsParams)
    vp = ctypes.c_void_p
    L.qs_last_error.restype = ctypes.c_char_p
    L.qs_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
    L.qs_ctx_destroy.argtypes = [vp]
    L.qs_ctx_stream.restype = vp
    L.qs_ctx_stream.argtypes = [vp]
    L.qs_params_finalize.argtypes = [P]
    L.qs_thickness_count.argtypes = [P]
    L.qs_lut_build.argtypes = [vp, P, ctypes.c_int, ctypes.c_double, ctypes.c_int, vp,
                               ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                               ctypes.POINTER(ctypes.c_int), ctypes.c_uint]
    L.qs_slices_build.argtypes = [vp, P, vp, ctypes.c_int, vp, ctypes.c_uint]
    L.qs_slab_build.argtypes = [vp, P, vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_uint]
    L.qs_slices_build_custom.argtypes = [vp, P, vp, ctypes.c_int, vp, ctypes.c_int, vp, vp, ctypes.c_int, vp,
                                         ctypes.c_uint]
    L.qs_probe.argtypes = [vp, P, ctypes.c_double, ctypes.c_double, vp, ctypes.c_uint]
    L.qs_multislice_run.argtypes = [vp, P, vp, vp, ctypes.POINTER(abi.QsBatch), vp, vp, vp, ctypes.c_uint]
    L.qs_collect.argtypes = [vp, P, vp, vp, vp, ctypes.c_uint]
    L.qs_stem_run.argtypes = [vp, P, vp, ctypes.c_int, ctypes.POINTER(abi.QsBatch), vp, vp]
    L.qs_tem_run.argtypes = [vp, P, vp, vp, ctypes.c_int, ctypes.POINTER(abi.QsCtf), ctypes.c_int, vp, vp, vp, vp]
    L.qs_tem_run_tilted.argtypes = [vp, P, ctypes.c_double, ctypes.c_double, vp, vp, ctypes.c_int,
                                    ctypes.POINTER(abi.QsCtf), ctypes.c_int, vp, vp, vp, vp]
    L.qs_cbed_batch_run.argtypes = [vp, vp, ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(abi.QsCbedReport)]
    L.qs_ctx_profile.argtypes = [vp, ctypes.c_int]
    L.qs_ctx_stats.argtypes = [vp, ctypes.POINTER(abi.QsStats)]
    L.qs_multislice_run_noalloc.argtypes = [vp, P, vp, vp, ctypes.POINTER(abi.QsBatch), vp, vp, vp]
    L.qs_phase_grating.argtypes = [vp, P, vp, vp, ctypes.c_uint]
    L.qs_adjoint_run.argtypes = [vp, P, vp, vp, ctypes.POINTER(abi.QsBatch), vp, ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_double), vp, vp, ctypes.c_uint]
    L.qs_atoms_grad.argtypes = [vp, P, vp, ctypes.c_int, vp, vp, ctypes.c_uint]
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise QsError(rc, load().qs_last_error().decode(errors="replace"))


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _ptr(a):
    if a is None:
        return None
    if _is_torch(a):
        if not a.is_cuda or not a.is_contiguous():
            raise ValueError("torch tensors must be contiguous CUDA tensors")
        return ctypes.c_void_p(a.data_ptr())
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("numpy arrays must be C-contiguous")
    return a.ctypes.data_as(ctypes.c_void_p)


def _io_flags(*arrays):
    kinds = {(_is_torch(a)) for a in arrays if a is not None}
    if len(kinds) > 1:
        raise ValueError("mix of host (numpy) and device (torch) buffers")
    return 0 if kinds == {True} else abi.QS_HOST_IO


def _batch(p, positions):
    if positions is None:
        return abi.QsBatch(p.scanXN * p.scanYN, None, None, None, None), ()
    arrs = [np.ascontiguousarray(a, dtype=np.int32) for a in positions]
    ip = [a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) for a in arrs]
    return abi.QsBatch(len(arrs[0]), *ip), arrs


class Context:
    """One device + one CUDA stream (qs_ctx_create)."""

    def __init__(self, device=0):
        self.lib = load()
        h = ctypes.c_void_p()
        _check(self.lib.qs_ctx_create(device, ctypes.byref(h)))
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            self.lib.qs_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream_handle(self):
        return self.lib.qs_ctx_stream(self.h)

    # -------------------------------------------------------------- LUTs
    def lut(self, p, Z, B=0.0, charged=False):
        nz, nr, ns = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(self.lib.qs_lut_build(self.h, ctypes.byref(p), Z, B, int(charged), None, ctypes.byref(nz),
                                     ctypes.byref(nr), ctypes.byref(ns), 0))
        out = np.zeros((nz.value, nr.value), np.float32)
        _check(self.lib.qs_lut_build(self.h, ctypes.byref(p), Z, B, int(charged), _ptr(out), None, None, None,
                                     abi.QS_HOST_IO))
        return out, ns.value

    # ------------------------------------------------------------ slices
    def slices(self, p, atoms, out=None, potential_only=False, sync=True, slab=0):
        """make3DSlices + initSTEMSlices -> trans[slices][potNx][potNy][2]
        (slab `slab` of a cell divided into cellDiv slabs)."""
        a = abi.atoms_to_numpy(atoms)
        if out is None:
            out = np.zeros((p.slices, p.potNx, p.potNy, 2), np.float32)
        flags = _io_flags(out) | (abi.QS_OUT_POTENTIAL if potential_only else 0) | (abi.QS_SYNC if sync else 0)
        _check(self.lib.qs_slab_build(self.h, ctypes.byref(p), a.ctypes.data_as(ctypes.c_void_p), len(a),
                                      int(slab), _ptr(out), flags))
        return out

    def slices_custom(self, p, atoms, k, Zs, f, out=None, potential_only=False, sync=True):
        """make3DSlicesFT + initSTEMSlices with the custom scattering-factor
        table k[nk] (1/A), f[kind][nk] (A) of the elements Zs[kind]."""
        a = abi.atoms_to_numpy(atoms)
        k = np.ascontiguousarray(k, np.float64)
        Z = np.ascontiguousarray(Zs, np.int32)
        f = np.ascontiguousarray(f, np.float64)
        if f.shape != (len(Z), len(k)):
            raise ValueError("f must be [len(Zs)][len(k)]")
        if out is None:
            out = np.zeros((p.slices, p.potNx, p.potNy, 2), np.float32)
        flags = _io_flags(out) | (abi.QS_OUT_POTENTIAL if potential_only else 0) | (abi.QS_SYNC if sync else 0)
        _check(self.lib.qs_slices_build_custom(self.h, ctypes.byref(p), a.ctypes.data_as(ctypes.c_void_p), len(a),
                                               _ptr(k), len(k), _ptr(Z), _ptr(f), len(Z), _ptr(out), flags))
        return out

    # ------------------------------------------------------------- probe
    def probe(self, p, dx=None, dy=None, out=None, sync=True):
        if dx is None:
            dx = float(np.float32(p.nx // 2 * np.float32(p.resolutionX)))
        if dy is None:
            dy = float(np.float32(p.ny // 2 * np.float32(p.resolutionY)))
        if out is None:
            out = np.zeros((p.nx, p.ny, 2), np.float32)
        flags = _io_flags(out) | (abi.QS_SYNC if sync else 0)
        _check(self.lib.qs_probe(self.h, ctypes.byref(p), dx, dy, _ptr(out), flags))
        return out

    # -------------------------------------------------------- multislice
    def multislice(self, p, trans, probe=None, positions=None, det=None, diffpats=None, exit_waves=None,
                   want_det=True, want_diffpats=False, want_exit_waves=False, sync=True, slab_stacks=False,
                   series=False, graph=False, resident=False):
        """Run probe positions through the slice stack.

        positions: None (the full scan raster) or (iPosX, iPosY, detPosX, detPosY) int arrays.
        Output buffers are allocated (numpy, host) when not given and requested.
        series: diffraction patterns and exit waves of every thickness slot
        ([slot][position]...), not only the final slice's (QS_SERIES).
        graph: replay the slice loop as a CUDA graph on repeated calls with
        the same parameters and device buffers (QS_GRAPH).
        resident: 256^2 waves through the wave-resident loop (one launch,
        each wave on chip for all of its slices) instead of a row and a
        column pass per slice (QS_RESIDENT)."""
        bx, keep = _batch(p, positions)
        npos = bx.npos
        host = not _is_torch(trans)
        nt = p.thickness_count()
        lead = (nt, npos) if series else (npos,)
        if det is None and want_det and p.detectorNum > 0:
            det = np.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), np.float32) if host else None
        if diffpats is None and want_diffpats:
            diffpats = np.zeros(lead + (p.nx, p.ny), np.float32) if host else None
        if exit_waves is None and want_exit_waves:
            exit_waves = np.zeros(lead + (p.nx, p.ny, 2), np.float32) if host else None
        flags = (_io_flags(trans, probe, det, diffpats, exit_waves) | (abi.QS_SYNC if sync else 0) |
                 (abi.QS_SLAB_STACKS if slab_stacks else 0) | (abi.QS_SERIES if series else 0) |
                 (abi.QS_GRAPH if graph else 0) | (abi.QS_RESIDENT if resident else 0))
        _check(self.lib.qs_multislice_run(self.h, ctypes.byref(p), _ptr(trans), _ptr(probe), ctypes.byref(bx),
                                          _ptr(det), _ptr(diffpats), _ptr(exit_waves), flags))
        del keep
        return det, diffpats, exit_waves

    def stem_run(self, p, atoms, positions=None, det=None, diffpats=None):
        """One frozen-phonon configuration end to end (host atoms in, host
        detector images out): qs_stem_run."""
        a = abi.atoms_to_numpy(atoms)
        bx, keep = _batch(p, positions)
        if det is None and p.detectorNum > 0:
            det = np.zeros((p.thickness_count(), p.detectorNum, p.scanXN, p.scanYN), np.float32)
        _check(self.lib.qs_stem_run(self.h, ctypes.byref(p), a.ctypes.data_as(ctypes.c_void_p), len(a),
                                    ctypes.byref(bx), _ptr(det), _ptr(diffpats)))
        del keep
        return det

    def cbed_batch(self, jobs, max_bytes=0):
        """doCBED for many instances (qs_cbed_batch_run).

        jobs: list of (params, atoms).  Returns (list of diffraction patterns
        [nx][ny] as host numpy arrays, report dict)."""
        arr = (abi.QsCbedJob * len(jobs))()
        keep, outs = [], []
        for k, (p, atoms) in enumerate(jobs):
            a = abi.atoms_to_numpy(atoms)
            dp = np.zeros((p.nx, p.ny), np.float32)
            keep.append(a)
            outs.append(dp)
            arr[k].params = p
            arr[k].atoms = a.ctypes.data_as(ctypes.c_void_p).value if len(a) else None
            arr[k].natom = len(a)
            arr[k].diffpat = dp.ctypes.data_as(ctypes.c_void_p).value
        rep = abi.QsCbedReport()
        _check(self.lib.qs_cbed_batch_run(self.h, ctypes.cast(arr, ctypes.c_void_p), len(jobs), int(max_bytes),
                                          ctypes.byref(rep)))
        del keep
        return outs, {n: getattr(rep, n) for n, _ in abi.QsCbedReport._fields_}

    def tem(self, p, configs, ctf=None, defoci=(), want_exit_waves=False, beam_tilt=(0.0, 0.0)):
        """doTEM over frozen-phonon configurations (qs_tem_run, or
        qs_tem_run_tilted with a beam tilt in rad).

        configs: list of atom arrays (abi.ATOM_DTYPE), one per configuration.
        ctf: abi.QsCtf or a dict of its fields; defoci: defocus per CTF image
        (Angstrom).  Returns (mean |psi_exit|^2, CTF images [ndef][nx][ny] or
        None, exit waves [nconf][nx][ny][2] or None), host numpy arrays."""
        arrs = [abi.atoms_to_numpy(a) for a in configs]
        cat = np.ascontiguousarray(np.concatenate(arrs)) if arrs else np.zeros(0, abi.ATOM_DTYPE)
        nat = np.array([len(a) for a in arrs], np.int32)
        mean = np.zeros((p.nx, p.ny), np.float32)
        defs = np.ascontiguousarray(defoci, dtype=np.float64)
        imgs = np.zeros((len(defs), p.nx, p.ny), np.float32) if len(defs) else None
        ew = np.zeros((len(arrs), p.nx, p.ny, 2), np.float32) if want_exit_waves else None
        c = ctf if isinstance(ctf, abi.QsCtf) else abi.QsCtf(**(ctf or {}))
        args = (cat.ctypes.data_as(ctypes.c_void_p), nat.ctypes.data_as(ctypes.c_void_p), len(arrs),
                ctypes.byref(c), len(defs), defs.ctypes.data_as(ctypes.c_void_p) if len(defs) else None, _ptr(mean),
                _ptr(imgs), _ptr(ew))
        if beam_tilt[0] or beam_tilt[1]:
            _check(self.lib.qs_tem_run_tilted(self.h, ctypes.byref(p), float(beam_tilt[0]), float(beam_tilt[1]),
                                              *args))
        else:
            _check(self.lib.qs_tem_run(self.h, ctypes.byref(p), *args))
        return mean, imgs, ew

    def phase_grating(self, p, V, out=None):
        """t = exp(i lambda gamma V) for a device potential stack V (torch)."""
        import torch
        if out is None:
            out = torch.empty((p.slices, p.potNx, p.potNy, 2), dtype=torch.float32, device=V.device)
        _check(self.lib.qs_phase_grating(self.h, ctypes.byref(p), _ptr(V), _ptr(out), abi.QS_SYNC))
        return out

    def adjoint(self, p, trans, probe, target, positions=None, ckpt=0, want_diffpats=False, slab_stacks=False,
                deterministic=False):
        """Loss sum (I - target)^2 and dL/dV (device torch tensors in and out).
        ckpt: keep the forward waves every ckpt slices (1: all; 0: all when
        they fit in device memory, else the smallest interval that fits).
        slab_stacks: trans holds one stack per slab of a cell divided into
        cellDiv slabs (dL/dV then too); else one stack serves every slab.
        deterministic: sum dL/dV over positions in a fixed order
        (QS_DETERMINISTIC; bit-reproducible) instead of with float atomics."""
        import torch
        bx, keep = _batch(p, positions)
        nst = p.cellDiv if (slab_stacks and p.cellDiv > 1) else 1
        dV = torch.empty((p.slices * nst, p.potNx, p.potNy), dtype=torch.float32, device=trans.device)
        dps = torch.empty((bx.npos, p.nx, p.ny), dtype=torch.float32, device=trans.device) if want_diffpats else None
        loss = ctypes.c_double()
        _check(self.lib.qs_adjoint_run(self.h, ctypes.byref(p), _ptr(trans), _ptr(probe), ctypes.byref(bx),
                                       _ptr(target), int(ckpt), ctypes.byref(loss), _ptr(dV), _ptr(dps),
                                       abi.QS_SYNC | (abi.QS_SLAB_STACKS if slab_stacks else 0) |
                                       (abi.QS_DETERMINISTIC if deterministic else 0)))
        del keep
        return loss.value, dV, dps

    def atoms_grad(self, p, atoms, dV, slab_stacks=False):
        a = abi.atoms_to_numpy(atoms)
        g = np.zeros((len(a), 2), np.float64)
        _check(self.lib.qs_atoms_grad(self.h, ctypes.byref(p), a.ctypes.data_as(ctypes.c_void_p), len(a), _ptr(dV),
                                      g.ctypes.data_as(ctypes.c_void_p),
                                      abi.QS_SLAB_STACKS if slab_stacks else 0))
        return g

    def profile(self, enable=True):
        _check(self.lib.qs_ctx_profile(self.h, int(enable)))

    def stats(self):
        st = abi.QsStats()
        _check(self.lib.qs_ctx_stats(self.h, ctypes.byref(st)))
        return {n: getattr(st, n) for n, _ in abi.QsStats._fields_}

    # ----------------------------------------------------------- collect
    def collect(self, p, wave_k, diffpat=False):
        w = np.ascontiguousarray(wave_k, dtype=np.float32)
        sums = np.zeros(max(p.detectorNum, 1), np.float64)
        dp = np.zeros((p.nx, p.ny), np.float32) if diffpat else None
        _check(self.lib.qs_collect(self.h, ctypes.byref(p), _ptr(w), _ptr(sums), _ptr(dp), abi.QS_HOST_IO))
        return sums[:p.detectorNum], dp


def thickness_count(p):
    return load().qs_thickness_count(ctypes.byref(p))
