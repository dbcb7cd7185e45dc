"""ctypes mirror of include/qstem_gpu.h (the C ABI of libqstem_gpu.so).

The structures have exactly the C layout; numpy structured dtypes are given
for arrays of atoms.
"""
import ctypes

import numpy as np

QS_OK = 0
QS_ERR_ARG = -1
QS_ERR_CUDA = -2
QS_ERR_NOMEM = -3
QS_ERR_UNSUPPORTED = -4
QS_ERR_TIMEOUT = -5

QS_HOST_IO = 1
QS_OUT_POTENTIAL = 2
QS_SYNC = 4
QS_SLAB_STACKS = 8
QS_SERIES = 16
QS_GRAPH = 32
QS_DETERMINISTIC = 64
QS_RESIDENT = 128

QS_MODE_STEM = 1
QS_MODE_CBED = 2
QS_MODE_TEM = 3

QS_MAX_DETECTORS = 16

# struct atom of libs/stemtypes_fftw3.h:70-77 (z first), 28 bytes
ATOM_DTYPE = np.dtype([("z", "<f4"), ("y", "<f4"), ("x", "<f4"), ("dw", "<f4"),
                       ("occ", "<f4"), ("q", "<f4"), ("Znum", "<i4")])


class QsAtom(ctypes.Structure):
    _fields_ = [("z", ctypes.c_float), ("y", ctypes.c_float), ("x", ctypes.c_float),
                ("dw", ctypes.c_float), ("occ", ctypes.c_float), ("q", ctypes.c_float),
                ("Znum", ctypes.c_int)]


class QsDetector(ctypes.Structure):
    _fields_ = [("rInside", ctypes.c_float), ("rOutside", ctypes.c_float),
                ("k2Inside", ctypes.c_float), ("k2Outside", ctypes.c_float),
                ("shiftX", ctypes.c_float), ("shiftY", ctypes.c_float)]


_INT_FIELDS = ["mode", "nx", "ny", "potNx", "potNy", "slices", "cellDiv", "outputInterval",
               "centerSlices", "nonPeriod", "nonPeriodZ", "potential3D", "fftpotential",
               "bandlimittrans", "tds"]
_FLOAT_FIELDS_A = ["resolutionX", "resolutionY", "sliceThickness", "czOffset", "potOffsetX",
                   "potOffsetY", "potSizeX", "potSizeY", "ax", "by", "c", "atomRadius", "v0",
                   "alpha", "Cs", "C5", "df0", "astigMag", "astigAngle", "Cc", "dE_E",
                   "a33", "a31", "a44", "a42", "a55", "a53", "a51", "a66", "a64", "a62",
                   "phi33", "phi31", "phi44", "phi42", "phi55", "phi53", "phi51", "phi66",
                   "phi64", "phi62"]


class QsParams(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_int) for n in _INT_FIELDS] +
                [(n, ctypes.c_float) for n in _FLOAT_FIELDS_A] +
                [("ismoth", ctypes.c_int), ("gaussFlag", ctypes.c_int),
                 ("gaussScale", ctypes.c_float), ("aAIS", ctypes.c_float),
                 ("scanXStart", ctypes.c_float), ("scanXStop", ctypes.c_float),
                 ("scanYStart", ctypes.c_float), ("scanYStop", ctypes.c_float),
                 ("scanXN", ctypes.c_int), ("scanYN", ctypes.c_int),
                 ("electronScale", ctypes.c_float), ("detectorNum", ctypes.c_int),
                 ("detectors", QsDetector * QS_MAX_DETECTORS), ("equalDivs", ctypes.c_int),
                 ("mulsRepeat1", ctypes.c_int), ("mulsRepeat2", ctypes.c_int)])

    def copy(self):
        out = QsParams()
        ctypes.pointer(out)[0] = self
        return out

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            if name == "detectors":
                d[name] = [(self.detectors[i].rInside, self.detectors[i].rOutside,
                            self.detectors[i].shiftX, self.detectors[i].shiftY)
                           for i in range(self.detectorNum)]
            else:
                d[name] = getattr(self, name)
        return d

    def thickness_count(self):
        """tCount+1 thickness outputs (stem3/stemlib.cpp:2589)."""
        return (self.slices * self.cellDiv) // self.outputInterval + 1


class QsBatch(ctypes.Structure):
    _fields_ = [("npos", ctypes.c_int), ("iPosX", ctypes.POINTER(ctypes.c_int)),
                ("iPosY", ctypes.POINTER(ctypes.c_int)), ("detPosX", ctypes.POINTER(ctypes.c_int)),
                ("detPosY", ctypes.POINTER(ctypes.c_int))]


class QsCtf(ctypes.Structure):
    """qs_ctf: objective-lens transfer of GUI_Matlab/simImageFromWave.m:57-73
    (Angstrom, radians, 1/Angstrom)."""
    _fields_ = [("Cs", ctypes.c_double), ("astig", ctypes.c_double), ("astigPhi", ctypes.c_double),
                ("focalSpread", ctypes.c_double), ("alpha", ctypes.c_double), ("kmax", ctypes.c_double),
                ("edge", ctypes.c_double)]


class QsCbedJob(ctypes.Structure):
    _fields_ = [("params", QsParams), ("atoms", ctypes.c_void_p), ("natom", ctypes.c_int),
                ("diffpat", ctypes.c_void_p)]


class QsCbedReport(ctypes.Structure):
    _fields_ = [("groups", ctypes.c_int), ("rounds", ctypes.c_int), ("streams", ctypes.c_int),
                ("admitted_bytes", ctypes.c_double), ("budget_bytes", ctypes.c_double)]


class QsStats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_longlong), ("row_launches", ctypes.c_longlong),
                ("col_launches", ctypes.c_longlong), ("row_ms", ctypes.c_double), ("col_ms", ctypes.c_double),
                ("row_bytes", ctypes.c_double), ("col_bytes", ctypes.c_double)]


def atoms_to_numpy(atoms):
    a = np.ascontiguousarray(atoms)
    if a.dtype != ATOM_DTYPE:
        raise TypeError("atoms must have dtype ATOM_DTYPE")
    return a
