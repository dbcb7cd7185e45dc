"""Thermal displacements and vacancies drawn the way the reference's
readUnitCell draws them while it replicates the unit cell
(replicateUnitCell, libs/fileio_fftw3.cpp:1188-1310, and
phononDisplacement, :367-659).

The walk: unit-cell sites from the last sorted atom down (a site is an atom
and the atoms before it at the same position), and for each site the cells
(icx, icy, icz) from the last down.  Per site and cell: one uniform draw
picks the occupant when the site holds several atoms or a total occupancy
below 1 (the others become vacancies, Znum 0), then the displacement u of
the chosen atom moves every atom of the site:
  Einstein     u = sqrt(T/300) sqrt(dw / (8 pi^2)) / sqrt(3) (g0, g1, g2),
               three normal draws, turned into fractional coordinates by the
               inverse of the cell matrix;
  phonon file  u = sum over modes l and k-points k of
               q1[l,k] Re(e exp(i 2 pi k.R)) - q2[l,k] Im(e exp(i 2 pi k.R)),
               e the mode's eigenvector component of the chosen atom, R the
               cell index (icx, icy, icz), q1, q2 = w[k,l] times normal draws
               made once per configuration (before the first atom's
               displacement), w the mode's Bose-Einstein amplitude at the
               temperature; u / (a, b, c) in fractional units.
Positions are (x + icx) in float, plus u in double, stored as float.

The draws come from a generator: the reference's own (RefRandom: ran1, the
Park-Miller generator with a Bays-Durham shuffle, and gasdev, the polar
Box-Muller method, as published in Numerical Recipes in C, 2nd ed.,
sec. 7.1-7.2; libs/fileio_fftw3.cpp:2565-2640), which the reference seeds
with its clock (-time(NULL)), or numpy's default_rng.
"""
import math
import struct
from dataclasses import dataclass

import numpy as np

F32 = np.float32

# Park-Miller / Bays-Durham constants of ran1 (libs/fileio_fftw3.cpp:2565-2573)
_IA, _IM, _IQ, _IR, _NTAB = 16807, 2147483647, 127773, 2836, 32
_NDIV = 1 + (_IM - 1) // _NTAB
_AM = 1.0 / _IM
_RNMX = 1.0 - 1.2e-7
# phononDisplacement's constants (libs/fileio_fftw3.cpp:61-70)
PID = 3.14159265358979
THZ_HBAR_KB = 1.90963567802059   # THz hbar / kB
THZ_AMU_HBAR = 0.15745702964189  # A^2 THz amu / hbar
SQRT_2 = 1.4142135               # doCBED's source-offset factor (stem3/stem3.cpp:75)


class RefRandom:
    """The reference's uniform (ran1) and normal (gasdev) deviates.  The
    shuffle table and gasdev's spare deviate are shared by every caller (they
    are function statics); each caller keeps its own seed, passed as a
    one-element list (the reference's `long *idum`).  A seed <= 0 restarts
    the table, as does the first call of all."""

    def __init__(self):
        self.iy = 0
        self.iv = [0] * _NTAB
        self.iset = 0
        self.gset = 0.0

    @staticmethod
    def _next(idum):
        k = idum // _IQ  # idum > 0 here: C's truncating division
        idum = _IA * (idum - k * _IQ) - _IR * k
        return idum + _IM if idum < 0 else idum

    def ran1(self, seed):
        if seed[0] <= 0 or not self.iy:
            seed[0] = 1 if -seed[0] < 1 else -seed[0]
            for j in range(_NTAB + 7, -1, -1):
                seed[0] = self._next(seed[0])
                if j < _NTAB:
                    self.iv[j] = seed[0]
            self.iy = self.iv[0]
        seed[0] = self._next(seed[0])
        j = self.iy // _NDIV
        self.iy = self.iv[j]
        self.iv[j] = seed[0]
        temp = _AM * self.iy
        return _RNMX if temp > _RNMX else temp

    def gasdev(self, seed):
        if seed[0] < 0:
            self.iset = 0
        if self.iset == 0:
            while True:
                v1 = 2.0 * self.ran1(seed) - 1.0
                v2 = 2.0 * self.ran1(seed) - 1.0
                rsq = v1 * v1 + v2 * v2
                if not (rsq >= 1.0 or rsq == 0.0):
                    break
            fac = math.sqrt(-2.0 * math.log(rsq) / rsq)
            self.gset = float(F32(v1 * fac))  # kept in a float
            self.iset = 1
            return v2 * fac
        self.iset = 0
        return self.gset


class _RefDraws:
    """The deviates of one reference process: readUnitCell's vacancy draws
    (replicateUnitCell's own seed, a static starting at -1), its thermal
    draws (phononDisplacement's seed, -clock at its first call) and doCBED's
    source offsets (seed -clock per doCBED call), all on one RefRandom."""

    def __init__(self, clock):
        self.g = RefRandom()
        self.clock = int(clock)
        self.vac = [-1]
        self.cube = [-1]  # tiltBoxed's own seed (libs/fileio_fftw3.cpp:1691)
        self.thermal = None
        self.cbed = None

    def uniform(self):
        return self.g.ran1(self.vac)

    def cube_uniform(self):
        return self.g.ran1(self.cube)

    def normal(self):
        if self.thermal is None:
            self.thermal = [-self.clock]
        return self.g.gasdev(self.thermal)

    def source(self):
        if self.cbed is None:
            self.cbed = [-self.clock]
        return self.g.gasdev(self.cbed)


class _NumpyDraws:
    """Seeded numpy deviates in the same roles (buffered)."""

    def __init__(self, seed):
        self.rng = np.random.default_rng(seed)
        self._n, self._u = [], []

    def uniform(self):
        if not self._u:
            self._u = list(self.rng.random(1024)[::-1])
        return float(self._u.pop())

    def normal(self):
        if not self._n:
            self._n = list(self.rng.standard_normal(4096)[::-1])
        return float(self._n.pop())

    source = normal
    cube_uniform = uniform


@dataclass
class PhononModes:
    """A phonon file (format of libs/fileio_fftw3.cpp:465-483, read at
    :507-529): int32 Nk, int32 Ns, float32 masses[Ns] (amu), then per
    k-point float32 k[3] (reciprocal-lattice units) and per mode float32
    omega (THz, 2 pi included) followed by its eigenvector, 3 Ns complex
    float32 (x, y, z of each atom of the primitive cell)."""
    masses: np.ndarray  # [Ns] float32
    kvecs: np.ndarray   # [Nk, 3] float32
    omega: np.ndarray   # [Nk, 3 Ns] float32
    eig: np.ndarray     # [Nk, 3 Ns (mode), 3 Ns (component), 2] float32

    @property
    def nk(self):
        return self.kvecs.shape[0]

    @property
    def ns(self):
        return self.masses.shape[0]

    def amplitudes(self, temperature):
        """phononDisplacement's per-mode amplitude (:531-552), stored back
        as float: sqrt((n + 1/2) / (2 pi Nk 2 M omega THZ_AMU_HBAR)) with
        n = 1/(exp(THZ_HBAR_KB omega / T) - 1) the Bose-Einstein occupation
        (0 at T = 0), and 0 for omega <= 1e-4."""
        T = float(F32(temperature))
        w = np.zeros_like(self.omega)
        Nk = self.nk
        for ik in range(Nk):
            for idd in range(self.ns):
                for iy in range(3):
                    om = float(self.omega[ik, iy + 3 * idd])
                    if om > 1e-4:
                        n = (1.0 / (math.exp(THZ_HBAR_KB * om / T) - 1)) if T > 0 else 0.0
                        den = 2 * PID * Nk * 2 * float(self.masses[idd]) * om * THZ_AMU_HBAR
                        w[ik, iy + 3 * idd] = F32(math.sqrt((n + 0.5) / den))
        return w


def read_phonon_file(path):
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 8:
        raise ValueError("%s: not a phonon file" % path)
    Nk, Ns = struct.unpack_from("<ii", data, 0)
    if Nk < 1 or Ns < 1:
        raise ValueError("%s: %d k-points, %d atoms" % (path, Nk, Ns))
    m = 3 * Ns
    need = 8 + 4 * Ns + Nk * (12 + m * (4 + 8 * m))
    if len(data) < need:
        raise ValueError("%s: %d bytes, %d k-points of %d atoms need %d" % (path, len(data), Nk, Ns, need))
    off = 8
    masses = np.frombuffer(data, "<f4", Ns, off).astype(F32)
    off += 4 * Ns
    kv = np.zeros((Nk, 3), F32)
    om = np.zeros((Nk, m), F32)
    eig = np.zeros((Nk, m, m, 2), F32)
    for ik in range(Nk):
        kv[ik] = np.frombuffer(data, "<f4", 3, off)
        off += 12
        for iy in range(m):
            om[ik, iy] = np.frombuffer(data, "<f4", 1, off)[0]
            off += 4
            eig[ik, iy] = np.frombuffer(data, "<f4", 2 * m, off).reshape(m, 2)
            off += 8 * m
    return PhononModes(masses, kv, om, eig)


def write_phonon_file(path, modes):
    """The inverse of read_phonon_file."""
    m = 3 * modes.ns
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", modes.nk, modes.ns))
        f.write(np.asarray(modes.masses, "<f4").tobytes())
        for ik in range(modes.nk):
            f.write(np.asarray(modes.kvecs[ik], "<f4").tobytes())
            for iy in range(m):
                f.write(np.asarray([modes.omega[ik, iy]], "<f4").tobytes())
                f.write(np.asarray(modes.eig[ik, iy], "<f4").reshape(-1).tobytes())


def _offset(d, radius):
    gx = d.source()
    gy = d.source()
    return float(F32(radius)) * gx * SQRT_2, float(F32(radius)) * gy * SQRT_2


def source_offset(seed, j, radius):
    """A CBED probe source offset of run j from numpy draws
    (default_rng([seed, j, 2]))."""
    return _offset(_NumpyDraws([seed, j, 2]), radius)


def _inverse_3x3(a):
    """inverse_3x3 (libs/matrixlib.cpp:197-257) of a row-major 3x3 list:
    the adjugate over the determinant, the identity when |det| < 5e-4."""
    det = (a[0] * (a[4] * a[8] - a[7] * a[5]) - a[1] * (a[3] * a[8] - a[6] * a[5])
           + a[2] * (a[3] * a[7] - a[6] * a[4]))
    if abs(det) < float(F32(0.0005)):
        return [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0]
    d = 1.0 / det
    return [(a[4] * a[8] - a[5] * a[7]) * d, -(a[1] * a[8] - a[7] * a[2]) * d, (a[1] * a[5] - a[4] * a[2]) * d,
            -(a[3] * a[8] - a[5] * a[6]) * d, (a[0] * a[8] - a[6] * a[2]) * d, -(a[0] * a[5] - a[3] * a[2]) * d,
            (a[3] * a[7] - a[6] * a[4]) * d, -(a[0] * a[7] - a[6] * a[1]) * d, (a[0] * a[4] - a[1] * a[3]) * d]


class Replicator:
    """readUnitCell's replication of one unit cell, configuration after
    configuration, with vacancies and thermal displacements drawn as
    replicateUnitCell draws them.

    frac: the unit cell's atoms sorted as readUnitCell sorts them, fractional
    (ATOM_DTYPE records); ncell: (ncx, ncy, ncz); H: cell vectors as rows
    (the reference's Mm); abc: the cell lengths the reference holds as
    floats (phonon-mode units); tds: thermal displacements on; modes: a
    PhononModes for the phonon-file model (None: Einstein).
    rng "reference": the reference's generator at clock `clock`; the
    configurations are drawn in order, as one reference process draws them
    (configuration 0 by readFile, then one per further run), interleaved
    with doCBED's source offsets when those are asked for.  rng "numpy":
    configuration j from default_rng(seed + j), in any order."""

    def __init__(self, frac, ncell, H, abc, tds, temperature, modes=None, rng="numpy", seed=0, clock=0):
        if rng not in ("numpy", "reference"):
            raise ValueError("rng must be 'numpy' or 'reference'")
        self.frac = frac
        self.ncell = tuple(int(v) for v in ncell)
        self.tds = bool(tds)
        self.temperature = float(F32(temperature))
        self.modes = modes
        self.rng = rng
        self.seed = int(seed)
        self.abc = tuple(float(F32(v)) for v in abc)
        Ht = np.asarray(H, np.float64).T  # phononDisplacement's Mm: the transpose of MULS's
        self.minv = _inverse_3x3([float(v) for v in Ht.reshape(-1)])
        if modes is not None:
            if modes.ns < len(frac):
                raise ValueError("the phonon file describes %d atoms, the unit cell has %d" % (modes.ns, len(frac)))
            self.w = modes.amplitudes(self.temperature)
        self._ref = _RefDraws(clock) if rng == "reference" else None
        self._next = 0

    def configuration(self, j):
        """Fractional atoms (ATOM_DTYPE, readUnitCell's order, j = (icz +
        icy ncz + icx ncy ncz) ncoord + i) of configuration j."""
        return self._walk(self._draws(j))

    def cube_configuration(self, j, cell, size, tilt, offset):
        """Cartesian atoms of configuration j of a "Cube:" box (tiltBoxed,
        libs/fileio_fftw3.cpp:1661-1940): its site draws and Einstein
        displacements in its order (config.cube)."""
        from . import config
        d = self._draws(j)
        disp = (lambda dw: self._einstein(d, dw)) if self.tds else None
        atoms, _, _, _ = config.cube(cell, size, tilt, offset, draws=d, displace=disp)
        return atoms

    def _draws(self, j):
        if self._ref is not None:
            if j != self._next:
                raise ValueError("the reference generator draws configuration %d next, not %d" % (self._next, j))
            self._next += 1
            return self._ref
        return _NumpyDraws(self.seed + j)

    def _einstein(self, draws, dw):
        """phononDisplacement's Einstein model (:586-607): three normal
        draws scaled by sqrt(T/300) sqrt(dw / (8 pi^2)) / sqrt(3), turned
        into fractional coordinates (u times the inverse cell matrix)."""
        scale = float(F32(math.sqrt(self.temperature / 300.0)))
        wob = scale * math.sqrt(dw * (1.0 / (8 * PID * PID)))
        sq3 = 1.0 / math.sqrt(3.0)
        g = [wob * sq3 * draws.normal() for _ in range(3)]
        M = self.minv
        return tuple(((0.0 + g[0] * M[k]) + g[1] * M[3 + k]) + g[2] * M[6 + k] for k in range(3))

    def source_offset(self, j, radius):
        """doCBED's probe offset of run j (stem3/stem3.cpp:2096-2097):
        radius * g * SQRT_2 for x, then y."""
        if self._ref is None:
            return source_offset(self.seed, j, radius)
        return _offset(self._ref, radius)

    def _sites(self):
        f = self.frac
        sites = []
        i = len(f) - 1
        while i >= 0:
            je, tot = i - 1, 1.0
            if f["Znum"][i] > 0:  # readUnitCell passes handleVacancies = 1
                tot = float(f["occ"][i])
                while je >= 0 and all(abs(F32(f[k][i] - f[k][je])) < 1e-6 for k in ("x", "y", "z")):
                    tot += float(f["occ"][je])
                    je -= 1
            sites.append((i, je, tot))
            i = je
        return sites

    def _walk(self, draws):
        from .abi import ATOM_DTYPE
        f = self.frac
        n = len(f)
        ncx, ncy, ncz = self.ncell
        natom = n * ncx * ncy * ncz
        out = np.zeros(natom, ATOM_DTYPE)
        for c in range(ncx * ncy * ncz):
            out[c * n:(c + 1) * n] = f
        occ = [float(v) for v in f["occ"]]
        einstein = self.tds and self.modes is None
        phonon = self.tds and self.modes is not None
        rec_src, rec_dst, rec_cell, rec_u = [], [], [], []
        ph_rec = []  # phonon mode: (record index, chosen atom, cell)
        q1 = q2 = None
        for i, je, tot in self._sites():
            members = list(range(i, je, -1))
            for icx in range(ncx - 1, -1, -1):
                for icy in range(ncy - 1, -1, -1):
                    for icz in range(ncz - 1, -1, -1):
                        jcell = (icz + icy * ncz + icx * ncy * ncz) * n
                        jch = i
                        if tot < 1 or je < i - 1:
                            ch = draws.uniform()
                            if tot >= 1.0:
                                ch = tot * ch
                            last = 0.0
                            for i2 in members:
                                if ch < last or ch >= last + occ[i2]:
                                    out["Znum"][jcell + i2] = 0
                                else:
                                    jch = i2
                                last += occ[i2]
                        u = (0.0, 0.0, 0.0)
                        if einstein:
                            u = self._einstein(draws, float(f["dw"][jch]))
                        elif phonon:
                            if jcell + i == natom - 1:
                                q1, q2 = self._draw_modes(draws)
                            ph_rec.append((len(rec_u), jch, icx, icy, icz))
                        rec_u.append(u)
                        rec_src.append(members)
                        rec_dst.append(jcell)
                        rec_cell.append((icx, icy, icz))
        U = np.asarray(rec_u, np.float64).reshape(-1, 3)
        if ph_rec:
            U[[r[0] for r in ph_rec]] = self._phonon_sum(ph_rec, q1, q2)
        # positions: (x + icx) in float, + u in double, stored as float
        src = np.concatenate([np.asarray(m, np.int64) for m in rec_src])
        cnt = np.asarray([len(m) for m in rec_src])
        dst = np.repeat(np.asarray(rec_dst, np.int64), cnt) + src
        cell = np.repeat(np.asarray(rec_cell, np.int64), cnt, axis=0)
        Ud = np.repeat(U, cnt, axis=0)
        for k, key in enumerate(("x", "y", "z")):
            base = (f[key][src].astype(F32) + cell[:, k].astype(F32)).astype(F32)
            out[key][dst] = (base.astype(np.float64) + Ud[:, k]).astype(F32)
        return out

    def _draw_modes(self, draws):
        m, Nk = 3 * self.modes.ns, self.modes.nk
        q1 = np.zeros((m, Nk))
        q2 = np.zeros((m, Nk))
        for lam in range(m):
            for ik in range(Nk):
                q1[lam, ik] = float(self.w[ik, lam]) * draws.normal()
                q2[lam, ik] = float(self.w[ik, lam]) * draws.normal()
        return q1, q2

    def _phonon_sum(self, recs, q1, q2):
        """phononDisplacement's mode sum (libs/fileio_fftw3.cpp:609-640) for
        every (chosen atom, cell) record, in its order of terms; the phase
        2 pi (icx kx + icy ky + icz kz) with the sum in float."""
        md = self.modes
        m, Nk = 3 * md.ns, md.nk
        cells = sorted({r[2:] for r in recs})
        cidx = {c: k for k, c in enumerate(cells)}
        cosT = np.zeros((len(cells), Nk))
        sinT = np.zeros((len(cells), Nk))
        for k, (icx, icy, icz) in enumerate(cells):
            for ik in range(Nk):
                kx, ky, kz = md.kvecs[ik]
                t = F32(F32(F32(F32(icx) * kx) + F32(F32(icy) * ky)) + F32(F32(icz) * kz))
                kR = 2 * PID * float(t)
                cosT[k, ik], sinT[k, ik] = math.cos(kR), math.sin(kR)
        ci = np.asarray([cidx[r[2:]] for r in recs])
        at = np.asarray([r[1] for r in recs])
        u = np.zeros((len(recs), 3))
        for lam in range(m):
            for ik in range(Nk):
                kRr, kRi = cosT[ci, ik], sinT[ci, ik]
                for c in range(3):
                    er = md.eig[ik, lam, c + 3 * at, 0].astype(np.float64)
                    ei = md.eig[ik, lam, c + 3 * at, 1].astype(np.float64)
                    u[:, c] += q1[lam, ik] * (er * kRr - ei * kRi) - q2[lam, ik] * (er * kRi + ei * kRr)
        return u / np.asarray(self.abc)
