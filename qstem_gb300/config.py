"""Host front end: stem3 .qsc parameters and .cfg atoms -> qs_params / atoms.

The derived quantities follow stem3's readFile (stem3/stem3.cpp:612-1559)
with the reference's float (MULS float_tt) arithmetic reproduced through
numpy float32, and the atom list follows readUnitCell/replicateUnitCell
(libs/fileio_fftw3.cpp:1313-1657, :1188-1306) for orthogonal unit cells
without tilt, thermal displacement or partial occupancy.  `write_qsc` /
`write_cfg` produce input files the reference's own stem3 reads, so that the
same run can be driven through both.
"""
import math

import numpy as np

from . import abi

F32 = np.float32
ELECTRON_CHARGE = 1.6021773e-19
MILLISEC_PICOAMP = 1e-3 * (1e-12 / ELECTRON_CHARGE)  # libs/stemtypes_fftw3.h:47-49
RAD2DEG = 57.2958                                   # stem3/stem3.cpp:73

ELEMENTS = {"H": 1, "He": 2, "Li": 3, "Be": 4, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9, "Ne": 10,
            "Na": 11, "Mg": 12, "Al": 13, "Si": 14, "P": 15, "S": 16, "Cl": 17, "Ar": 18,
            "K": 19, "Ca": 20, "Sc": 21, "Ti": 22, "V": 23, "Cr": 24, "Mn": 25, "Fe": 26,
            "Co": 27, "Ni": 28, "Cu": 29, "Zn": 30, "Ga": 31, "Ge": 32, "As": 33, "Se": 34,
            "Br": 35, "Kr": 36, "Rb": 37, "Sr": 38, "Y": 39, "Zr": 40, "Nb": 41, "Mo": 42,
            "Tc": 43, "Ru": 44, "Rh": 45, "Pd": 46, "Ag": 47, "Cd": 48, "In": 49, "Sn": 50,
            "Sb": 51, "Te": 52, "I": 53, "Xe": 54, "Cs": 55, "Ba": 56, "La": 57, "Ce": 58,
            "Pr": 59, "Nd": 60, "Pm": 61, "Sm": 62, "Eu": 63, "Gd": 64, "Tb": 65, "Dy": 66,
            "Ho": 67, "Er": 68, "Tm": 69, "Yb": 70, "Lu": 71, "Hf": 72, "Ta": 73, "W": 74,
            "Re": 75, "Os": 76, "Ir": 77, "Pt": 78, "Au": 79, "Hg": 80, "Tl": 81, "Pb": 82,
            "Bi": 83, "Po": 84, "At": 85, "Rn": 86, "Fr": 87, "Ra": 88, "Ac": 89, "Th": 90,
            "Pa": 91, "U": 92}
SYMBOL = {v: k for k, v in ELEMENTS.items()}
MASS = {8: 16.0, 14: 28.0855, 22: 47.867, 38: 87.62, 79: 196.97}


def wavelength(kev):
    """Electron wavelength in A (stem3/stemutil.cpp:714-725)."""
    return 12.3984244 / math.sqrt(kev * (2 * 510.99906 + kev))


# --------------------------------------------------------------- unit cells
class UnitCell:
    """Unit cell: fractional atoms (Z, fx, fy, fz, dw, occ, q) and the cell
    vectors as the rows of H (A); a, b, c are their lengths.  Orthogonal
    cells are built from a, b, c alone."""

    def __init__(self, a, b, c, atoms, H=None):
        self.a, self.b, self.c = float(a), float(b), float(c)
        self.H = np.diag([self.a, self.b, self.c]) if H is None else np.asarray(H, dtype=np.float64)
        self.atoms = [tuple(t) for t in atoms]

    @property
    def orthogonal(self):
        return bool(np.all(self.H == np.diag(np.diag(self.H))))


def srtio3_cell(dw=0.0):
    a = 3.905
    return UnitCell(a, a, a, [(38, 0, 0, 0, dw, 1, 0), (22, .5, .5, .5, dw, 1, 0),
                              (8, 0, .5, .5, dw, 1, 0), (8, .5, 0, .5, dw, 1, 0),
                              (8, .5, .5, 0, dw, 1, 0)])


def fcc_cell(Z, a, dw=0.0):
    return UnitCell(a, a, a, [(Z, 0, 0, 0, dw, 1, 0), (Z, .5, .5, 0, dw, 1, 0),
                              (Z, .5, 0, .5, dw, 1, 0), (Z, 0, .5, .5, dw, 1, 0)])


def diamond_cell(Z=14, a=5.431, dw=0.0):
    """Cubic diamond (Si by default) along [001]: 8 atoms."""
    base = [(0, 0, 0), (.5, .5, 0), (.5, 0, .5), (0, .5, .5)]
    frac = base + [(x + .25, y + .25, z + .25) for x, y, z in base]
    return UnitCell(a, a, a, [(Z, fx, fy, fz, dw, 1, 0) for fx, fy, fz in frac])


def si110_cell(dw=0.0):
    """Si diamond (a = 5.431 A) viewed along [110]: orthorhombic cell
    a/sqrt2 x a x a/sqrt2 with 4 atoms."""
    a = 5.431
    ax, by = a / math.sqrt(2), a
    frac = [(0.0, 0.0, 0.0), (0.5, 0.5, 0.5), (0.0, 0.25, 0.5), (0.5, 0.75, 0.0)]
    return UnitCell(ax, by, ax, [(14, fx, fy, fz, dw, 1, 0) for fx, fy, fz in frac])


def write_cfg(cell, path):
    """AtomEye .cfg with dw, occupancy and charge columns (the format
    readCFGCellParams/readNextCFGAtom read, libs/fileio_fftw3.cpp:721-989)."""
    lines = ["Number of particles = %d" % len(cell.atoms), "A = 1.0 Angstrom (basic length-scale)"]
    H = [[cell.a, 0, 0], [0, cell.b, 0], [0, 0, cell.c]]
    for i in range(3):
        for j in range(3):
            lines.append("H0(%d,%d) = %r A" % (i + 1, j + 1, float(H[i][j])))
    lines += [".NO_VELOCITY.", "entry_count = 6"]
    last = None
    for Z, fx, fy, fz, dw, occ, q in cell.atoms:
        if Z != last:
            lines += ["%g" % MASS.get(Z, 2.0 * Z), SYMBOL[Z]]
            last = Z
        lines.append("%r %r %r %r %r %r" % (float(fx), float(fy), float(fz), float(dw), float(occ), float(q)))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _cmp_zyx_key(row):
    return (row[3], row[2], row[1])


def cell_vectors(ax, by, c, alpha, beta, gamma):
    """makeCellVectMuls (libs/matrixlib.cpp:722-747): cell vectors (rows)
    from lengths and angles (degrees) held as floats, as the reference
    builds them -- including its b vector of (b cos(gamma), b cos(gamma), 0)
    for non-orthogonal cells."""
    ax, by, c, al, be, ga = (float(F32(v)) for v in (ax, by, c, alpha, beta, gamma))
    if al == 90 and be == 90 and ga == 90:
        return np.diag([ax, by, c])
    d = 1.7453292519943e-2  # PI180
    ca, cb, cg, sg = math.cos(al * d), math.cos(be * d), math.cos(ga * d), math.sin(ga * d)
    return np.array([[ax, 0.0, 0.0],
                     [by * cg, by * cg, 0.0],
                     [c * cb, c * (ca - cb * cg) / sg, c * (math.sqrt(1 - ca * ca - cb * cb + 2 * ca * cb * cg) / sg)]])


def sorted_fractional(cell):
    """The unit cell's atoms as records in fractional coordinates, sorted by
    (z, y, x) as readUnitCell sorts them (libs/fileio_fftw3.cpp:1497-1500).
    readUnitCell stores the file's atoms last to first (:1421) and sorts
    with the C library's qsort, whose merge sort keeps atoms at equal
    positions in that stored order."""
    n = len(cell.atoms)
    frac = np.zeros(n, dtype=abi.ATOM_DTYPE)
    for i, (Z, fx, fy, fz, dw, occ, q) in enumerate(cell.atoms):
        frac[n - 1 - i] = (fz, fy, fx, dw, occ, q, Z)
    order = sorted(range(n), key=lambda i: (frac["z"][i], frac["y"][i], frac["x"][i]))
    return frac[order]


def rotation(phi_x, phi_y, phi_z):
    """rotateVect's matrix (libs/matrixlib.cpp:599-635): rotations by
    phi_x, phi_y, phi_z (rad) about x, then y, then z, in double with the
    same products and sums."""
    cx, sx = math.cos(phi_x), math.sin(phi_x)
    cy, sy = math.cos(phi_y), math.sin(phi_y)
    cz, sz = math.cos(phi_z), math.sin(phi_z)
    return np.array([[cz * cy, cz * sy * sx - sz * cx, cz * sy * cx + sz * sx],
                     [sz * cy, sz * sy * sx + cz * cx, sz * sy * cx - cz * sx],
                     [-sy, cy * sx, cy * cx]])


def _mat_vec(M, u0, u1, u2):
    """M (3x3) times the vectors (u0, u1, u2), each row summed left to right."""
    return [(M[i, 0] * u0 + M[i, 1] * u1) + M[i, 2] * u2 for i in range(3)]


def supercell(cell, ncx, ncy, ncz, tilt=(0.0, 0.0, 0.0), offset=(0.0, 0.0), replicated=None):
    """readUnitCell's NCELL mode (libs/fileio_fftw3.cpp:1512-1645): the unit
    cell replicated ncx x ncy x ncz times in fractional coordinates (atom
    j = (icz + icy*ncz + icx*ncy*ncz)*ncoord + i), converted to Cartesian by
    the cell vectors, rotated by the crystal tilt about the centre of the
    super-cell, shifted so that the bounding box of the (rotated) super-cell
    starts at 0, then offset by (xOffset, yOffset).  Double arithmetic with
    float32 storage where the reference stores floats.
    replicated: the replicated fractional atoms in that order, when drawn
    elsewhere (thermal.Replicator: vacancies and thermal displacements).
    Returns (atoms[ATOM_DTYPE], ax, by, c): the bounding box size, float32."""
    if replicated is not None:
        out = np.array(replicated, dtype=abi.ATOM_DTYPE)
    else:
        frac = sorted_fractional(cell)
        n = len(frac)
        out = np.zeros(n * ncx * ncy * ncz, dtype=abi.ATOM_DTYPE)
        for icx in range(ncx):
            for icy in range(ncy):
                for icz in range(ncz):
                    j0 = (icz + icy * ncz + icx * ncy * ncz) * n
                    blk = out[j0:j0 + n]
                    blk[:] = frac
                    blk["x"] = (frac["x"].astype(np.float64) + icx).astype(F32)
                    blk["y"] = (frac["y"].astype(np.float64) + icy).astype(F32)
                    blk["z"] = (frac["z"].astype(np.float64) + icz).astype(F32)
    # Cartesian: x_j = sum_k Mm[k][j] * frac_k with Mm's rows the cell vectors
    Mt = cell.H.T
    fx, fy, fz = (out[k].astype(np.float64) for k in ("x", "y", "z"))
    cart = _mat_vec(Mt, fx, fy, fz)
    for k, v in zip(("x", "y", "z"), cart):
        out[k] = v.astype(F32)
    bc = (ncx / 2.0, ncy / 2.0, ncz / 2.0)
    centre = _mat_vec(Mt, *bc)
    R = rotation(*tilt)
    lo, hi = None, None
    for icx in (0, ncx):
        for icy in (0, ncy):
            for icz in (0, ncz):
                u = _mat_vec(Mt, icx - bc[0], icy - bc[1], icz - bc[2])
                u = _mat_vec(R, *u)
                c = [u[k] + centre[k] for k in range(3)]
                lo = list(c) if lo is None else [min(lo[k], c[k]) for k in range(3)]
                hi = list(c) if hi is None else [max(hi[k], c[k]) for k in range(3)]
    if any(t != 0 for t in tilt):
        u = [out[k].astype(np.float64) - centre[i] for i, k in enumerate(("x", "y", "z"))]
        u = _mat_vec(R, *u)
        for i, k in enumerate(("x", "y", "z")):
            out[k] = (u[i] + centre[i]).astype(F32)
    for i, k in enumerate(("x", "y", "z")):
        out[k] = (out[k].astype(np.float64) - lo[i]).astype(F32)
    if offset[0] != 0 or offset[1] != 0:
        out["x"] = (out["x"] + F32(offset[0])).astype(F32)
        out["y"] = (out["y"] + F32(offset[1])).astype(F32)
    return out, F32(hi[0] - lo[0]), F32(hi[1] - lo[1]), F32(hi[2] - lo[2])


def cube(cell, size, tilt=(0.0, 0.0, 0.0), offset=(0.0, 0.0), seed=None, draws=None, displace=None):
    """tiltBoxed (libs/fileio_fftw3.cpp:1661-1940): the atoms of the crystal,
    rotated by the crystal tilt about the origin and shifted by (xOffset,
    yOffset), that fall inside the box [0, size] (the "Cube:" sizes).  Unit
    cells are walked over the range that covers the box's corners; atoms are
    listed per unit-cell atom (sorted as readUnitCell sorts them), then by
    cell (x, y, z).  Unit-cell atoms at equal positions are one site: one of
    them is kept per cell, chosen by a uniform draw over their occupancies
    (numpy.random.default_rng(seed); the reference draws with ran1); the
    first stays when the draw falls past a total occupancy below 1, as in
    the reference.  draws / displace (thermal.Replicator): the site draws
    from draws.cube_uniform() instead, and each (site, cell) moved by the
    fractional displacement displace(dw) (drawn for every cell of the walk,
    inside the box or not, and once more after it, as tiltBoxed calls
    phononDisplacement; the box test uses the undisplaced position).
    Returns (atoms[ATOM_DTYPE], ax, by, c) = the box."""
    frac = sorted_fractional(cell)
    n = len(frac)
    cx, cy, cz = (F32(v) for v in size)
    dx, dy, dz = float(F32(offset[0])), float(F32(offset[1])), 0.0
    # rotateMatrix(Mm) with Mm the transposed cell matrix: Mrot * Mm, sums from 0
    R = rotation(*tilt)
    Mt = cell.H.T
    M = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            acc = 0.0
            for k in range(3):
                acc += R[i, k] * Mt[k, j]
            M[i, j] = acc
    Minv = np.linalg.inv(M)
    b = Minv @ np.zeros(3)
    nmin = [int(math.floor(b[0] - dx)), int(math.floor(b[1] - dy)), int(math.floor(b[2] - dz))]
    nmax = list(nmin)
    for ix in (0, 1):
        for iy in (0, 1):
            for iz in (0, 1):
                b = Minv @ np.array([ix * float(cx) - dx, iy * float(cy) - dy, iz * float(cz) - dz])
                for k in range(3):
                    nmin[k] = min(nmin[k], int(math.floor(b[k])))
                    nmax[k] = max(nmax[k], int(math.ceil(b[k])))
    rng = np.random.default_rng(seed)
    cells = np.array([(i, j, k) for i in range(nmin[0], nmax[0] + 1) for j in range(nmin[1], nmax[1] + 1)
                      for k in range(nmin[2], nmax[2] + 1)], dtype=np.float64)
    kept = []
    i = 0
    while i < n:
        j = i + 1
        occ = float(frac["occ"][i])
        if frac["Znum"][i] > 0:
            while j < n and all(abs(float(frac[k][j]) - float(frac[k][i])) < 1e-6 for k in ("x", "y", "z")):
                occ += float(frac["occ"][j])
                j += 1
        else:
            occ = 1.0
        # ix + newAtom.x: an int plus a float, added in float
        pos = [(cells[:, k].astype(F32) + frac[c][i]).astype(np.float64) for k, c in enumerate(("x", "y", "z"))]
        cart = _mat_vec(M, *pos)
        x, y, z = cart[0] + dx, cart[1] + dy, cart[2] + dz
        inside = (x >= 0) & (x <= float(cx)) & (y >= 0) & (y <= float(cy)) & (z >= 0) & (z <= float(cz))
        if draws is not None or displace is not None:
            for c in range(len(cells)):
                jch = i
                if occ < 1.0 or j > i + 1:
                    ch = draws.cube_uniform() if draws is not None else rng.random()
                    if occ >= 1.0:
                        ch = occ * ch
                    last = 0.0
                    for m in range(i, j):
                        o = float(frac["occ"][m])
                        if last <= ch < last + o:
                            jch = m
                        last += o
                u = displace(float(frac["dw"][jch])) if displace is not None else (0.0, 0.0, 0.0)
                if inside[c]:
                    b = _mat_vec(M, *(float(pos[k][c]) + u[k] for k in range(3)))
                    rec = frac[jch].copy()
                    rec["x"], rec["y"], rec["z"] = F32(b[0] + dx), F32(b[1] + dy), F32(b[2] + dz)
                    kept.append(rec)
            last_site = i
            i = j
            continue
        choice = np.full(len(cells), i)
        if occ < 1.0 or j > i + 1:
            u = rng.random(len(cells)) * (1.0 if occ < 1.0 else occ)
            last = 0.0
            for m in range(i, j):
                o = float(frac["occ"][m])
                choice[(u >= last) & (u < last + o)] = m
                last += o
        for c in np.nonzero(inside)[0]:
            rec = frac[choice[c]].copy()
            rec["x"], rec["y"], rec["z"] = F32(x[c]), F32(y[c]), F32(z[c])
            kept.append(rec)
        i = j
    if displace is not None and n:
        displace(float(frac["dw"][last_site]))  # tiltBoxed's closing phononDisplacement call (:1935)
    atoms = np.array(kept, dtype=abi.ATOM_DTYPE) if kept else np.zeros(0, abi.ATOM_DTYPE)
    return atoms, cx, cy, cz


def replicate(cell, ncx, ncy, ncz):
    """Cartesian atoms of an ncx x ncy x ncz super-cell without tilt or
    offset (supercell).  Returns (atoms[ATOM_DTYPE], ax, by, c) with the
    super-cell size as float32."""
    return supercell(cell, ncx, ncy, ncz)


# ------------------------------------------------------------------ params
def make_params(*, mode=abi.QS_MODE_STEM, nx, ny=None, resolutionX, resolutionY=None, v0,
                slices, sliceThickness, ax, by, c, scan=None, detectors=(), alpha=20.0,
                Cs_mm=0.0, C5_mm=0.0, defocus_nm=0.0, Cc_mm=0.0, dE_E=0.0,
                astig_nm=0.0, astig_deg=0.0, outputInterval=None, czOffset=0.0,
                centerSlices=False, periodicXY=False, periodicZ=False, bandlimit=False,
                atomRadius=5.0, smooth=True, gaussian=None, aAIS=0.0, beamCurrent=1.0,
                dwellTime=1.6021773e-4, tds=False, cellDiv=1, nCellZ=None, potential3D=True):
    """qs_params as stem3's readFile would fill them from the corresponding
    .qsc keys (units as in the .qsc: mm, nm, mrad, deg).
    scan = (x_start, x_stop, x_pixels, y_start, y_stop, y_pixels) in A.
    cellDiv, nCellZ: "NCELLZ: nCellZ/cellDiv" (slabs along z); nCellZ is only
    needed for readFile's equalDivs test."""
    ny = nx if ny is None else ny
    resolutionY = resolutionX if resolutionY is None else resolutionY
    p = abi.QsParams()
    p.mode = mode
    p.nx, p.ny = nx, ny
    p.resolutionX, p.resolutionY = F32(resolutionX), F32(resolutionY)
    p.v0 = F32(v0)
    p.slices = slices + (1 if centerSlices else 0)
    p.sliceThickness = F32(sliceThickness)
    p.centerSlices = int(bool(centerSlices))
    p.cellDiv = max(1, int(cellDiv))
    # stem3/stem3.cpp:930-931, in the reference's float fields
    ncz = p.cellDiv if nCellZ is None else int(nCellZ)
    p.equalDivs = int((not tds) and ncz % p.cellDiv == 0 and
                      abs(float(F32(F32(p.slices) * F32(sliceThickness)) - F32(F32(c) / F32(p.cellDiv)))) < 1e-5)
    p.outputInterval = p.slices if (outputInterval is None or outputInterval < 1) else outputInterval
    p.mulsRepeat1 = p.mulsRepeat2 = 1  # "sequence: 1 1"
    p.czOffset = F32(czOffset)
    p.ax, p.by, p.c = F32(ax), F32(by), F32(c)
    p.nonPeriod = 0 if periodicXY else 1
    p.nonPeriodZ = 0 if periodicZ else 1
    p.bandlimittrans = int(bool(bandlimit))
    p.fftpotential = 1
    p.potential3D = int(bool(potential3D))
    p.tds = int(bool(tds))
    p.atomRadius = F32(atomRadius)
    # scan window and potential array (stem3/stem3.cpp:1054-1068, :1436-1455)
    if mode == abi.QS_MODE_STEM:
        x0, x1, xn, y0, y1, yn = scan
        p.scanXStart, p.scanXStop, p.scanXN = F32(x0), F32(x1), max(1, int(xn))
        p.scanYStart, p.scanYStop, p.scanYN = F32(y0), F32(y1), max(1, int(yn))
    else:
        if scan is None:
            x0, y0 = float(F32(ax)) / 2.0, float(F32(by)) / 2.0
        else:
            x0, y0 = scan[0], scan[3] if len(scan) > 3 else scan[1]
        p.scanXStart = p.scanXStop = F32(x0)
        p.scanYStart = p.scanYStop = F32(y0)
        p.scanXN = p.scanYN = 1
    if mode in (abi.QS_MODE_STEM, abi.QS_MODE_CBED):
        p.potOffsetX = F32(float(p.scanXStart) - 0.5 * nx * float(p.resolutionX))
        p.potOffsetY = F32(float(p.scanYStart) - 0.5 * ny * float(p.resolutionY))
        pnx = int(F32(F32(p.scanXStop) - F32(p.scanXStart)) / F32(p.resolutionX))
        pny = int(F32(F32(p.scanYStop) - F32(p.scanYStart)) / F32(p.resolutionY))
        p.scanXStop = F32(F32(p.scanXStart) + F32(p.resolutionX) * F32(pnx))
        p.scanYStop = F32(F32(p.scanYStart) + F32(p.resolutionY) * F32(pny))
        p.potNx, p.potNy = pnx + nx, pny + ny
        p.potSizeX = F32(F32(p.potNx) * F32(p.resolutionX))
        p.potSizeY = F32(F32(p.potNy) * F32(p.resolutionY))
    else:
        p.potNx, p.potNy = nx, ny
        p.potSizeX = F32(F32(nx) * F32(p.resolutionX))
        p.potSizeY = F32(F32(ny) * F32(p.resolutionY))
        p.potOffsetX = F32(float(p.scanXStart) - 0.5 * float(p.potSizeX))
        p.potOffsetY = F32(float(p.scanYStart) - 0.5 * float(p.potSizeY))
    # optics (stem3/stem3.cpp:1128-1275)
    p.Cc = F32(1e7 * Cc_mm)
    p.dE_E = F32(dE_E)
    p.Cs = F32(F32(Cs_mm) * 1.0e7)
    p.C5 = F32(F32(C5_mm) * 1.0e7)
    if defocus_nm is None or (isinstance(defocus_nm, str) and defocus_nm.lower().startswith("s")):
        p.df0 = F32(-math.sqrt(1.5 * float(p.Cs) * wavelength(float(p.v0))))
    else:
        p.df0 = F32(10.0 * float(F32(defocus_nm)))
    p.astigMag = F32(10.0 * float(F32(astig_nm)))
    p.astigAngle = F32(float(F32(astig_deg)) * 3.1415926535897 / 180.0)
    p.alpha = F32(alpha)
    p.aAIS = F32(aAIS)
    p.electronScale = F32(float(F32(F32(beamCurrent) * F32(dwellTime))) * MILLISEC_PICOAMP)
    p.ismoth = int(bool(smooth))
    p.gaussFlag = 0 if gaussian is None else 1
    p.gaussScale = F32(0.05 if gaussian is None else gaussian)
    # detectors (stem3/stem3.cpp:1316-1355)
    dets = list(detectors)
    if len(dets) > abi.QS_MAX_DETECTORS:
        raise ValueError("at most %d detectors" % abi.QS_MAX_DETECTORS)
    p.detectorNum = len(dets) if mode == abi.QS_MODE_STEM else 0
    wl = wavelength(float(p.v0))
    for i, d in enumerate(dets[:p.detectorNum]):
        rin, rout = d[0], d[1]
        sx = d[3] if len(d) > 3 else 0.0
        sy = d[4] if len(d) > 4 else 0.0
        det = p.detectors[i]
        det.rInside, det.rOutside = F32(rin), F32(rout)
        ki = F32(math.sin(float(F32(rin)) * 0.001) / wl)
        ko = F32(math.sin(float(F32(rout)) * 0.001) / wl)
        det.k2Inside, det.k2Outside = F32(ki * ki), F32(ko * ko)
        det.shiftX, det.shiftY = F32(sx), F32(sy)
    return p


def scan_offsets(p):
    """(iPosX, iPosY) of every raster position p = ix*scanYN + iy
    (stem3/stem3.cpp:2860-2871)."""
    ix = np.arange(p.scanXN, dtype=np.int64)
    iy = np.arange(p.scanYN, dtype=np.int64)
    fx = (ix.astype(F32) * F32(F32(p.scanXStop) - F32(p.scanXStart))) / (F32(p.scanXN) * F32(p.resolutionX))
    fy = (iy.astype(F32) * F32(F32(p.scanYStop) - F32(p.scanYStart))) / (F32(p.scanYN) * F32(p.resolutionY))
    px = np.minimum(fx.astype(F32).astype(np.int64), p.potNx - p.nx)
    py = np.minimum(fy.astype(F32).astype(np.int64), p.potNy - p.ny)
    PX = np.repeat(px, p.scanYN)
    PY = np.tile(py, p.scanXN)
    DX = np.repeat(ix, p.scanYN)
    DY = np.tile(iy, p.scanXN)
    return (PX.astype(np.int32), PY.astype(np.int32), DX.astype(np.int32), DY.astype(np.int32))


def write_qsc(path, *, cfg_file, ncell, nx, resolutionX, v0, slices, sliceThickness, scan=None,
              detectors=(), alpha=20.0, Cs_mm=0.0, C5_mm=0.0, defocus_nm=0.0, outputInterval=None,
              mode="STEM", bandlimit=False, periodicXY=False, periodicZ=False, folder="out",
              saveLevel=0, smooth=True, czOffset=0.0, atomRadius=5.0, centerSlices=False, cellDiv=1,
              sequence=(1, 1), potential3D=True, custom_sf=None):
    """A stem3 input file for the same run make_params describes
    (sequence: the stacking sequence m1 m2; custom_sf: (k values, {Z: f
    values}) for "Structure Factors: custom", the table readSFactLUT reads,
    stem3/stem3.cpp:555-600)."""
    yn = lambda b: "yes" if b else "no"
    L = ["mode: %s" % mode, "print level: 1", "save level: %d" % saveLevel,
         "filename: %s" % cfg_file, "resolutionX: %r" % float(resolutionX),
         "resolutionY: %r" % float(resolutionX), "NCELLX: %d" % ncell[0], "NCELLY: %d" % ncell[1],
         ("NCELLZ: %d/%d" % (ncell[2], cellDiv) if cellDiv > 1 else "NCELLZ: %d" % ncell[2]),
         "v0: %r" % float(v0), "tds: no",
         "slice-thickness: %r" % float(sliceThickness), "slices: %d" % slices,
         "center slices: %s" % yn(centerSlices)]
    if outputInterval:
        L.append("slices between outputs: %d" % outputInterval)
    L += ["zOffset: %r" % float(czOffset), "periodicXY: %s" % yn(periodicXY),
          "periodicZ: %s" % yn(periodicZ)]
    if scan is not None:
        if mode == "STEM":
            L += ["scan_x_start: %r" % float(scan[0]), "scan_x_stop: %r" % float(scan[1]),
                  "scan_x_pixels: %d" % scan[2], "scan_y_start: %r" % float(scan[3]),
                  "scan_y_stop: %r" % float(scan[4]), "scan_y_pixels: %d" % scan[5]]
        else:
            L += ["scan_x_start: %r" % float(scan[0]), "scan_y_start: %r" % float(scan[3])]
    for d in detectors:
        sx = d[3] if len(d) > 3 else 0.0
        sy = d[4] if len(d) > 4 else 0.0
        L.append("detector: %r %r %s %r %r" % (float(d[0]), float(d[1]), d[2], float(sx), float(sy)))
    L += ["nx: %d" % nx, "ny: %d" % nx, "Cs: %r" % float(Cs_mm), "C5: %r" % float(C5_mm),
          "Cc: 0", "alpha: %r" % float(alpha), "defocus: %r" % float(defocus_nm),
          "beam current: 1", "dwell time: 1.6021773e-4", "smooth: %s" % yn(smooth),
          "gaussian: no", "potential3D: %s" % yn(potential3D), "atom radius: %r" % float(atomRadius),
          "bandlimit f_trans: %s" % yn(bandlimit), "one time integration: yes",
          'Folder: "%s"' % folder, "Runs for averaging: 1"]
    if custom_sf is None:
        L.append("Structure Factors: WK")
    else:
        kv, table = custom_sf
        L += ["Structure Factors: custom", "Nk: %d" % len(kv), "k: " + " ".join("%.6g" % v for v in kv)]
        for Z, f in table.items():
            L.append("%s: " % SYMBOL[Z] + " ".join("%.6g" % v for v in f))
    L.append("sequence: %d %d" % tuple(sequence))
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")
