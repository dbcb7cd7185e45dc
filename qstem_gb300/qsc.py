"""Read unmodified stem3 inputs: a .qsc parameter file and its unit cell
(AtomEye .cfg, .dat or .cssr), into qs_params and the atom list.

The parameter file is read the way the reference's readFile does
(stem3/stem3.cpp:600-1460): every key is looked up with readparam's rule
(libs/readparams.cpp:173-212) -- search forward from where the previous
look-up stopped, wrap to the start once, cut each line at '%', match the key
anywhere in the line -- in readFile's order, so that a key such as "slices:"
resolves to the same line it does there (it is also a substring of
"center slices:").  The derived fields (potential grid, offsets, k^2 of the
detectors, ...) then come from config.make_params, which follows the rest of
readFile.  The unit cell is read as readCFGCellParams / readNextCFGAtom
(and the .dat / .cssr readers) read it (libs/fileio_fftw3.cpp:664-1051) and
built as readUnitCell builds it: NCELL replication with crystal tilt, or a
"Cube:" box cut from the tilted crystal (config.supercell, config.cube).

Thermal displacements (tds) follow the Einstein model or a phonon file
("phonon-File:"), vacancies the occupancies; their random draws come from
numpy's generator or, on request, from the reference's own clock-seeded
generator in the reference's order (qstem_gb300.thermal).

"Structure Factors: custom" tables (Nk, k and one array per element) are
read as readSFactLUT reads them; CBED runs build their slices from them
(qs_slices_build_custom), STEM and TEM runs keep the parameterised
potential, as doSTEM and doTEM do.

Inputs that need parts of the reference outside this library, or that the
reference cannot run, are refused with NotImplementedError: the 2-D
potential (potential3D: no) on a non-periodic potential array (the
reference reads its table outside the array there), more than one
stacking-sequence line, a phonon file with a "Cube:" box (the reference
exits there), custom scattering factors on a divided cell or with fewer
than four k values in CBED mode, and modes other than STEM, CBED and TEM.
"""
import math
import os
import re
from dataclasses import dataclass, field

import numpy as np

from . import abi, config

F32 = np.float32

# element symbols (index = Z), as getZNumber resolves them
_SYMBOLS = ["", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl",
            "Ar", "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se",
            "Br", "Kr", "Rb", "Sr", "Y", "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In", "Sn", "Sb",
            "Te", "I", "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho", "Er",
            "Tm", "Yb", "Lu", "Hf", "Ta", "W", "Re", "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi", "Po", "At",
            "Rn", "Fr", "Ra", "Ac", "Th", "Pa", "U", "Np", "Pu", "Am", "Cm", "Bk", "Cf", "Es", "Fm", "Md", "No"]
_Z = {s.lower(): z for z, s in enumerate(_SYMBOLS) if s}


class ParamFile:
    """readparam over the lines of a parameter file: a position that
    advances with every successful look-up, one wrap to the start."""

    def __init__(self, path, comment="%"):
        with open(path, "r", errors="replace") as f:
            self.lines = f.read().splitlines()
        self.comment = comment
        self.pos = 0  # index of the next line to read

    def _line(self, i):
        s = self.lines[i]
        c = s.find(self.comment)
        return s if c < 0 else s[:c]

    def get(self, title, wrap=True):
        """The rest of the first line at or after the current position that
        contains `title` (None if there is none)."""
        n = len(self.lines)
        for start, stop in ((self.pos, n), (0, n) if wrap else (0, 0)):
            for i in range(start, stop):
                s = self._line(i)
                k = s.find(title)
                if k >= 0:
                    self.pos = i + 1
                    return s[k + len(title):]
            self.pos = n
        return None

    def array(self, title, n):
        """readArray (stem3/stem3.cpp:531-549): n numbers that start after
        `title` and run on over the following lines (comments cut, blank
        lines skipped), each read as atof reads it; None when the title is
        missing, ValueError when the file ends first."""
        v = self.get(title)
        if v is None:
            return None
        toks = v.split()
        while len(toks) < n:
            if self.pos >= len(self.lines):
                raise ValueError("incomplete reading of the %s array (%d of %d values)" % (title, len(toks), n))
            toks += self._line(self.pos).split()
            self.pos += 1
        return np.array([_atof(t) for t in toks[:n]], np.float64)

    def all(self, title):
        """Every line containing `title`, in file order (readparam with
        wrapFlag 0 from the start, as the detector loop reads them)."""
        self.pos = 0
        out = []
        while True:
            v = self.get(title, wrap=False)
            if v is None:
                return out
            out.append(v)


def _word(v, default=""):
    t = (v or "").split()
    return t[0] if t else default


def _num(v, default):
    """sscanf("%g")-style: the leading number, else the default."""
    t = (v or "").split()
    if not t:
        return default
    try:
        return float(t[0])
    except ValueError:
        return default


_ATOF = re.compile(r"[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?")


def _atof(t):
    """atof: the longest leading decimal number, 0 without one."""
    m = _ATOF.match(t)
    return float(m.group(0)) if m else 0.0


def _yes(v, default=False):
    w = _word(v)
    return default if not w else w[0].lower() == "y"


def read_cfg(path):
    """A unit cell from an AtomEye .cfg: the cell vectors H0 (rows, times
    the length scale "A =") and fractional coordinates with the dw,
    occupancy and charge columns when present (default dw = 0.45*28/mass,
    occupancy 1, charge 0)."""
    pf = ParamFile(path, comment="#")
    ncoord = int(_num(pf.get("Number of particles ="), 0))
    scale = _num(pf.get("A ="), 1.0)
    H = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            H[i, j] = _num(pf.get("H0(%d,%d) =" % (i + 1, j + 1)), 0.0) * scale
    # the atom lines follow the header: readNextCFGAtom reads on from the
    # "entry_count =" line (with .NO_VELOCITY., else 3 velocity columns too)
    pf.pos = 0
    novel = pf.get(".NO_VELOCITY.") is not None
    pf.pos = 0
    ec = pf.get("entry_count =")
    entry = int(_num(ec, 3))
    start = pf.pos if ec is not None else 0
    if not novel:
        entry += 3
    off = 0 if novel else 3
    atoms = []
    mass, Z = 28.0, 1
    lines = pf.lines[start:]
    i = 0
    while i < len(lines):
        raw = lines[i]
        i += 1
        tok = raw.split()
        if not tok:
            continue
        try:
            first = float(tok[0])
        except ValueError:
            continue
        if first >= 1.0 and (len(tok) == 1 or tok[1].startswith("#")):
            # a mass line, then the element symbol, then the first atom
            mass = first
            if i >= len(lines):
                break
            Z = _Z.get(lines[i].split()[0].lower(), 0) if lines[i].split() else 0
            i += 1
            continue
        vals = [float(t) for t in tok[:entry]]
        if len(vals) < entry:
            raise ValueError("%s: incomplete atom line %r" % (path, raw))
        dw = vals[3 + off] if entry > 3 + off else 0.45 * 28.0 / mass
        occ = vals[4 + off] if entry > 4 + off else 1.0
        q = vals[5 + off] if entry > 5 + off else 0.0
        atoms.append((Z, vals[0], vals[1], vals[2], dw, occ, q))
    if ncoord and len(atoms) != ncoord:
        raise ValueError("%s: %d atoms listed, %d announced" % (path, len(atoms), ncoord))
    return config.UnitCell(*(float(np.sqrt(np.dot(H[i], H[i]))) for i in range(3)), atoms, H=H)


def _element(field):
    """getZNumber (libs/fileio_fftw3.cpp:2299-2321): the first two characters
    of a symbol field, a digit or line end in the second read as a blank,
    looked up case-sensitively; 0 when unknown."""
    f = (field + "  ")[:2]
    if f[1].isdigit() or f[1] in "\n\r\0 ":
        f = f[0] + " "
    sym = f.rstrip()
    return _SYMBOLS.index(sym) if sym in _SYMBOLS and sym else 0


def read_dat(path):
    """A unit cell from a .dat file (readDATCellParams / readNextDATAtom,
    libs/fileio_fftw3.cpp:664-707, 825-890): "a =", "b =", "c =" and the
    angles after "Number of atoms =" ('#' comments), then one atom per line
    after the "gamma =" line -- element in the first two characters,
    fractional x y z -- with dw = 0.45*28/(2 Z), occupancy 1, charge 0.  The
    reference stores alpha as the cell's gamma and gamma as its alpha."""
    pf = ParamFile(path, comment="#")
    ncoord = int(_num(pf.get("Number of atoms ="), 0))
    a = _num(pf.get("a ="), 0.0)
    b = _num(pf.get("b ="), 0.0)
    c = _num(pf.get("c ="), 0.0)
    al = _num(pf.get("alpha ="), 90.0)
    be = _num(pf.get("beta ="), 90.0)
    ga = _num(pf.get("gamma ="), 90.0)
    H = config.cell_vectors(a, b, c, ga, be, al)
    pf.pos = 0
    pf.get("gamma =")
    atoms = []
    for line in pf.lines[pf.pos:]:
        Z = _element(line[:2]) if line else 0
        if Z == 0:
            continue
        tok = line[2:].split()
        if len(tok) < 3:
            raise ValueError("%s: incomplete atom line %r" % (path, line))
        atoms.append((Z, float(tok[0]), float(tok[1]), float(tok[2]), 0.45 * 28.0 / (2.0 * Z), 1.0, 0.0))
        if len(atoms) == ncoord:
            break
    if ncoord and len(atoms) != ncoord:
        raise ValueError("%s: %d atoms listed, %d announced" % (path, len(atoms), ncoord))
    return config.UnitCell(*(float(np.sqrt(np.dot(H[i], H[i]))) for i in range(3)), atoms, H=H)


def read_cssr(path):
    """A unit cell from a .cssr file (readCSSRCellParams / readNextCSSRAtom,
    libs/fileio_fftw3.cpp:785-815, 998-1051): lengths on line 1, angles on
    line 2 (space group 1 only), the atom count on line 3, atoms from line 5
    as "n element x y z" + 8 integers + dw; occupancy 1, charge 0."""
    with open(path) as fh:
        lines = fh.read().split("\n")
    a, b, c = (float(t) for t in lines[0].split()[:3])
    al, be, ga = (float(t) for t in lines[1].split()[:3])
    if "SPGR =" in lines[1]:
        grp = lines[1].split("SPGR =")[1].split()
        if grp and grp[0].isdigit() and int(grp[0]) != 1:
            raise NotImplementedError("%s: space group %s" % (path, grp[0]))
    ncoord = int(lines[2].split()[0])
    H = config.cell_vectors(a, b, c, al, be, ga)
    atoms = []
    for line in lines[4:4 + ncoord]:
        tok = line.split()
        dw = float(tok[13]) if len(tok) > 13 else 0.0
        atoms.append((_element(tok[1]), float(tok[2]), float(tok[3]), float(tok[4]), dw, 1.0, 0.0))
    return config.UnitCell(*(float(np.sqrt(np.dot(H[i], H[i]))) for i in range(3)), atoms, H=H)


def read_cell(path):
    """readUnitCell's formats by file extension: .cfg, .dat, .cssr."""
    if path.endswith(".cssr"):
        return read_cssr(path)
    if path.endswith(".dat"):
        return read_dat(path)
    if path.endswith(".cfg"):
        return read_cfg(path)
    raise NotImplementedError("%s: unit cell format not supported (.cfg, .dat, .cssr)" % path)


@dataclass
class QscRun:
    """What a .qsc asks for: params (qs_params of run 0), the replicated
    atoms, and the run settings the library leaves to its caller."""
    params: abi.QsParams
    atoms: np.ndarray
    cell: config.UnitCell
    ncell: tuple
    mode: str
    tds: bool
    temperature: float
    avg_runs: int
    folder: str
    detector_names: list = field(default_factory=list)
    dE_E: list = field(default_factory=list)    # energy deviation of each run (dE_EArray)
    scan_step: tuple = (1.0, 1.0)               # detector image sampling, from the .qsc's scan range
    save_level: int = 0                         # "save level:"
    beam_tilt: tuple = (0.0, 0.0)               # rad (TEM: a tilted incident plane wave)
    tilt: tuple = (0.0, 0.0, 0.0)               # crystal tilt, rad
    offset: tuple = (0.0, 0.0)                  # xOffset, yOffset
    source_radius: float = 0.0                  # CBED probe source radius (A)
    replicator: object = None                   # thermal.Replicator drawing the runs' atoms
    cube: tuple = None                          # "Cube:" box size (None: NCELL mode)
    tilt_back: bool = True                      # "Tilt back:" (TEM: wave.img tilted back)
    spread: tuple = (0.0, 0.0, 0.0)             # dE/E, dI/I, dV/V as read (CBED/TEM use them as such)
    custom_sf: tuple = None                     # (k[nk], Z[kinds], f[kinds][nk]): "Structure Factors: custom"

    def einstein_sigma(self):
        """Per-atom, per-axis rms displacement of the Einstein model with
        this temperature (libs/fileio_fftw3.cpp:489-591):
        sqrt(T/300) * sqrt(dw / (8 pi^2)) / sqrt(3)."""
        dw = self.atoms["dw"].astype(np.float64)
        return math.sqrt(self.temperature / 300.0) * np.sqrt(dw / (8 * math.pi ** 2)) / math.sqrt(3.0)


def draw_vacancies(atoms, seed):
    """Vacancies from partial occupancies, seeded (the reference draws them
    with its time-seeded ran1 while replicating, libs/fileio_fftw3.cpp:
    1205-1290): atoms sharing a position form a group; one uniform draw u in
    [0, max(1, total occupancy)) keeps the member whose occupancy interval
    holds u and marks the others Znum = 0 (all of them when u falls past the
    total).  Atoms of occupancy 1 alone at their position are kept."""
    a = abi.atoms_to_numpy(atoms).copy()
    rng = np.random.default_rng(seed)
    key = np.stack([a["x"], a["y"], a["z"]], 1)
    order = np.lexsort((key[:, 2], key[:, 1], key[:, 0]))
    i = 0
    while i < len(order):
        j = i + 1
        while j < len(order) and np.array_equal(key[order[j]], key[order[i]]):
            j += 1
        grp = order[i:j]
        occ = a["occ"][grp].astype(np.float64)
        tot = occ.sum()
        if len(grp) > 1 or tot < 1.0:
            u = rng.random() * max(1.0, tot)
            edges = np.concatenate([[0.0], np.cumsum(occ)])
            for k, idx in enumerate(grp):
                if not (edges[k] <= u < edges[k + 1]):
                    a["Znum"][idx] = 0
        i = j
    return a


def _energy_spread_series(dE_E0, avg_runs):
    """readFile's deterministic energy deviations per run
    (stem3/stem3.cpp:1100-1139): a Gaussian sampled at equal-area points,
    alternating signs, the first run at zero."""
    arr = [0.0] * (avg_runs + 1)
    dy = 1.772453850905 / (2.0 * avg_runs)
    dx = math.pi / ((avg_runs + 1) * 20)
    ix, x, y = 1, 0.0, 0.0
    while ix < avg_runs:
        y += math.exp(-x * x) * dx
        if y >= ix * dy:
            arr[ix] = x * 2 * dE_E0 / math.pi
            ix += 1
            if ix < avg_runs:
                arr[ix] = -arr[ix - 1]
                ix += 1
        x += dx
    return arr[:avg_runs]


def read_qsc(path, seed=20261203, rng="numpy", clock=0):
    """Parse a stem3 .qsc (and the .cfg it names, relative to the .qsc's
    folder) into a QscRun.

    rng "numpy": random draws from numpy.random.default_rng -- the thermal
    displacements of run j from seed + j (phonons.displaced for the Einstein
    model, thermal.Replicator for a phonon file), vacancies likewise, the
    site choice of a "Cube:" box from seed.  rng "reference": the
    reference's own generator, seeded as the reference seeds it from its
    clock (time(NULL) = clock), drawing in the reference's order from
    readFile on (thermal.Replicator), so that runs reproduce a reference run
    made at that clock (NCELL mode)."""
    pf = ParamFile(path)
    g = pf.get
    unsupported = []
    # readFile parses yes/no answers into one buffer, `answer`; a key that
    # is absent leaves the previous answer there, and "smooth:" is decided
    # from whatever it holds (stem3/stem3.cpp:1262-1263)
    answer = [""]

    def ans(v, k=0, reset=False):
        if reset:
            answer[0] = ""
        if v is not None and len(v.split()) > k:
            answer[0] = v.split()[k]
        return v

    mode_s = g("mode:") or ""
    mode = "STEM" if "STEM" in mode_s else "TEM" if "TEM" in mode_s else "CBED" if "CBED" in mode_s else (
        "NBED" if "NBED" in mode_s else "STEM" if not mode_s.strip() else mode_s.strip())
    if mode not in ("STEM", "TEM", "CBED"):
        unsupported.append("mode %s" % mode)
    g("print level:")
    save_level = int(_num(g("save level:"), 0))
    cfg = _word(g("filename:"))
    ncx = int(_num(g("NCELLX:"), 1))
    ncy = int(_num(g("NCELLY:"), 1))
    nz_s = _word(ans(g("NCELLZ:")), "1")
    cellDiv = 1
    if "/" in nz_s:
        nz_s, d = nz_s.split("/", 1)
        cellDiv = int(float(d))
    ncz = int(float(nz_s))
    # beam tilt in rad, or in degrees with a unit word starting with "d"
    # (stem3/stem3.cpp:699-717; floats); tilt back on unless said otherwise
    beam_tilt = []
    for key in ("Beam tilt X:", "Beam tilt Y:"):
        v = ans(g(key), 1, reset=True)
        t = F32(_num(v, 0.0))
        words = (v or "").split()
        if len(words) > 1 and words[1][:1].lower() == "d":
            t = F32(float(t) * (3.1415926535897 / 180.0))
        beam_tilt.append(float(t))
    tb = ans(g("Tilt back:"))
    tilt_back = True if tb is None else _yes(tb)
    # crystal tilt in rad, or in degrees with a unit word starting with "d"
    # (stem3/stem3.cpp:723-743; the values are floats)
    tilt = []
    for key in ("Crystal tilt X:", "Crystal tilt Y:", "Crystal tilt Z:"):
        v = ans(g(key), 1, reset=True)
        t = F32(_num(v, 0.0))
        words = (v or "").split()
        if len(words) > 1 and words[1][:1].lower() == "d":
            t = F32(float(t) * (3.1415926535897 / 180.0))
        tilt.append(float(t))
    cube_v = g("Cube:")
    cube = None
    if cube_v is not None:
        vals = [float(F32(float(t))) for t in cube_v.split()[:3] if _isnum(t)]
        if len(vals) == 3 and all(v > 0 for v in vals):
            cube = vals
    ans(g("Adjust cube size with tilt:"))
    tds = _yes(ans(g("tds:")))
    temperature = float(F32(_num(g("temperature:"), 300.0)))
    here = os.path.dirname(os.path.abspath(path))
    modes = None
    pv = g("phonon-File:")
    if pv is not None and pv.split():
        # a file that cannot be opened leaves the Einstein model
        # (libs/fileio_fftw3.cpp:500-504)
        pfile = os.path.join(here, pv.split()[0])
        if os.path.isfile(pfile):
            from . import thermal
            modes = thermal.read_phonon_file(pfile)
    if rng not in ("numpy", "reference"):
        raise ValueError("rng must be 'numpy' or 'reference'")
    # the unit cell (readUnitCell: .cfg read, replicated, then shifted)
    cell = read_cell(os.path.join(here, cfg))
    xoff = _num(g("xOffset:"), 0.0)
    yoff = _num(g("yOffset:"), 0.0)
    replicator = None
    if cube is not None:  # a box cut from the tilted crystal (tiltBoxed)
        if tds and modes is not None:
            unsupported.append("phonon-File with Cube")  # tiltBoxed exits (libs/fileio_fftw3.cpp:1893-1896)
        if rng == "reference":
            from . import thermal
            replicator = thermal.Replicator(config.sorted_fractional(cell), (1, 1, 1), cell.H,
                                            (cell.a, cell.b, cell.c), tds, temperature, rng=rng, seed=seed,
                                            clock=clock)
            atoms = replicator.cube_configuration(0, cell, cube, tuple(tilt), (xoff, yoff))
            ax, by, c = (F32(v) for v in cube)
        else:
            atoms, ax, by, c = config.cube(cell, cube, tuple(tilt), (xoff, yoff), seed=seed)
    else:  # NCELL mode
        if rng == "reference" or (tds and modes is not None):
            from . import thermal
            replicator = thermal.Replicator(config.sorted_fractional(cell), (ncx, ncy, ncz), cell.H,
                                            (cell.a, cell.b, cell.c), tds, temperature, modes=modes, rng=rng,
                                            seed=seed, clock=clock)
            if not unsupported:  # readFile's own configuration
                atoms, ax, by, c = config.supercell(cell, ncx, ncy, ncz, tuple(tilt), (xoff, yoff),
                                                    replicated=replicator.configuration(0))
        if replicator is None or unsupported:
            atoms, ax, by, c = config.supercell(cell, ncx, ncy, ncz, tuple(tilt), (xoff, yoff))
    nx = int(_num(g("nx:"), 0))
    ny_v = g("ny:")
    ny = int(_num(ny_v, nx)) if ny_v is not None else nx
    resX = _num(g("resolutionX:"), 0.0)
    resY = _num(g("resolutionY:"), 0.0)
    v0 = _num(g("v0:"), 0.0)
    if nx < 1 or v0 <= 0:
        raise ValueError("%s: nx and v0 are required" % path)
    centerSlices = _yes(ans(g("center slices:")))
    dz_v = g("slice-thickness:")
    if dz_v is not None:
        dz = _num(dz_v, 0.0)
        sl_v = g("slices:")
        if sl_v is not None:
            slices = int(_num(sl_v, 0))
        else:
            slices = int(float(F32(c)) / (cellDiv * dz) + 0.99)
    else:
        sl_v = g("slices:")
        slices = int(_num(sl_v, 0))
        if slices == 1 and cellDiv == 1:
            if cube is not None:
                dz = float(F32(2.0 * float(F32(c)) / cellDiv)) if centerSlices else float(F32(float(F32(c)) / cellDiv))
            else:
                dz = float(F32(c)) if centerSlices else float(F32(c)) / cellDiv
        elif cube is not None:
            dz = float(F32(F32(c) / F32(cellDiv * slices - int(centerSlices))))
        else:
            dz = float(F32(F32(c) / F32(cellDiv * slices)))
    if slices < 1:
        raise ValueError("%s: number of slices = 0" % path)
    # only the slice-thickness branch adds the centre slice
    # (stem3/stem3.cpp:880-892); make_params adds it, so take it off here
    if dz_v is None:
        slices -= int(centerSlices)
    out_v = g("slices between outputs:")
    outputInterval = int(_num(out_v, 0)) if out_v is not None else None
    czOffset = _num(g("zOffset:"), 0.0)
    if resX == 0.0:  # stem3/stem3.cpp:949-952
        resX = float(F32(float(F32(ax)) / nx))
    if resY == 0.0:
        resY = float(F32(float(F32(by)) / ny))
    periodicXY = _yes(ans(g("periodicXY:")))
    periodicZ = _yes(ans(g("periodicZ:")))
    bandlimit = _yes(ans(g("bandlimit f_trans:")), True)  # on unless said otherwise
    for key in ("read potential:", "save potential:", "save projected potential:", "plot V(r)*r:",
                "one time integration:"):
        ans(g(key))
    pot3d = ans(g("potential3D:"))
    potential3D = pot3d is None or _yes(pot3d, True)
    if not potential3D and not periodicXY:
        unsupported.append("potential3D: no (the 2-D potential) without periodicXY")
    avg_runs = int(_num(g("Runs for averaging:"), 10))
    ans(g("Store TDS diffr. patt. series:"))
    if not tds:  # stem3/stem3.cpp:1023
        avg_runs = 1
    scan_step = (1.0, 1.0)
    if mode == "STEM":
        scan = (_num(g("scan_x_start:"), 0.0), _num(g("scan_x_stop:"), 0.0), int(_num(g("scan_x_pixels:"), 0)),
                _num(g("scan_y_start:"), 0.0), _num(g("scan_y_stop:"), 0.0), int(_num(g("scan_y_pixels:"), 0)))
        # Detector images are sampled at (stop - start)/N of the values as
        # read, before readFile moves the stops onto the pixel grid
        # (stem3/stem3.cpp:1335-1337)
        scan_step = (float(F32(F32(F32(scan[1]) - F32(scan[0])) / F32(max(scan[2], 1)))),
                     float(F32(F32(F32(scan[4]) - F32(scan[3])) / F32(max(scan[5], 1)))))
    elif mode == "CBED":  # the probe position; TEM keeps the cell centre (:1025-1041)
        xs, ys = g("scan_x_start:"), g("scan_y_start:")
        scan = None if xs is None and ys is None else (
            _num(xs, float(F32(ax)) / 2), 0, 1, _num(ys, float(F32(by)) / 2), 0, 1)
    else:
        scan = None
    dE_E = _num(g("dE/E:"), 0.0)
    dI_I = _num(g("dI/I:"), 0.0)
    dV_V = _num(g("dV/V:"), 0.0)
    Cc = _num(g("Cc:"), 0.0)
    Cs = _num(g("Cs:"), 0.0)
    C5 = _num(g("C5:"), 0.0)
    df = ans(g("defocus:"))
    df_w = _word(df)
    astig = _num(g("astigmatism:"), 0.0)
    astig_deg = _num(g("astigmatism angle:"), 0.0)
    aberr = {}
    for k in ("33", "31", "44", "42", "55", "53", "51", "66", "64", "62"):
        aberr["a" + k] = _num(g("a_%s:" % k), 0.0)
    for k in ("33", "31", "44", "42", "55", "53", "51", "66", "64", "62"):
        aberr["phi" + k] = _num(g("phi_%s:" % k), 0.0)
    alpha = _num(g("alpha:"), 0.0)
    aAIS = _num(g("AIS aperture:"), 0.0)
    beam = _num(g("beam current:"), 1.0)
    dwell = _num(g("dwell time:"), 1.0)
    # doCBED's probe source: offsets of radius * normal draw * sqrt 2 per run
    source_radius = float(F32(_num(g("Source Size (diameter):"), 0.0) / 2.0))
    ans(g("smooth:"))
    smooth = answer[0][:1].lower() == "y"
    gv = g("gaussian:")
    gaussian = None
    if gv is not None and _yes(gv):
        t = gv.split()
        gaussian = float(t[1]) if len(t) > 1 and _isnum(t[1]) else 0.05
    folder = (g("Folder:") or "").strip().strip('"')
    dets = []
    names = []
    for v in pf.all("detector:"):
        t = v.split()
        if len(t) < 3:
            continue
        sx = float(t[3]) if len(t) > 3 and _isnum(t[3]) else 0.0
        sy = float(t[4]) if len(t) > 4 and _isnum(t[4]) else 0.0
        dets.append((float(t[0]), float(t[1]), t[2], sx, sy))
        names.append(t[2])
    pf.pos = 0
    atomRadius = _num(g("atom radius:"), 5.0)
    # "Structure Factors: custom": the k table and one f table per element
    # kind, in the order the unit cell names the kinds (readSFactLUT,
    # stem3/stem3.cpp:555-600, 1402-1419).  doCBED builds its slices from
    # them (make3DSlicesFT); doSTEM and doTEM read them and keep the
    # parameterised potential.
    custom_sf = None
    if _word(g("Structure Factors:"))[:1].lower() == "c":
        nk_v = g("Nk:")
        if nk_v is None:
            raise ValueError("%s: custom scattering factors without Nk" % path)
        nk = int(_atof(nk_v.strip()))
        kv = pf.array("k:", nk)
        if kv is None:
            raise ValueError("%s: custom scattering factors without the k: array" % path)
        kinds = []
        for t in cell.atoms:
            if int(t[0]) > 0 and int(t[0]) not in kinds:
                kinds.append(int(t[0]))
        tables = []
        for Z in kinds:
            fz = pf.array(_SYMBOLS[Z] + ":", nk)
            if fz is None:
                raise ValueError("%s: custom scattering factors without the %s: array" % (path, _SYMBOLS[Z]))
            tables.append(fz)
        custom_sf = (kv, np.array(kinds, np.int32), np.array(tables, np.float64))
        if mode == "CBED" and cellDiv > 1:
            unsupported.append("custom scattering factors with a divided cell")
        if mode == "CBED" and nk < 4:
            unsupported.append("custom scattering factors with Nk < 4")
    # the stacking sequence (doSTEM/doTEM/doCBED's "sequence: m1 m2" loop,
    # stem3/stem3.cpp:2761-2790): m1 repeats each slab's stack inside
    # runMulsSTEM, m2 the slab loop (m2 < 1 reads as 1).  One line is
    # supported (each further line restarts the scan; without any line the
    # reference runs no scan at all, this reader runs the one pass).
    seqs = pf.all("sequence: ")
    m1, m2 = 1, 1
    if len(seqs) > 1:
        unsupported.append("%d stacking-sequence lines" % len(seqs))
    elif seqs:
        tok = seqs[0].split()
        if tok and tok[0][:1].isalnum():
            m = [int(float(t)) if _isnum(t) else 1 for t in tok[:2]] + [1, 1]
            m1, m2 = m[0], max(m[1], 1)
            if m1 < 1:
                unsupported.append("sequence: %s (no slices)" % seqs[0].strip())
    if mode == "STEM" and cube is not None:
        m2 = 1  # doSTEM ignores m2 with a Cube box (stem3/stem3.cpp:2788-2791)
    if mode == "STEM" and m2 * cellDiv > 1 and not (save_level > 1 or cellDiv > 1):
        # doSTEM continues every pass from mulswav_<ix>_<iy>.img, which
        # runMulsSTEM writes only at save level > 1 or with slabs
        unsupported.append("sequence: %d %d at save level %d (the reference reads wave files it did not "
                           "write)" % (m1, m2, save_level))
    if unsupported:
        raise NotImplementedError("%s: not supported by this library: %s" % (path, ", ".join(unsupported)))

    mode_code = {"STEM": abi.QS_MODE_STEM, "TEM": abi.QS_MODE_TEM, "CBED": abi.QS_MODE_CBED}[mode]
    # defocus: Scherzer by default or "s...", "optimum" for "o...", else nm
    if df is None or df_w[:1].lower() == "s":
        defocus = "scherzer"
    elif df_w[:1].lower() == "o":
        defocus = 0.0  # replaced below
    else:
        defocus = _num(df, 0.0)
    p = config.make_params(mode=mode_code, nx=nx, ny=ny, resolutionX=resX, resolutionY=resY, v0=v0, slices=slices,
                           sliceThickness=dz, ax=ax, by=by, c=c, scan=scan, detectors=dets, alpha=alpha, Cs_mm=Cs,
                           C5_mm=C5, defocus_nm=defocus, Cc_mm=Cc, dE_E=0.0, astig_nm=astig,
                           astig_deg=astig_deg, outputInterval=outputInterval, czOffset=czOffset,
                           centerSlices=centerSlices, periodicXY=periodicXY, periodicZ=periodicZ,
                           bandlimit=bandlimit, atomRadius=atomRadius, smooth=smooth, gaussian=gaussian, aAIS=aAIS,
                           beamCurrent=beam, dwellTime=dwell, tds=tds, cellDiv=cellDiv, nCellZ=ncz,
                           potential3D=potential3D)
    p.mulsRepeat1, p.mulsRepeat2 = m1, m2
    if df is not None and df_w[:1].lower() == "o":  # "optimum" defocus, stem3/stem3.cpp:1160-1163
        p.df0 = F32(-float(F32(math.sqrt(float(p.Cs) * config.wavelength(float(p.v0))))))
    for k, v in aberr.items():
        setattr(p, k, F32(v / config.RAD2DEG) if k.startswith("phi") else F32(v))
    dE0 = math.sqrt(dE_E * dE_E + dI_I * dI_I + dV_V * dV_V)
    series = _energy_spread_series(dE0, max(avg_runs, 1))
    return QscRun(params=p, atoms=atoms, cell=cell, ncell=(ncx, ncy, ncz), mode=mode, tds=tds,
                  temperature=temperature, avg_runs=avg_runs, folder=folder, detector_names=names, dE_E=series,
                  scan_step=scan_step, save_level=save_level, spread=(dE_E, dI_I, dV_V),
                  beam_tilt=tuple(beam_tilt), tilt_back=tilt_back, tilt=tuple(tilt), offset=(xoff, yoff),
                  source_radius=source_radius, replicator=replicator,
                  cube=tuple(cube) if cube is not None else None, custom_sf=custom_sf)


def _isnum(t):
    try:
        float(t)
        return True
    except ValueError:
        return False


def _slot_writers(SA, oi, nT):
    """The absolute slice whose collectIntensity call a thickness slot keeps
    (stem3/stemlib.cpp:2597-2610): slices before the last write slot a // oi,
    the last slice slot nT - 1; -1 for a slot nothing writes."""
    last = [-1] * nT
    for a in range(SA):
        t = a // oi if a < SA - 1 else nT - 1
        if t < nT:
            last[t] = a
    return last


def _interim_files(SA, oi):
    """interimWave's writes (stem3/stemlib.cpp:2538-2565): file index -> the
    last absolute slice writing wave_<index>.img (after slice a when a + 1 is
    a multiple of oi, and after the last slice)."""
    files = {}
    for a in range(SA):
        if a == SA - 1 or (a + 1) % oi == 0:
            files[a // oi] = a
    return files


def _steps(p):
    """The wave's steps through the stacking sequence: mulsRepeat2 passes
    through the cellDiv slabs (the slab loop of doSTEM/doCBED/doTEM,
    stem3/stem3.cpp:2795-2949), each slab's stack mulsRepeat1 times
    (runMulsSTEM, stem3/stemlib.cpp:2403-2486).  Per step: (slab, slice,
    collectIntensity's index totalSliceCount + islice*(1 + repeat),
    interimWave's index absolute_slice*(1 + repeat), absolute_slice =
    totalSliceCount + islice)."""
    S, D = p.slices, p.cellDiv
    out = []
    for pc in range(max(1, p.mulsRepeat2) * D):
        for r in range(max(1, p.mulsRepeat1)):
            for i in range(S):
                tsc = pc * S
                out.append((pc % D, i, tsc + i * (1 + r), (tsc + i) * (1 + r), tsc + i))
    return out


def _slot(x, SA, oi, nT):
    """collectIntensity's thickness slot of index x (stem3/stemlib.cpp:2597-2610)."""
    return x // oi if x < SA - 1 else nT - 1


def _repeats(p):
    return max(1, p.mulsRepeat1) > 1 or max(1, p.mulsRepeat2) > 1


# run CBED/TEM through _chain even without repeats (tests compare both paths)
_ALWAYS_CHAIN = False


def _chain(ctx, p, T, slabs, wave0, stops):
    """The wave after chosen steps: one multislice call per stretch of steps
    (their stack slices gathered into one stack), each starting from the
    previous stretch's exit wave.  Returns {step: (k-space pattern after the
    step, real-space wave after it)}."""
    steps = _steps(p)
    S = p.slices
    pos = tuple(np.zeros(1, np.int32) for _ in range(4))
    out, w, a0 = {}, wave0, 0
    for stop in sorted(set(stops)):
        seg = steps[a0:stop + 1]
        stack = np.ascontiguousarray(T[[(st[0] * S if slabs else 0) + st[1] for st in seg]])
        q = p.copy()
        q.slices = q.outputInterval = len(seg)
        q.cellDiv, q.equalDivs, q.mulsRepeat1, q.mulsRepeat2 = 1, 0, 1, 1
        _, dps, ews = ctx.multislice(q, stack, w, positions=pos, want_det=False, want_diffpats=True,
                                     want_exit_waves=True)
        out[stop] = (dps[0], ews[0])
        w, a0 = ews[0], stop + 1
    return out


def _wave_events(p, real_space, sl_diff):
    """What runMulsSTEM writes step by step, reduced to each file's last
    write: {("diff", t): (kind, step, thickness in slices)} for
    collectIntensity's CBED patterns (sl_diff; kind "k" the k-space pattern,
    written with the thickness before the step, "r" the real-space intensity
    of the second collectIntensity), {("wave", f): (step, thickness)} for
    interimWave (real_space: TEM, CBED at save level > 1;
    stem3/stemlib.cpp:2429, 2475-2482, 2538-2565)."""
    steps = _steps(p)
    SA = p.slices * p.cellDiv
    oi, nT = p.outputInterval, p.thickness_count()
    last = {}
    before = None  # thickness before the step: the previous step's
    for a, (_, _, s1, s2, ab) in enumerate(steps):
        if sl_diff:
            last[("diff", _slot(s1, SA, oi, nT))] = ("k", a, before)
        if real_space:
            if s2 >= SA - 1 or (s2 + 1) % oi == 0:
                last[("wave", s2 // oi)] = (a, ab + 1)
            if sl_diff:
                last[("diff", _slot(s2, SA, oi, nT))] = ("r", a, ab + 1)
        before = ab + 1
    return last, len(steps)


def _thick(n, dz):
    """wave->thickness = n * sliceThickness in float (stem3/stemlib.cpp:2455)."""
    return float(F32(F32(n) * F32(dz)))


def _stacks(ctx, p, atoms):
    """Every slab's slice stack (one, reused, for equal divisions), host."""
    if p.cellDiv > 1 and not p.equalDivs:
        return np.concatenate([ctx.slices(p, atoms, slab=k) for k in range(p.cellDiv)]), True
    return ctx.slices(p, atoms), False


def _run_atoms(run, j, seed):
    """The atoms of run j: readFile's for run 0, redrawn for later runs
    (make3DSlices re-reads the cell, stem3/stemlib.cpp:465-485)."""
    if run.replicator is not None:
        if j == 0:
            return run.atoms
        if run.cube is not None:
            return run.replicator.cube_configuration(j, run.cell, run.cube, run.tilt, run.offset)
        atoms, _, _, _ = config.supercell(run.cell, *run.ncell, run.tilt, run.offset,
                                          replicated=run.replicator.configuration(j))
        return atoms
    atoms = run.atoms
    if run.tds:
        from . import phonons
        atoms = phonons.displaced(atoms, j, seed, run.einstein_sigma())
    if np.any(run.atoms["occ"] < 1):
        atoms = draw_vacancies(atoms, seed + 7919 * (j + 1))
    return atoms


def _kspace_pattern(wave, scale):
    """collectIntensity's diffpat of a wave (stem3/stemlib.cpp:2626-2630):
    |psi|^2 at ((ix + nx/2) % nx, (iy + ny/2) % ny), times scale."""
    w = np.asarray(wave, np.float32)
    I = (w[..., 0] * w[..., 0] + w[..., 1] * w[..., 1]).astype(np.float64) * scale
    return np.roll(I.astype(np.float32), (w.shape[0] // 2, w.shape[1] // 2), axis=(0, 1))


def run_qsc(path, ctx=None, folder=None, seed=20261203, chunk=256, rng="numpy", clock=0):
    """Run a stem3 input through the library and write what stem3 writes to
    its output folder.

    Every run of a frozen-phonon average draws its Einstein displacements
    from numpy.random.default_rng(seed + run) when tds is on (and seeded
    vacancies where occupancies are partial).  The files follow doSTEM,
    doCBED and doTEM (stem3/stem3.cpp:2722-2961, 2048-2344, 2354-2710) and
    runMulsSTEM's collectIntensity / interimWave (stem3/stemlib.cpp:
    2538-2749); the writers below say which file comes from where.

    rng, clock: the generator of the runs' random draws (read_qsc); with
    "reference" a run reproduces the reference's run at that clock.
    folder: where to write (default the .qsc's "Folder:", relative to it;
    None writes nothing when the .qsc names none).  chunk: positions per
    multislice call when per-position files are written (bounds host memory).
    Returns a dict of the results (STEM: {detector name: images [slot][x][y]};
    CBED: {"diffpat": mean final pattern, "series": mean slot patterns};
    TEM: {"exit_intensity": mean |psi_exit|^2, "exit_wave": run 0's})."""
    from . import lib
    run = read_qsc(path, seed=seed, rng=rng, clock=clock)
    where = folder if folder is not None else (
        os.path.join(os.path.dirname(os.path.abspath(path)), run.folder) if run.folder else None)
    if where:
        os.makedirs(where, exist_ok=True)
    own = ctx is None
    ctx = ctx or lib.Context(0)
    try:
        if run.mode == "STEM":
            return _run_stem(ctx, run, where, seed, chunk)
        if run.mode == "CBED":
            return _run_cbed(ctx, run, where, seed)
        return _run_tem(ctx, run, where, seed)
    finally:
        if own:
            ctx.close()


def _run_stem(ctx, run, where, seed, chunk):
    """doSTEM: detector images averaged over the runs, saved as
    saveSTEMImages does (stem3/stemlib.cpp:2693-2749): <name>_<t>.img for
    the thickness slots before the last, <name>.img for the last, comment
    "STEM image", the thickness, the scan sampling, and params [runs, error,
    image2 per pixel] with image2 = image^2 and error 0: the values of a
    single-threaded reference run (collectIntensity squares a detector sum
    that its OpenMP threads share, stem3/stemlib.cpp:2614-2681, so threaded
    runs write racy ones).  At save level > 0 also
    each position's diffraction pattern, averaged over the runs in the file
    itself as doSTEM does (diffAvg_<ix>_<iy>.img, "Average Array",
    stem3/stem3.cpp:2890-2930), and at save level > 1 or with slabs its exit
    wave (mulswav_<ix>_<iy>.img, runMulsSTEM's WriteWave,
    stem3/stemlib.cpp:2525-2532; the last run's)."""
    from . import imageio
    p = run.params.copy()
    nt = p.thickness_count()
    SA = p.slices * p.cellDiv
    want_dp = bool(where) and run.save_level > 0
    want_ew = bool(where) and (run.save_level > 1 or p.cellDiv > 1)
    per_pos = want_dp or want_ew
    acc = np.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), np.float64)
    offs = config.scan_offsets(p)
    npos = len(offs[0])
    t_end = _thick(SA * max(1, p.mulsRepeat2), p.sliceThickness)
    rk = (1.0 / float(F32(p.nx * F32(p.resolutionX))), 1.0 / float(F32(p.ny * F32(p.resolutionY))))
    for j in range(run.avg_runs):
        atoms = _run_atoms(run, j, seed)
        p.dE_E = F32(run.dE_E[j]) if j < len(run.dE_E) else F32(0.0)
        if not per_pos:
            acc += ctx.stem_run(p, atoms)
            continue
        T, slabs = _stacks(ctx, p, atoms)
        for c0 in range(0, npos, chunk):
            pos = tuple(a[c0:c0 + chunk] for a in offs)
            det, dps, ews = ctx.multislice(p, T, positions=pos, want_det=p.detectorNum > 0, want_diffpats=want_dp,
                                           want_exit_waves=want_ew and j == run.avg_runs - 1,
                                           slab_stacks=slabs)
            if det is not None:
                acc += det
            for k in range(len(pos[0])):
                ix, iy = int(pos[2][k]), int(pos[3][k])
                if want_dp:
                    fn = os.path.join(where, "diffAvg_%d_%d.img" % (ix, iy))
                    avg = dps[k]
                    if j > 0:  # (avgCount * avg + diffpat) / (avgCount + 1) in float
                        old = imageio.read_img(fn).data.astype(np.float32)
                        avg = ((F32(j) * old + dps[k]) / F32(j + 1)).astype(np.float32)
                    imageio.write_img(fn, avg, t=t_end, dx=rk[0], dy=rk[1], comment="Average Array")
                if ews is not None:
                    imageio.write_img(os.path.join(where, "mulswav_%d_%d.img" % (ix, iy)), ews[k], t=t_end,
                                      dx=float(F32(p.resolutionX)), dy=float(F32(p.resolutionY)),
                                      comment="Wavefunction")
    mean = (acc / run.avg_runs).astype(np.float32)
    out = {name: mean[:, i] for i, name in enumerate(run.detector_names[:p.detectorNum])}
    if where:
        for t in range(nt):
            thick = ((t + 1) * p.outputInterval if t < nt - 1 else SA) * float(p.sliceThickness)
            for name, img in out.items():
                im = img[t]
                # error = sum(image2 - image^2) / sum(image^2): 0 with image2 = image^2
                params = [float(run.avg_runs), 0.0] + list((im.astype(np.float64) ** 2).ravel())
                fn = "%s_%d.img" % (name, t) if t < nt - 1 else "%s.img" % name
                imageio.write_img(os.path.join(where, fn), im, t=float(F32(thick)), dx=run.scan_step[0],
                                  dy=run.scan_step[1], params=params, comment="STEM image")
    return out


def _wave_params(p, spread, beam_tilt=(0.0, 0.0)):
    """interimWave's nine header parameters (stem3/stemlib.cpp:2545-2556):
    v0, Cs, df0, astigmatism and its angle, Cc * total energy spread, alpha,
    beam tilt x and y."""
    dE, dI, dV = (float(F32(v)) for v in spread)
    return [float(p.v0), float(p.Cs), float(p.df0), float(p.astigMag), float(p.astigAngle),
            float(F32(float(p.Cc) * math.sqrt(dE * dE + dV * dV + dI * dI))), float(p.alpha),
            float(beam_tilt[0]), float(beam_tilt[1])]


def _beam_phase(p, beam_tilt, sign):
    """The phase of doTEM's tilted plane wave per row ix
    (stem3/stem3.cpp:2409-2419, and -tilt for the tilt back at :2498-2508):
    k_t = sign * 2 pi sin(tilt) / lambda, x = dx (ix - nx/2), and y taken as
    dy (ix - nx/2) as the reference does, so the wave is constant along y."""
    lam = config.wavelength(float(F32(p.v0)))
    pi = 3.1415926535897
    ktx = sign * 2.0 * pi * math.sin(beam_tilt[0]) / lam
    kty = sign * 2.0 * pi * math.sin(beam_tilt[1]) / lam
    d = (np.arange(p.nx) - p.nx // 2).astype(F32)
    x = (F32(p.resolutionX) * d).astype(F32).astype(np.float64)
    y = (F32(p.resolutionY) * d).astype(F32).astype(np.float64)
    return [ktx * a + kty * b for a, b in zip(x, y)]


def _run_cbed(ctx, run, where, seed):
    """doCBED: one probe at the scan start through every run's stack.

    Files of the first run, as the reference writes them:
      diff_<t>.img   save level > 0: collectIntensity's pattern of thickness
                     slot t ("Diffraction Pattern"; the thickness is the
                     wave's before the slice, as collectIntensity runs before
                     runMulsSTEM updates it).  At save level > 1 runMulsSTEM's
                     second, real-space collectIntensity overwrites it with
                     the real-space intensity after the slice
                     (stem3/stemlib.cpp:2475-2482, 2663-2676).
      wave_<t>.img   save level > 1: interimWave's real-space wave.
      wave_probe.img, wave_final.img   save level > 2: the probe and the
                     final wave (stem3/stem3.cpp:2101-2104, 2210-2213).
      diffAvg_1.img  the final pattern ("DEBUG Wave intensity",
                     stem3/stem3.cpp:2224-2250).
    Later runs (tds): diff_<t>.img hold the mean over the runs so far
    ("Average Array"), diffAvg_<n>.img the mean of the first n runs'
    final patterns ("Averaged Diffraction pattern, unit: 1/A", params
    [tilt 0, 1/lambda]; the previous one is removed unless n - 1 is a
    multiple of the save level) and avgresults.dat the mean squared change
    of each step (stem3/stem3.cpp:2252-2295).  The reference's own averaging
    re-reads the second run's pattern from a leftover diff.img for every
    later run and averages every slice of a thickness group into diff_<t>;
    the files here hold the plain means instead."""
    from . import imageio
    p = run.params.copy()
    p.dE_E = F32(run.spread[0])
    nx, ny = p.nx, p.ny
    SA = p.slices * p.cellDiv
    nT = p.thickness_count()
    oi = p.outputInterval
    writers = _slot_writers(SA, oi, nT)
    sl = run.save_level
    dz = float(p.sliceThickness)
    t_end = _thick(SA * max(1, p.mulsRepeat2), dz)  # the wave's thickness after its last step
    rx, ry = float(F32(p.resolutionX)), float(F32(p.resolutionY))
    rk = (1.0 / float(F32(nx * F32(p.resolutionX))), 1.0 / float(F32(ny * F32(p.resolutionY))))
    scale = 1.0 / math.sqrt(float(nx * ny))
    # doCBED's probe position (stem3/stem3.cpp:2096-2100)
    probes = {}

    def probe_at(off):
        """doCBED's probe at the scan start moved by the run's source
        offset (stem3/stem3.cpp:2096-2100), all positions floats."""
        if off not in probes:
            sx = F32(float(F32(p.scanXStart)) + off[0])
            sy = F32(float(F32(p.scanYStart)) + off[1])
            probes[off] = ctx.probe(p, float(F32(sx - F32(p.potOffsetX))), float(F32(sy - F32(p.potOffsetY))))
        return probes[off]
    pos = tuple(np.zeros(1, np.int32) for _ in range(4))
    inv_lambda = 1.0 / config.wavelength(float(p.v0))
    series_avg = [None] * nT
    avg = None
    chisq = []
    rep = run.replicator
    for j in range(run.avg_runs):
        off = (0.0, 0.0)
        if rep is not None and rep.rng == "reference":
            off = rep.source_offset(j, run.source_radius)  # drawn at radius 0 too: it moves the generator on
        elif run.source_radius > 0:
            from . import thermal
            off = thermal.source_offset(seed, j, run.source_radius)
        probe = probe_at(off)
        if run.custom_sf is not None:
            # make3DSlicesFT builds from readFile's atoms every run (it draws
            # no new configuration, stem3/customslice.cpp:115): one stack
            if j == 0:
                T, slabs = ctx.slices_custom(p, run.atoms, *run.custom_sf), False
        else:
            atoms = _run_atoms(run, j, seed)
            T, slabs = _stacks(ctx, p, atoms)
        # the pattern each slot's file ends the run with and its thickness,
        # interimWave's files, the final wave
        slot_pat, slot_t = [None] * nT, [0.0] * nT
        if _ALWAYS_CHAIN or _repeats(p):
            ev, NS = _wave_events(p, sl > 1, True)
            res = _chain(ctx, p, T, slabs, probe, {v[1] if k[0] == "diff" else v[0] for k, v in ev.items()} | {NS - 1})
            for (kind, t), v in ev.items():
                if kind == "diff" and v[0] == "k":
                    slot_pat[t] = res[v[1]][0]
                    slot_t[t] = t_end if (v[2] is None and j > 0) else _thick(v[2] or 0, dz)
                elif kind == "diff":
                    slot_pat[t], slot_t[t] = _kspace_pattern(res[v[1]][1], scale), _thick(v[2], dz)
            last_wave = res[NS - 1][1]
            final = _kspace_pattern(last_wave, scale) if sl > 1 else res[NS - 1][0]
            wave_files = {k[1]: (res[v[0]][1], _thick(v[1], dz)) for k, v in ev.items() if k[0] == "wave"}
        else:
            _, dps, ews = ctx.multislice(p, T, probe, positions=pos, want_det=False, want_diffpats=True,
                                         want_exit_waves=sl > 1, slab_stacks=slabs, series=True)
            for t, a in enumerate(writers):
                if a < 0:
                    continue
                if sl > 1:
                    slot_pat[t], slot_t[t] = _kspace_pattern(ews[t, 0], scale), _thick(a + 1, dz)
                else:
                    stale = t_end if (a == 0 and j > 0) else _thick(a, dz)
                    slot_pat[t], slot_t[t] = dps[t, 0], stale
            final = slot_pat[nT - 1]
            last_wave = ews[nT - 1, 0] if sl > 1 else None
            wave_files = {f: (ews[nT - 1 if a == SA - 1 else a // oi, 0], _thick(a + 1, dz))
                          for f, a in _interim_files(SA, oi).items()} if sl > 1 else {}
        if where and sl > 2:
            imageio.write_img(os.path.join(where, "wave_probe.img"), probe, t=0.0 if j == 0 else t_end, dx=rx,
                              dy=ry, comment="Wavefunction")
            if j == 0:
                imageio.write_img(os.path.join(where, "wave_final.img"), last_wave, t=t_end, dx=rx, dy=ry,
                                  comment="Wavefunction")
        if where and sl > 1:
            for f, (w, th) in wave_files.items():
                name = "wave_%d_%d.img" % (j, f) if run.tds else "wave_%d.img" % f
                imageio.write_img(os.path.join(where, name), w, t=th, dx=rx, dy=ry,
                                  params=_wave_params(p, run.spread, run.beam_tilt), comment="Wave Function")
        for t in range(nT):
            if slot_pat[t] is None:
                continue
            series_avg[t] = slot_pat[t] if j == 0 else ((F32(j) * series_avg[t] + slot_pat[t]) / F32(j + 1)).astype(
                np.float32)
            if where and sl > 0:
                imageio.write_img(os.path.join(where, "diff_%d.img" % t), series_avg[t], t=slot_t[t], dx=rk[0],
                                  dy=rk[1], comment="Diffraction Pattern" if j == 0 else "Average Array")
        if j == 0:
            avg = final.copy()
            if where:
                imageio.write_img(os.path.join(where, "diffAvg_1.img"), avg, t=t_end, dx=rk[0], dy=rk[1],
                                  comment="DEBUG Wave intensity")
            continue
        new = ((F32(j) * avg + final) / F32(j + 1)).astype(np.float32)
        chisq.append(float(np.sum((avg.astype(np.float64) - new) ** 2)) / float(nx * ny))
        avg = new
        if where:
            imageio.write_img(os.path.join(where, "diffAvg_%d.img" % (j + 1)), avg, t=t_end, dx=rk[0], dy=rk[1],
                              params=[0.0, inv_lambda], comment="Averaged Diffraction pattern, unit: 1/A")
            if sl == 0 or j % sl != 0:
                prev = os.path.join(where, "diffAvg_%d.img" % j)
                if os.path.exists(prev):
                    os.remove(prev)
            with open(os.path.join(where, "avgresults.dat"), "w") as fh:
                for k, c in enumerate(chisq):
                    fh.write("%d %g\n" % (k + 1, c))
    return {"diffpat": avg, "series": series_avg}


def _run_tem(ctx, run, where, seed):
    """doTEM: an incident plane wave through every run's stack.

    Files: interimWave's real-space waves wave_<t>.img ("Wave Function",
    nine parameters; wave_<run>_<t>.img with tds) after the slices it writes
    (stem3/stemlib.cpp:2538-2565), and the first run's exit wave wave.img
    ("Exit face wave function for no TDS", or "Test wave function for run 0"
    with tds; stem3/stem3.cpp:2494-2513).  The reference stops there: it
    then reads a diff.img that TEM never writes (stem3/stem3.cpp:2545-2547).
    This also writes the mean exit-wave intensity over all runs,
    waveIntensity.img ("Wave intensity", params [runs]), which the
    reference intends but never reaches; CTF images are Context.tem's."""
    from . import imageio
    p = run.params.copy()
    nx, ny = p.nx, p.ny
    SA = p.slices * p.cellDiv
    nT = p.thickness_count()
    oi = p.outputInterval
    dz = float(p.sliceThickness)
    t_end = _thick(SA * max(1, p.mulsRepeat2), dz)  # the wave's thickness after its last step
    rx, ry = float(F32(p.resolutionX)), float(F32(p.resolutionY))
    plane = np.zeros((nx, ny, 2), np.float32)
    plane[..., 0] = 1.0  # stem3/stem3.cpp:2403-2407
    tilted = run.beam_tilt[0] != 0 or run.beam_tilt[1] != 0
    if tilted:
        ph = _beam_phase(p, run.beam_tilt, 1.0)
        plane[..., 0] = np.array([F32(math.cos(v)) for v in ph], np.float32)[:, None]
        plane[..., 1] = np.array([F32(math.sin(v)) for v in ph], np.float32)[:, None]
    pos = tuple(np.zeros(1, np.int32) for _ in range(4))
    files = _interim_files(SA, oi)
    acc = np.zeros((nx, ny), np.float64)
    first = None
    for j in range(run.avg_runs):
        atoms = _run_atoms(run, j, seed)
        T, slabs = _stacks(ctx, p, atoms)
        if _ALWAYS_CHAIN or _repeats(p):
            ev, NS = _wave_events(p, True, False)
            res = _chain(ctx, p, T, slabs, plane, {a for a, _ in ev.values()} | {NS - 1})
            exit_wave = res[NS - 1][1]
            wave_files = {f: (res[a][1], _thick(th, dz)) for (_, f), (a, th) in ev.items()}
        else:
            _, _, ews = ctx.multislice(p, T, plane, positions=pos, want_det=False, want_exit_waves=True,
                                       slab_stacks=slabs, series=True)
            exit_wave = ews[nT - 1, 0]
            wave_files = {f: (ews[nT - 1 if a == SA - 1 else a // oi, 0], _thick(a + 1, dz)) for f, a in files.items()}
        acc += exit_wave[..., 0].astype(np.float64) ** 2 + exit_wave[..., 1].astype(np.float64) ** 2
        if j == 0:
            first = exit_wave
        if not where:
            continue
        for f, (w, th) in wave_files.items():
            name = "wave_%d_%d.img" % (j, f) if run.tds else "wave_%d.img" % f
            imageio.write_img(os.path.join(where, name), w, t=th, dx=rx, dy=ry,
                              params=_wave_params(p, run.spread, run.beam_tilt), comment="Wave Function")
        if j == 0:
            saved = exit_wave
            if run.tilt_back and tilted:
                # re *= cos(phase), im *= sin(phase): the reference scales the
                # two parts separately (stem3/stem3.cpp:2498-2508)
                ph = _beam_phase(p, run.beam_tilt, -1.0)
                c = np.array([math.cos(v) for v in ph])[:, None]
                sn = np.array([math.sin(v) for v in ph])[:, None]
                saved = np.stack([(exit_wave[..., 0].astype(np.float64) * c).astype(F32),
                                  (exit_wave[..., 1].astype(np.float64) * sn).astype(F32)], -1)
            imageio.write_img(os.path.join(where, "wave.img"), saved, t=t_end, dx=rx, dy=ry,
                              comment="Test wave function for run 0" if run.tds else
                              "Exit face wave function for no TDS")
    mean = (acc / run.avg_runs).astype(np.float32)
    if where:
        imageio.write_img(os.path.join(where, "waveIntensity.img"), mean, t=t_end, dx=rx, dy=ry,
                          params=[float(run.avg_runs)], comment="Wave intensity")
    return {"exit_intensity": mean, "exit_wave": first}
