"""Read unmodified stem3 inputs: a .qsc parameter file and its AtomEye .cfg
unit cell, into qs_params and the replicated atom list.

The parameter file is read the way the reference's readFile does
(stem3/stem3.cpp:600-1460): every key is looked up with readparam's rule
(libs/readparams.cpp:173-212) -- search forward from where the previous
look-up stopped, wrap to the start once, cut each line at '%', match the key
anywhere in the line -- in readFile's order, so that a key such as "slices:"
resolves to the same line it does there (it is also a substring of
"center slices:").  The derived fields (potential grid, offsets, k^2 of the
detectors, ...) then come from config.make_params, which follows the rest of
readFile.  The unit cell is read as readCFGCellParams / readNextCFGAtom read
it (libs/fileio_fftw3.cpp:721-989) and replicated as readUnitCell does.

Inputs that need parts of the reference outside this library are refused
with NotImplementedError: a "Cube" box, crystal or beam tilt, phonon files,
the 2-D potential, and non-orthogonal cells.
"""
import math
import os
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


def _yes(v, default=False):
    w = _word(v)
    return default if not w else w[0].lower() == "y"


def read_cfg(path):
    """A unit cell from an AtomEye .cfg (orthogonal H0 only): fractional
    coordinates with the dw, occupancy and charge columns when present
    (default dw = 0.45*28/mass, occupancy 1, charge 0)."""
    pf = ParamFile(path, comment="#")
    ncoord = int(_num(pf.get("Number of particles ="), 0))
    scale = _num(pf.get("A ="), 1.0)
    H = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            H[i, j] = _num(pf.get("H0(%d,%d) =" % (i + 1, j + 1)), 0.0) * scale
    if np.abs(H - np.diag(np.diag(H))).max() > 0:
        raise NotImplementedError("%s: non-orthogonal cells are not supported" % path)
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
    return config.UnitCell(H[0, 0], H[1, 1], H[2, 2], atoms)


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


def read_qsc(path):
    """Parse a stem3 .qsc (and the .cfg it names, relative to the .qsc's
    folder) into a QscRun."""
    pf = ParamFile(path)
    g = pf.get
    unsupported = []
    mode_s = g("mode:") or ""
    mode = "STEM" if "STEM" in mode_s else "TEM" if "TEM" in mode_s else "CBED" if "CBED" in mode_s else (
        "NBED" if "NBED" in mode_s else "STEM" if not mode_s.strip() else mode_s.strip())
    if mode not in ("STEM", "TEM", "CBED"):
        unsupported.append("mode %s" % mode)
    g("print level:")
    g("save level:")
    cfg = _word(g("filename:"))
    ncx = int(_num(g("NCELLX:"), 1))
    ncy = int(_num(g("NCELLY:"), 1))
    nz_s = _word(g("NCELLZ:"), "1")
    cellDiv = 1
    if "/" in nz_s:
        nz_s, d = nz_s.split("/", 1)
        cellDiv = int(float(d))
    ncz = int(float(nz_s))
    for key in ("Beam tilt X:", "Beam tilt Y:", "Tilt back:", "Crystal tilt X:", "Crystal tilt Y:",
                "Crystal tilt Z:"):
        v = g(key)
        if key != "Tilt back:" and _num(v, 0.0) != 0.0:
            unsupported.append(key.rstrip(":"))
    cube = g("Cube:")
    if cube is not None and any(float(t) != 0 for t in cube.split()[:3] if _isnum(t)):
        unsupported.append("Cube")
    tds = _yes(g("tds:"))
    temperature = _num(g("temperature:"), 300.0)
    if g("phonon-File:") is not None:
        unsupported.append("phonon-File")
    # the unit cell (readUnitCell: .cfg read, replicated, then shifted)
    cfg_path = os.path.join(os.path.dirname(os.path.abspath(path)), cfg)
    cell = read_cfg(cfg_path)
    atoms, ax, by, c = config.replicate(cell, ncx, ncy, ncz)
    xoff = _num(g("xOffset:"), 0.0)
    yoff = _num(g("yOffset:"), 0.0)
    if xoff != 0 or yoff != 0:  # libs/fileio_fftw3.cpp:1634-1640
        atoms["x"] = (atoms["x"] + F32(xoff)).astype(F32)
        atoms["y"] = (atoms["y"] + F32(yoff)).astype(F32)
    nx = int(_num(g("nx:"), 0))
    ny_v = g("ny:")
    ny = int(_num(ny_v, nx)) if ny_v is not None else nx
    resX = _num(g("resolutionX:"), 0.0)
    resY = _num(g("resolutionY:"), 0.0)
    v0 = _num(g("v0:"), 0.0)
    if nx < 1 or v0 <= 0:
        raise ValueError("%s: nx and v0 are required" % path)
    centerSlices = _yes(g("center slices:"))
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
            dz = float(F32(c)) if centerSlices else float(F32(c)) / cellDiv
        else:
            dz = float(F32(F32(c) / F32(cellDiv * slices)))
    if slices < 1:
        raise ValueError("%s: number of slices = 0" % path)
    out_v = g("slices between outputs:")
    outputInterval = int(_num(out_v, 0)) if out_v is not None else None
    czOffset = _num(g("zOffset:"), 0.0)
    if resX == 0.0:  # stem3/stem3.cpp:949-952
        resX = float(F32(float(F32(ax)) / nx))
    if resY == 0.0:
        resY = float(F32(float(F32(by)) / ny))
    periodicXY = _yes(g("periodicXY:"))
    periodicZ = _yes(g("periodicZ:"))
    bandlimit = _yes(g("bandlimit f_trans:"), False)
    g("one time integration:")
    pot3d = g("potential3D:")
    if pot3d is not None and not _yes(pot3d, True):
        unsupported.append("potential3D: no (the 2-D potential)")
    avg_runs = int(_num(g("Runs for averaging:"), 10))
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
    df = g("defocus:")
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
    smooth = _yes(g("smooth:"), True)
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
                           beamCurrent=beam, dwellTime=dwell, tds=tds, cellDiv=cellDiv, nCellZ=ncz)
    if df is not None and df_w[:1].lower() == "o":  # "optimum" defocus, stem3/stem3.cpp:1160-1163
        p.df0 = F32(-float(F32(math.sqrt(float(p.Cs) * config.wavelength(float(p.v0))))))
    for k, v in aberr.items():
        setattr(p, k, F32(v / config.RAD2DEG) if k.startswith("phi") else F32(v))
    dE0 = math.sqrt(dE_E * dE_E + dI_I * dI_I + dV_V * dV_V)
    series = _energy_spread_series(dE0, max(avg_runs, 1))
    return QscRun(params=p, atoms=atoms, cell=cell, ncell=(ncx, ncy, ncz), mode=mode, tds=tds,
                  temperature=temperature, avg_runs=avg_runs, folder=folder, detector_names=names, dE_E=series,
                  scan_step=scan_step)


def _isnum(t):
    try:
        float(t)
        return True
    except ValueError:
        return False


def run_qsc(path, ctx=None, folder=None, seed=20261203):
    """Run a stem3 input through the library and write what stem3 writes.

    STEM: every run of the frozen-phonon average (Einstein displacements
    drawn from numpy.random.default_rng(seed + run) when tds is on, and
    seeded vacancies where occupancies are partial) through qs_stem_run;
    the mean detector images are written as saveSTEMImages does
    (stem3/stemlib.cpp:2693-2749): <folder>/<name>_<t>.img for the thickness
    slots before the last, <folder>/<name>.img for the last, comment
    "STEM image", the thickness, the scan sampling, and params [runs, error,
    image^2 per pixel] (the reference's image2 sums the squares over the
    slices of a slot; this writes the final slice's).  Returns
    {detector name: images [thickness slot][scanX][scanY]}.
    folder: where to write (default the .qsc's "Folder:", relative to it;
    None writes nothing when the .qsc names none)."""
    from . import imageio, lib, phonons
    run = read_qsc(path)
    if run.mode != "STEM":
        raise NotImplementedError("run_qsc writes STEM outputs; use Context.cbed_batch / Context.tem")
    own = ctx is None
    ctx = ctx or lib.Context(0)
    try:
        p = run.params.copy()
        nt = p.thickness_count()
        acc = np.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), np.float64)
        partial = bool(np.any(run.atoms["occ"] < 1))
        for j in range(run.avg_runs):
            atoms = run.atoms
            if run.tds:
                atoms = phonons.displaced(atoms, j, seed, run.einstein_sigma())
            if partial:
                atoms = draw_vacancies(atoms, seed + 7919 * (j + 1))
            p.dE_E = F32(run.dE_E[j]) if j < len(run.dE_E) else F32(0.0)
            acc += ctx.stem_run(p, atoms)
        mean = (acc / run.avg_runs).astype(np.float32)
    finally:
        if own:
            ctx.close()
    out = {name: mean[:, i] for i, name in enumerate(run.detector_names[:p.detectorNum])}
    where = folder if folder is not None else (
        os.path.join(os.path.dirname(os.path.abspath(path)), run.folder) if run.folder else None)
    if where:
        os.makedirs(where, exist_ok=True)
        for t in range(nt):
            thick = ((t + 1) * p.outputInterval if t < nt - 1 else p.slices * p.cellDiv) * float(p.sliceThickness)
            for name, img in out.items():
                im = img[t]
                # error = sum(image2 - image^2) / sum(image^2): 0 with image2 = image^2
                params = [float(run.avg_runs), 0.0] + list((im.astype(np.float64) ** 2).ravel())
                fn = "%s_%d.img" % (name, t) if t < nt - 1 else "%s.img" % name
                imageio.write_img(os.path.join(where, fn), im, t=float(F32(thick)), dx=run.scan_step[0],
                                  dy=run.scan_step[1], params=params, comment="STEM image")
    return out
