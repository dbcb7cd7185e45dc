"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own CPU path (compiled from its sources by
`make -C oracle ref`, FFTW supplied by the project's FFT shim) through
oracle/ref_harness on small seeded cases, and stores its inputs and outputs
as compressed .npz files:

  params    the qs_params the case describes (as a dict)
  meta      the MULS fields readFile derived (to pin qstem_gb300.config)
  atoms     readFile's atoms (struct atom records)
  lut_*     getAtomPotential3D / getAtomPotentialOffset3D tables
  V, T      trans after make3DSlices and after initSTEMSlices
  probe     probe() at the window centre
  det       detector images after doSTEM (STEM cases that run)
  diffpat_* / wave_*   diffAvg_ix_iy.img / mulswav_ix_iy.img the reference
            wrote for the first positions (saveLevel 2)
  V_slabs, T_slabs   every slab's potential/transmission of an unequally
            divided cell (cellDiv > 1)
  cbed_diffpat  doCBED's diffraction pattern (diffAvg_1.img)
  exit_wave     doTEM's exit wave (wave.img)

Usage: QS_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py [case ...]
(the fixtures are committed so the tests do not need the reference)
"""
import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from qstem_gb300 import abi, config, imageio  # noqa: E402

CASES = {
    # configuration-1-like: non-periodic, neutral atoms, one output group
    "sto64": dict(cell="sto", ncell=(3, 3, 4), nx=64, resolutionX=0.0915, v0=200.0, slices=8,
                  sliceThickness=1.9525, scan=(3.905, 7.81, 4, 3.905, 7.81, 4),
                  detectors=[(0.0, 20.0, "BF"), (20.0, 40.0, "ADF"), (40.0, 90.0, "HAADF")],
                  alpha=20.0, outputInterval=4, mode="STEM", run=True),
    # periodic in x-y, charged atoms with Debye-Waller factors, centred slices,
    # z offset, uneven output groups, aberrated probe
    "sto64q": dict(cell="stoq", ncell=(3, 3, 3), nx=64, resolutionX=0.0915, v0=300.0, slices=6,
                   sliceThickness=1.9525, scan=(2.0, 5.905, 3, 2.5, 6.405, 3),
                   detectors=[(10.0, 40.0, "A"), (40.0, 80.0, "B")], alpha=15.0, outputInterval=4,
                   Cs_mm=0.5, defocus_nm=-5.0, czOffset=0.3, centerSlices=True, periodicXY=True,
                   mode="STEM", run=True),
    # the transmission band limit on a 106 x 110 potential grid (sizes the
    # line FFTs do not cover: the DFT-matrix path)
    "sto64bl": dict(cell="sto", ncell=(3, 3, 4), nx=64, resolutionX=0.0915, v0=200.0, slices=6,
                    sliceThickness=1.9525, scan=(3.905, 7.81, 3, 3.905, 8.2, 3),
                    detectors=[(0.0, 20.0, "BF"), (40.0, 90.0, "HAADF")], alpha=20.0, bandlimit=True,
                    mode="STEM", run=True),
    # a cell divided into two equal slabs (NCELLZ: 4/2): slab 0's stack reused,
    # thickness slots counted over both
    "sto64d2": dict(cell="sto", ncell=(3, 3, 4), nx=64, resolutionX=0.0915, v0=200.0, slices=4,
                    sliceThickness=1.9525, scan=(3.905, 7.81, 3, 3.905, 7.81, 3),
                    detectors=[(0.0, 20.0, "BF"), (40.0, 90.0, "HAADF")], alpha=20.0, outputInterval=3,
                    cellDiv=2, mode="STEM", run=True),
    # two unequal slabs (NCELLZ: 3/2): every slab built from shifted atoms
    "sto64d2u": dict(cell="sto", ncell=(3, 3, 3), nx=64, resolutionX=0.0915, v0=200.0, slices=3,
                     sliceThickness=1.9525, scan=(3.905, 7.81, 3, 3.905, 7.81, 3),
                     detectors=[(0.0, 20.0, "BF"), (40.0, 90.0, "HAADF")], alpha=20.0, cellDiv=2,
                     mode="STEM", run=True),
    # CBED geometry (potential grid = wave grid) with the transmission band limit
    "si64cbed": dict(cell="si", ncell=(4, 3, 3), nx=64, resolutionX=0.06788, v0=300.0, slices=5, sliceThickness=2.0,
                     scan=None, detectors=[], alpha=10.0, Cs_mm=1.2, defocus_nm=-60.0, bandlimit=True,
                     mode="CBED", run=True, saveLevel=1),
    # the 2-D potential (potential3D: no) on a periodic potential array: the
    # periodic 2-D branch of make3DSlices and getAtomPotential2D's tables
    "sto64p2d": dict(cell="sto", ncell=(3, 3, 4), nx=64, resolutionX=0.0915, v0=200.0, slices=8,
                     sliceThickness=1.9525, scan=(3.905, 7.81, 3, 3.905, 7.81, 3),
                     detectors=[(0.0, 20.0, "BF"), (40.0, 90.0, "HAADF")], alpha=20.0, periodicXY=True,
                     potential3D=False, mode="STEM", run=True),
    # custom scattering factors ("Structure Factors: custom"): doCBED builds
    # its slices with make3DSlicesFT (stem3/customslice.cpp:56-317)
    "sto64ft": dict(cell="sto", ncell=(3, 3, 2), nx=64, resolutionX=0.18, v0=200.0, slices=4,
                    sliceThickness=1.9525, scan=None, detectors=[], alpha=10.0, mode="CBED", run=True,
                    saveLevel=1, custom_sf="sto"),
    # TEM: plane wave through a band-limited Si [110] slab (doTEM's exit wave)
    "si64tem": dict(cell="si", ncell=(4, 3, 4), nx=64, resolutionX=0.06, v0=300.0, slices=7, sliceThickness=2.0,
                    scan=None, detectors=[], alpha=0.0, bandlimit=True, mode="TEM", run=True),
}


def cell_of(name):
    if name == "sto":
        return config.srtio3_cell()
    if name == "stoq":
        a = 3.905
        return config.UnitCell(a, a, a, [(38, 0, 0, 0, 0.6214, 1, 2.0), (22, .5, .5, .5, 0.4390, 1, 4.0),
                                         (8, 0, .5, .5, 0.7323, 1, -2.0), (8, .5, 0, .5, 0.7323, 1, -2.0),
                                         (8, .5, .5, 0, 0.7323, 1, -2.0)])
    if name == "si":
        return config.si110_cell()
    raise KeyError(name)


def custom_table(name):
    """A synthetic custom scattering-factor table (k in 1/A, f in A): f_Z(k)
    = A_Z / (1 + (k / 0.6)^2)^2, A_Z = 0.28 Z^0.7, written with 6 significant
    digits; returns (k, {Z: f}) as the reference parses them back."""
    if name != "sto":
        raise KeyError(name)
    k = [float("%.6g" % (0.25 * i)) for i in range(25)]
    table = {}
    for Z in (38, 22, 8):
        A = 0.28 * Z ** 0.7
        table[Z] = [float("%.6g" % (A / (1.0 + (kk / 0.6) ** 2) ** 2)) for kk in k]
    return k, table


def params_for(case):
    cell = cell_of(case["cell"])
    atoms, ax, by, c = config.replicate(cell, *case["ncell"])
    mode = {"STEM": abi.QS_MODE_STEM, "CBED": abi.QS_MODE_CBED, "TEM": abi.QS_MODE_TEM}[case["mode"]]
    p = config.make_params(mode=mode, nx=case["nx"], resolutionX=case["resolutionX"], v0=case["v0"],
                           slices=case["slices"], sliceThickness=case["sliceThickness"], ax=ax, by=by, c=c,
                           scan=case["scan"], detectors=case["detectors"], alpha=case["alpha"],
                           Cs_mm=case.get("Cs_mm", 0.0), defocus_nm=case.get("defocus_nm", 0.0),
                           outputInterval=case.get("outputInterval"), czOffset=case.get("czOffset", 0.0),
                           centerSlices=case.get("centerSlices", False),
                           periodicXY=case.get("periodicXY", False), bandlimit=case.get("bandlimit", False),
                           cellDiv=case.get("cellDiv", 1), nCellZ=case["ncell"][2],
                           potential3D=case.get("potential3D", True))
    return cell, atoms, p


def run_case(name, case, workdir):
    cell, atoms, p = params_for(case)
    cfg = os.path.join(workdir, "cell.cfg")
    config.write_cfg(cell, cfg)
    qsc = os.path.join(workdir, "run.qsc")
    config.write_qsc(qsc, cfg_file="cell.cfg", ncell=case["ncell"], nx=case["nx"],
                     resolutionX=case["resolutionX"], v0=case["v0"], slices=case["slices"],
                     sliceThickness=case["sliceThickness"], scan=case["scan"], detectors=case["detectors"],
                     alpha=case["alpha"], Cs_mm=case.get("Cs_mm", 0.0), defocus_nm=case.get("defocus_nm", 0.0),
                     outputInterval=case.get("outputInterval"), mode=case["mode"],
                     bandlimit=case.get("bandlimit", False), periodicXY=case.get("periodicXY", False),
                     folder="out", saveLevel=case.get("saveLevel", 2 if case["run"] else 0), czOffset=case.get("czOffset", 0.0),
                     centerSlices=case.get("centerSlices", False), cellDiv=case.get("cellDiv", 1),
                     potential3D=case.get("potential3D", True),
                     custom_sf=custom_table(case["custom_sf"]) if "custom_sf" in case else None)
    dump = os.path.join(workdir, "dump")
    oracle.run_reference(qsc, dump, run=case["run"])
    meta = dict(l.split(" = ", 1) for l in open(os.path.join(dump, "meta.txt")).read().strip().split("\n"))
    out = {}
    out["atoms"] = np.fromfile(os.path.join(dump, "atoms.bin"), dtype=abi.ATOM_DTYPE)
    shp = (p.slices, p.potNx, p.potNy, 2)
    assert int(meta["potNx"]) == p.potNx and int(meta["potNy"]) == p.potNy, (meta, p.potNx)
    out["V"] = np.fromfile(os.path.join(dump, "potential.bin"), np.float32).reshape(shp)
    out["T"] = np.fromfile(os.path.join(dump, "trans.bin"), np.float32).reshape(shp)
    out["probe"] = np.fromfile(os.path.join(dump, "probe.bin"), np.float32).reshape(p.nx, p.ny, 2)
    if p.cellDiv > 1 and not p.equalDivs:
        # slabs 1..cellDiv-1 of an unequally divided cell
        out["V_slabs"] = np.stack([out["V"]] + [np.fromfile(os.path.join(dump, "potential_%d.bin" % k), np.float32)
                                                .reshape(shp) for k in range(1, p.cellDiv)])
        out["T_slabs"] = np.stack([out["T"]] + [np.fromfile(os.path.join(dump, "trans_%d.bin" % k), np.float32)
                                                .reshape(shp) for k in range(1, p.cellDiv)])
    for line in open(os.path.join(dump, "lut_dims.txt")):
        Z, Nz, Nr, ns = map(int, line.split())
        out["lut_%d" % Z] = np.fromfile(os.path.join(dump, "lut_%d.bin" % Z), np.float32).reshape(Nz, Nr, 2)[..., 0]
        qf = os.path.join(dump, "lutq_%d.bin" % Z)
        if os.path.exists(qf):
            out["lutq_%d" % Z] = np.fromfile(qf, np.float32).reshape(Nz, Nr, 2)[..., 0]
        out["nzsub"] = np.int32(ns)
    l2d = os.path.join(dump, "lut2d_dims.txt")
    if os.path.exists(l2d):
        for line in open(l2d):
            Z, nx2, ny2 = map(int, line.split())
            out["lut2d_%d" % Z] = np.fromfile(os.path.join(dump, "lut2d_%d.bin" % Z), np.float32).reshape(nx2, ny2, 2)
    if case["run"] and case["mode"] == "STEM":
        nt = p.thickness_count()
        det = np.zeros((nt, p.detectorNum, p.scanXN, p.scanYN), np.float32)
        for t in range(nt):
            for i in range(p.detectorNum):
                det[t, i] = np.fromfile(os.path.join(dump, "det_%d_%d.bin" % (t, i)), np.float32).reshape(
                    p.scanXN, p.scanYN)
        out["det"] = det
        folder = os.path.join(workdir, "out")
        for ix, iy in [(0, 0), (0, 1), (1, 0), (p.scanXN - 1, p.scanYN - 1)]:
            dp = imageio.read_img(os.path.join(folder, "diffAvg_%d_%d.img" % (ix, iy)))
            out["diffpat_%d_%d" % (ix, iy)] = dp.data.astype(np.float32)
            ww = imageio.read_img(os.path.join(folder, "mulswav_%d_%d.img" % (ix, iy)))
            out["wave_%d_%d" % (ix, iy)] = np.stack([ww.data.real, ww.data.imag], -1).astype(np.float32)
    folder = os.path.join(workdir, "out")
    if case["run"] and case["mode"] == "CBED":
        # doCBED moves the last collectIntensity pattern to diffAvg_1.img (at
        # save level <= 1; above it runMulsSTEM's extra real-space
        # collectIntensity, stem3/stemlib.cpp:2475-2482, overwrites it)
        out["cbed_diffpat"] = imageio.read_img(os.path.join(folder, "diffAvg_1.img")).data.astype(np.float32)
    if case["run"] and case["mode"] == "TEM":
        # doTEM writes the exit wave of its first run before it fails on the
        # diff.img it never wrote (stem3/stem3.cpp:2494-2517, 2545-2547)
        ww = imageio.read_img(os.path.join(folder, "wave.img"))
        out["exit_wave"] = np.stack([ww.data.real, ww.data.imag], -1).astype(np.float32)
    if "custom_sf" in case:
        kv, table = custom_table(case["custom_sf"])
        out["sf_k"] = np.array(kv, np.float64)
        out["sf_Z"] = np.array(list(table), np.int32)
        out["sf_f"] = np.array([table[Z] for Z in table], np.float64)
    out["params_json"] = np.array(json.dumps(p.as_dict()))
    out["meta_json"] = np.array(json.dumps(meta))
    out["case_json"] = np.array(json.dumps({k: v for k, v in case.items()}))
    return out


def qsc_case():
    """readFile on a hand-written .qsc + .cfg (tests/golden/qsc/): the MULS
    fields it derives and the atoms of readUnitCell, with the input texts,
    to pin qstem_gb300.qsc.read_qsc."""
    src = os.path.join(HERE, "qsc")
    work = tempfile.mkdtemp(prefix="qs_golden_")
    try:
        for f in ("run.qsc", "cell.cfg"):
            shutil.copy(os.path.join(src, f), work)
        dump = os.path.join(work, "dump")
        oracle.run_reference(os.path.join(work, "run.qsc"), dump, run=True)
        meta = dict(l.split(" = ", 1) for l in open(os.path.join(dump, "meta.txt")).read().strip().split("\n"))
        out = {"atoms": np.fromfile(os.path.join(dump, "atoms.bin"), dtype=abi.ATOM_DTYPE),
               "meta_json": np.array(json.dumps(meta)),
               "qsc_text": np.array(open(os.path.join(src, "run.qsc")).read()),
               "cfg_text": np.array(open(os.path.join(src, "cell.cfg")).read())}
        # the run: detector images of every thickness slot and the .img
        # files saveSTEMImages wrote (name, thickness, sampling, comment)
        nt = (int(meta["slices"]) * int(meta["cellDiv"])) // int(meta["outputInterval"]) + 1
        nd, sx, sy = int(meta["detectorNum"]), int(meta["scanXN"]), int(meta["scanYN"])
        det = np.zeros((nt, nd, sx, sy), np.float32)
        for t in range(nt):
            for i in range(nd):
                det[t, i] = np.fromfile(os.path.join(dump, "det_%d_%d.bin" % (t, i)), np.float32).reshape(sx, sy)
        out["det"] = det
        files = sorted(f for f in os.listdir(os.path.join(work, "out")) if f.endswith(".img"))
        heads = {}
        for f in files:
            im = imageio.read_img(os.path.join(work, "out", f))
            heads[f] = [float(im.t), float(im.dx), float(im.dy), im.comment]
        out["img_headers_json"] = np.array(json.dumps(heads))
    finally:
        shutil.rmtree(work, ignore_errors=True)
    path = os.path.join(HERE, "qscread.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def qsc_geometry_case(name, qsc_file, cfg_file):
    """readFile on a hand-written input of tests/golden/qsc/ (crystal tilt,
    non-orthogonal cells, "Cube:" boxes): the MULS fields it derives and the
    atoms readUnitCell builds, with the input texts."""
    src = os.path.join(HERE, "qsc")
    work = tempfile.mkdtemp(prefix="qs_golden_")
    try:
        for f in (qsc_file, cfg_file):
            shutil.copy(os.path.join(src, f), work)
        dump = os.path.join(work, "dump")
        oracle.run_reference(os.path.join(work, qsc_file), dump, run=True)
        meta = dict(l.split(" = ", 1) for l in open(os.path.join(dump, "meta.txt")).read().strip().split("\n"))
        out = {"atoms": np.fromfile(os.path.join(dump, "atoms.bin"), dtype=abi.ATOM_DTYPE),
               "meta_json": np.array(json.dumps(meta)),
               "qsc_text": np.array(open(os.path.join(src, qsc_file)).read()),
               "cfg_name": np.array(cfg_file),
               "cfg_text": np.array(open(os.path.join(src, cfg_file)).read())}
        # doSTEM's detector images of every thickness slot
        nt = (int(meta["slices"]) * int(meta["cellDiv"])) // int(meta["outputInterval"]) + 1
        nd, sx, sy = int(meta["detectorNum"]), int(meta["scanXN"]), int(meta["scanYN"])
        out["det"] = np.stack([np.stack([np.fromfile(os.path.join(dump, "det_%d_%d.bin" % (t, i)), np.float32)
                                         .reshape(sx, sy) for i in range(nd)]) for t in range(nt)])
    finally:
        shutil.rmtree(work, ignore_errors=True)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes", len(out["atoms"]), "atoms")


GEOMETRY_CASES = {"qsctilt": ("tilt.qsc", "hex.cfg"), "qsccube": ("cube.qsc", "cell.cfg"),
                  "qscdat": ("dat.qsc", "cell.dat"), "qsccssr": ("cssr.qsc", "cell.cssr")}


def phonon_modes_fixture():
    """The phonon file of tests/golden/qsc/phonon.qsc: a 2-atom cell (Al, N
    masses) at 4 k-points, seeded eigenvectors (unit length per mode), the
    three modes at k = 0 acoustic (omega 0)."""
    from qstem_gb300 import thermal
    rng = np.random.default_rng(20261203 + 400)
    Nk, Ns = 4, 2
    m = 3 * Ns
    kv = np.array([[0, 0, 0], [0.5, 0, 0], [0, 0.25, 0.5], [0.25, 0.25, 0.25]], np.float32)
    om = rng.uniform(3.0, 30.0, (Nk, m)).astype(np.float32)
    om[0, :3] = 0.0
    e = rng.standard_normal((Nk, m, m, 2))
    e /= np.sqrt((e ** 2).sum(axis=(2, 3), keepdims=True))
    return thermal.PhononModes(np.array([26.98, 14.007], np.float32), kv, om, e.astype(np.float32))


# readFile and doSTEM with thermal displacements at a fixed reference clock
# (the reference seeds them with time(NULL)): qsc file, its other inputs
THERMAL_CLOCK = 1764000000
THERMAL_CASES = {"qsctds": ("tds.qsc", ["vac.cfg"]), "qscphonon": ("phonon.qsc", ["ph.cfg", "modes.phonon"]),
                  "qsctdscube": ("tdscube.qsc", ["vac.cfg"])}


def qsc_thermal_case(name, qsc_file, others):
    """readFile's atoms (thermal displacements and vacancies of the first
    run), doSTEM's detector images (those of the last run: collectIntensity
    overwrites them, Navg being 0) and its per-position patterns averaged
    over the runs (diffAvg_<ix>_<iy>.img), with the reference's clock fixed."""
    from qstem_gb300 import thermal
    src = os.path.join(HERE, "qsc")
    if "modes.phonon" in others:
        thermal.write_phonon_file(os.path.join(src, "modes.phonon"), phonon_modes_fixture())
    work = tempfile.mkdtemp(prefix="qs_golden_")
    try:
        for f in [qsc_file] + others:
            shutil.copy(os.path.join(src, f), work)
        dump = os.path.join(work, "dump")
        oracle.run_reference(os.path.join(work, qsc_file), dump, run=True, clock=THERMAL_CLOCK)
        meta = dict(l.split(" = ", 1) for l in open(os.path.join(dump, "meta.txt")).read().strip().split("\n"))
        out = {"atoms": np.fromfile(os.path.join(dump, "atoms.bin"), dtype=abi.ATOM_DTYPE),
               "meta_json": np.array(json.dumps(meta)), "clock": np.array(THERMAL_CLOCK)}
        nt = (int(meta["slices"]) * int(meta["cellDiv"])) // int(meta["outputInterval"]) + 1
        nd, sx, sy = int(meta["detectorNum"]), int(meta["scanXN"]), int(meta["scanYN"])
        out["det"] = np.stack([np.stack([np.fromfile(os.path.join(dump, "det_%d_%d.bin" % (t, i)), np.float32)
                                         .reshape(sx, sy) for i in range(nd)]) for t in range(nt)])
        out["diffavg"] = np.stack([np.stack([imageio.read_img(os.path.join(work, "out", "diffAvg_%d_%d.img" % (ix, iy)))
                                             .data.astype(np.float32) for iy in range(sy)]) for ix in range(sx)])
    finally:
        shutil.rmtree(work, ignore_errors=True)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes", len(out["atoms"]), "atoms")

# whole stem3 runs whose output folders pin qstem_gb300.qsc.run_qsc: every
# .img file the reference wrote (name, header, data)
RUN_CASES = {
    # CBED with a thickness series (diff_<t>.img, save level 1) and diffAvg_1.img
    "qsccbed": dict(cell="si", ncell=(4, 3, 3), nx=64, resolutionX=0.06788, v0=300.0, slices=5,
                    sliceThickness=2.0, scan=None, detectors=[], alpha=10.0, Cs_mm=1.2, defocus_nm=-60.0,
                    bandlimit=True, outputInterval=2, mode="CBED", saveLevel=1),
    # CBED at save level 3: wave_probe.img, wave_final.img, and the patterns
    # that runMulsSTEM's real-space collectIntensity overwrites
    "qsccbed3": dict(cell="si", ncell=(4, 3, 3), nx=64, resolutionX=0.06788, v0=300.0, slices=4,
                     sliceThickness=2.0, scan=None, detectors=[], alpha=10.0, Cs_mm=1.2, defocus_nm=-60.0,
                     bandlimit=True, outputInterval=3, mode="CBED", saveLevel=3),
    # TEM: interimWave's wave_<t>.img and the exit wave wave.img
    "qsctem": dict(cell="si", ncell=(4, 3, 4), nx=64, resolutionX=0.06, v0=300.0, slices=7, sliceThickness=2.0,
                   scan=None, detectors=[], alpha=0.0, Cs_mm=1.2, defocus_nm=-60.0, bandlimit=True,
                   outputInterval=3, mode="TEM", saveLevel=0),
    # TEM with a tilted incident beam (and the exit wave tilted back)
    "qsctemtilt": dict(cell="si", ncell=(4, 3, 3), nx=64, resolutionX=0.06, v0=300.0, slices=5, sliceThickness=2.0,
                       scan=None, detectors=[], alpha=0.0, Cs_mm=1.2, defocus_nm=-60.0, bandlimit=True,
                       outputInterval=2, mode="TEM", saveLevel=0,
                       extra=["Beam tilt X: 0.004", "Beam tilt Y: 0.2 deg", "Tilt back: yes"]),
    # CBED from a probe source of finite size: doCBED's source offset, drawn
    # with the reference's clock-seeded generator (fixed here)
    "qsccbedsrc": dict(cell="si", ncell=(4, 3, 3), nx=64, resolutionX=0.06788, v0=300.0, slices=5,
                       sliceThickness=2.0, scan=None, detectors=[], alpha=10.0, Cs_mm=1.2, defocus_nm=-60.0,
                       bandlimit=True, outputInterval=2, mode="CBED", saveLevel=1,
                       extra=["Source Size (diameter): 0.9"], clock=1764000000),
    # stacking sequences "sequence: m1 m2": each slab's stack m1 times in a
    # row, the slab loop m2 times.  CBED at save level 1 (k-space patterns,
    # their stale thicknesses) and 3 (interimWave and the real-space
    # collectIntensity at absolute_slice*(1 + repeat), files past the
    # thickness slots), TEM, STEM through two unequal slabs at save level 1
    "qsccbedseq": dict(cell="si", ncell=(4, 3, 2), nx=64, resolutionX=0.06788, v0=300.0, slices=3,
                       sliceThickness=2.0, scan=None, detectors=[], alpha=10.0, Cs_mm=1.2, defocus_nm=-60.0,
                       bandlimit=True, outputInterval=2, mode="CBED", saveLevel=1, sequence=(2, 2)),
    "qsccbedseq3": dict(cell="si", ncell=(4, 3, 2), nx=64, resolutionX=0.06788, v0=300.0, slices=3,
                        sliceThickness=2.0, scan=None, detectors=[], alpha=10.0, Cs_mm=1.2, defocus_nm=-60.0,
                        bandlimit=True, outputInterval=2, mode="CBED", saveLevel=3, sequence=(2, 2)),
    "qsctemseq": dict(cell="si", ncell=(4, 3, 2), nx=64, resolutionX=0.06, v0=300.0, slices=4, sliceThickness=2.0,
                      scan=None, detectors=[], alpha=0.0, Cs_mm=1.2, defocus_nm=-60.0, bandlimit=True,
                      outputInterval=3, mode="TEM", saveLevel=0, sequence=(3, 2)),
    # CBED through two unequal slabs (NCELLZ: 3/2): every slab's stack
    "qsccbedd2u": dict(cell="si", ncell=(4, 3, 3), nx=64, resolutionX=0.06788, v0=300.0, slices=3,
                       sliceThickness=2.0, scan=None, detectors=[], alpha=10.0, Cs_mm=1.2, defocus_nm=-60.0,
                       bandlimit=True, outputInterval=2, mode="CBED", saveLevel=1, cellDiv=2),
    # TEM through two equal slabs (NCELLZ: 4/2, slab 0's stack reused)
    "qsctemd2": dict(cell="si", ncell=(4, 3, 4), nx=64, resolutionX=0.06, v0=300.0, slices=4,
                     sliceThickness=float(np.float32(np.float32(4 * 5.431 / np.sqrt(2)) / np.float32(8))),
                     scan=None, detectors=[], alpha=0.0, Cs_mm=1.2, defocus_nm=-60.0, bandlimit=True,
                     outputInterval=3, mode="TEM", saveLevel=0, cellDiv=2),
    # STEM at save level 2: per-position diffAvg_ix_iy.img and mulswav_ix_iy.img
    "qscstem": dict(cell="sto", ncell=(3, 3, 4), nx=64, resolutionX=0.0915, v0=200.0, slices=8,
                    sliceThickness=1.9525, scan=(3.905, 7.81, 2, 3.905, 7.81, 2),
                    detectors=[(0.0, 20.0, "BF"), (40.0, 90.0, "HAADF")], alpha=20.0, outputInterval=4,
                    mode="STEM", saveLevel=2),
    # STEM through a stacking sequence over two equal slabs
    "qscstemseq": dict(cell="sto", ncell=(3, 3, 4), nx=64, resolutionX=0.0915, v0=200.0, slices=4,
                       sliceThickness=1.9525, scan=(3.905, 7.81, 2, 3.905, 7.81, 2),
                       detectors=[(0.0, 20.0, "BF"), (40.0, 90.0, "HAADF")], alpha=20.0, outputInterval=2,
                       mode="STEM", saveLevel=1, cellDiv=2, sequence=(2, 2)),
}


def qsc_run_case(name, case):
    """The reference run end to end on a .qsc written for `case`; stores the
    input texts and every .img file of its output folder."""
    work = tempfile.mkdtemp(prefix="qs_golden_")
    try:
        cell = cell_of(case["cell"])
        config.write_cfg(cell, os.path.join(work, "cell.cfg"))
        qsc = os.path.join(work, "run.qsc")
        config.write_qsc(qsc, cfg_file="cell.cfg", ncell=case["ncell"], nx=case["nx"],
                         resolutionX=case["resolutionX"], v0=case["v0"], slices=case["slices"],
                         sliceThickness=case["sliceThickness"], scan=case["scan"], detectors=case["detectors"],
                         alpha=case["alpha"], Cs_mm=case.get("Cs_mm", 0.0), defocus_nm=case.get("defocus_nm", 0.0),
                         outputInterval=case.get("outputInterval"), mode=case["mode"],
                         bandlimit=case.get("bandlimit", False), folder="out", saveLevel=case["saveLevel"],
                         cellDiv=case.get("cellDiv", 1), sequence=case.get("sequence", (1, 1)))
        if case.get("extra"):
            with open(qsc, "a") as f:
                f.write("\n".join(case["extra"]) + "\n")
        oracle.run_reference(qsc, os.path.join(work, "dump"), run=True, clock=case.get("clock"))
        out = {"qsc_text": np.array(open(qsc).read()),
               "cfg_text": np.array(open(os.path.join(work, "cell.cfg")).read())}
        if case.get("clock") is not None:
            out["clock"] = np.array(case["clock"])
        heads = {}
        for f in sorted(os.listdir(os.path.join(work, "out"))):
            if not f.endswith(".img"):
                continue
            im = imageio.read_img(os.path.join(work, "out", f))
            heads[f] = [float(im.t), float(im.dx), float(im.dy), im.comment, [float(v) for v in im.params]]
            d = im.data
            out["img_" + f] = (np.stack([d.real, d.imag], -1) if np.iscomplexobj(d) else d).astype(np.float32)
        out["img_headers_json"] = np.array(json.dumps(heads))
    finally:
        shutil.rmtree(work, ignore_errors=True)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes", sorted(heads))


def main(names=None):
    if not os.environ.get("QS_REFERENCE_DIR"):
        raise SystemExit("set QS_REFERENCE_DIR to the reference checkout")
    oracle.build(quiet=False)
    if not names or "qscread" in names:
        qsc_case()
    for name, case in RUN_CASES.items():
        if not names or name in names:
            qsc_run_case(name, case)
    for name, (q, c) in GEOMETRY_CASES.items():
        if not names or name in names:
            qsc_geometry_case(name, q, c)
    for name, (q, others) in THERMAL_CASES.items():
        if not names or name in names:
            qsc_thermal_case(name, q, others)
    for name, case in CASES.items():
        if names and name not in names:
            continue
        work = tempfile.mkdtemp(prefix="qs_golden_")
        try:
            out = run_case(name, case, work)
        finally:
            shutil.rmtree(work, ignore_errors=True)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **out)
        print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(sys.argv[1:])
