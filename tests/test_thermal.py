"""Thermal displacements and vacancies (qstem_gb300.thermal) against the
reference's own draws.

The reference seeds its thermal displacements with its clock
(-time(NULL), libs/fileio_fftw3.cpp:496).  The fixtures qsctds / qscphonon
were made by the reference with time() fixed (oracle/fixed_clock.c): its
readFile atoms (Einstein displacements plus vacancy draws in a
non-orthogonal cell, in NCELL mode and in a tilted "Cube:" box;
displacements from a phonon file), its doSTEM images
(those of the last run: Navg stays 0, so collectIntensity overwrites them)
and its per-position patterns averaged over two runs.  read_qsc with the
reference generator at that clock must give readFile's atoms bit for bit,
and run_qsc the same runs (through the oracle here; on the GPU in
test_gpu_thermal.py)."""
import os
import shutil

import numpy as np
import pytest

from conftest import rel_l2
from oracle_ctx import OracleContext
from qstem_gb300 import config, qsc, thermal

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
CASES = {"qsctds": ("tds.qsc", ["vac.cfg"]), "qscphonon": ("phonon.qsc", ["ph.cfg", "modes.phonon"]),
         "qsctdscube": ("tdscube.qsc", ["vac.cfg"])}


def _inputs(tmp_path, name):
    q, others = CASES[name]
    for f in [q] + others:
        shutil.copy(os.path.join(GOLDEN, "qsc", f), tmp_path)
    return str(tmp_path / q), np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.mark.parametrize("name", sorted(CASES))
def test_reference_generator_gives_readfiles_atoms(tmp_path, name):
    path, z = _inputs(tmp_path, name)
    run = qsc.read_qsc(path, rng="reference", clock=int(z["clock"]))
    assert np.array_equal(run.atoms, z["atoms"])
    # the displacements are there: the undisplaced cell differs
    plain = qsc.read_qsc(path)
    assert np.abs(plain.atoms["x"] - z["atoms"]["x"]).max() > 1e-3
    # another clock, other draws
    other = qsc.read_qsc(path, rng="reference", clock=int(z["clock"]) + 1)
    assert not np.array_equal(other.atoms, z["atoms"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_runs_reproduce_the_references_stem_run(tmp_path, name):
    """run_qsc with the reference generator, through the oracle: run 1
    redraws the atoms as make3DSlices re-reads them; the per-position
    patterns averaged over both runs and the last run's detector images
    equal the reference's."""
    path, z = _inputs(tmp_path, name)
    ctx = OracleContext()
    out = str(tmp_path / "out")
    qsc.run_qsc(path, ctx=ctx, folder=out, rng="reference", clock=int(z["clock"]))
    runs = [entry for kind, entry in ctx.log if kind == "multislice"]
    assert len(runs) == 2
    assert rel_l2(runs[1][0][:, 0], z["det"][:, 0]) <= 1e-5
    assert rel_l2(runs[0][0][:, 0], z["det"][:, 0]) > 1e-3  # run 0 differs: other draws
    from qstem_gb300 import imageio
    sx, sy = z["diffavg"].shape[:2]
    for ix in range(sx):
        for iy in range(sy):
            got = imageio.read_img(os.path.join(out, "diffAvg_%d_%d.img" % (ix, iy))).data
            assert rel_l2(got, z["diffavg"][ix, iy]) <= 1e-5


def test_generator_restarts_and_shares_its_table():
    g = thermal.RefRandom()
    a = [-5]
    u = [g.ran1(a) for _ in range(5)]
    assert all(0.0 < v < 1.0 for v in u) and len(set(u)) == 5
    assert thermal.RefRandom().ran1([-5]) == u[0]  # the seed decides the sequence
    # a second caller with a negative seed restarts the shared table
    assert g.ran1([-5]) == u[0]
    # gasdev: the spare deviate is the first one's partner, stored as a float
    g = thermal.RefRandom()
    s = [-7]
    n0, n1 = g.gasdev(s), g.gasdev(s)
    assert n1 == float(np.float32(n1)) and n0 != n1


def test_phonon_file_round_trip(tmp_path):
    m = thermal.read_phonon_file(os.path.join(GOLDEN, "qsc", "modes.phonon"))
    assert (m.nk, m.ns) == (4, 2)
    thermal.write_phonon_file(str(tmp_path / "m.phonon"), m)
    assert (tmp_path / "m.phonon").read_bytes() == open(os.path.join(GOLDEN, "qsc", "modes.phonon"), "rb").read()
    w = m.amplitudes(300.0)
    assert np.all(w[0, :3] == 0) and np.all(w[1:] > 0)  # acoustic modes at k = 0 carry nothing
    assert np.all(m.amplitudes(0.0)[1:] < w[1:])  # zero-point motion only
    with open(tmp_path / "short.phonon", "wb") as f:
        f.write(open(os.path.join(GOLDEN, "qsc", "modes.phonon"), "rb").read()[:100])
    with pytest.raises(ValueError):
        thermal.read_phonon_file(str(tmp_path / "short.phonon"))


def test_numpy_generator_phonon_runs(tmp_path):
    """A phonon file with the default (numpy) generator: run j's atoms
    depend on the seed and j only, runs differ, and the displacements are of
    the modes' size."""
    path, z = _inputs(tmp_path, "qscphonon")
    run = qsc.read_qsc(path, seed=3)
    assert run.replicator is not None and run.replicator.rng == "numpy"
    a1 = qsc._run_atoms(run, 1, 3)
    assert np.array_equal(a1, qsc._run_atoms(qsc.read_qsc(path, seed=3), 1, 3))
    assert not np.array_equal(a1, run.atoms)
    undisplaced, *_ = config.supercell(run.cell, *run.ncell)
    dx = a1["x"].astype(np.float64) - undisplaced["x"]
    assert 0.01 < np.sqrt(np.mean(dx ** 2)) < 1.0


def test_missing_phonon_file_leaves_the_einstein_model(tmp_path):
    path, z = _inputs(tmp_path, "qscphonon")
    os.remove(str(tmp_path / "modes.phonon"))
    run = qsc.read_qsc(path, rng="reference", clock=int(z["clock"]))
    assert run.replicator.modes is None
    assert not np.array_equal(run.atoms, z["atoms"])


def test_replication_without_draws_is_the_plain_supercell():
    cell = config.srtio3_cell(dw=0.5)
    frac = config.sorted_fractional(cell)
    r = thermal.Replicator(frac, (3, 2, 2), cell.H, (cell.a, cell.b, cell.c), tds=False, temperature=300,
                           rng="reference", clock=5)
    got, *_ = config.supercell(cell, 3, 2, 2, replicated=r.configuration(0))
    want, *_ = config.supercell(cell, 3, 2, 2)
    assert np.array_equal(got, want)
    with pytest.raises(ValueError):
        r.configuration(2)  # the reference generator draws in order
