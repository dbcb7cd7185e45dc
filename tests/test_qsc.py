"""Reading unmodified stem3 inputs (qstem_gb300.qsc): the .qsc/.cfg pair in
tests/golden/qsc/ against what the reference's own readFile derived from it
(tests/golden/qscread.npz), and the fixtures' inputs read back."""
import json
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES, Golden
from qstem_gb300 import abi, config, qsc

F32 = np.float32


def _write(texts):
    d = tempfile.mkdtemp()
    for name, text in texts.items():
        with open(os.path.join(d, name), "w") as f:
            f.write(text)
    return d


@pytest.fixture(scope="module")
def pinned():
    z = np.load(os.path.join(GOLDEN, "qscread.npz"))
    d = _write({"run.qsc": str(z["qsc_text"]), "cell.cfg": str(z["cfg_text"])})
    return qsc.read_qsc(os.path.join(d, "run.qsc")), json.loads(str(z["meta_json"])), z["atoms"]


def test_params_match_the_references_readfile(pinned):
    run, meta, _ = pinned
    p = run.params
    for k, v in meta.items():
        if k.startswith("det"):
            continue
        if k == "avgRuns":
            assert run.avg_runs == int(v)
        elif k == "natom":
            assert len(run.atoms) == int(v)
        elif k in ("ax", "by", "c"):
            assert F32(getattr(p, k)) == F32(float(v)), k
        else:
            got = getattr(p, k)
            if isinstance(got, int):
                assert got == int(v), k
            else:
                assert F32(got) == F32(float(v)), (k, got, v)
    assert p.detectorNum == int(meta["detectorNum"])
    for i in range(p.detectorNum):
        want = [F32(float(t)) for t in meta["det%d" % i].split()]
        d = p.detectors[i]
        assert [F32(d.rInside), F32(d.rOutside), F32(d.k2Inside), F32(d.k2Outside), F32(d.shiftX),
                F32(d.shiftY)] == want
    assert run.detector_names == ["adf", "bf"]


def test_atoms_match_the_references_readunitcell(pinned):
    run, _, atoms = pinned
    assert run.atoms.dtype == abi.ATOM_DTYPE
    assert np.array_equal(run.atoms, atoms)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_fixture_inputs_read_back(name):
    """The .qsc each fixture was made from (config.write_qsc) reads back to
    the fixture's params and atoms."""
    g = Golden(name)
    case = g.case
    from tests.golden import make_golden  # noqa: F401  (path set up by conftest)
    cell, atoms, p = make_golden.params_for(case)
    d = tempfile.mkdtemp()
    config.write_cfg(cell, os.path.join(d, "cell.cfg"))
    config.write_qsc(os.path.join(d, "run.qsc"), cfg_file="cell.cfg", ncell=case["ncell"], nx=case["nx"],
                     resolutionX=case["resolutionX"], v0=case["v0"], slices=case["slices"],
                     sliceThickness=case["sliceThickness"], scan=case["scan"], detectors=case["detectors"],
                     alpha=case["alpha"], Cs_mm=case.get("Cs_mm", 0.0), defocus_nm=case.get("defocus_nm", 0.0),
                     outputInterval=case.get("outputInterval"), mode=case["mode"],
                     bandlimit=case.get("bandlimit", False), periodicXY=case.get("periodicXY", False),
                     czOffset=case.get("czOffset", 0.0), centerSlices=case.get("centerSlices", False),
                     cellDiv=case.get("cellDiv", 1), potential3D=case.get("potential3D", True))
    run = qsc.read_qsc(os.path.join(d, "run.qsc"))
    for f, _ in abi.QsParams._fields_:
        # equalDivs means nothing for an undivided cell (and older fixtures
        # predate the field)
        if f == "detectors" or (f == "equalDivs" and g.params.cellDiv == 1):
            continue
        if f.startswith("mulsRepeat"):  # 0 (fixtures older than the field) reads as 1
            assert max(1, getattr(run.params, f)) == max(1, getattr(g.params, f)), (name, f)
            continue
        assert getattr(run.params, f) == getattr(g.params, f), (name, f)
    assert np.array_equal(run.atoms, g["atoms"])


def test_refused_inputs():
    z = np.load(os.path.join(GOLDEN, "qscread.npz"))
    base = str(z["qsc_text"])
    for extra in ("potential3D: no", "mode: NBED", "sequence: 0 1", "sequence: 1 1\nsequence: 2 1"):
        text = base.replace("print level: 1", extra + "\nprint level: 1")
        if extra.startswith("potential3D"):
            # the 2-D potential on a non-periodic array (the periodic one runs)
            text = base.replace("potential3D: yes", extra).replace("periodicXY: yes", "periodicXY: no")
        if extra.startswith("mode"):
            text = base.replace("mode: STEM", extra)
        if extra.startswith("sequence"):
            text = base.replace("sequence: 1 1", extra)
        d = _write({"run.qsc": text, "cell.cfg": str(z["cfg_text"])})
        with pytest.raises(NotImplementedError):
            qsc.read_qsc(os.path.join(d, "run.qsc"))
    # doSTEM continues a second pass from wave files it writes only at save
    # level > 1 or with slabs
    text = base.replace("sequence: 1 1", "sequence: 1 2").replace("NCELLZ: 4/2", "NCELLZ: 4")
    d = _write({"run.qsc": text, "cell.cfg": str(z["cfg_text"])})
    with pytest.raises(NotImplementedError):
        qsc.read_qsc(os.path.join(d, "run.qsc"))
    text = base.replace("sequence: 1 1", "sequence: 2 3")
    d = _write({"run.qsc": text, "cell.cfg": str(z["cfg_text"])})
    run = qsc.read_qsc(os.path.join(d, "run.qsc"))
    assert (run.params.mulsRepeat1, run.params.mulsRepeat2) == (2, 3)


def test_energy_spread_series_and_einstein_sigma(pinned):
    s = qsc._energy_spread_series(1e-5, 5)
    assert s[0] == 0.0 and len(s) == 5
    assert s[1] > 0 and s[2] == -s[1] and s[3] > s[1] and s[4] == -s[3]
    run, _, _ = pinned
    sig = run.einstein_sigma()
    dw = run.atoms["dw"].astype(np.float64)
    assert np.allclose(sig, np.sqrt(290 / 300.0) * np.sqrt(dw / (8 * np.pi ** 2)) / np.sqrt(3))


def test_seeded_vacancies():
    cell = config.UnitCell(4.0, 4.0, 4.0, [(8, 0, 0, 0, 0.5, 0.5, 0), (14, 0.5, 0.5, 0.5, 0.5, 1.0, 0),
                                           (26, 0.25, 0.25, 0.25, 0.5, 0.3, 0), (28, 0.25, 0.25, 0.25, 0.5, 0.7, 0)])
    atoms, *_ = config.replicate(cell, 10, 10, 10)
    a = qsc.draw_vacancies(atoms, 7)
    assert np.array_equal(a, qsc.draw_vacancies(atoms, 7))
    kept_o = np.mean(a["Znum"][atoms["Znum"] == 8] == 8)
    assert 0.4 < kept_o < 0.6
    assert np.all(a["Znum"][atoms["Znum"] == 14] == 14)
    # a shared Fe/Ni site keeps exactly one of the two
    fe, ni = atoms["Znum"] == 26, atoms["Znum"] == 28
    assert np.sum(a["Znum"][fe] == 26) + np.sum(a["Znum"][ni] == 28) == np.sum(fe)


def _read_geometry(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = _write({"run.qsc": str(z["qsc_text"]), str(z["cfg_name"]): str(z["cfg_text"])})
    return qsc.read_qsc(os.path.join(d, "run.qsc")), json.loads(str(z["meta_json"])), z["atoms"]


@pytest.mark.parametrize("name", ["qsctilt", "qsccube", "qscdat", "qsccssr"])
def test_tilted_and_boxed_crystals_match_the_references_readfile(name):
    """Crystal tilt about x and y of a non-orthogonal cell replicated in
    NCELL mode, a "Cube:" box cut from a crystal tilted about x and z (with
    centre slices and no slice thickness), and .dat / .cssr unit cells: the
    atoms readUnitCell / tiltBoxed produce, bit for bit, and the fields
    readFile derives."""
    run, meta, atoms = _read_geometry(name)
    assert len(run.atoms) == len(atoms) == int(meta["natom"])
    for k in ("x", "y", "z", "dw", "occ", "Znum"):
        np.testing.assert_array_equal(run.atoms[k], atoms[k], err_msg=k)
    if name == "qsccssr":
        # readNextCSSRAtom never sets the charge (libs/fileio_fftw3.cpp:
        # 1034-1039): the reference's are whatever the buffer held; 0 here
        assert np.all(run.atoms["q"] == 0) and np.abs(atoms["q"]).max() < 1e-6
    else:
        np.testing.assert_array_equal(run.atoms["q"], atoms["q"])
    p = run.params
    for k, v in meta.items():
        if k.startswith("det") or k in ("natom", "avgRuns"):
            continue
        got = getattr(p, k)
        if isinstance(got, int):
            assert got == int(v), k
        else:
            assert F32(got) == F32(float(v)), (k, got, v)


def test_param_file_arrays_read_as_readarray():
    """readArray (stem3/stem3.cpp:531-549): numbers after the title, running
    on over following lines (comments cut, blank lines skipped), each read as
    atof reads it; a missing title gives None, a file that ends first an
    error."""
    d = _write({"a.qsc": "x: 1\nk: 1 2.5e-1   % three of five\n\n% note\n  -3 4x .5\nO: 7\n"})
    pf = qsc.ParamFile(os.path.join(d, "a.qsc"))
    np.testing.assert_array_equal(pf.array("k:", 5), [1.0, 0.25, -3.0, 4.0, 0.5])
    np.testing.assert_array_equal(pf.array("O:", 1), [7.0])
    assert pf.array("Sr:", 3) is None
    pf.pos = 0
    with pytest.raises(ValueError):
        pf.array("k:", 9)
    assert qsc._atof("1e3x") == 1000.0 and qsc._atof("abc") == 0.0 and qsc._atof("-.5e-1") == -0.05
