"""Host logic of qstem_gb300.qsc.run_qsc on the CPU: the files a stem3 run
writes (names, headers, data) and the averaging over frozen-phonon runs,
with the oracle standing in for the GPU library (tests/oracle_ctx.py).

The folders are pinned against the reference's own runs (tests/golden/
qsc*.npz); the oracle is bit-exact with the reference on these cases, so
data agree to 1e-6 relative L2.  The multi-run cases check the averages
against the per-run results the stand-in logged."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, custom_qsc, rel_l2
from oracle import oracle
from oracle_ctx import OracleContext
from qstem_gb300 import imageio, qsc

EXTRA = {"qsctem": {"waveIntensity.img"}, "qsctemtilt": {"waveIntensity.img"}, "qsctemd2": {"waveIntensity.img"},
         "qsctemseq": {"waveIntensity.img"}}


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    oracle.build()


def _inputs(tmp_path, name, edit=None):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    texts = {"run.qsc": str(z["qsc_text"]), "cell.cfg": str(z["cfg_text"])}
    if edit:
        texts = edit(texts)
    for fn, text in texts.items():
        (tmp_path / fn).write_text(text)
    return z, str(tmp_path / "run.qsc"), str(tmp_path / "out")


def _read(folder, fn):
    im = imageio.read_img(os.path.join(folder, fn))
    d = im.data
    return im, (np.stack([d.real, d.imag], -1) if np.iscomplexobj(d) else d)


@pytest.mark.parametrize("name", ["qsccbed", "qsccbed3", "qsccbedsrc", "qsccbedd2u", "qsctem", "qsctemtilt",
                                  "qsctemd2", "qscstem", "qsccbedseq", "qsccbedseq3", "qsctemseq", "qscstemseq"])
def test_output_folder_as_the_reference_writes_it(tmp_path, name):
    z, path, out = _inputs(tmp_path, name)
    # a case made at a fixed reference clock runs with the reference's generator
    kw = {"rng": "reference", "clock": int(z["clock"])} if "clock" in z.files else {}
    qsc.run_qsc(path, ctx=OracleContext(), folder=out, **kw)
    heads = json.loads(str(z["img_headers_json"]))
    assert set(os.listdir(out)) == set(heads) | EXTRA.get(name, set())
    for fn, (t, dx, dy, comment, params) in heads.items():
        im, data = _read(out, fn)
        assert (np.float32(im.t), np.float32(im.dx), np.float32(im.dy)) == (
            np.float32(t), np.float32(dx), np.float32(dy)), fn
        assert im.comment == comment, fn
        if comment != "STEM image":
            np.testing.assert_allclose(im.params, params, rtol=1e-6, err_msg=fn)
        assert rel_l2(data, z["img_" + fn]) <= 1e-6, fn


@pytest.mark.parametrize("name", ["qsccbed", "qsccbed3", "qsccbedd2u", "qsctem", "qsctemtilt", "qsctemd2"])
def test_step_chaining_writes_the_same_folder(tmp_path, monkeypatch, name):
    """The path run_qsc takes for stacking sequences -- every file's last
    write found step by step, the wave run in stretches between those steps
    -- on the cases without repeats: the same folder as the reference's."""
    monkeypatch.setattr(qsc, "_ALWAYS_CHAIN", True)
    test_output_folder_as_the_reference_writes_it(tmp_path, name)


def _tds(runs, save_level):
    def edit(texts):
        q = texts["run.qsc"].replace("tds: no", "tds: yes\ntemperature: 300")
        q = q.replace("Runs for averaging: 1", "Runs for averaging: %d" % runs)
        q = "\n".join("save level: %d" % save_level if l.startswith("save level:") else l for l in q.split("\n"))
        # a Debye-Waller factor, so that the Einstein displacements are not zero
        c = texts["cell.cfg"].replace(" 0.0 1.0 0.0", " 0.5 1.0 0.0")
        return {"run.qsc": q, "cell.cfg": c}
    return edit


def _running_mean(values):
    avg = values[0]
    for j, v in enumerate(values[1:], 1):
        avg = ((np.float32(j) * avg + v) / np.float32(j + 1)).astype(np.float32)
    return avg


def test_cbed_runs_averaged(tmp_path):
    _, path, out = _inputs(tmp_path, "qsccbed", _tds(3, 2))
    ctx = OracleContext()
    res = qsc.run_qsc(path, ctx=ctx, folder=out)
    series = [entry for kind, entry in ctx.log if kind == "series"]
    assert len(series) == 3
    # save level 2: the patterns are the real-space intensities of the waves
    finals = [qsc._kspace_pattern(ew[-1, 0], 1 / 64.0) for _, _, ew in series]
    assert rel_l2(finals[1], finals[0]) > 1e-3  # the runs differ
    files = set(os.listdir(out))
    # diffAvg_2 stays (run index 2 is a multiple of the save level), diffAvg_1 does not
    assert {"diffAvg_2.img", "diffAvg_3.img"} <= files and "diffAvg_1.img" not in files
    im, data = _read(out, "diffAvg_3.img")
    assert im.comment == "Averaged Diffraction pattern, unit: 1/A"
    np.testing.assert_array_equal(data, _running_mean(finals))
    np.testing.assert_allclose(data, np.mean(finals, 0), rtol=1e-5, atol=1e-6 * np.abs(data).max())
    np.testing.assert_array_equal(res["diffpat"], data)
    lines = open(os.path.join(out, "avgresults.dat")).read().split("\n")
    assert [l.split()[0] for l in lines if l] == ["1", "2"]
    # thickness series averaged over the runs; interimWave per run with tds
    for t in range(3):
        im, data = _read(out, "diff_%d.img" % t)
        assert im.comment == "Average Array"
        pats = [qsc._kspace_pattern(ew[t, 0], 1 / 64.0) for _, _, ew in series]
        np.testing.assert_array_equal(data, _running_mean(pats))
    for j in range(3):
        for f in range(3):
            assert "wave_%d_%d.img" % (j, f) in files


def test_tem_runs_averaged(tmp_path):
    _, path, out = _inputs(tmp_path, "qsctem", _tds(2, 0))
    ctx = OracleContext()
    res = qsc.run_qsc(path, ctx=ctx, folder=out)
    waves = [entry[2][-1, 0].astype(np.float64) for kind, entry in ctx.log if kind == "series"]
    assert len(waves) == 2
    mean = np.mean([w[..., 0] ** 2 + w[..., 1] ** 2 for w in waves], 0)
    im, data = _read(out, "waveIntensity.img")
    assert im.params[0] == 2 and rel_l2(data, mean) <= 1e-6
    assert rel_l2(res["exit_intensity"], mean) <= 1e-6
    im, data = _read(out, "wave.img")
    assert im.comment == "Test wave function for run 0" and rel_l2(data, waves[0]) <= 1e-6
    files = set(os.listdir(out))
    assert {"wave_%d_%d.img" % (j, f) for j in range(2) for f in range(3)} <= files


def test_stem_position_patterns_averaged(tmp_path):
    _, path, out = _inputs(tmp_path, "qscstem", _tds(2, 1))
    ctx = OracleContext()
    qsc.run_qsc(path, ctx=ctx, folder=out, chunk=3)  # two chunks of the 2 x 2 raster
    runs = [entry for kind, entry in ctx.log if kind == "multislice"]
    assert len(runs) == 4  # 2 runs x 2 chunks
    pats = [np.concatenate([runs[2 * j][1], runs[2 * j + 1][1]]) for j in range(2)]
    assert rel_l2(pats[1], pats[0]) > 1e-4
    for k, (ix, iy) in enumerate([(0, 0), (0, 1), (1, 0), (1, 1)]):
        im, data = _read(out, "diffAvg_%d_%d.img" % (ix, iy))
        assert im.comment == "Average Array"
        np.testing.assert_array_equal(data, _running_mean([pats[0][k], pats[1][k]]))
    # save level 1, one slab: no exit waves
    assert not any(f.startswith("mulswav") for f in os.listdir(out))


@pytest.mark.parametrize("name", ["qsctilt", "qsccube", "qscdat", "qsccssr"])
def test_tilted_and_boxed_crystals_through_the_oracle(tmp_path, name):
    """The detector images of the tilted / boxed inputs through the oracle
    stand-in match the reference's doSTEM (the atom front end feeds the
    slice builder what readUnitCell feeds make3DSlices)."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    (tmp_path / "run.qsc").write_text(str(z["qsc_text"]))
    (tmp_path / str(z["cfg_name"])).write_text(str(z["cfg_text"]))
    out = qsc.run_qsc(str(tmp_path / "run.qsc"), ctx=OracleContext(), folder=str(tmp_path / "out"))
    assert rel_l2(out["adf"], z["det"][:, 0]) <= 1e-6


def test_step_helpers_reduce_to_the_plain_slot_rule():
    """Without repeats the steps are the absolute slices and the file writes
    found step by step are the plain slot rule's last writers; with repeats
    collectIntensity's index and interimWave's part ways once a pass starts
    past slice 0 (totalSliceCount > 0)."""
    from qstem_gb300 import config
    p = config.make_params(nx=64, resolutionX=0.1, v0=200, slices=5, sliceThickness=2.0, ax=6.4, by=6.4, c=10.0,
                           outputInterval=2, scan=(3.2, 3.2, 1, 3.2, 3.2, 1))
    p.cellDiv = 2
    steps = qsc._steps(p)
    assert [s[4] for s in steps] == list(range(10)) and all(s[2] == s[3] == s[4] for s in steps)
    nT, SA = p.thickness_count(), 10
    ev, NS = qsc._wave_events(p, True, True)
    writers = qsc._slot_writers(SA, 2, nT)
    for t, a in enumerate(writers):
        if a >= 0:
            assert ev[("diff", t)][:2] == ("r", a)
    assert {f for (k, f) in ev if k == "wave"} == set(qsc._interim_files(SA, 2))
    p.mulsRepeat1, p.mulsRepeat2 = 2, 2
    steps = qsc._steps(p)
    assert len(steps) == 2 * 2 * 2 * 5
    # second repeat of the second pass: index 5 + 2i against (5 + i) * 2
    s = [st for st in steps if st[4] == 5 + 3][1]
    assert (s[2], s[3]) == (5 + 3 * 2, (5 + 3) * 2)


@pytest.mark.parametrize("split", [False, True])
def test_custom_scattering_factors_read_and_run(tmp_path, split):
    """A "Structure Factors: custom" table read as readSFactLUT reads it (k,
    then one array per element kind in the cell's order, running on over
    lines), and a CBED run built from it (make3DSlicesFT through the
    stand-in): the final pattern against the reference's doCBED run."""
    from conftest import Golden
    g = Golden("sto64ft")
    path, out = custom_qsc(tmp_path, split)
    run = qsc.read_qsc(path)
    k, Z, f = run.custom_sf
    np.testing.assert_array_equal(k, g["sf_k"])
    np.testing.assert_array_equal(Z, g["sf_Z"])
    np.testing.assert_array_equal(f, g["sf_f"])
    res = qsc.run_qsc(path, ctx=OracleContext(), folder=out)
    assert rel_l2(res["diffpat"], g["cbed_diffpat"]) <= 1e-5


def test_custom_scattering_factors_refused_or_missing(tmp_path):
    path, _ = custom_qsc(tmp_path)
    text = open(path).read()
    # an element kind without its table: the reference exits
    open(path, "w").write("\n".join(l for l in text.split("\n") if not l.startswith("Ti:")))
    with pytest.raises(ValueError):
        qsc.read_qsc(path)
    # a divided cell in CBED mode
    open(path, "w").write(text.replace("NCELLZ: 2", "NCELLZ: 2/2"))
    with pytest.raises(NotImplementedError):
        qsc.read_qsc(path)
    # STEM and TEM read the table and keep the parameterised potential
    open(path, "w").write(text.replace("mode: CBED", "mode: TEM"))
    assert qsc.read_qsc(path).custom_sf is not None
