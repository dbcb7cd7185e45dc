"""An unmodified stem3 input run end to end through the library
(qstem_gb300.qsc.run_qsc): the detector images of every thickness slot
against the reference's own run of the same .qsc/.cfg (tests/golden/
qscread.npz: readFile, doSTEM through two slabs, saveSTEMImages), and the
.img files it writes against the names and headers the reference wrote;
whole output folders of CBED, TEM and STEM runs at several save levels
(tests/golden/qsc*.npz).
Tolerance 1e-4 relative L2 (complex FP32 slice loops on both sides)."""
import json
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2
from qstem_gb300 import imageio, qsc

pytestmark = pytest.mark.gpu


def test_stem3_input_end_to_end():
    z = np.load(os.path.join(GOLDEN, "qscread.npz"))
    d = tempfile.mkdtemp()
    for name, key in (("run.qsc", "qsc_text"), ("cell.cfg", "cfg_text")):
        with open(os.path.join(d, name), "w") as f:
            f.write(str(z[key]))
    out = qsc.run_qsc(os.path.join(d, "run.qsc"), folder=os.path.join(d, "out"))
    ref = z["det"]
    assert list(out) == ["adf", "bf"]
    for i, name in enumerate(out):
        assert out[name].shape == ref[:, i].shape
        assert rel_l2(out[name], ref[:, i]) <= 1e-4, name
    heads = json.loads(str(z["img_headers_json"]))
    written = sorted(os.listdir(os.path.join(d, "out")))
    # the cell is divided into slabs, so doSTEM also wrote every position's
    # exit wave (mulswav_<ix>_<iy>.img: names and headers pinned here)
    assert written == sorted(heads)
    for fn, (t, dx, dy, comment) in heads.items():
        im = imageio.read_img(os.path.join(d, "out", fn))
        assert np.float32(im.t) == np.float32(t) and np.float32(im.dx) == np.float32(dx), fn
        assert np.float32(im.dy) == np.float32(dy) and im.comment == comment, fn
        if fn.startswith("mulswav"):
            continue
        stem = fn[:-4].split("_")
        slot = int(stem[1]) if len(stem) > 1 else ref.shape[0] - 1
        assert rel_l2(im.data, ref[slot, ["adf", "bf"].index(stem[0])]) <= 1e-4, fn


# this library's own addition to the TEM output folder (the reference stops
# before it writes its averages)
EXTRA = {"qsctem": {"waveIntensity.img"}, "qsctemtilt": {"waveIntensity.img"}, "qsctemd2": {"waveIntensity.img"},
         "qsctemseq": {"waveIntensity.img"}}


@pytest.mark.parametrize("name", ["qsccbed", "qsccbed3", "qsccbedsrc", "qsccbedd2u", "qsctem", "qsctemtilt",
                                  "qsctemd2", "qscstem", "qsccbedseq", "qsccbedseq3", "qsctemseq", "qscstemseq"])
def test_output_folder_matches_the_references(name):
    """The whole output folder of a stem3 run: CBED thickness series
    (diff_<t>.img) at save level 1 and 3 (real-space overwrite, interimWave,
    probe and final wave), TEM interimWave series and exit wave, STEM
    per-position patterns and exit waves at save level 2 -- every file the
    reference wrote, with its header (thickness, sampling, comment,
    parameters) and data."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = tempfile.mkdtemp()
    for fn, key in (("run.qsc", "qsc_text"), ("cell.cfg", "cfg_text")):
        with open(os.path.join(d, fn), "w") as f:
            f.write(str(z[key]))
    # a case made at a fixed reference clock (CBED source offsets) runs with
    # the reference's generator
    kw = {"rng": "reference", "clock": int(z["clock"])} if "clock" in z.files else {}
    qsc.run_qsc(os.path.join(d, "run.qsc"), folder=os.path.join(d, "out"), **kw)
    heads = json.loads(str(z["img_headers_json"]))
    written = set(os.listdir(os.path.join(d, "out")))
    assert written == set(heads) | EXTRA.get(name, set())
    for fn, (t, dx, dy, comment, params) in heads.items():
        im = imageio.read_img(os.path.join(d, "out", fn))
        assert np.float32(im.t) == np.float32(t), (fn, im.t, t)
        assert np.float32(im.dx) == np.float32(dx) and np.float32(im.dy) == np.float32(dy), (fn, im.dx, dx)
        assert im.comment == comment, (fn, im.comment)
        if comment == "STEM image":
            # [runs, error, image2...]: the reference's threads share the sum
            # image2 squares, so only its run count is reproducible
            assert im.params[0] == params[0], fn
        else:
            np.testing.assert_allclose(im.params, params, rtol=1e-6, err_msg=fn)
        data = im.data
        if np.iscomplexobj(data):
            data = np.stack([data.real, data.imag], -1)
        assert rel_l2(data, z["img_" + fn]) <= 1e-4, fn


@pytest.mark.parametrize("name", ["qsctilt", "qsccube", "qscdat", "qsccssr"])
def test_tilted_and_boxed_crystals_end_to_end(name):
    """A non-orthogonal cell tilted about x and y, and a Cube box cut from a
    crystal tilted about x and z: run_qsc's detector images of every
    thickness slot against the reference's doSTEM on the same input."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = tempfile.mkdtemp()
    for fn, text in (("run.qsc", str(z["qsc_text"])), (str(z["cfg_name"]), str(z["cfg_text"]))):
        with open(os.path.join(d, fn), "w") as f:
            f.write(text)
    out = qsc.run_qsc(os.path.join(d, "run.qsc"), folder=os.path.join(d, "out"))
    ref = z["det"]
    assert out["adf"].shape == ref[:, 0].shape
    assert rel_l2(out["adf"], ref[:, 0]) <= 1e-4


def test_custom_scattering_factors_end_to_end(tmp_path):
    """A doCBED input with "Structure Factors: custom" (the table spread
    over lines with comments): the slices built from it on the GPU
    (qs_slices_build_custom) and the final pattern against the reference's
    own run."""
    from conftest import Golden, custom_qsc
    path, out = custom_qsc(tmp_path, split=True)
    res = qsc.run_qsc(path, folder=out)
    assert rel_l2(res["diffpat"], Golden("sto64ft")["cbed_diffpat"]) <= 1e-4
