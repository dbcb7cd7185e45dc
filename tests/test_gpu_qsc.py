"""An unmodified stem3 input run end to end through the library
(qstem_gb300.qsc.run_qsc): the detector images of every thickness slot
against the reference's own run of the same .qsc/.cfg (tests/golden/
qscread.npz: readFile, doSTEM through two slabs, saveSTEMImages), and the
.img files it writes against the names and headers the reference wrote.
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
    heads = {k: v for k, v in json.loads(str(z["img_headers_json"])).items() if not k.startswith("mulswav")}
    written = sorted(os.listdir(os.path.join(d, "out")))
    assert written == sorted(heads)
    for fn, (t, dx, dy, comment) in heads.items():
        im = imageio.read_img(os.path.join(d, "out", fn))
        assert np.float32(im.t) == np.float32(t) and np.float32(im.dx) == np.float32(dx), fn
        assert np.float32(im.dy) == np.float32(dy) and im.comment == comment, fn
        stem = fn[:-4].split("_")
        slot = int(stem[1]) if len(stem) > 1 else ref.shape[0] - 1
        assert rel_l2(im.data, ref[slot, ["adf", "bf"].index(stem[0])]) <= 1e-4, fn
