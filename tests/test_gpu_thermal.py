"""Frozen-phonon runs on the GPU reproduce the reference's runs made at a
fixed clock (tests/golden/qsctds, qscphonon): with the reference's own
generator, run_qsc draws readFile's atoms and the second run's redraw as
the reference does (Einstein displacements and vacancies in a
non-orthogonal cell; displacements from a phonon file).  The last run's
detector images (the reference keeps only the last run's: Navg stays 0)
and the per-position patterns averaged over the runs (diffAvg_<ix>_<iy>.img)
agree to 1e-4 relative L2."""
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2
from qstem_gb300 import imageio, lib, qsc

pytestmark = pytest.mark.gpu

CASES = {"qsctds": ("tds.qsc", ["vac.cfg"]), "qscphonon": ("phonon.qsc", ["ph.cfg", "modes.phonon"]),
         "qsctdscube": ("tdscube.qsc", ["vac.cfg"])}


class _Logged:
    """The library context, recording what each multislice call returned."""

    def __init__(self, ctx):
        self.ctx, self.log = ctx, []

    def __getattr__(self, name):
        return getattr(self.ctx, name)

    def multislice(self, *a, **k):
        out = self.ctx.multislice(*a, **k)
        self.log.append(out)
        return out


@pytest.fixture(scope="module")
def ctx():
    c = lib.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_thermal_runs_match_the_reference(tmp_path, ctx, name):
    q, others = CASES[name]
    for f in [q] + others:
        shutil.copy(os.path.join(GOLDEN, "qsc", f), tmp_path)
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    logged = _Logged(ctx)
    out = str(tmp_path / "out")
    qsc.run_qsc(str(tmp_path / q), ctx=logged, folder=out, rng="reference", clock=int(z["clock"]))
    assert len(logged.log) == 2
    assert rel_l2(logged.log[1][0][:, 0], z["det"][:, 0]) <= 1e-4
    sx, sy = z["diffavg"].shape[:2]
    for ix in range(sx):
        for iy in range(sy):
            got = imageio.read_img(os.path.join(out, "diffAvg_%d_%d.img" % (ix, iy))).data
            assert rel_l2(got, z["diffavg"][ix, iy]) <= 1e-4
