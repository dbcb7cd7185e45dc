"""TEM (qs_tem_run): plane wave through frozen-phonon configurations, the
mean exit intensity and through-focus CTF images, against the reference's
exit wave (doTEM's wave.img, tests/golden/si64tem.npz) and the oracle
(oracle.tem: the C restatement's slice loop + a float64 restatement of
GUI_Matlab/simImageFromWave.m:57-73).

Tolerances: 1e-4 relative L2 (complex FP32 slice loops on both sides)."""
import numpy as np
import pytest

from conftest import Golden, rel_l2
from qstem_gb300 import lib

pytestmark = pytest.mark.gpu

TOL = 1e-4
CTF = dict(Cs=1.2e7, kmax=0.9, edge=0.05, alpha=1e-4, focalSpread=30.0, astig=20.0, astigPhi=0.5)
DEFOCI = [-600.0, 0.0, 300.0]


def displaced(atoms, sigma, seed):
    rng = np.random.default_rng(seed)
    a = atoms.copy()
    for k in ("x", "y", "z"):
        a[k] = (a[k].astype(np.float64) + rng.standard_normal(len(a)) * sigma).astype(np.float32)
    return a


@pytest.fixture(scope="module")
def case():
    from oracle import oracle
    oracle.build()
    g = Golden("si64tem")
    p = g.params
    configs = [g["atoms"]] + [displaced(g["atoms"], 0.05, 20261203 + 400 + j) for j in range(2)]
    ctx = lib.Context(0)
    out = ctx.tem(p, configs, ctf=CTF, defoci=DEFOCI, want_exit_waves=True)
    stacks = [oracle.transmission(p, oracle.potential(p, a)) for a in configs]
    ref = oracle.tem(p, stacks, CTF, DEFOCI)
    yield dict(g=g, p=p, out=out, ref=ref, ctx=ctx, configs=configs)
    ctx.close()


def test_exit_wave_matches_reference(case):
    _, _, ew = case["out"]
    assert rel_l2(ew[0], case["g"]["exit_wave"]) <= TOL


def test_exit_waves_and_mean_intensity_match_oracle(case):
    mean, _, ew = case["out"]
    rmean, _, rew = case["ref"]
    for k in range(len(ew)):
        assert rel_l2(ew[k], rew[k]) <= TOL, k
    assert rel_l2(mean, rmean) <= TOL


def test_ctf_images_match_oracle(case):
    _, imgs, _ = case["out"]
    _, rimgs, _ = case["ref"]
    assert imgs.shape == (len(DEFOCI), case["p"].nx, case["p"].ny)
    for d in range(len(DEFOCI)):
        assert rel_l2(imgs[d], rimgs[d]) <= TOL, DEFOCI[d]


def test_identity_transfer_gives_the_exit_intensity(case):
    mean, imgs, _ = case["ctx"].tem(case["p"], case["configs"], ctf={}, defoci=[0.0])
    assert rel_l2(imgs[0], mean) <= 1e-5


def _qsc_run(name):
    import os
    import tempfile
    from conftest import GOLDEN
    from qstem_gb300 import qsc
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = tempfile.mkdtemp()
    for fn, key in (("run.qsc", "qsc_text"), ("cell.cfg", "cfg_text")):
        with open(os.path.join(d, fn), "w") as f:
            f.write(str(z[key]))
    return qsc.read_qsc(os.path.join(d, "run.qsc")), z


def test_slabs_exit_wave_matches_reference(case):
    """A cell divided into two equal slabs (NCELLZ 4/2): qs_tem_run's exit
    wave against the reference's wave.img of the same input."""
    run, z = _qsc_run("qsctemd2")
    assert run.params.cellDiv == 2 and run.params.equalDivs
    _, _, ew = case["ctx"].tem(run.params, [run.atoms], want_exit_waves=True)
    assert rel_l2(ew[0], z["img_wave.img"]) <= TOL


def test_beam_tilt_exit_wave_matches_reference(case):
    """qs_tem_run_tilted: doTEM's tilted incident wave (beam tilt 0.004 rad
    and 0.2 degrees) through the reference's input; the exit wave against
    interimWave's wave_<last>.img (wave.img itself is tilted back)."""
    run, z = _qsc_run("qsctemtilt")
    assert run.beam_tilt[0] != 0 and run.beam_tilt[1] != 0
    _, _, ew = case["ctx"].tem(run.params, [run.atoms], want_exit_waves=True, beam_tilt=run.beam_tilt)
    assert rel_l2(ew[0], z["img_wave_2.img"]) <= TOL
    _, _, flat = case["ctx"].tem(run.params, [run.atoms], want_exit_waves=True)
    assert rel_l2(flat[0], z["img_wave_2.img"]) > 10 * TOL  # the tilt matters
