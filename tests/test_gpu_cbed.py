"""CBED batches (qs_cbed_batch_run) against the reference's doCBED pattern
(tests/golden/si64cbed.npz) and the oracle (the C restatement's probe and
slice loop): mixed grids, thicknesses and convergence angles in one call,
admission rounds under a memory cap, and the batch against single runs.

Tolerances: 1e-4 relative L2 against the reference and the oracle; 1e-6
between runs of the same instance (the slice builder's float atomics may
reorder last bits)."""
import numpy as np
import pytest

from conftest import Golden, rel_l2
from qstem_gb300 import abi, config, lib

pytestmark = pytest.mark.gpu

TOL = 1e-4


def cbed_job(cell, ncell, nx, slices, alpha, v0=200.0, **kw):
    atoms, ax, by, c = config.replicate(cell, *ncell)
    p = config.make_params(mode=abi.QS_MODE_CBED, nx=nx, resolutionX=float(np.float32(ax)) / nx,
                           resolutionY=float(np.float32(by)) / nx, v0=v0, slices=slices, sliceThickness=2.0, ax=ax,
                           by=by, c=c, scan=None, alpha=alpha, bandlimit=True, **kw)
    return p, atoms


def oracle_pattern(p, atoms):
    from oracle import oracle
    T = oracle.transmission(p, oracle.potential(p, atoms))
    dx = float(np.float32(p.scanXStart) - np.float32(p.potOffsetX))
    dy = float(np.float32(p.scanYStart) - np.float32(p.potOffsetY))
    return oracle.run_position(p, T, 0, 0, oracle.probe(p, dx, dy))[2]


@pytest.fixture(scope="module")
def ctx():
    from oracle import oracle
    oracle.build()
    c = lib.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def mixed():
    si, sto = config.diamond_cell(), config.srtio3_cell()
    return [cbed_job(si, (2, 2, 2), 64, 5, 10.0),
            cbed_job(si, (2, 2, 2), 64, 3, 15.0, Cs_mm=1.0, defocus_nm=-20.0),
            cbed_job(si, (2, 2, 2), 64, 7, 8.0),
            cbed_job(sto, (3, 3, 3), 64, 6, 20.0),
            cbed_job(sto, (4, 4, 2), 128, 4, 12.0)]


def test_pattern_matches_reference(ctx):
    g = Golden("si64cbed")
    (dp,), rep = ctx.cbed_batch([(g.params, g["atoms"])])
    assert rel_l2(dp, g["cbed_diffpat"]) <= TOL
    assert rep["groups"] == 1 and rep["rounds"] == 1


def test_mixed_batch_matches_oracle(ctx, mixed):
    dps, rep = ctx.cbed_batch(mixed)
    assert rep["groups"] == 2  # one batch per grid: 64^2 (4 instances of two samplings), 128^2
    for k, (p, atoms) in enumerate(mixed):
        assert dps[k].shape == (p.nx, p.ny)
        assert rel_l2(dps[k], oracle_pattern(p, atoms)) <= TOL, k


def test_batch_equals_single_runs(ctx, mixed):
    dps, _ = ctx.cbed_batch(mixed)
    for k, job in enumerate(mixed):
        (one,), _ = ctx.cbed_batch([job])
        assert rel_l2(one, dps[k]) <= 1e-6, k


def test_admission_rounds_under_a_memory_cap(ctx, mixed):
    ref, rep0 = ctx.cbed_batch(mixed)
    assert rep0["rounds"] == 1
    # a cap below the whole set's footprint (~2.3 MiB): the 64^2 batch is
    # split into units that fit, and the rounds take them one after another
    cap = 1 << 20
    dps, rep = ctx.cbed_batch(mixed, max_bytes=cap)
    assert rep["rounds"] > 1 and rep["admitted_bytes"] <= cap
    for k in range(len(mixed)):
        assert rel_l2(dps[k], ref[k]) <= 1e-6, k


def test_instance_larger_than_the_cap_is_rejected(ctx, mixed):
    with pytest.raises(lib.QsError) as e:
        ctx.cbed_batch(mixed, max_bytes=100 << 10)
    assert e.value.code == abi.QS_ERR_NOMEM


def test_slabs_pattern_matches_reference(ctx):
    """Two unequal slabs (NCELLZ 3/2): every slab built from its shifted
    atoms; the pattern against the reference's diffAvg_1.img, alone and in
    a batch with an undivided instance of the same grid."""
    import os
    import tempfile
    from conftest import GOLDEN
    from qstem_gb300 import qsc
    z = np.load(os.path.join(GOLDEN, "qsccbedd2u.npz"))
    d = tempfile.mkdtemp()
    for fn, key in (("run.qsc", "qsc_text"), ("cell.cfg", "cfg_text")):
        with open(os.path.join(d, fn), "w") as f:
            f.write(str(z[key]))
    run = qsc.read_qsc(os.path.join(d, "run.qsc"))
    p = run.params
    assert p.cellDiv == 2 and not p.equalDivs
    p.dE_E = np.float32(run.spread[0])
    ref = z["img_diffAvg_1.img"]
    (dp,), _ = ctx.cbed_batch([(p, run.atoms)])
    assert rel_l2(dp, ref) <= TOL
    q = p.copy()
    q.cellDiv = 1
    (dp2, dq), _ = ctx.cbed_batch([(p, run.atoms), (q, run.atoms)])
    assert rel_l2(dp2, ref) <= TOL
    (dq1,), _ = ctx.cbed_batch([(q, run.atoms)])
    assert rel_l2(dq, dq1) <= 1e-6
