"""GPU library (through the C ABI) against the oracle and against the
reference's own outputs (golden fixtures).

Tolerances (relative L2 unless noted):
  LUT, potential, transmission  1e-5   (FP64 table build; float atomics)
  probe                         1e-5
  detectors / diffraction patterns / exit waves after the slice loop
                                1e-4   (the contract's bound for the
                                        complex-FP32 multislice)
"""
import numpy as np
import pytest

from conftest import Golden, rel_l2, scan_stack
from oracle import oracle
from qstem_gb300 import config, lib

pytestmark = pytest.mark.gpu

TOL_BUILD = 1e-5
TOL_MS = 1e-4


@pytest.fixture(scope="module")
def ctx():
    oracle.build()
    c = lib.Context(0)
    yield c
    c.close()


def _B(g, Z, charged):
    a = g["atoms"]
    sel = a[(a["Znum"] == Z) & ((a["q"] != 0) if charged else True)]
    return 0.0 if (g.params.tds or len(sel) == 0) else float(sel["dw"][0])


def test_lut_vs_oracle_and_reference(ctx, golden):
    p = golden.params
    for k in golden.keys():
        if not (k.startswith("lut_") or k.startswith("lutq_")):
            continue
        Z = int(k.split("_")[1])
        charged = k.startswith("lutq_")
        B = _B(golden, Z, charged)
        gpu, ns = ctx.lut(p, Z, B, charged)
        cpu, _ = oracle.lut(p, Z, B, charged)
        assert ns == int(golden["nzsub"])
        assert rel_l2(gpu, cpu) <= TOL_BUILD, k
        assert rel_l2(gpu, golden[k]) <= TOL_BUILD, k


def test_potential_and_transmission(ctx, golden):
    p = golden.params
    V = ctx.slices(p, golden["atoms"], potential_only=True)
    assert rel_l2(V, golden["V"]) <= TOL_BUILD
    T = ctx.slices(p, golden["atoms"])
    assert rel_l2(T, golden["T"]) <= TOL_BUILD
    # |t| = 1 without band limit
    if not p.bandlimittrans:
        assert np.abs(np.hypot(T[..., 0], T[..., 1]) - 1).max() < 1e-5


def test_probe(ctx, golden):
    p = golden.params
    pr = ctx.probe(p)
    assert rel_l2(pr, golden["probe"]) <= TOL_BUILD
    assert rel_l2(pr, oracle.probe(p)) <= TOL_BUILD
    assert abs(np.sum(pr.astype(np.float64) ** 2) / (p.nx * p.ny) - 1) < 1e-5


def test_multislice_vs_reference(ctx, golden):
    if "det" not in golden:
        pytest.skip("case does not run the scan")
    p = golden.params
    T, slabs = scan_stack(golden)
    det, dps, ews = ctx.multislice(p, T, golden["probe"], want_diffpats=True, want_exit_waves=True,
                                   slab_stacks=slabs)
    assert rel_l2(det, golden["det"]) <= TOL_MS
    ocd, ocp, ocw = oracle.stem(p, T, golden["probe"], diffpats=True, exit_waves=True, slab_stacks=slabs)
    assert rel_l2(det, ocd) <= TOL_MS
    assert rel_l2(dps, ocp) <= TOL_MS
    assert rel_l2(ews, ocw) <= TOL_MS
    for k in golden.keys():
        if k.startswith("diffpat_") or k.startswith("wave_"):
            ix, iy = map(int, k.split("_")[1:])
            pos = ix * p.scanYN + iy
            mine = dps[pos] if k.startswith("diffpat_") else ews[pos]
            assert rel_l2(mine, golden[k]) <= TOL_MS, k


@pytest.mark.parametrize("name", ["sto64d2", "sto64d2u"])
def test_slabs_from_atoms(ctx, name):
    """Cells divided into slabs (NCELLZ n/2): every slab's stack against the
    reference's, and qs_stem_run (atoms in, detector images out: slab 0 reused
    for equal divisions, every slab built otherwise) against the reference's
    detector images of every thickness slot."""
    g = Golden(name)
    p = g.params
    refs = g["T_slabs"] if "T_slabs" in g else [g["T"]]
    for k, ref in enumerate(refs):
        assert rel_l2(ctx.slices(p, g["atoms"], slab=k), ref) <= TOL_BUILD, k
    det = ctx.stem_run(p, g["atoms"])
    assert det.shape == g["det"].shape
    assert rel_l2(det, g["det"]) <= TOL_MS


def test_2d_potential_from_atoms(ctx):
    """The periodic 2-D potential (potential3D: no; make3DSlices' 2-D branch
    with getAtomPotential2D's tables): qs_stem_run from atoms against the
    reference's detector images, and a 256^2 stack of 1,000 atoms against the
    oracle's; the non-periodic 2-D branch is refused."""
    g = Golden("sto64p2d")
    p = g.params
    det = ctx.stem_run(p, g["atoms"])
    assert rel_l2(det, g["det"]) <= TOL_MS
    cell = config.srtio3_cell()
    atoms, ax, by, c = config.replicate(cell, 5, 5, 10)
    q = config.make_params(nx=256, resolutionX=0.0763, v0=200, slices=20, sliceThickness=1.9525, ax=ax, by=by, c=c,
                           scan=(7.81, 11.715, 2, 7.81, 11.715, 2), detectors=[(70, 200, "HAADF")], alpha=20,
                           periodicXY=True, potential3D=False)
    V = ctx.slices(q, atoms, potential_only=True)
    Vo = oracle.potential(q, atoms)
    assert rel_l2(V, Vo) <= TOL_BUILD
    q.nonPeriod = 1
    with pytest.raises(lib.QsError):
        ctx.slices(q, atoms, potential_only=True)


def test_custom_scattering_factors(ctx):
    """make3DSlicesFT (custom scattering factors; qs_slices_build_custom)
    against the reference's own doCBED run of it: potential, transmission, and
    the CBED pattern through the GPU's stack; an element without a table is
    refused."""
    g = Golden("sto64ft")
    p = g.params
    args = (g["atoms"], g["sf_k"], g["sf_Z"], g["sf_f"])
    V = ctx.slices_custom(p, *args, potential_only=True)
    assert rel_l2(V, g["V"]) <= TOL_BUILD
    T = ctx.slices_custom(p, *args)
    assert rel_l2(T, g["T"]) <= TOL_BUILD
    dx = float(np.float32(p.scanXStart) - np.float32(p.potOffsetX))
    dy = float(np.float32(p.scanYStart) - np.float32(p.potOffsetY))
    pr = ctx.probe(p, dx, dy)
    z = np.zeros(1, np.int32)
    _, dps, _ = ctx.multislice(p, T, pr, positions=(z, z, z, z), want_det=False, want_diffpats=True)
    assert rel_l2(dps[0], g["cbed_diffpat"]) <= TOL_MS
    with pytest.raises(lib.QsError):
        ctx.slices_custom(p, g["atoms"], g["sf_k"], g["sf_Z"][:2], g["sf_f"][:2])


def test_end_to_end_from_atoms(ctx):
    """atoms -> slices -> probe -> scan entirely on the GPU vs the oracle chain."""
    g = Golden("sto64")
    p = g.params
    T = ctx.slices(p, g["atoms"])
    det, _, _ = ctx.multislice(p, T)
    To = oracle.transmission(p, oracle.potential(p, g["atoms"]))
    dco, _, _ = oracle.stem(p, To)
    assert rel_l2(det, dco) <= TOL_MS
    assert rel_l2(det, g["det"]) <= TOL_MS


def sto_case(nx, res, slices, ncell, scan_px, dets, v0=200.0, alpha=20.0, out_every=None, periodic=False):
    cell = config.srtio3_cell()
    atoms, ax, by, c = config.replicate(cell, *ncell)
    a = 3.905
    x0 = a * (ncell[0] // 2)
    y0 = a * (ncell[1] // 2)
    p = config.make_params(nx=nx, resolutionX=res, v0=v0, slices=slices, sliceThickness=1.9525, ax=ax, by=by,
                           c=c, scan=(x0, x0 + a, scan_px, y0, y0 + a, scan_px), detectors=dets, alpha=alpha,
                           outputInterval=out_every, periodicXY=periodic)
    return p, atoms


@pytest.mark.parametrize("nx,res,ncell", [(256, 0.0763, (5, 5, 4)), (128, 0.0915, (4, 4, 4)),
                                          (384, 0.0763, (7, 7, 3)), (512, 0.07627, (10, 10, 2)),
                                          (768, 0.0763, (15, 15, 2)), (1024, 0.0763, (20, 20, 2))])
def test_larger_grids_vs_oracle(ctx, nx, res, ncell):
    """Every line length the slice loop has a transform for, radix-3 ones
    (384 = 8*6*8, 768 = 8*12*8) included, through both passes, the detector
    sums, the patterns and the exit waves."""
    dets = [(0, 10, "BF"), (10, 25, "LA"), (25, 70, "MA"), (70, 200, "HAADF")]
    p, atoms = sto_case(nx, res, 2 * ncell[2], ncell, 2, dets, out_every=3)
    T = ctx.slices(p, atoms)
    To = oracle.transmission(p, oracle.potential(p, atoms))
    assert rel_l2(T, To) <= TOL_BUILD
    det, dps, ews = ctx.multislice(p, To, want_diffpats=True, want_exit_waves=True)
    dco, dpo, ewo = oracle.stem(p, To, diffpats=True, exit_waves=True)
    assert rel_l2(det, dco) <= TOL_MS
    assert rel_l2(dps, dpo) <= TOL_MS
    assert rel_l2(ews, ewo) <= TOL_MS


def test_bandlimited_cbed(ctx):
    g = Golden("si64cbed")
    p = g.params
    T = ctx.slices(p, g["atoms"])
    assert rel_l2(T, g["T"]) <= TOL_BUILD
    # one CBED position at the window origin, diffraction pattern out
    pos = (np.zeros(1), np.zeros(1), np.zeros(1), np.zeros(1))
    _, dp, ew = ctx.multislice(p, g["T"], g["probe"], positions=pos, want_det=False, want_diffpats=True,
                               want_exit_waves=True)
    w, _, dpo = oracle.run_position(p, g["T"], 0, 0, g["probe"])
    assert rel_l2(dp[0], dpo) <= TOL_MS
    assert rel_l2(ew[0], w) <= TOL_MS


def test_collect_matches_oracle_semantics(ctx):
    g = Golden("sto64")
    p = g.params
    rng = np.random.default_rng(3)
    w = rng.standard_normal((p.nx, p.ny, 2)).astype(np.float32)
    sums, dp = ctx.collect(p, w, diffpat=True)
    I = (w[..., 0] * w[..., 0] + w[..., 1] * w[..., 1]).astype(np.float64)
    t = config  # noqa
    ax = np.float32(np.float32(p.resolutionX) * p.nx)
    k = np.arange(p.nx)
    kx = np.where(k > p.nx // 2, (k - p.nx).astype(np.float32) / ax, k.astype(np.float32) / ax).astype(np.float32)
    k2 = (kx[:, None] * kx[:, None] + (kx * kx)[None, :]).astype(np.float32)
    for d in range(p.detectorNum):
        m = (k2 >= np.float32(p.detectors[d].k2Inside)) & (k2 <= np.float32(p.detectors[d].k2Outside))
        assert abs(sums[d] - I[m].sum()) <= 1e-9 * I.sum()
    ref_dp = np.fft.fftshift(I) / np.sqrt(p.nx * p.ny)
    assert rel_l2(dp, ref_dp) <= 1e-6


def test_errors_are_codes_not_exits(ctx):
    g = Golden("sto64")
    p = g.params.copy()
    p.nx = p.ny = 100  # no FFT kernel for 100
    with pytest.raises(lib.QsError) as e:
        ctx.probe(p)
    assert e.value.code == -4
    p2 = g.params.copy()
    p2.slices = 0
    with pytest.raises(lib.QsError) as e:
        ctx.slices(p2, g["atoms"])
    assert e.value.code == -1


def test_thickness_series(ctx):
    """QS_SERIES: the pattern and real-space wave of every thickness slot
    (collectIntensity's diff_<t>.img, interimWave's wave_<t>.img) against
    the oracle run truncated after the slot's writer slice; the last slot
    is bit-identical to the final outputs of a run without the flag."""
    g = Golden("sto64")
    p = g.params
    T = g["T"]
    _, dps, ews = ctx.multislice(p, T, g["probe"], want_det=False, want_diffpats=True, want_exit_waves=True,
                                 series=True)
    nt = p.thickness_count()
    assert dps.shape == (nt, p.scanXN * p.scanYN, p.nx, p.ny) and ews.shape[:2] == dps.shape[:2]
    _, dpf, ewf = ctx.multislice(p, T, g["probe"], want_det=False, want_diffpats=True, want_exit_waves=True)
    np.testing.assert_array_equal(dps[-1], dpf)
    np.testing.assert_array_equal(ews[-1], ewf)
    S = p.slices
    for t in range(nt):
        a = min((t + 1) * p.outputInterval - 1, S - 2) if t < nt - 1 else S - 1
        q = p.copy()
        q.slices = q.outputInterval = a + 1
        _, dpo, ewo = oracle.stem(q, T[:a + 1], g["probe"], det=False, diffpats=True, exit_waves=True)
        assert rel_l2(dps[t], dpo) <= TOL_MS, t
        assert rel_l2(ews[t], ewo) <= TOL_MS, t
