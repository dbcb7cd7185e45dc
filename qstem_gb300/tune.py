"""Autotune the slice-loop kernels per line length: the factorisation of the
row and of the column transforms, the column-pass tile, the row-pass shape
and the register budgets (CTAs per SM).

    python -m qstem_gb300.tune [--candidates 1,2,3,4,6,8] [--sizes 256,384,...] [--write]

Phase 0, factorisations and tiles: variant k compiles every line length
with its k-th factorisation (QS_RADIX_ROW_<N> = QS_RADIX_COL_<N> = k, where
that length has a k-th one that fits the thread layout of its row or column
lines; qs_fft.cuh lists them), plus one variant with
16-column tiles wherever the double-buffered tile fits (QS_COL_TILE_<N>);
the row transform keeps the factorisation with the fastest row pass, the
column transform the one with the fastest column pass, independently.

Phase 1, row and column passes: for each candidate budget k and row-pass
shape L (line transforms per CTA, --lines) the slice-loop translation unit
(qs_multislice.cu, qs_rows.cu) is compiled with every QS_ROW_LINES_<N> = L and
QS_ROW_MIN_BLOCKS_<N> = QS_COL_MIN_BLOCKS_<N> = k and linked with the other
objects of the normal build into a variant library in a temporary folder
(the candidates compile in parallel).  Each variant times, in a fresh
process on the GPU, the row and column passes of every line length through
the library's own CUDA-event counters (qs_ctx_profile / qs_ctx_stats): a
random slice stack of 8 slices, 1024 waves at 256^2 down to 128 at 1024^2,
best of 4.  Phase 2, row adjoint: the row and column tables fixed at the
phase-1 winners, qs_adjoint.cu is compiled with every
QS_ADJ_MIN_BLOCKS_<N> = k and the whole adjoint (every state kept) is timed
per size with CUDA events.  The fastest candidate per pass and size is
printed and, with --write, stored in csrc/qs_tuned.h (then rebuild).  Needs
nvcc and a GPU.
"""
import argparse
import concurrent.futures
import json
import os
import subprocess
import sys
import tempfile

from . import build as _build

SIZES = (256, 384, 512, 768, 1024)
WAVES = {64: 2048, 128: 2048, 256: 1024, 384: 512, 512: 512, 768: 192, 1024: 128}
# factorisations per line length (the lists of qs_fft.cuh's Line / LineCol)
RADIX_LISTS = {384: [(8, 6, 8), (6, 8, 8), (8, 8, 6), (12, 4, 8), (24, 4, 4), (8, 48), (48, 8)],
               512: [(32, 16), (16, 32)],
               768: [(8, 12, 8), (12, 8, 8), (8, 8, 12), (24, 4, 8), (24, 8, 4), (16, 48), (48, 16)],
               1024: [(32, 32), (8, 16, 8)]}
RADIX_ALTS = {n: len(v) for n, v in RADIX_LISTS.items()}
# threads per row / column line of the lengths whose layout qs_tuned.h sets
# (QS_LINE_T_<N>, QS_COL_LINE_T_<N>); the others: qs_fft.cuh's line_threads
ROW_T = {384: 8, 768: 16}
COL_T = {384: 8, 768: 16}


def _line_threads(n, col=False):
    t = (COL_T if col else ROW_T).get(n)
    return t if t else (8 if n <= 128 else 16 if n <= 512 else 32)


def radix_ok(n, k, col=False):
    """Factorisation k of length n fits its thread layout (every radix
    divides the elements a thread holds)."""
    e = n // _line_threads(n, col)
    return k < RADIX_ALTS.get(n, 1) and all(e % r == 0 for r in RADIX_LISTS[n][k])
# lengths whose double-buffered 16-column tile fits in shared memory
TILE16 = (64, 128, 256, 384, 512, 768)


# the slice-loop translation units (row pass, column pass and transforms)
SLICE_LOOP = ("qs_multislice.cu", "qs_rows.cu")


def _variant(tag, sources, defs, tmp, extra_objs=()):
    """Compile `sources` (one name or several) with -D`defs` and link them
    with the normal build's other objects (or `extra_objs` in their place)
    into a variant library.  Returns (library, [objects])."""
    sources = [sources] if isinstance(sources, str) else list(sources)
    replaced = {os.path.basename(o).split("@")[0] for o in extra_objs} | set(sources)
    objs = [os.path.join(_build.BUILD, s.replace(".cu", ".o")) for s in _build.SOURCES if s not in replaced]
    built = []
    for source in sources:
        obj = os.path.join(tmp, "%s@%s.o" % (source, tag))
        cmd = ([_build.nvcc()] + _build.ARCH + _build.FLAGS + ["-D" + d for d in defs] +
               ["-c", os.path.join(_build.SRC, source), "-o", obj])
        subprocess.run(cmd, check=True, capture_output=True)
        built.append(obj)
    lib = os.path.join(tmp, "libqstem_gpu_%s.so" % tag)
    subprocess.run([_build.nvcc()] + _build.ARCH + ["-shared", "-o", lib] + built + list(extra_objs) + objs +
                   ["-lcudart"], check=True, capture_output=True)
    return lib, built


def measure(lib_path, sizes, reps=4):
    """{N: (row, col) microseconds per position-slice} of one library build."""
    import numpy as np
    import torch
    from . import config, lib
    lib.load(lib_path)
    ctx = lib.Context(0)
    out = {}
    try:
        for n in sizes:
            dx = 0.05
            ax = n * dx * 1.2
            p = config.make_params(nx=n, resolutionX=dx, v0=200, slices=8, sliceThickness=2.0, ax=ax, by=ax, c=16.0,
                                   scan=(ax / 2, ax / 2 + 0.5, 4, ax / 2, ax / 2 + 0.5, 4),
                                   detectors=[(70, 200, "A")], alpha=20)
            ph = np.random.default_rng(1).standard_normal((p.slices, p.potNx, p.potNy)).astype(np.float32) * 0.3
            T = torch.from_numpy(np.stack([np.cos(ph), np.sin(ph)], -1)).cuda()
            probe = torch.from_numpy(ctx.probe(p)).cuda()
            nw = WAVES[n]
            z = np.zeros(nw, np.int32)
            pos = (z, z, z, z)
            ctx.multislice(p, T, probe, positions=pos, want_det=False)
            best = None
            for _ in range(reps):
                ctx.profile(True)
                ctx.multislice(p, T, probe, positions=pos, want_det=False, sync=False)
                st = ctx.stats()
                ctx.profile(False)
                r = st["row_ms"] / st["row_launches"] * 1e3 / nw
                c = st["col_ms"] / st["col_launches"] * 1e3 / nw
                best = (r, c) if best is None or r + c < sum(best) else best
            out[n] = best
    finally:
        ctx.close()
    return out


def measure_adjoint(lib_path, sizes, reps=3):
    """{N: ms} of the adjoint (every state kept) of one library build."""
    import numpy as np
    import torch
    from . import config, lib
    lib.load(lib_path)
    ctx = lib.Context(0)
    out = {}
    try:
        stream = torch.cuda.ExternalStream(ctx.stream_handle)
        for n in sizes:
            dx = 0.05
            ax = n * dx * 1.2
            side = {64: 32, 128: 32, 256: 32, 384: 16, 512: 16, 768: 8, 1024: 8}[n]
            p = config.make_params(nx=n, resolutionX=dx, v0=200, slices=8, sliceThickness=2.0, ax=ax, by=ax, c=16.0,
                                   scan=(ax / 2, ax / 2 + 0.5, side, ax / 2, ax / 2 + 0.5, side), detectors=[],
                                   alpha=20)
            ph = np.random.default_rng(1).standard_normal((p.slices, p.potNx, p.potNy)).astype(np.float32) * 0.3
            T = torch.from_numpy(np.stack([np.cos(ph), np.sin(ph)], -1)).cuda()
            probe = torch.from_numpy(ctx.probe(p)).cuda()
            target = torch.rand((side * side, n, n), device="cuda")
            ctx.adjoint(p, T, probe, target, ckpt=1)
            best = None
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                e0.record(stream)
                ctx.adjoint(p, T, probe, target, ckpt=1)
                e1.record(stream)
                torch.cuda.synchronize()
                t = e0.elapsed_time(e1)
                best = t if best is None else min(best, t)
            out[n] = best
    finally:
        ctx.close()
    return out


MACRO = {"LINES": "QS_ROW_LINES_%d", "RROW": "QS_RADIX_ROW_%d", "RCOL": "QS_RADIX_COL_%d",
         "TILE": "QS_COL_TILE_%d", "STAGES": "QS_COL_STAGES_%d"}


def write_table(best):
    """Store the chosen values ({(kind, N): k}, kind one of ROW, COL, ADJ
    (register budgets), LINES, RROW, RCOL, TILE, STAGES) as the defaults of
    csrc/qs_tuned.h."""
    path = os.path.join(_build.SRC, "qs_tuned.h")
    lines = open(path).read().split("\n")
    for i, line in enumerate(lines):
        for (kind, n), k in best.items():
            name = (MACRO[kind] if kind in MACRO else "QS_" + kind + "_MIN_BLOCKS_%d") % n
            if line.startswith("#define %s " % name):
                lines[i] = "#define %s %d" % (name, k)
    with open(path, "w") as f:
        f.write("\n".join(lines))


def tune_factorisations(sizes, tmp):
    """Phase 0: {("RROW"|"RCOL"|"TILE"|"STAGES", N): choice} and the defines fixing them."""
    nalt = max([RADIX_ALTS.get(n, 1) for n in sizes])
    variants = {"r%d" % k: ["QS_RADIX_ROW_%d=%d" % (n, k) for n in sizes if n in RADIX_LISTS and radix_ok(n, k)] +
                ["QS_RADIX_COL_%d=%d" % (n, k) for n in sizes if n in RADIX_LISTS and radix_ok(n, k, True)]
                for k in range(nalt)}
    # column tiles: (columns, stages); a double-buffered 16-column tile only
    # where it fits
    tiles = {"t8s2": (8, 2), "t16s2": (16, 2), "t8s1": (8, 1), "t16s1": (16, 1)}
    for v, (c, st) in tiles.items():
        variants[v] = ["QS_COL_TILE_%d=%d" % (n, c if (st == 1 or c == 8 or n in TILE16) else 8) for n in sizes] + \
                      ["QS_COL_STAGES_%d=%d" % (n, st) for n in sizes]
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(variants)) as ex:
        libs = dict(zip(variants, ex.map(lambda v: _variant(v, SLICE_LOOP, variants[v], tmp)[0], variants)))
    res = {v: _run_measure("--measure", sizes, libs[v]) for v in variants}
    best = {}
    print("factorisation k: row | column pass, us per position-slice")
    print("N     " + "".join("%16s" % v for v in variants))
    for n in sizes:
        print("%-6d" % n + "".join("%8.3f%8.3f" % tuple(res[v][n]) for v in variants))
        if n in RADIX_ALTS:
            best[("RROW", n)] = min([k for k in range(RADIX_ALTS[n]) if radix_ok(n, k)],
                                    key=lambda k: res["r%d" % k][n][0])
            best[("RCOL", n)] = min([k for k in range(RADIX_ALTS[n]) if radix_ok(n, k, True)],
                                    key=lambda k: res["r%d" % k][n][1])
        cand = [v for v in tiles if v != "t16s2" or n in TILE16]
        tv = min(cand, key=lambda v: res[v][n][1])
        best[("TILE", n)], best[("STAGES", n)] = tiles[tv]
        print("      -> row factorisation %s, column factorisation %s, column tile %d x %d stage(s)" %
              (best.get(("RROW", n), 0), best.get(("RCOL", n), 0), best[("TILE", n)], best[("STAGES", n)]))
    defs = ["%s=%d" % (MACRO[kind] % n, k) for (kind, n), k in best.items()]
    return best, defs


def compare(specs, sizes, tmp):
    """Time slice-loop builds with -D overrides side by side (best of two
    measurements of each): specs "tag:DEF1,DEF2" ("tag:" for the defaults)."""
    variants = {}
    for spec in specs:
        tag, _, defs = spec.partition(":")
        variants[tag] = [d for d in defs.split(",") if d]
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(variants)) as ex:
        libs = dict(zip(variants, ex.map(lambda v: _variant(v, SLICE_LOOP, variants[v], tmp)[0], variants)))
    res = {}
    for _ in range(2):
        for v in variants:
            r = _run_measure("--measure", sizes, libs[v])
            res[v] = r if v not in res else {n: tuple(min(x, y) for x, y in zip(res[v][n], r[n])) for n in sizes}
    print("row | column pass, us per position-slice")
    print("N     " + "".join("%18s" % v for v in variants))
    for n in sizes:
        print("%-6d" % n + "".join("%9.3f%9.3f" % tuple(res[v][n]) for v in variants))
    return 0


def _run_measure(mode, sizes, path):
    r = subprocess.run([sys.executable, "-m", "qstem_gb300.tune", "--sizes", ",".join(map(str, sizes)), mode, path],
                       capture_output=True, text=True, check=True, cwd=os.path.dirname(_build.HERE))
    return {int(n): v for n, v in json.loads(r.stdout.strip().splitlines()[-1]).items()}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--candidates", default="1,2,3,4,6,8")
    ap.add_argument("--sizes", default=",".join(map(str, SIZES)))
    ap.add_argument("--lines", default="4,8")
    ap.add_argument("--write", action="store_true")
    ap.add_argument("--compare", nargs="+", metavar="TAG:DEF,DEF",
                    help="time the row and column passes of slice-loop builds with the given -D overrides "
                         "(e.g. base: t8:QS_COL_TILE_256=8,QS_COL_MIN_BLOCKS_256=4) side by side and stop")
    ap.add_argument("--measure", help=argparse.SUPPRESS)          # internal: time one library
    ap.add_argument("--measure-adjoint", help=argparse.SUPPRESS)  # internal
    a = ap.parse_args(argv)
    sizes = [int(s) for s in a.sizes.split(",")]
    if a.measure:
        print(json.dumps(measure(a.measure, sizes)))
        return 0
    if a.measure_adjoint:
        print(json.dumps(measure_adjoint(a.measure_adjoint, sizes)))
        return 0
    _build.build()
    tmp = tempfile.mkdtemp(prefix="qs_tune_")
    if a.compare:
        return compare(a.compare, sizes, tmp)
    cands = [int(k) for k in a.candidates.split(",")]
    # phase 0: factorisations and column tiles
    best, fdefs = tune_factorisations(sizes, tmp)
    # phase 1: row and column passes
    shapes = [int(x) for x in a.lines.split(",")]
    combos = [(L, k) for L in shapes for k in cands]
    defs = {(L, k): fdefs + ["QS_ROW_LINES_%d=%d" % (n, L) for n in sizes] +
            ["QS_%s_MIN_BLOCKS_%d=%d" % (kind, n, k) for n in sizes for kind in ("ROW", "COL")] for L, k in combos}
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(combos)) as ex:
        libs = dict(zip(combos, ex.map(
            lambda c: _variant("rc%d_%d" % c, SLICE_LOOP, defs[c], tmp)[0], combos)))
    res = {c: _run_measure("--measure", sizes, libs[c]) for c in combos}
    print("row pass, us per position-slice (lines per CTA x CTAs per SM)")
    print("N     " + "".join("%8s" % ("%dx%d" % c) for c in combos))
    for n in sizes:
        times = {c: res[c][n][0] for c in combos}
        L, k = min(times, key=times.get)
        best[("ROW", n)], best[("LINES", n)] = k, L
        print("%-6d" % n + "".join("%8.3f" % times[c] for c in combos) + "   -> %dx%d" % (L, k))
    print("col pass, us per position-slice (CTAs per SM)")
    print("N     " + "".join("%8d" % k for k in cands))
    for n in sizes:
        times = {k: min(res[(L, k)][n][1] for L in shapes) for k in cands}
        best[("COL", n)] = min(times, key=times.get)
        print("%-6d" % n + "".join("%8.3f" % times[k] for k in cands) + "   -> %d" % best[("COL", n)])
    # phase 2: row adjoint, with the phase-1 winners
    fixed = (fdefs + ["QS_%s_MIN_BLOCKS_%d=%d" % (kind, n, best[(kind, n)]) for n in sizes for kind in ("ROW", "COL")] +
             ["QS_ROW_LINES_%d=%d" % (n, best[("LINES", n)]) for n in sizes])
    _, ms_objs = _variant("fixed", SLICE_LOOP, fixed, tmp)
    # the adjoint's kernels share the factorisations and tiles (their twiddle
    # tables come from the slice-loop object)
    adefs = {k: fdefs + ["QS_ADJ_MIN_BLOCKS_%d=%d" % (n, k) for n in sizes] for k in cands}
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(cands)) as ex:
        alibs = dict(zip(cands, ex.map(
            lambda k: _variant("adj%d" % k, "qs_adjoint.cu", adefs[k], tmp, extra_objs=ms_objs)[0], cands)))
    ares = {k: _run_measure("--measure-adjoint", sizes, alibs[k]) for k in cands}
    print("adjoint (every state kept, 8 slices), ms")
    print("N     " + "".join("%8d" % k for k in cands))
    for n in sizes:
        times = {k: ares[k][n] for k in cands}
        best[("ADJ", n)] = min(times, key=times.get)
        print("%-6d" % n + "".join("%8.3f" % times[k] for k in cands) + "   -> %d" % best[("ADJ", n)])
    if a.write:
        write_table(best)
        print("wrote", os.path.join(_build.SRC, "qs_tuned.h"))
    return 0


if __name__ == "__main__":
    sys.exit(main())
