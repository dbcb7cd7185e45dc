"""Autotune the row pass's register budget per line length.

    python -m qstem_gb300.tune [--candidates 1,2,3,4,6,8] [--sizes 256,384,...] [--write]

For each candidate k the row-pass translation unit (qs_multislice.cu) is
compiled with every QS_ROW_MIN_BLOCKS_<N> = k and linked with the other
objects of the normal build into a variant library in a temporary folder
(the candidates compile in parallel).  Each variant then times, in a fresh
process on the GPU, the row and column passes of every line length through
the library's own CUDA-event counters (qs_ctx_profile / qs_ctx_stats): a
random slice stack of 8 slices, 1024 waves at 256^2 down to 128 at 1024^2,
best of 4.  The fastest candidate per size is printed as a table and, with
--write, stored in csrc/qs_tuned.h (then rebuild).  Needs nvcc and a GPU.
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


def _variant(k, sizes, tmp):
    """Compile the row pass with register budget k for all sizes; link a library."""
    objs = [os.path.join(_build.BUILD, s.replace(".cu", ".o")) for s in _build.SOURCES if s != "qs_multislice.cu"]
    obj = os.path.join(tmp, "qs_multislice_%d.o" % k)
    defs = ["-DQS_ROW_MIN_BLOCKS_%d=%d" % (n, k) for n in sizes]
    cmd = ([_build.nvcc()] + _build.ARCH + _build.FLAGS + defs +
           ["-c", os.path.join(_build.SRC, "qs_multislice.cu"), "-o", obj])
    subprocess.run(cmd, check=True, capture_output=True)
    lib = os.path.join(tmp, "libqstem_gpu_%d.so" % k)
    subprocess.run([_build.nvcc()] + _build.ARCH + ["-shared", "-o", lib, obj] + objs + ["-lcudart"], check=True,
                   capture_output=True)
    return k, lib


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


def write_table(best):
    """Store the chosen values as the defaults of csrc/qs_tuned.h."""
    path = os.path.join(_build.SRC, "qs_tuned.h")
    lines = open(path).read().split("\n")
    for i, line in enumerate(lines):
        for n, k in best.items():
            if line.startswith("#define QS_ROW_MIN_BLOCKS_%d " % n):
                lines[i] = "#define QS_ROW_MIN_BLOCKS_%d %d" % (n, k)
    with open(path, "w") as f:
        f.write("\n".join(lines))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--candidates", default="1,2,3,4,6,8")
    ap.add_argument("--sizes", default=",".join(map(str, SIZES)))
    ap.add_argument("--write", action="store_true")
    ap.add_argument("--measure", help=argparse.SUPPRESS)  # internal: time one library, print JSON
    a = ap.parse_args(argv)
    sizes = [int(s) for s in a.sizes.split(",")]
    if a.measure:
        print(json.dumps(measure(a.measure, sizes)))
        return 0
    _build.build()
    cands = [int(k) for k in a.candidates.split(",")]
    tmp = tempfile.mkdtemp(prefix="qs_tune_")
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(cands)) as ex:
        libs = dict(ex.map(lambda k: _variant(k, sizes, tmp), cands))
    results = {}
    for k, path in sorted(libs.items()):
        r = subprocess.run([sys.executable, "-m", "qstem_gb300.tune", "--sizes", a.sizes, "--measure", path],
                           capture_output=True, text=True, check=True, cwd=os.path.dirname(_build.HERE))
        results[k] = {int(n): v for n, v in json.loads(r.stdout.strip().splitlines()[-1]).items()}
    print("row pass, us per position-slice (candidate = CTAs per SM)")
    print("N     " + "".join("%8d" % k for k in sorted(results)))
    best = {}
    for n in sizes:
        times = {k: results[k][n][0] for k in results}
        best[n] = min(times, key=times.get)
        print("%-6d" % n + "".join("%8.3f" % times[k] for k in sorted(times)) + "   -> %d" % best[n])
    if a.write:
        write_table(best)
        print("wrote", os.path.join(_build.SRC, "qs_tuned.h"))
    return 0


if __name__ == "__main__":
    sys.exit(main())
