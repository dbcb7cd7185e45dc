"""A stand-in for qstem_gb300.lib.Context that answers from the oracle.

TEST INFRASTRUCTURE ONLY: it lets the CPU suite check the host-side logic
of qstem_gb300.qsc.run_qsc (which files a run writes, their headers, the
averaging over runs) without a GPU.  It implements the calls run_qsc makes
-- slices, probe, stem_run, multislice (with thickness series) -- through
the oracle's C restatement of the reference (oracle/qs_oracle.c).  It
records every multislice result in `log` so that tests can rebuild the
averages they expect.
"""
import numpy as np

from oracle import oracle


class OracleContext:
    def __init__(self):
        self.log = []

    def close(self):
        pass

    def slices(self, p, atoms, slab=0):
        return oracle.transmission(p, oracle.potential(p, atoms, slab=slab))

    def probe(self, p, dx=None, dy=None):
        return oracle.probe(p, dx, dy)

    def stem_run(self, p, atoms):
        det = oracle.stem(p, self.slices(p, atoms))[0]
        self.log.append(("stem_run", det))
        return det

    def multislice(self, p, trans, probe=None, positions=None, want_det=True, want_diffpats=False,
                   want_exit_waves=False, slab_stacks=False, series=False):
        if probe is None:
            probe = oracle.probe(p)
        px, py, dx, dy = positions
        n = len(px)
        if not series:
            # positions are a contiguous run of raster indices
            p0 = int(dx[0]) * p.scanYN + int(dy[0])
            out = oracle.stem(p, trans, probe, p0, p0 + n, det=want_det and p.detectorNum > 0,
                              diffpats=want_diffpats, exit_waves=want_exit_waves, slab_stacks=slab_stacks)
            self.log.append(("multislice", out))
            return out
        # thickness series: slot t is the run truncated after its writer
        # slice (collectIntensity's slot rule, stem3/stemlib.cpp:2597-2610);
        # slabs are one stack of all absolute slices
        nt, S = p.thickness_count(), p.slices * p.cellDiv
        if p.cellDiv > 1 and not slab_stacks:
            trans = np.concatenate([trans] * p.cellDiv)
        last = [-1] * nt
        for a in range(S):
            t = a // p.outputInterval if a < S - 1 else nt - 1
            if t < nt:
                last[t] = a
        dps = np.zeros((nt, n, p.nx, p.ny), np.float32)
        ews = np.zeros((nt, n, p.nx, p.ny, 2), np.float32)
        for t, a in enumerate(last):
            if a < 0:
                continue
            q = p.copy()
            q.slices = q.outputInterval = a + 1
            q.cellDiv = 1
            for k in range(n):
                ews[t, k], _, dps[t, k] = oracle.run_position(q, trans[:a + 1], int(px[k]), int(py[k]), probe)
        out = (None, dps if want_diffpats else None, ews if want_exit_waves else None)
        self.log.append(("series", out))
        return out
