"""A stand-in for qstem_gb300.lib.Context that answers from the oracle.

TEST INFRASTRUCTURE ONLY: it lets the CPU suite check the host-side logic
of qstem_gb300.qsc.run_qsc (which files a run writes, their headers, the
averaging over runs) without a GPU.  It implements the calls run_qsc makes
-- slices, slices_custom, probe, stem_run, multislice (with thickness series) -- through
the oracle's C restatement of the reference (oracle/qs_oracle.c).  It
records every multislice result in `log` so that tests can rebuild the
averages they expect.
"""
import numpy as np

from oracle import oracle
from qstem_gb300 import config


class OracleContext:
    def __init__(self):
        self.log = []

    def close(self):
        pass

    def slices(self, p, atoms, slab=0):
        return oracle.transmission(p, oracle.potential(p, atoms, slab=slab))

    def slices_custom(self, p, atoms, k, Zs, f):
        return oracle.transmission(p, oracle.potential_ft(p, atoms, k, Zs, f))

    def probe(self, p, dx=None, dy=None):
        return oracle.probe(p, dx, dy)

    def stem_run(self, p, atoms):
        if max(1, p.mulsRepeat1) > 1 or max(1, p.mulsRepeat2) > 1:
            offs = config.scan_offsets(p)
            return self.multislice(p, self.slices(p, atoms), positions=offs)[0]
        det = oracle.stem(p, self.slices(p, atoms))[0]
        self.log.append(("stem_run", det))
        return det

    @staticmethod
    def _sequence(p, trans, slab_stacks):
        """A stacking sequence unrolled: the stack slice of every step (m2
        passes through the slabs, each slab's stack m1 times) and the
        step that keeps each thickness slot (collectIntensity's slot of
        totalSliceCount + islice*(1 + repeat), last writer wins)."""
        S, D = p.slices, p.cellDiv
        idx, index = [], []
        for pc in range(max(1, p.mulsRepeat2) * D):
            for r in range(max(1, p.mulsRepeat1)):
                for i in range(S):
                    idx.append(((pc % D) * S if (D > 1 and slab_stacks) else 0) + i)
                    index.append(pc * S + i * (1 + r))
        nt, SA = p.thickness_count(), S * D
        last = [-1] * nt
        for a, x in enumerate(index):
            last[x // p.outputInterval if x < SA - 1 else nt - 1] = a
        return np.ascontiguousarray(np.asarray(trans)[idx]), last

    def _repeated(self, p, trans, probe, px, py, dx, dy, want_det, want_diffpats, want_exit_waves, slab_stacks):
        """qs_multislice_run through a stacking sequence: every slot's
        detector values from a run truncated after the slot's writer step;
        patterns and exit waves after the last step."""
        steps, last = self._sequence(p, trans, slab_stacks)
        n = len(px)
        det = np.zeros((p.thickness_count(), p.detectorNum, p.scanXN, p.scanYN), np.float32)
        dps = np.zeros((n, p.nx, p.ny), np.float32)
        ews = np.zeros((n, p.nx, p.ny, 2), np.float32)
        for t, a in enumerate(last):
            if a < 0:
                continue
            q = p.copy()
            q.slices = q.outputInterval = a + 1
            q.cellDiv, q.mulsRepeat1, q.mulsRepeat2 = 1, 1, 1
            for k in range(n):
                w, d, dp = oracle.run_position(q, steps[:a + 1], int(px[k]), int(py[k]), probe)
                det[t, :, int(dx[k]), int(dy[k])] = d[-1]
                if a == len(steps) - 1:
                    dps[k], ews[k] = dp, w
        out = (det if want_det and p.detectorNum > 0 else None, dps if want_diffpats else None,
               ews if want_exit_waves else None)
        self.log.append(("multislice", out))
        return out

    def multislice(self, p, trans, probe=None, positions=None, want_det=True, want_diffpats=False,
                   want_exit_waves=False, slab_stacks=False, series=False):
        if probe is None:
            probe = oracle.probe(p)
        px, py, dx, dy = positions
        n = len(px)
        if max(1, p.mulsRepeat1) > 1 or max(1, p.mulsRepeat2) > 1:
            assert not series, "thickness series through a stacking sequence: run_qsc chains steps instead"
            return self._repeated(p, trans, probe, px, py, dx, dy, want_det, want_diffpats, want_exit_waves,
                                  slab_stacks)
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
