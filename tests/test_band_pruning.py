"""The registers the line transforms never store (qs_fft.cuh,
always_out_of_band<N, T>) hold only frequencies that propagate_slow's 2/3
band limit removes, whatever the cell: propagate_slow's tables
(stem3/stemlib.cpp:2783-2824, restated in float as prop_tables does) for
random samplings of every length, against every thread layout in use."""
import numpy as np
import pytest

from qstem_gb300 import tune

F32 = np.float32


def always_out_of_band(N, T, e):
    return T * e >= N // 3 + 1 and T * e + T - 1 <= (2 * N + 2) // 3 - 1


def k2_tables(n, d):
    a = F32(F32(d) * F32(n))
    i = np.arange(n)
    k = np.where(i > n // 2, (i - n).astype(F32) / a, i.astype(F32) / a).astype(F32)
    return (k * k).astype(F32), a


@pytest.mark.parametrize("N", [64, 128, 256, 384, 512, 768, 1024])
def test_pruned_registers_are_out_of_band(N):
    rng = np.random.default_rng(N)
    layouts = {tune._line_threads(N), tune._line_threads(N, col=True)}
    for _ in range(200):
        dx = float(rng.uniform(0.02, 0.3))
        dy = dx * float(rng.uniform(0.5, 2.0))
        kx2, ax = k2_tables(N, dx)
        ky2, by = k2_tables(N, dy)
        k2max = F32(N) / (F32(2.0) * ax)
        k2max = min(k2max, F32(N) / (F32(2.0) * by))
        k2max = F32(2.0 / 3.0 * float(k2max))
        k2max = F32(k2max * k2max)
        for T in layouts:
            for e in range(N // T):
                if not always_out_of_band(N, T, e):
                    continue
                idx = np.arange(T) + T * e
                # the propagator zeroes them in x (kx2 >= k2max) and the band
                # limit drops them in y (ky2 >= k2max)
                assert np.all(kx2[idx] >= k2max), (N, T, e, dx)
                assert np.all(ky2[idx] >= k2max), (N, T, e, dy)
