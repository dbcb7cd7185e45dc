"""The line transforms' schedule (qstem_gb300/csrc/qs_fft.cuh, line_fft_sync)
restated in numpy: T threads hold E = N/T elements each (element t + T*e in
register e); pass p of radix R takes butterflies j = t + T*q, q < E/R, from
registers q + r*E/R, multiplies input r by the pass twiddle
exp(-2 pi i r (j mod Ns) / (Ns R)) (Ns = product of the earlier radices),
transforms, and writes output r to exchange slot (j div Ns)*Ns*R + (j mod Ns)
+ r*Ns, from which every thread reads its registers t + T*e back.  Every
length, thread layout and factorisation the tables allow must give the DFT
in natural order."""
import numpy as np
import pytest

from qstem_gb300 import tune


def schedule(x, T, radices, inverse=False):
    N = len(x)
    E = N // T
    reg = np.array([[x[t + T * e] for e in range(E)] for t in range(T)], dtype=np.complex128)
    sgn = 1.0 if inverse else -1.0
    Ns = 1
    for p, R in enumerate(radices):
        assert E % R == 0
        Q = E // R
        last = p == len(radices) - 1
        sm = np.zeros(N, dtype=np.complex128)
        out = reg.copy()
        for t in range(T):
            for q in range(Q):
                j = t + T * q
                jm = j % Ns
                v = np.array([reg[t, q + r * Q] for r in range(R)])
                if Ns > 1:
                    v = v * np.exp(sgn * 2j * np.pi * np.arange(R) * jm / (Ns * R))
                v = np.fft.fft(v) if not inverse else np.fft.ifft(v) * R
                for r in range(R):
                    if last:
                        out[t, q + r * Q] = v[r]
                    else:
                        sm[(j // Ns) * Ns * R + jm + r * Ns] = v[r]
        if not last:
            out = np.array([[sm[t + T * e] for e in range(E)] for t in range(T)])
        reg = out
        Ns *= R
    y = np.zeros(N, dtype=np.complex128)
    for t in range(T):
        for e in range(E):
            y[t + T * e] = reg[t, e]
    return y


def configurations():
    out = []
    for n, lists in tune.RADIX_LISTS.items():
        for col in (False, True):
            T = tune._line_threads(n, col)
            for k, rad in enumerate(lists):
                if tune.radix_ok(n, k, col):
                    out.append((n, T, rad))
    # the fixed lengths (qs_fft.cuh Line<64>, <128>, <256>)
    out += [(64, 8, (8, 8)), (128, 8, (16, 8)), (256, 16, (16, 16))]
    return sorted(set(out))


@pytest.mark.parametrize("n,T,rad", configurations())
def test_schedule_gives_the_dft(n, T, rad):
    rng = np.random.default_rng(n + T)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    np.testing.assert_allclose(schedule(x, T, rad), np.fft.fft(x), rtol=0, atol=1e-9 * n)
    np.testing.assert_allclose(schedule(x, T, rad, inverse=True), np.fft.ifft(x) * n, rtol=0, atol=1e-9 * n)
