"""The slice builders' atom order (qstem_gb300/csrc/qs_zorder.h: a stable radix
sort on the float bit pattern) against std::stable_sort by z, compiled with
the host C++ compiler: ties, signed zeros, negative and large values, and
sizes on both sides of the switch to the radix sort."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "qstem_gb300", "csrc")

PROG = r"""
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>
#include "qs_zorder.h"
int main() {
    std::mt19937 rng(7);
    int bad = 0;
    for (int n : {0, 1, 5, 2047, 2048, 3000, 70000, 200000}) {
        for (int kind = 0; kind < 4; kind++) {
            std::vector<float> z(n);
            for (int i = 0; i < n; i++) {
                if (kind == 0) z[i] = std::uniform_real_distribution<float>(-50.f, 300.f)(rng);
                if (kind == 1) z[i] = (float)(rng() % 40) * 1.9525f - 20.f;         // many ties
                if (kind == 2) z[i] = (rng() % 3 == 0) ? -0.0f : ((rng() % 2) ? 0.0f : 1e-30f);
                if (kind == 3) z[i] = ldexpf(1.0f, (int)(rng() % 200) - 100) * ((rng() % 2) ? 1.f : -1.f);
            }
            std::vector<int> want(n), got;
            for (int i = 0; i < n; i++) want[i] = i;
            std::stable_sort(want.begin(), want.end(), [&](int a, int b) { return z[a] < z[b]; });
            qs::z_order(n, [&](int i) { return z[i]; }, got);
            if (got != want) { std::printf("mismatch n=%d kind=%d\n", n, kind); bad++; }
        }
    }
    std::printf("%s\n", bad ? "FAIL" : "OK");
    return bad ? 1 : 0;
}
"""


def test_z_order_matches_stable_sort(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "zorder.cpp"
    src.write_text(PROG)
    exe = tmp_path / "zorder"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout
