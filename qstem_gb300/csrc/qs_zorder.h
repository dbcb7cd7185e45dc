// qs_zorder.h -- the order in which the slice builders visit atoms: sorted
// by z, ties in input order (the reference sorts with qsort and atomCompare,
// stem3/stemlib.cpp:540, stem3/stemutil.cpp:1524; glibc's qsort keeps ties in
// input order), i.e. std::stable_sort with a < b on z.
//
// A stable least-significant-digit radix sort on the float's order-preserving
// bit pattern gives that same order in two passes of 16 bits: for floats
// that are not NaN, a < b exactly when key(a) < key(b) once -0 is read as +0.
// Host code only (C++, no CUDA).
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

// below this many atoms the comparison sort is as fast
#ifndef QS_ZORDER_RADIX_MIN
#define QS_ZORDER_RADIX_MIN 2048
#endif

namespace qs {

inline uint32_t z_key(float z) {
    if (z == 0.0f) z = 0.0f;  // -0 sorts with +0, as a < b treats them
    uint32_t u;
    std::memcpy(&u, &z, sizeof(u));
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// order[k] = index of the k-th atom in z order; zof(i) = z of atom i
template <class ZOf>
void z_order(int n, ZOf zof, std::vector<int>& order) {
    order.resize(n > 0 ? n : 0);
    for (int i = 0; i < n; i++) order[i] = i;
    if (n < QS_ZORDER_RADIX_MIN) {
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return zof(a) < zof(b); });
        return;
    }
    std::vector<uint32_t> key(n);
    for (int i = 0; i < n; i++) key[i] = z_key(zof(i));
    std::vector<int> tmp(n);
    std::vector<uint32_t> count(65537);
    for (int shift = 0; shift < 32; shift += 16) {
        std::fill(count.begin(), count.end(), 0u);
        for (int k = 0; k < n; k++) count[((key[order[k]] >> shift) & 0xffffu) + 1]++;
        for (int b = 0; b < 65536; b++) count[b + 1] += count[b];
        for (int k = 0; k < n; k++) tmp[count[(key[order[k]] >> shift) & 0xffffu]++] = order[k];
        order.swap(tmp);
    }
}

}  // namespace qs
