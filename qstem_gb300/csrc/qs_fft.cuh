// qs_fft.cuh -- register/shared-memory line FFTs for sm_103a.
//
// A "line" is one row or column of a wave.  T threads cooperate on a line of
// N = T*E complex values; thread t holds elements t + T*e (e < E) in
// registers, which is also the coalesced global-memory order for rows
// (consecutive threads, consecutive addresses) and for column tiles.
//
// The transform is a self-sorting (Stockham) mixed-radix factorisation
// N = R_0 * R_1 * ... executed as passes.  At pass p (radix R, Ns = product
// of the earlier radices) butterfly j = t + T*q takes its R inputs
// j + r*N/R -- which are exactly the thread's own registers q + r*E/R -- so
// no data moves before a butterfly.  Outputs go to (j/Ns)*Ns*R + j%Ns + r*Ns;
// for every pass but the last they are exchanged through a padded shared
// memory line (one float2 of padding per first-pass radix, so that the
// stride-R writes of the first pass hit distinct banks).  The last pass writes its outputs
// straight back to the thread's registers in natural order.  A line's
// threads are one warp or half-warp, so the exchanges need only __syncwarp.
//
// Inter-pass twiddles exp(-+2 pi i r (j%Ns)/(Ns R)) come from a per-pass
// table (rounded from double) staged in shared memory; the in-register DFTs
// use compile-time constants.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>
#include <utility>

#include "qs_tuned.h"

namespace qs {

// ---------------------------------------------------------------- complex
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// the same with one packed two-lane instruction (add/sub.rn.f32x2, sm_100
// family; each lane rounds as the scalar operation does)
__device__ __forceinline__ float2 cadd_x2(float2 a, float2 b) {
    float2 r;
    asm("{\n .reg .b64 ra, rb, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
        " add.rn.f32x2 rd, ra, rb;\n mov.b64 {%0, %1}, rd;\n}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 csub_x2(float2 a, float2 b) {
    float2 r;
    asm("{\n .reg .b64 ra, rb, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
        " sub.rn.f32x2 rd, ra, rb;\n mov.b64 {%0, %1}, rd;\n}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
template <bool PK>
__device__ __forceinline__ float2 cadd_p(float2 a, float2 b) {
    if constexpr (PK) return cadd_x2(a, b);
    else return cadd(a, b);
}
template <bool PK>
__device__ __forceinline__ float2 csub_p(float2 a, float2 b) {
    if constexpr (PK) return csub_x2(a, b);
    else return csub(a, b);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// ------------------------------------------------ asynchronous copies
// global -> shared copies that bypass the registers (cp.async, 8 bytes)
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}

// --------------------------------------------------- compile-time twiddles
// sin/cos evaluated by the compiler (argument in [-pi, pi], reduced to
// [-pi/4, pi/4] by quadrant, then a Taylor series to double precision).
constexpr double kPi = 3.14159265358979323846264338327950288;

constexpr double taylor_sin(double x) {
    double x2 = x * x, term = x, sum = x;
    for (int k = 1; k < 14; ++k) {
        term *= -x2 / ((2.0 * k) * (2.0 * k + 1.0));
        sum += term;
    }
    return sum;
}
constexpr double taylor_cos(double x) {
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 14; ++k) {
        term *= -x2 / ((2.0 * k - 1.0) * (2.0 * k));
        sum += term;
    }
    return sum;
}
// exp(-2 pi i k/n) as (cos, sin) of angle -2 pi k/n, computed from the
// exact rational k/n by octant reduction.
constexpr double tw_cos(int k, int n) {
    // angle in turns, reduced to [0, 1)
    long kk = ((long)k % n + n) % n;
    // cos(-2 pi kk/n) = cos(2 pi kk/n)
    // reduce 8*kk/n to octant
    double t = (double)kk / (double)n;  // [0,1)
    int oct = (int)(t * 8.0);
    double rem = t * 8.0 - oct;          // [0,1)
    double a = rem * (kPi / 4.0);        // [0, pi/4)
    switch (oct & 7) {
        case 0: return taylor_cos(a);
        case 1: return taylor_sin(kPi / 4.0 - a);
        case 2: return -taylor_sin(a);
        case 3: return -taylor_cos(kPi / 4.0 - a);
        case 4: return -taylor_cos(a);
        case 5: return -taylor_sin(kPi / 4.0 - a);
        case 6: return taylor_sin(a);
        default: return taylor_cos(kPi / 4.0 - a);
    }
}
constexpr double tw_sin(int k, int n) {
    // sin(-2 pi k/n) = -sin(2 pi k/n) = -cos(2 pi k/n - pi/2) = -cos(2pi (k - n/4)/n)
    // evaluate sin(2 pi t) by octant as well
    long kk = ((long)k % n + n) % n;
    double t = (double)kk / (double)n;
    int oct = (int)(t * 8.0);
    double rem = t * 8.0 - oct;
    double a = rem * (kPi / 4.0);
    double s = 0;
    switch (oct & 7) {
        case 0: s = taylor_sin(a); break;
        case 1: s = taylor_cos(kPi / 4.0 - a); break;
        case 2: s = taylor_cos(a); break;
        case 3: s = taylor_sin(kPi / 4.0 - a); break;
        case 4: s = -taylor_sin(a); break;
        case 5: s = -taylor_cos(kPi / 4.0 - a); break;
        case 6: s = -taylor_cos(a); break;
        default: s = -taylor_sin(kPi / 4.0 - a); break;
    }
    return -s;
}

template <int I, int END, class F>
__device__ __forceinline__ void sfor(F&& f) {
    if constexpr (I < END) {
        f(std::integral_constant<int, I>{});
        sfor<I + 1, END>(f);
    }
}

// multiply by exp(s * 2 pi i k/n) with s = -1 (forward) or +1 (inverse), k,n compile time
template <int K, int N, bool INV>
__device__ __forceinline__ float2 ctw(float2 a) {
    constexpr int kk = ((K % N) + N) % N;
    if constexpr (kk == 0) {
        return a;
    } else if constexpr (4 * kk == N) {  // -i (forward) or +i (inverse)
        return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
    } else if constexpr (2 * kk == N) {
        return make_float2(-a.x, -a.y);
    } else if constexpr (4 * kk == 3 * N) {
        return INV ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
    } else {
        constexpr float c = (float)tw_cos(kk, N);
        constexpr float s = (float)tw_sin(kk, N);  // forward: exp(-2 pi i k/N) = (c, s)
        constexpr float si = INV ? -s : s;
        return make_float2(a.x * c - a.y * si, a.x * si + a.y * c);
    }
}

// ------------------------------------------------------ in-register DFTs
// In-place DFT of x[OFF + STRIDE*i], i < N; output in natural order at the
// same positions.  Decimation in time: N = R*M with R = 4, 2 or 3.
template <int N>
struct first_radix {
    static constexpr int value = (N % 4 == 0 && N != 8) ? 4 : (N % 2 == 0 ? 2 : (N % 3 == 0 ? 3 : N));
};

// PK: additions as packed two-lane instructions
template <int N, bool INV, int STRIDE, int OFF, bool PK = false, int L>
__device__ __forceinline__ void dft_reg(float2 (&x)[L]) {
    if constexpr (N == 1) {
        return;
    } else if constexpr (N == 2) {
        float2 a = x[OFF], b = x[OFF + STRIDE];
        x[OFF] = cadd_p<PK>(a, b);
        x[OFF + STRIDE] = csub_p<PK>(a, b);
    } else if constexpr (N == 3) {
        constexpr float h = 0.86602540378443864676f;
        float2 a = x[OFF], b = x[OFF + STRIDE], c = x[OFF + 2 * STRIDE];
        float2 t1 = cadd_p<PK>(b, c), t2 = csub_p<PK>(b, c);
        float2 m = make_float2(a.x - 0.5f * t1.x, a.y - 0.5f * t1.y);
        // n = (s*h) * i * t2, s = -1 forward
        float2 n = INV ? make_float2(-h * t2.y, h * t2.x) : make_float2(h * t2.y, -h * t2.x);
        x[OFF] = cadd_p<PK>(a, t1);
        x[OFF + STRIDE] = cadd_p<PK>(m, n);
        x[OFF + 2 * STRIDE] = csub_p<PK>(m, n);
    } else if constexpr (N == 4) {
        float2 a = x[OFF], b = x[OFF + STRIDE], c = x[OFF + 2 * STRIDE], d = x[OFF + 3 * STRIDE];
        float2 t0 = cadd_p<PK>(a, c), t1 = csub_p<PK>(a, c), t2 = cadd_p<PK>(b, d), dd = csub_p<PK>(b, d);
        float2 t3 = INV ? make_float2(-dd.y, dd.x) : make_float2(dd.y, -dd.x);
        x[OFF] = cadd_p<PK>(t0, t2);
        x[OFF + STRIDE] = cadd_p<PK>(t1, t3);
        x[OFF + 2 * STRIDE] = csub_p<PK>(t0, t2);
        x[OFF + 3 * STRIDE] = csub_p<PK>(t1, t3);
    } else {
        constexpr int R = first_radix<N>::value;
        constexpr int M = N / R;
        static_assert(R * M == N, "unsupported radix");
        // sub-DFTs of the decimated sequences x[OFF + STRIDE*(r + R*m)]
        sfor<0, R>([&](auto r) { dft_reg<M, INV, STRIDE * R, OFF + STRIDE * decltype(r)::value, PK>(x); });
        // combine: y[m + M*k] = sum_r W_N^{r m} X_r[m] W_R^{r k}
        float2 y[N];
        sfor<0, M>([&](auto mi) {
            constexpr int m = decltype(mi)::value;
            float2 v[R];
            sfor<0, R>([&](auto ri) {
                constexpr int r = decltype(ri)::value;
                v[r] = ctw<r * m, N, INV>(x[OFF + STRIDE * (r + R * m)]);
            });
            dft_reg<R, INV, 1, 0, PK>(v);
            sfor<0, R>([&](auto ki) {
                constexpr int k = decltype(ki)::value;
                y[m + M * k] = v[k];
            });
        });
        sfor<0, N>([&](auto ii) {
            constexpr int i = decltype(ii)::value;
            x[OFF + STRIDE * i] = y[i];
        });
    }
}

// -------------------------------------------------------- line transforms
template <int... Rs>
struct radices {
    static constexpr int count = sizeof...(Rs);
    static constexpr int arr[count] = {Rs...};
    static constexpr int at(int i) { return arr[i]; }
    static constexpr int prefix(int i) {  // product of the first i radices
        int p = 1;
        for (int k = 0; k < i; ++k) p *= arr[k];
        return p;
    }
};

// threads per line for a supported length (usable in __launch_bounds__)
constexpr int line_threads(int n) {
    return n == 384 ? QS_LINE_T_384 : n == 768 ? QS_LINE_T_768 : (n <= 128 ? 8 : (n <= 512 ? 16 : 32));
}
// threads per column line (the column transforms may hold more elements a
// thread than the row transforms of the same length)
constexpr int col_line_threads(int n) {
    return n == 384 ? QS_COL_LINE_T_384 : n == 768 ? QS_COL_LINE_T_768 : line_threads(n);
}

// Line configuration: N points, T threads per line.
//
// Shared-memory exchange scratch of a row line: element i lives at
// i + i / R0 (R0 = first radix), so the stride-R0 writes of the first pass
// land on an odd float2 stride and a half-warp hits 16 distinct 8-byte bank
// pairs.  Inter-pass twiddles: pass p >= 1 (radix R, Ns = product of the
// earlier radices) multiplies input r of butterfly j by
// exp(-+2 pi i r (j mod Ns)/(Ns R)); the table stores them per pass as
// [r-1][j mod Ns] so that consecutive lanes read consecutive words.
template <int N_, int T_, class RAD, int PK_ = 0>
struct LineCfg {
    static constexpr int N = N_;
    static constexpr int T = T_;
    // butterflies' additions packed (cadd_x2): bit 0 forward, bit 1 inverse
    static constexpr int PK = PK_;
    static constexpr int E = N / T;
    static constexpr int PASSES = RAD::count;
    static constexpr int R0 = RAD::at(0);
    static constexpr int SMEM = N + N / R0 + 1;  // padded float2 per row line
    using rad = RAD;
    // offset of pass p's twiddles in the table (pass 0 has none)
    static constexpr int tw_offset(int p) {
        int o = 0;
        for (int k = 1; k < p; ++k) o += (RAD::at(k) - 1) * RAD::prefix(k);
        return o;
    }
    static constexpr int TW = tw_offset(RAD::count);  // table length
    static_assert(RAD::prefix(RAD::count) == N, "radices must multiply to N");
    static_assert(T <= 32 && (32 % T) == 0, "row lines must live inside one warp");
    static_assert(TW <= N, "twiddle table must fit in N entries");
};

// The same line configuration with other packed-addition bits (the
// transforms, twiddle tables and shared-memory layout are unchanged).
template <class Cfg, int PK>
struct with_packing;
template <int N_, int T_, class RAD, int P_, int PK>
struct with_packing<LineCfg<N_, T_, RAD, P_>, PK> {
    using type = LineCfg<N_, T_, RAD, PK>;
};

// Shared-memory views of a line's exchange scratch.
// Row lines: one padded line of Cfg::SMEM float2 per line.
template <int R0>
struct SmemRow {
    float2* p;
    __device__ __forceinline__ float2& operator()(int i) const { return p[i + i / R0]; }
};
// Column tiles: element i of column c at p[i*C + c] (columns interleaved, so a
// half-warp of consecutive columns touches consecutive words).
template <int C>
struct SmemCol {
    float2* p;
    int c;
    __device__ __forceinline__ float2& operator()(int i) const { return p[i * C + c]; }
};

template <bool BLOCK>
__device__ __forceinline__ void line_sync() {
    if constexpr (BLOCK) __syncthreads();
    else __syncwarp();
}
// the synchronisation between the passes of a line transform, as a type
template <bool BLOCK>
struct LineSync {
    __device__ __forceinline__ static void sync() { line_sync<BLOCK>(); }
};
// named barrier ID over the first COUNT threads of the block (COUNT a
// multiple of 32): lines spread over a subset of the block's warps
template <int ID, int COUNT>
struct NamedBarrier {
    static_assert(COUNT % 32 == 0, "a named barrier counts whole warps");
    __device__ __forceinline__ static void sync() { asm volatile("bar.sync %0, %1;" ::"n"(ID), "n"(COUNT) : "memory"); }
};

// Transform the E registers of thread t (elements t + T*e) in place.
// sm: this line's shared scratch view; tw: the per-pass twiddle table of Cfg.
// SYNC::sync() orders the exchanges between passes (every thread that takes
// part in it must call).
template <class Cfg, bool INV, class SYNC, class SM>
__device__ __forceinline__ void line_fft_sync(float2 (&reg)[Cfg::E], const SM& sm, const float2* __restrict__ tw,
                                              int t);
// BLOCK selects __syncthreads (a line spread over several warps) instead of
// __syncwarp; with BLOCK every thread of the block must call.
template <class Cfg, bool INV, bool BLOCK = false, class SM>
__device__ __forceinline__ void line_fft(float2 (&reg)[Cfg::E], const SM& sm, const float2* __restrict__ tw,
                                         int t) {
    line_fft_sync<Cfg, INV, LineSync<BLOCK>>(reg, sm, tw, t);
}

template <class Cfg, bool INV, class SYNC, class SM>
__device__ __forceinline__ void line_fft_sync(float2 (&reg)[Cfg::E], const SM& sm, const float2* __restrict__ tw,
                                              int t) {
    constexpr int T = Cfg::T, E = Cfg::E;
    using RAD = typename Cfg::rad;
    sfor<0, Cfg::PASSES>([&](auto pi) {
        constexpr int p = decltype(pi)::value;
        constexpr int R = RAD::at(p);
        constexpr int Ns = RAD::prefix(p);
        constexpr int Q = E / R;
        constexpr bool last = (p == Cfg::PASSES - 1);
        static_assert(E % R == 0, "each thread must own whole butterflies");
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int j = t + T * q;
            const int jm = (Ns == 1) ? 0 : (j % Ns);
            float2 v[R];
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = reg[q + r * Q];
            if constexpr (Ns > 1) {
                constexpr int off = Cfg::tw_offset(p);
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    const float2 w = tw[off + (r - 1) * Ns + jm];
                    v[r] = INV ? cmulc(v[r], w) : cmul(v[r], w);
                }
            }
            dft_reg<R, INV, 1, 0, ((Cfg::PK >> (INV ? 1 : 0)) & 1) != 0>(v);
            if constexpr (last) {
#pragma unroll
                for (int r = 0; r < R; ++r) reg[q + r * Q] = v[r];
            } else {
                const int base = (j / Ns) * Ns * R + jm;
#pragma unroll
                for (int r = 0; r < R; ++r) sm(base + r * Ns) = v[r];
            }
        }
        if constexpr (!last) {
            SYNC::sync();
#pragma unroll
            for (int e = 0; e < E; ++e) reg[e] = sm(t + T * e);
            SYNC::sync();
        }
    });
}

// Register e of a line held by T threads (elements t + T*e) lies, for every
// t, in [N/3 + 1, ceil(2N/3) - 1]: frequencies that the 2/3 band limit of
// propagate_slow always removes (|k| < k_max <= N/3 grid steps in each
// direction, whatever the cell; the margin of one step keeps the float
// comparisons at |k| = N/3 out of it).  Kernels leave those registers
// unstored or zero, and the compiler drops the butterfly outputs that only
// fed them.
template <int N, int T>
__host__ __device__ constexpr bool always_out_of_band(int e) {
    return T * e >= N / 3 + 1 && T * e + T - 1 <= (2 * N + 2) / 3 - 1;
}

// ------------------------------------------------------- size dispatching
// One configuration per supported line length.  Where several
// factorisations fit the thread layout (each radix must divide E = N/T), the
// row transforms (Line) and the column transforms (LineCol) pick one each:
// QS_RADIX_ROW_<N> and QS_RADIX_COL_<N> in qs_tuned.h index the lists below.
template <int... Rs>
using rad_t = radices<Rs...>;
template <int I, class... Alts>
struct pick;
template <class A, class... Rest>
struct pick<0, A, Rest...> { using type = A; };
template <int I, class A, class... Rest>
struct pick<I, A, Rest...> { using type = typename pick<I - 1, Rest...>::type; };
template <int I>
using Rad384 = typename pick<I, rad_t<8, 6, 8>, rad_t<6, 8, 8>, rad_t<8, 8, 6>, rad_t<12, 4, 8>, rad_t<24, 4, 4>,
                             rad_t<8, 48>, rad_t<48, 8>>::type;
template <int I>
using Rad512 = typename pick<I, rad_t<32, 16>, rad_t<16, 32>>::type;
template <int I>
using Rad768 = typename pick<I, rad_t<8, 12, 8>, rad_t<12, 8, 8>, rad_t<8, 8, 12>, rad_t<24, 4, 8>, rad_t<24, 8, 4>,
                             rad_t<16, 48>, rad_t<48, 16>>::type;
template <int I>
using Rad1024 = typename pick<I, rad_t<32, 32>, rad_t<8, 16, 8>>::type;

// (the product kernels size __launch_bounds__ with line_threads(N) and col_line_threads(N))
template <int N>
struct Line;
template <> struct Line<64> { using cfg = LineCfg<64, 8, radices<8, 8>>; };
template <> struct Line<128> { using cfg = LineCfg<128, 8, radices<16, 8>>; };
template <> struct Line<256> { using cfg = LineCfg<256, 16, radices<16, 16>, QS_PACKED_256>; };
template <> struct Line<384> { using cfg = LineCfg<384, QS_LINE_T_384, Rad384<QS_RADIX_ROW_384>, QS_PACKED_ROWS>; };
template <> struct Line<512> { using cfg = LineCfg<512, 16, Rad512<QS_RADIX_ROW_512>, QS_PACKED_ROWS>; };
template <> struct Line<768> { using cfg = LineCfg<768, QS_LINE_T_768, Rad768<QS_RADIX_ROW_768>, QS_PACKED_ROWS>; };
template <> struct Line<1024> { using cfg = LineCfg<1024, 32, Rad1024<QS_RADIX_ROW_1024>, QS_PACKED_ROWS>; };
// column transforms
template <int N>
struct LineCol { using cfg = typename Line<N>::cfg; };
template <> struct LineCol<384> { using cfg = LineCfg<384, QS_COL_LINE_T_384, Rad384<QS_RADIX_COL_384>, QS_PACKED_COLS_384>; };
template <> struct LineCol<512> { using cfg = LineCfg<512, 16, Rad512<QS_RADIX_COL_512>, QS_PACKED_COLS_512>; };
template <> struct LineCol<768> { using cfg = LineCfg<768, QS_COL_LINE_T_768, Rad768<QS_RADIX_COL_768>, QS_PACKED_COLS_768>; };
template <> struct LineCol<1024> { using cfg = LineCfg<1024, 32, Rad1024<QS_RADIX_COL_1024>, QS_PACKED_COLS_1024>; };

// columns per column-pass tile (qs_tuned.h: 16 = 128-byte row segments)
template <int N>
constexpr int col_tile() {
    return N == 64     ? QS_COL_TILE_64
           : N == 128  ? QS_COL_TILE_128
           : N == 256  ? QS_COL_TILE_256
           : N == 384  ? QS_COL_TILE_384
           : N == 512  ? QS_COL_TILE_512
           : N == 768  ? QS_COL_TILE_768
           : N == 1024 ? QS_COL_TILE_1024
                       : 8;
}

template <int N>
constexpr bool line_threads_match() {
    return Line<N>::cfg::T == line_threads(N) && LineCol<N>::cfg::T == col_line_threads(N);
}
static_assert(line_threads_match<64>() && line_threads_match<128>() && line_threads_match<256>() &&
                  line_threads_match<384>() && line_threads_match<512>() && line_threads_match<768>() &&
                  line_threads_match<1024>(),
              "line_threads() and col_line_threads() must match the Line<N> / LineCol<N> configurations");

inline bool line_supported(int n) {
    return n == 64 || n == 128 || n == 256 || n == 384 || n == 512 || n == 768 || n == 1024;
}

}  // namespace qs
