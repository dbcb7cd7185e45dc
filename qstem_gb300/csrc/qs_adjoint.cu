// qs_adjoint.cu -- the adjoint of the multislice scan (differentiable 4D-STEM)
// and of the slice builder's scatter-sum.
//
// Loss  L = sum_p sum_k (I_p(k) - T_p(k))^2 with I_p the diffraction pattern
// of position p after the last slice (|psi(k)|^2/sqrt(nx*ny), the reference's
// wave->diffpat, stem3/stemlib.cpp:2630) and T_p a target pattern.
//
// Gradients use the conjugate convention g_z = dL/d(conj z), so that
// dL = 2 Re sum conj(g_z) dz.  Per slice the forward step
//   psi = IFFT_y(h)/N;  phi = psi * t;  A = FFT_y(phi)      (row pass)
//   B' = P * FFT_x(A);  h' = IFFT_x(B')                      (column pass)
// has the adjoint
//   g_A = IFFT_x(conj(P) * FFT_x(g_h'))                      (column pass, conj P)
//   g_phi = IFFT_y(g_A);  g_t = conj(psi) g_phi;  g_psi = conj(t) g_phi;
//   g_h = FFT_y(g_psi)/N                                      (row adjoint)
//   dL/dV = -2 sigma Im(conj(sum_p g_t,p) t)                  (window gather)
// with t = exp(i sigma V), sigma = lambda*gamma (initSTEMSlices,
// stem3/stemlib.cpp:2290-2299).  The last slice seeds g_B' = 2(I - T) c B'.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "qs_fft.cuh"
#include "qs_internal.h"
#include "qs_tuned.h"

namespace qs {

// lines per CTA of the row adjoint
#ifndef QS_ADJ_ROW_LINES
#define QS_ADJ_ROW_LINES 8
#endif
constexpr int ADJ_ROW_LINES = QS_ADJ_ROW_LINES;
// the row adjoint's register budget (qs_tuned.h)
constexpr int adj_min_blocks(int n) {
    return n == 64     ? QS_ADJ_MIN_BLOCKS_64
           : n == 128  ? QS_ADJ_MIN_BLOCKS_128
           : n == 256  ? QS_ADJ_MIN_BLOCKS_256
           : n == 384  ? QS_ADJ_MIN_BLOCKS_384
           : n == 512  ? QS_ADJ_MIN_BLOCKS_512
           : n == 768  ? QS_ADJ_MIN_BLOCKS_768
           : n == 1024 ? QS_ADJ_MIN_BLOCKS_1024
                       : 1;
}

// ---------------------------------------------- last slice: loss and seed
// One block per (wave, column tile), all tiles of the grid: forward FFT_x
// and propagator of the last slice, loss terms, g_B' = 2 (I - T) c B',
// g_A = IFFT_x(conj(P) g_B').
template <int N>
__global__ void __launch_bounds__(col_tile<N>() * col_line_threads(N))
    adj_last_cols(AdjLastArgs a) {
    using Cfg = typename LineCol<N>::cfg;
    constexpr int T = Cfg::T, E = Cfg::E, C = col_tile<N>();
    constexpr int NT = C * T;
    constexpr int NWARPS = (NT + 31) / 32;
    extern __shared__ float2 dsm[];
    float2* s_tw = dsm;
    float2* s_tile = dsm + N;
    __shared__ double s_loss[NWARPS];
    const int tid = threadIdx.x + C * threadIdx.y;
    for (int i = tid; i < Cfg::TW; i += NT) s_tw[i] = a.tw[i];
    __syncthreads();
    const int c = threadIdx.x, t = threadIdx.y;
    const int ntiles = a.ny / C;
    const int tile = blockIdx.x % ntiles;
    const int b = blockIdx.x / ntiles;
    const int ky = tile * C + c;
    const float2* col = a.waves + (size_t)b * a.nx * a.ny + ky;
    float2* out = a.waves_out + (size_t)b * a.nx * a.ny + ky;
    const bool inband = (ky <= a.yA || ky >= a.yB);
    float2 reg[E];
#pragma unroll
    for (int e = 0; e < E; ++e) reg[e] = inband ? col[(size_t)(t + T * e) * a.ny] : make_float2(0.f, 0.f);
    const SmemCol<C> sm{s_tile, c};
    line_fft<Cfg, false, true>(reg, sm, s_tw, t);
    const float ky2 = a.ky2[ky];
    const float2 pyv = a.py[ky];
    const float* tgt = a.target + (size_t)b * a.nx * a.ny + (ky + a.ny / 2) % a.ny;
    float* dp = a.diffpat ? a.diffpat + (size_t)b * a.nx * a.ny + (ky + a.ny / 2) % a.ny : nullptr;
    // FP32 per pixel (FP64 runs at a small fraction of the FP32 rate here);
    // a thread's E squared residuals are summed in FP32, the rest in double
    const float sc = (float)a.scaleDiff;
    float loss = 0.f;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int kx = t + T * e;
        const float kx2 = a.kx2[kx];
        const float2 pxv = a.px[kx];
        const bool pass = !always_out_of_band<N, T>(e) && inband && kx2 < a.k2max && (kx2 + ky2) < a.k2max;
        const float2 Bp = pass ? cmul(cmul(reg[e], pyv), pxv) : make_float2(0.f, 0.f);
        const float I = (Bp.x * Bp.x + Bp.y * Bp.y) * sc;
        const size_t ik = (size_t)((kx + a.nx / 2) % a.nx) * a.ny;
        const float dI = I - tgt[ik];
        loss += dI * dI;
        if (dp) dp[ik] = I;
        // g_B' = 2 dI c B', then g_B = conj(P) g_B'
        const float g = 2.f * dI * sc;
        const float2 gBp = make_float2(g * Bp.x, g * Bp.y);
        reg[e] = pass ? cmulc(cmulc(gBp, pyv), pxv) : make_float2(0.f, 0.f);
    }
    const int lane = tid & 31, warp = tid >> 5;
    double lsum = (double)loss;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0) s_loss[warp] = lsum;
    line_fft<Cfg, true, true>(reg, sm, s_tw, t);
#pragma unroll
    for (int e = 0; e < E; ++e) out[(size_t)(t + T * e) * a.ny] = reg[e];
    __syncthreads();
    if (tid == 0) {
        double s = 0.0;
        for (int w = 0; w < NWARPS; ++w) s += s_loss[w];
        a.loss_partial[blockIdx.x] = s;
    }
}

// ------------------------------------------------------------ row adjoint
// SUM: add g_t = conj(psi) g_phi into the slice's window sum a.gsum with
// float atomics (vector reductions into an L2-resident potNx x potNy array)
// instead of storing every position's g_t for the two-kernel gather.
// QS_PACKED_ADJ: packed-addition bits of the row adjoint's transforms at
// 256 points and below (-1: those of the forward row transforms).  The
// inverse transform packed (2) measured fastest on the 256^2 4D-STEM
// adjoint: 42.50 -> 42.01 ms at 6-slice checkpoints (both: 42.07, forward
// only: 42.71), the forward row pass unchanged.
#ifndef QS_PACKED_ADJ
#define QS_PACKED_ADJ 2
#endif
template <int N>
using AdjRowCfg = typename std::conditional<(N <= 256 && QS_PACKED_ADJ >= 0),
                                            typename with_packing<typename Line<N>::cfg,
                                                                  (QS_PACKED_ADJ < 0 ? 0 : QS_PACKED_ADJ)>::type,
                                            typename Line<N>::cfg>::type;
template <int N, bool FIRST, bool SUM>
__global__ void __launch_bounds__(line_threads(N) * ADJ_ROW_LINES, adj_min_blocks(N))
    adj_rows(AdjRowArgs a) {
    using Cfg = AdjRowCfg<N>;
    constexpr int T = Cfg::T, E = Cfg::E;
    extern __shared__ float2 dsm[];
    float2* s_tw = dsm;
    float2* s_line = dsm + N + threadIdx.y * Cfg::SMEM;
    const int tid = threadIdx.x + T * threadIdx.y;
    for (int i = tid; i < Cfg::TW; i += T * ADJ_ROW_LINES) s_tw[i] = a.tw[i];
    __syncthreads();
    const int t = threadIdx.x;
    const long line = (long)blockIdx.x * ADJ_ROW_LINES + threadIdx.y;
    const int b = (int)(line / a.nx);
    const int x = (int)(line - (long)b * a.nx);
    const SmemRow<Cfg::R0> sm{s_line};
    // g_phi = IFFT_y(g_A), and psi of this slice: the probe, or
    // IFFT_y(h)/N of the stored state.  With up to 16 elements a thread both
    // lines' loads are issued before either transform, so that their
    // latencies overlap (longer lines keep them apart: registers)
    constexpr bool EARLY = E <= 16;
    float2* grow = a.grad + ((size_t)b * a.nx + x) * N;
    float2 g[E], psi[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int y = t + T * e;
        g[e] = (y <= a.yA || y >= a.yB) ? grow[y] : make_float2(0.f, 0.f);
    }
    auto load_psi = [&]() {
        if constexpr (FIRST) {
            const float2* src = a.probe + (size_t)x * N;
#pragma unroll
            for (int e = 0; e < E; ++e) psi[e] = __ldg(src + t + T * e);
        } else {
            const float2* src = a.state + ((size_t)b * a.nx + x) * N;
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int y = t + T * e;
                psi[e] = (y <= a.yA || y >= a.yB) ? src[y] : make_float2(0.f, 0.f);
            }
        }
    };
    if constexpr (EARLY) load_psi();
    line_fft<Cfg, true>(g, sm, s_tw, t);
    if constexpr (!EARLY) load_psi();
    if constexpr (!FIRST) {
        line_fft<Cfg, true>(psi, sm, s_tw, t);
#pragma unroll
        for (int e = 0; e < E; ++e) psi[e] = cscale(psi[e], a.norm);
    }
    const size_t win = (size_t)(x + __ldg(a.posX + b)) * a.potNy + __ldg(a.posY + b);
    const float2* tr = a.trans_slice + win;
    if constexpr (SUM) {
        float2* gs = a.gsum + win;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const float2 tv = __ldg(tr + t + T * e);
            atomicAdd(gs + t + T * e, cmulc(g[e], psi[e]));  // conj(psi) g_phi
            g[e] = cmulc(g[e], tv);                          // conj(t) g_phi
        }
    } else {
        float2* gt = a.grad_t + ((size_t)b * a.nx + x) * N;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const float2 tv = __ldg(tr + t + T * e);
            gt[t + T * e] = cmulc(g[e], psi[e]);  // conj(psi) g_phi
            g[e] = cmulc(g[e], tv);               // conj(t) g_phi
        }
    }
    if constexpr (!FIRST) {
        line_fft<Cfg, false>(g, sm, s_tw, t);
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int y = t + T * e;
            if (!always_out_of_band<N, T>(e) && (y <= a.yA || y >= a.yB)) grow[y] = cscale(g[e], a.norm);
        }
    }
}

// dL/dV of one slice: sum the windows of all positions, then
// -2 sigma Im(conj(G) t).  Stage 1: blockIdx.z picks a chunk of DV_CHUNK
// positions, one thread per potential pixel sums that chunk in float
// (coalesced along Y; FP64 adds run at a small fraction of the FP32 rate on
// this part); stage 2 adds the chunks in double in a fixed order, so the
// result is deterministic.
constexpr int DV_CHUNK = 32;

__global__ void adj_dv_partial(const float2* __restrict__ grad_t, int npos, int nx, int ny, int potNx, int potNy,
                               const int* __restrict__ posX, const int* __restrict__ posY,
                               float2* __restrict__ partial) {
    const int Y = blockIdx.x * blockDim.x + threadIdx.x;
    const int X = blockIdx.y;
    if (Y >= potNy) return;
    const int p0 = blockIdx.z * DV_CHUNK, p1 = min(npos, p0 + DV_CHUNK);
    float gr = 0.f, gi = 0.f;
#pragma unroll 8
    for (int p = p0; p < p1; ++p) {
        const int lx = X - __ldg(posX + p), ly = Y - __ldg(posY + p);
        if (lx >= 0 && lx < nx && ly >= 0 && ly < ny) {
            const float2 v = __ldg(grad_t + ((size_t)p * nx + lx) * ny + ly);
            gr += v.x;
            gi += v.y;
        }
    }
    partial[((size_t)blockIdx.z * potNx + X) * potNy + Y] = make_float2(gr, gi);
}

__global__ void adj_dv_finish(const float2* __restrict__ partial, int nchunks, int potNx, int potNy,
                              const float2* __restrict__ trans_slice, double sigma, int accumulate,
                              float* __restrict__ dV) {
    const size_t n = (size_t)potNx * potNy;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double gr = 0.0, gi = 0.0;
        // unrolled so that several chunks' loads are in flight; the adds
        // stay in chunk order
#pragma unroll 8
        for (int c = 0; c < nchunks; ++c) {
            const float2 v = __ldg(partial + (size_t)c * n + i);
            gr += v.x;
            gi += v.y;
        }
        const float2 tv = trans_slice[i];
        // Im(conj(G) t) = gr*t.y - gi*t.x
        const float g = (float)(-2.0 * sigma * (gr * tv.y - gi * tv.x));
        dV[i] = accumulate ? dV[i] + g : g;
    }
}

// dL/dV of one slice from the summed windows, and the sum cleared for the
// next slice's row adjoint.
__global__ void adj_dv_from_sum(float2* __restrict__ gsum, size_t n, const float2* __restrict__ trans_slice,
                                float sigma2, int accumulate, float* __restrict__ dV) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 G = gsum[i], tv = trans_slice[i];
        // Im(conj(G) t) = G.x t.y - G.y t.x
        const float g = -sigma2 * (G.x * tv.y - G.y * tv.x);
        dV[i] = accumulate ? dV[i] + g : g;
        gsum[i] = make_float2(0.f, 0.f);
    }
}

// ---------------------------------------------- scatter-sum adjoint (atoms)
// dL/d(atomX, atomY) = sum over the atom's pixels and slices of
// dL/dV * dV/dr * dr/d(atom), dV/dr the slope of the radial linear
// interpolation (stem3/stemlib.cpp:957-1019), dr/datomX = -(x_pixel - atomX)/r.
// FP32 arithmetic (FP64 runs at a small fraction of the FP32 rate here): the
// per-thread sums over pixels are Kahan-compensated, because an atom's
// gradient is a small difference of large symmetric contributions, and the
// block reduction runs in double.  The radial interval is the forward's
// (stem3/stemlib.cpp:944-952: r and r/dr in double): the float radius is
// within 1e-6 relative of it, so only pixels whose r/dr lies within 2e-4 of
// a knot recompute it in double.
struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ void add(float v) {
        const float y = __fsub_rn(v, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
};

__global__ void __launch_bounds__(256) atoms_grad(const AtomJob* __restrict__ jobs, const float* const* __restrict__ luts,
                                                  int Nz, int Nr, int nzSub, float dx, float dy, double dr,
                                                  float inv_dr, float dzs,
                                                  int potNx, int potNy, int periodic, const float* __restrict__ dV,
                                                  double* __restrict__ grad) {
    const AtomJob J = jobs[blockIdx.x];
    const float* lut = luts[J.lut];
    const float* lutq = J.lutq >= 0 ? luts[J.lutq] : nullptr;
    const int w = J.iay1 - J.iay0 + 1;
    const int npx = (J.iax1 - J.iax0 + 1) * w;
    const size_t sliceStep = (size_t)potNx * potNy;
    const int limHi = Nr * (Nz - 1), limLo = -Nr * (Nz - 1), step = nzSub * Nr;
    const double dOffsZ = (double)(((float)(J.iAtomZ + J.iaz0) - J.atomZ / dzs) * (float)nzSub);
    const int iOffsZ0 = ((int)(dOffsZ + 0.5)) * Nr;
    const float q = J.q;
    Kahan gx, gy;
    for (int k = threadIdx.x; k < npx; k += blockDim.x) {
        const int iax = J.iax0 + k / w;
        const int iay = J.iay0 + k % w;
        // the reference's float offsets, rounded step by step (no FMA
        // contraction: an atom on a pixel must give r == 0 exactly)
        const float ddx = __fsub_rn(__fmul_rn((float)iax, dx), J.atomX);
        const float ddy = __fsub_rn(__fmul_rn((float)iay, dy), J.atomY);
        const float r2 = ddx * ddx + ddy * ddy;
        if (r2 <= 0.f) continue;
        const float rinv = rsqrtf(r2);
        const float r = r2 * rinv;
        const float rr = r * inv_dr;
        int ir = (int)floorf(rr);
        const float fr = rr - (float)ir;
        if (fr < 2e-4f || fr > 1.f - 2e-4f) {
            const double x2 = (double)ddx * ddx, y2 = (double)ddy * ddy;
            ir = (int)floor(sqrt(x2 + y2) / dr);
        }
        if (ir >= Nr - 1) continue;
        const int cx = periodic ? ((iax % potNx) + potNx) % potNx : iax;
        const int cy = periodic ? ((iay % potNy) + potNy) % potNy : iay;
        const float* g = dV + (size_t)(J.iAtomZ + J.iaz0) * sliceStep + (size_t)cx * potNy + cy;
        int iOffsZ = iOffsZ0;
        float dLdr = 0.f;
        for (int iaz = J.iaz0; iaz <= J.iaz1; iaz++) {
            int row = -1;
            if (iOffsZ < 0) {
                if (iOffsZ > limLo) row = -iOffsZ + Nr;
            } else if (iOffsZ < limHi) {
                row = iOffsZ;
            }
            if (row >= 0) {
                float slope = __ldg(lut + row + ir + 1) - __ldg(lut + row + ir);
                if (lutq) slope += q * (__ldg(lutq + row + ir + 1) - __ldg(lutq + row + ir));
                dLdr += __ldg(g) * slope;
            }
            g += sliceStep;
            iOffsZ += step;
        }
        // dV/dr = slope / dr
        dLdr *= inv_dr;
        gx.add(-dLdr * ddx * rinv);
        gy.add(-dLdr * ddy * rinv);
    }
    __shared__ double sx[256], sy[256];
    sx[threadIdx.x] = (double)gx.s - (double)gx.c;
    sy[threadIdx.x] = (double)gy.s - (double)gy.c;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sx[threadIdx.x] += sx[threadIdx.x + o];
            sy[threadIdx.x] += sy[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        grad[2 * (size_t)J.index] = sx[0];
        grad[2 * (size_t)J.index + 1] = sy[0];
    }
}

// --------------------------------------------------------------- launchers
template <int N>
static int last_n(const AdjLastArgs& a, cudaStream_t s) {
    using Cfg = typename LineCol<N>::cfg;
    constexpr int C = col_tile<N>();
    const size_t sm = sizeof(float2) * (N + (size_t)N * C);
    QS_TRY(smem_attr((const void*)adj_last_cols<N>, sm));
    const long nblk = (long)a.nwaves * (a.ny / C);
    adj_last_cols<N><<<(unsigned)nblk, dim3(C, Cfg::T), sm, s>>>(a);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

int launch_adj_last(const AdjLastArgs& a, cudaStream_t s) {
    if (!a.waves || !a.waves_out || !a.target || !a.loss_partial) {
        set_error("adjoint: last-slice pass given a null buffer");
        return QS_ERR_ARG;
    }
    switch (a.nx) {
        case 64: return last_n<64>(a, s);
        case 128: return last_n<128>(a, s);
        case 256: return last_n<256>(a, s);
        case 384: return last_n<384>(a, s);
        case 512: return last_n<512>(a, s);
        case 768: return last_n<768>(a, s);
        case 1024: return last_n<1024>(a, s);
    }
    set_error("adjoint: unsupported nx");
    return QS_ERR_UNSUPPORTED;
}

template <int N, bool FIRST, bool SUM>
static int adj_rows_n3(const AdjRowArgs& a, cudaStream_t s) {
    using Cfg = typename Line<N>::cfg;
    const size_t sm = sizeof(float2) * (N + ADJ_ROW_LINES * Cfg::SMEM);
    QS_TRY(smem_attr((const void*)adj_rows<N, FIRST, SUM>, sm));
    const long lines = (long)a.nwaves * a.nx;
    adj_rows<N, FIRST, SUM><<<(unsigned)(lines / ADJ_ROW_LINES), dim3(Cfg::T, ADJ_ROW_LINES), sm, s>>>(a);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

template <int N, bool FIRST>
static int adj_rows_n(const AdjRowArgs& a, cudaStream_t s) {
    return a.gsum ? adj_rows_n3<N, FIRST, true>(a, s) : adj_rows_n3<N, FIRST, false>(a, s);
}

template <bool FIRST>
static int adj_rows_any(const AdjRowArgs& a, cudaStream_t s) {
    switch (a.ny) {
        case 64: return adj_rows_n<64, FIRST>(a, s);
        case 128: return adj_rows_n<128, FIRST>(a, s);
        case 256: return adj_rows_n<256, FIRST>(a, s);
        case 384: return adj_rows_n<384, FIRST>(a, s);
        case 512: return adj_rows_n<512, FIRST>(a, s);
        case 768: return adj_rows_n<768, FIRST>(a, s);
        case 1024: return adj_rows_n<1024, FIRST>(a, s);
    }
    set_error("adjoint: unsupported ny");
    return QS_ERR_UNSUPPORTED;
}

int launch_adj_rows(const AdjRowArgs& a, bool first, cudaStream_t s) {
    if (!a.grad || !(a.grad_t || a.gsum) || (first ? !a.probe : !a.state)) {
        set_error("adjoint: row pass given a null buffer");
        return QS_ERR_ARG;
    }
    return first ? adj_rows_any<true>(a, s) : adj_rows_any<false>(a, s);
}

size_t dv_partial_bytes(int npos, int potNx, int potNy) {
    return sizeof(float2) * (size_t)((npos + DV_CHUNK - 1) / DV_CHUNK) * potNx * potNy;
}

int launch_dv_gather(const float2* grad_t, int npos, int nx, int ny, int potNx, int potNy, const int* posX,
                     const int* posY, const float2* trans_slice, double sigma, void* partial, float* dV,
                     bool accumulate, cudaStream_t s) {
    const int nchunks = (npos + DV_CHUNK - 1) / DV_CHUNK;
    adj_dv_partial<<<dim3((potNy + 127) / 128, potNx, nchunks), 128, 0, s>>>(grad_t, npos, nx, ny, potNx, potNy,
                                                                            posX, posY, (float2*)partial);
    QS_CUDA_TRY(cudaGetLastError());
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    adj_dv_finish<<<sms * 4, 256, 0, s>>>((const float2*)partial, nchunks, potNx, potNy, trans_slice, sigma,
                                          accumulate ? 1 : 0, dV);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(2);
    return QS_OK;
}

int launch_dv_from_sum(float2* gsum, int potNx, int potNy, const float2* trans_slice, double sigma, float* dV,
                       bool accumulate, cudaStream_t s) {
    const size_t n = (size_t)potNx * potNy;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long blocks = std::min<long>((long)sms * 4, (long)((n + 255) / 256));
    adj_dv_from_sum<<<(unsigned)std::max<long>(blocks, 1), 256, 0, s>>>(gsum, n, trans_slice, (float)(2.0 * sigma),
                                                                       accumulate ? 1 : 0, dV);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

int launch_atoms_grad(const AtomJob* d_jobs, int njobs, const float* const* d_luts, int Nz, int Nr, int nzSub,
                      const qs_params& p, const float* dV, double* grad, cudaStream_t s) {
    if (njobs <= 0) return QS_OK;
    const double dr = p.resolutionX / 2;
    const float inv_dr = (float)(1.0 / dr);
    atoms_grad<<<njobs, 256, 0, s>>>(d_jobs, d_luts, Nz, Nr, nzSub, p.resolutionX, p.resolutionY, dr, inv_dr,
                                     p.sliceThickness, p.potNx, p.potNy, p.nonPeriod ? 0 : 1, dV, grad);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

}  // namespace qs
