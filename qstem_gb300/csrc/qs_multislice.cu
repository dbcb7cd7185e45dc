// qs_multislice.cu -- the fused per-slice passes of the multislice loop: the
// column pass, the generic 2-D transforms and the band limit (the row pass
// is in qs_rows.cu, compiled in parallel).
//
// The reference's slice step (runMulsSTEM, stem3/stemlib.cpp:2403-2486) is
//   transmit -> FFT2 -> propagate_slow -> collectIntensity -> IFFT2 -> /N.
// Here the 2-D transforms are split into their row (y, contiguous) and
// column (x, strided) halves and the pointwise work is fused into them, so
// that a wave crosses HBM twice per slice:
//   row pass    IFFT_y of the previous slice, 1/N, transmit with slice s,
//               FFT_y                              (ms_rows)
//   column pass FFT_x, propagator and band limit, detector sums and the
//               diffraction pattern on output slices, IFFT_x   (ms_cols)
// The 2/3 band limit zeroes every column ky with ky^2 >= k2max, so those
// columns are neither stored by the row pass nor touched by the column pass,
// and the next row pass reads them as zeros.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <utility>
#include <vector>

#include "qs_fft.cuh"
#include "qs_internal.h"
#include "qs_tuned.h"

namespace qs {


// Column pass, persistent: each CTA walks the (wave, column tile) work items
// blockIdx.x, blockIdx.x + gridDim.x, ...  While one tile is transformed, the
// next one is copied into the other shared-memory stage with cp.async (16
// bytes a copy: a pair of columns of one row, half the copy instructions of
// one element a copy, and 12 % less time for the 1024-point pass); once every
// thread has read its elements of the current stage into registers, that
// stage serves as the FFT exchange scratch.
// the column pass's register budget (qs_tuned.h)
constexpr int col_min_blocks(int n) {
    return n == 64     ? QS_COL_MIN_BLOCKS_64
           : n == 128  ? QS_COL_MIN_BLOCKS_128
           : n == 256  ? QS_COL_MIN_BLOCKS_256
           : n == 384  ? QS_COL_MIN_BLOCKS_384
           : n == 512  ? QS_COL_MIN_BLOCKS_512
           : n == 768  ? QS_COL_MIN_BLOCKS_768
           : n == 1024 ? QS_COL_MIN_BLOCKS_1024
                       : 1;
}

// shared-memory tile stages of the column pass (qs_tuned.h)
constexpr int col_stages(int n) {
    return n == 64     ? QS_COL_STAGES_64
           : n == 128  ? QS_COL_STAGES_128
           : n == 256  ? QS_COL_STAGES_256
           : n == 384  ? QS_COL_STAGES_384
           : n == 512  ? QS_COL_STAGES_512
           : n == 768  ? QS_COL_STAGES_768
           : n == 1024 ? QS_COL_STAGES_1024
                       : 2;
}

// PW: per-wave work items and propagator/k^2 tables (waves of different
// samplings; no detectors), compiled only into that variant
template <int N, bool DET, bool INVERSE, bool PW>
__global__ void __launch_bounds__(col_tile<N>() * col_line_threads(N), col_min_blocks(N))
    ms_cols(ColArgs a, long nitems) {
    using Cfg = typename LineCol<N>::cfg;
    constexpr int T = Cfg::T, E = Cfg::E, C = col_tile<N>();
    constexpr int NT = C * T;
    constexpr int NWARPS = (NT + 31) / 32;
    constexpr int STAGES = col_stages(N);
    static_assert(STAGES == 1 || STAGES == 2, "one or two tile stages");
    extern __shared__ float2 dsm[];
    float2* s_tw = dsm;
    float2* s_stage = dsm + N;  // STAGES stages of N*C
    __shared__ double s_det[QS_MAX_DETECTORS][NWARPS];
    const int tid = threadIdx.x + C * threadIdx.y;
    const int c = threadIdx.x, t = threadIdx.y;
    for (int i = tid; i < Cfg::TW; i += NT) s_tw[i] = a.tw[i];

    // work item -> wave b, first column ky0 of its tile, tile index
    auto decode = [&](long item, int& b, int& ky0, int& tile) {
        if constexpr (PW) {
            const int2 v = __ldg(a.items + item);
            b = v.x;
            ky0 = v.y;
            tile = 0;
        } else {
            tile = (int)(item % a.ntiles);
            b = (int)(item / a.ntiles);
            ky0 = __ldg(a.tiles + tile);
        }
    };
    auto prefetch = [&](long item, int stage) {
        if (item < nitems) {
            // 16-byte copies of column pairs (consecutive threads take
            // consecutive pairs of one row); the elements a thread transforms
            // come from other threads' copies
            constexpr int P2 = C / 2, RS = NT / P2;
            static_assert(C % 2 == 0 && N % RS == 0, "whole column pairs and rows");
            const int c2 = tid % P2, r0 = tid / P2;
            int b, ky0, tile;
            decode(item, b, ky0, tile);
            const float2* src = a.waves + (size_t)b * a.nx * a.ny + ky0 + 2 * c2;
            float2* dst = s_stage + stage * N * C + 2 * c2;
#pragma unroll
            for (int k = 0; k < N / RS; ++k) {
                const int row = r0 + RS * k;
                cp_async16(dst + row * C, src + (size_t)row * a.ny);
            }
        }
        cp_async_commit();
    };

    long item = blockIdx.x;
    prefetch(item, 0);
    __syncthreads();
    for (int it = 0; item < nitems; ++it, item += gridDim.x) {
        if constexpr (STAGES == 2) {
            prefetch(item + gridDim.x, (it + 1) & 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        float2* stage = s_stage + (STAGES == 2 ? (it & 1) : 0) * N * C;
        __syncthreads();  // every thread's copies of this tile have landed
        float2 reg[E];
#pragma unroll
        for (int e = 0; e < E; ++e) reg[e] = stage[(t + T * e) * C + c];
        __syncthreads();  // all elements read before the stage becomes exchange scratch
        const SmemCol<C> sm{stage, c};
        line_fft<Cfg, false, true>(reg, sm, s_tw, t);

        int b, ky0, tile;
        decode(item, b, ky0, tile);
        const int ky = ky0 + c;
        // the wave's propagator and k^2 tables
        const float *kx2t = a.kx2, *ky2t = a.ky2;
        const float2 *pxt = a.px, *pyt = a.py;
        float k2max = a.k2max;
        if constexpr (PW) {
            kx2t += (size_t)b * a.nx;
            pxt += (size_t)b * a.nx;
            ky2t += (size_t)b * a.ny;
            pyt += (size_t)b * a.ny;
            k2max = __ldg(a.k2max_w + b);
        }
        // propagate_slow (stem3/stemlib.cpp:2831-2849)
        const float ky2 = __ldg(ky2t + ky);
        const float2 pyv = __ldg(pyt + ky);
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int kx = t + T * e;
            const float kx2 = __ldg(kx2t + kx);
            if (!always_out_of_band<N, T>(e) && kx2 < k2max && (kx2 + ky2) < k2max)
                reg[e] = cmul(cmul(reg[e], pyv), __ldg(pxt + kx));
            else
                reg[e] = make_float2(0.f, 0.f);
        }

        if constexpr (DET) {
            // collectIntensity (stem3/stemlib.cpp:2615-2657): |psi(k)|^2 in
            // float, summed per annulus.  The sums of a thread's E pixels and
            // of a warp are FP32 (positive terms: relative error ~1e-6; FP64
            // adds run at a small fraction of the FP32 rate on this part); the
            // warps of a CTA and the CTAs are added in double.
            const int lane = tid & 31, warp = tid >> 5;
            for (int d = 0; d < a.ndet; ++d) {
                float acc = 0.f;
                const float lo = a.k2in[d], hi = a.k2out[d];
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const float k2 = __ldg(kx2t + t + T * e) + ky2;
                    const float I = reg[e].x * reg[e].x + reg[e].y * reg[e].y;
                    if (k2 >= lo && k2 <= hi) acc += I;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0) s_det[d][warp] = (double)acc;
            }
            if (a.diffpat) {
                float* dp = a.diffpat + (size_t)b * a.nx * a.ny + (ky + a.ny / 2) % a.ny;
                const float sc = (float)a.scaleDiff;
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const int kx = t + T * e;
                    const float I = reg[e].x * reg[e].x + reg[e].y * reg[e].y;
                    dp[(size_t)((kx + a.nx / 2) % a.nx) * a.ny] = I * sc;
                }
            }
            __syncthreads();
            if (tid < a.ndet) {
                double sum = 0.0;
                for (int w = 0; w < NWARPS; ++w) sum += s_det[tid][w];
                a.partial[((size_t)b * a.ntiles + tile) * a.ndet + tid] = sum;
            }
        }
        if constexpr (INVERSE) {
            line_fft<Cfg, true, true>(reg, sm, s_tw, t);
            float2* col = (a.waves_out ? a.waves_out : a.waves) + (size_t)b * a.nx * a.ny + ky;
#pragma unroll
            for (int e = 0; e < E; ++e) col[(size_t)(t + T * e) * a.ny] = reg[e];
        }
        __syncthreads();  // scratch and s_det reads done before the stage is refilled
        if constexpr (STAGES == 1) prefetch(item + gridDim.x, 0);
    }
    cp_async_wait<0>();
}

__global__ void det_finalize(const double* __restrict__ partial, int nwaves, int ntiles, int ndet, double scale,
                             const int* __restrict__ detPosX, const int* __restrict__ detPosY, int scanYN,
                             int npix, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nwaves * ndet) return;
    const int b = i / ndet, d = i - b * ndet;
    double s = 0.0;
    for (int k = 0; k < ntiles; ++k) s += partial[((size_t)b * ntiles + k) * ndet + d];
    out[(size_t)d * npix + (size_t)detPosX[b] * scanYN + detPosY[b]] = (float)(s * scale);
}

// ------------------------------------------------------------- launchers
// A kernel's dynamic shared-memory limit belongs to one device's context:
// set it once per (device, kernel), under a lock (contexts may run on
// several threads and devices).
static std::mutex g_attr_mu;
static std::map<std::pair<int, const void*>, size_t> g_attr;
static std::map<std::tuple<int, const void*, int, size_t>, std::pair<int, int>> g_occ;

int smem_attr(const void* func, size_t bytes) {
    int dev = 0;
    QS_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_attr_mu);
    size_t& have = g_attr[{dev, func}];
    if (bytes > have) {
        QS_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        have = bytes;
    }
    return QS_OK;
}

// CTAs of `func` resident per SM on the current device for `threads` and
// `bytes` of dynamic shared memory, and the device's SM count (cached).
int resident_ctas(const void* func, int threads, size_t bytes, int* ctas, int* sms) {
    int dev = 0;
    QS_CUDA_TRY(cudaGetDevice(&dev));
    QS_TRY(smem_attr(func, bytes));
    std::lock_guard<std::mutex> lk(g_attr_mu);
    auto key = std::make_tuple(dev, func, threads, bytes);
    auto it = g_occ.find(key);
    if (it == g_occ.end()) {
        int r = 0, n = 0;
        QS_CUDA_TRY(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
        QS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, func, threads, bytes));
        it = g_occ.emplace(key, std::make_pair(r, n)).first;
    }
    *ctas = it->second.first;
    *sms = it->second.second;
    return QS_OK;
}

template <int N>
static size_t col_smem() {
    return sizeof(float2) * (N + (size_t)col_stages(N) * N * col_tile<N>());
}
template <int N>
static size_t col_smem_plain() {
    return sizeof(float2) * (N + (size_t)N * col_tile<N>());
}

template <int N, bool DET, bool INV, bool PW>
static int cols_n3(const ColArgs& a, cudaStream_t s) {
    using Cfg = typename LineCol<N>::cfg;
    const size_t sm = col_smem<N>();
    int resident = 0, sms = 0;  // CTAs per SM (occupancy calculator), SMs
    QS_TRY(resident_ctas((const void*)ms_cols<N, DET, INV, PW>, col_tile<N>() * Cfg::T, sm, &resident, &sms));
    if (resident < 1) {
        set_error("column pass does not fit on an SM");
        return QS_ERR_UNSUPPORTED;
    }
    dim3 block(col_tile<N>(), Cfg::T);
    const long nitems = PW ? a.nitems : (long)a.nwaves * a.ntiles;
    if (nitems <= 0) return QS_OK;
    const long grid = std::min<long>(nitems, (long)sms * resident);
    ms_cols<N, DET, INV, PW><<<(unsigned)grid, block, sm, s>>>(a, nitems);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

template <int N>
static int cols_n(const ColArgs& a, cudaStream_t s) {
    const bool det = a.ndet > 0 || a.diffpat != nullptr;
    if (a.items) {
        // per-wave work items and tables: no detector sums; the pattern of
        // the waves that end here, or the inverse for those that go on
        if (a.ndet > 0 || !a.per_wave || !a.k2max_w) {
            set_error("column pass: per-wave work items need per-wave tables and carry no detector sums");
            return QS_ERR_ARG;
        }
        if (a.inverse) return cols_n3<N, false, true, true>(a, s);
        return cols_n3<N, true, false, true>(a, s);
    }
    if (det) return a.inverse ? cols_n3<N, true, true, false>(a, s) : cols_n3<N, true, false, false>(a, s);
    return a.inverse ? cols_n3<N, false, true, false>(a, s) : cols_n3<N, false, false, false>(a, s);
}

int launch_cols(const ColArgs& a, cudaStream_t s) {
    if (!a.waves) {
        set_error("column pass given a null buffer");
        return QS_ERR_ARG;
    }
    switch (a.nx) {
        case 64: return cols_n<64>(a, s);
        case 128: return cols_n<128>(a, s);
        case 256: return cols_n<256>(a, s);
        case 384: return cols_n<384>(a, s);
        case 512: return cols_n<512>(a, s);
        case 768: return cols_n<768>(a, s);
        case 1024: return cols_n<1024>(a, s);
    }
    set_error("column pass: unsupported nx");
    return QS_ERR_UNSUPPORTED;
}

int col_tile_width(int nx) {
    switch (nx) {
        case 64: return col_tile<64>();
        case 128: return col_tile<128>();
        case 256: return col_tile<256>();
        case 384: return col_tile<384>();
        case 512: return col_tile<512>();
        case 768: return col_tile<768>();
        case 1024: return col_tile<1024>();
    }
    return 8;
}

int launch_det_finalize(const double* partial, int nwaves, int ntiles, int ndet, double scale,
                        const int* detPosX, const int* detPosY, int scanYN, int npix, float* det_out,
                        cudaStream_t s) {
    const int n = nwaves * ndet;
    if (n <= 0) return QS_OK;
    det_finalize<<<(n + 255) / 256, 256, 0, s>>>(partial, nwaves, ntiles, ndet, scale, detPosX, detPosY, scanYN,
                                                 npix, det_out);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

// ------------------------------------------------ generic 2-D transforms
template <int N, bool INV>
__global__ void __launch_bounds__(col_tile<N>() * col_line_threads(N))
    fft_cols(float2* data, int ncols, const float2* tw) {
    // columns of length N, row stride ncols; blockIdx.y = array index
    using Cfg = typename LineCol<N>::cfg;
    constexpr int T = Cfg::T, E = Cfg::E, C = col_tile<N>();
    extern __shared__ float2 dsm[];
    float2* s_tw = dsm;
    float2* s_tile = dsm + N;
    const int tid = threadIdx.x + C * threadIdx.y;
    for (int i = tid; i < Cfg::TW; i += C * T) s_tw[i] = tw[i];
    __syncthreads();
    const int c = threadIdx.x, t = threadIdx.y;
    const int col = blockIdx.x * C + c;
    const bool ok = col < ncols;
    float2* p = data + (size_t)blockIdx.y * N * ncols + (ok ? col : 0);
    float2 reg[E];
#pragma unroll
    for (int e = 0; e < E; ++e) reg[e] = ok ? p[(size_t)(t + T * e) * ncols] : make_float2(0.f, 0.f);
    line_fft<Cfg, INV, true>(reg, SmemCol<C>{s_tile, c}, s_tw, t);
    if (ok) {
#pragma unroll
        for (int e = 0; e < E; ++e) p[(size_t)(t + T * e) * ncols] = reg[e];
    }
}

template <int N, bool INV>
static int fft_cols_n(float2* data, int ncols, int howmany, cudaStream_t s) {
    const size_t sm = col_smem_plain<N>();
    QS_TRY(smem_attr((const void*)fft_cols<N, INV>, sm));
    constexpr int C = col_tile<N>();
    dim3 block(C, LineCol<N>::cfg::T);
    dim3 grid((ncols + C - 1) / C, howmany);
    fft_cols<N, INV><<<grid, block, sm, s>>>(data, ncols, twiddles(N, true));
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

template <bool INV>
static int fft_cols_any(float2* data, int n, int ncols, int howmany, cudaStream_t s) {
    switch (n) {
        case 64: return fft_cols_n<64, INV>(data, ncols, howmany, s);
        case 128: return fft_cols_n<128, INV>(data, ncols, howmany, s);
        case 256: return fft_cols_n<256, INV>(data, ncols, howmany, s);
        case 384: return fft_cols_n<384, INV>(data, ncols, howmany, s);
        case 512: return fft_cols_n<512, INV>(data, ncols, howmany, s);
        case 768: return fft_cols_n<768, INV>(data, ncols, howmany, s);
        case 1024: return fft_cols_n<1024, INV>(data, ncols, howmany, s);
    }
    set_error("fft2d: unsupported column length " + std::to_string(n));
    return QS_ERR_UNSUPPORTED;
}

int fft2d(float2* data, int n0, int n1, int howmany, bool inverse, cudaStream_t s) {
    if (!line_supported(n0) || !line_supported(n1)) {
        set_error("fft2d: size " + std::to_string(n0) + "x" + std::to_string(n1) + " not supported");
        return QS_ERR_UNSUPPORTED;
    }
    const long lines = (long)n0 * howmany;
    if (inverse) {
        QS_TRY(line_fft_rows(data, n1, lines, true, s));
        QS_TRY(fft_cols_any<true>(data, n0, n1, howmany, s));
    } else {
        QS_TRY(line_fft_rows(data, n1, lines, false, s));
        QS_TRY(fft_cols_any<false>(data, n0, n1, howmany, s));
    }
    return QS_OK;
}

// The transmission band limit of initSTEMSlices (stem3/stemlib.cpp:2305-2336)
// on every slice of `data` (howmany slices of n0 x n1) in three passes:
// forward line FFTs along y that store only the in-band columns
// (bl_rows_fwd); one column pass over the tiles holding them (FFT_x, the mask
// with its 1/N scale as a separable "propagator" of (1/N, 0) x (1, 0) limited
// to k^2 < k2max, IFFT_x); inverse line FFTs along y that read the other
// columns as zeros (bl_rows_inv).  Columns ky are in band iff ky <= yA or
// ky >= yB; tab: device tables kx2[n0], ky2[n1], px[n0] = (1/N, 0),
// py[n1] = (1, 0), tiles[ntiles] (first columns of the in-band tiles).
int bandlimit_lines(float2* data, int n0, int n1, int howmany, const float* kx2, const float* ky2,
                    const float2* px, const float2* py, const int* tiles, int ntiles, int yA, int yB, float k2max,
                    cudaStream_t s) {
    if (!line_supported(n0) || !line_supported(n1)) {
        set_error("band limit: size " + std::to_string(n0) + "x" + std::to_string(n1) + " not supported");
        return QS_ERR_UNSUPPORTED;
    }
    const float2* tw = twiddles(n0, true);
    if (!tw || !twiddles(n1)) {
        set_error("twiddle table allocation failed");
        return QS_ERR_NOMEM;
    }
    const long lines = (long)n0 * howmany;
    QS_TRY(bandlimit_rows(data, n1, lines, yA, yB, false, s));
    ColArgs ca{};
    ca.nx = n0;
    ca.ny = n1;
    ca.nwaves = howmany;
    ca.waves = data;
    ca.waves_out = nullptr;
    ca.tw = tw;
    ca.kx2 = kx2;
    ca.ky2 = ky2;
    ca.px = px;
    ca.py = py;
    ca.k2max = k2max;
    ca.tiles = tiles;
    ca.ntiles = ntiles;
    ca.inverse = 1;
    ca.ndet = 0;
    ca.diffpat = nullptr;
    QS_TRY(launch_cols(ca, s));
    QS_TRY(bandlimit_rows(data, n1, lines, yA, yB, true, s));
    return QS_OK;
}

template <class Cfg>
static void fill_twiddles(std::vector<float2>& h) {
    using RAD = typename Cfg::rad;
    constexpr int N = Cfg::N;
    h.assign(N, make_float2(0.f, 0.f));
    for (int p = 1; p < Cfg::PASSES; ++p) {
        const int R = RAD::at(p), Ns = RAD::prefix(p), off = Cfg::tw_offset(p);
        for (int r = 1; r < R; ++r)
            for (int jm = 0; jm < Ns; ++jm) {
                // exp(-2 pi i r jm/(Ns R)), angle reduced exactly in turns
                double turns = (double)(r * jm) / (double)(Ns * R);
                turns -= std::floor(turns + 0.5);
                const double ang = -2.0 * kPi * turns;
                h[off + (r - 1) * Ns + jm] = make_float2((float)std::cos(ang), (float)std::sin(ang));
            }
    }
}

template <int N>
static void fill_kind(std::vector<float2>& h, bool col) {
    if (col) fill_twiddles<typename LineCol<N>::cfg>(h);
    else fill_twiddles<typename Line<N>::cfg>(h);
}

int twiddle_host(int n, std::vector<float2>& h, bool col) {
    switch (n) {
        case 64: fill_kind<64>(h, col); return QS_OK;
        case 128: fill_kind<128>(h, col); return QS_OK;
        case 256: fill_kind<256>(h, col); return QS_OK;
        case 384: fill_kind<384>(h, col); return QS_OK;
        case 512: fill_kind<512>(h, col); return QS_OK;
        case 768: fill_kind<768>(h, col); return QS_OK;
        case 1024: fill_kind<1024>(h, col); return QS_OK;
    }
    set_error("no line transform of length " + std::to_string(n));
    return QS_ERR_UNSUPPORTED;
}

const float2* twiddles(int n, bool col) {
    static std::mutex mu;
    static std::map<std::tuple<int, int, bool>, float2*> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_tuple(dev, n, col);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    std::vector<float2> h;
    if (twiddle_host(n, h, col) != QS_OK) return nullptr;
    float2* d = nullptr;
    if (cudaMalloc(&d, sizeof(float2) * n) != cudaSuccess) return nullptr;
    cudaMemcpy(d, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
    cache[key] = d;
    return d;
}

}  // namespace qs
