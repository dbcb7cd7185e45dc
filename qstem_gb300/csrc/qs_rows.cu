// qs_rows.cu -- the row pass of the multislice loop (transforms along y, the
// contiguous index) and the plain row line-FFT kernels; the column pass,
// the 2-D transforms and the band limit are in qs_multislice.cu.
#include <cuda_runtime.h>

#include <algorithm>

#include <string>

#include "qs_fft.cuh"
#include "qs_internal.h"
#include "qs_tuned.h"

namespace qs {

// lines per CTA of the plain line-FFT kernels (fft_rows)
constexpr int ROW_LINES = 8;

// lines per CTA of the row pass, per line length (qs_tuned.h)
constexpr int row_lines(int n) {
    return n == 64     ? QS_ROW_LINES_64
           : n == 128  ? QS_ROW_LINES_128
           : n == 256  ? QS_ROW_LINES_256
           : n == 384  ? QS_ROW_LINES_384
           : n == 512  ? QS_ROW_LINES_512
           : n == 768  ? QS_ROW_LINES_768
           : n == 1024 ? QS_ROW_LINES_1024
                       : 8;
}

// CTAs per SM the row pass is compiled for (register budget), per line
// length, from the measured table in qs_tuned.h
constexpr int row_min_blocks(int n) {
    return n == 64     ? QS_ROW_MIN_BLOCKS_64
           : n == 128  ? QS_ROW_MIN_BLOCKS_128
           : n == 256  ? QS_ROW_MIN_BLOCKS_256
           : n == 384  ? QS_ROW_MIN_BLOCKS_384
           : n == 512  ? QS_ROW_MIN_BLOCKS_512
           : n == 768  ? QS_ROW_MIN_BLOCKS_768
           : n == 1024 ? QS_ROW_MIN_BLOCKS_1024
                       : 1;
}

// Shared memory of the row pass: the twiddle table (N float2) and one padded
// exchange line per line transform.
// PW: the waves come from instances of different samplings (per-wave bands
// and step-to-slice table); a compile-time choice, so that the scan of one
// sampling carries none of it (its kernels take the plain RowCore)
template <bool PW> struct RowK { using type = RowArgs; };
template <> struct RowK<false> { using type = RowCore; };

// QS_ROW_WALK: at 512 and 1024 points the row pass launches this many times
// the CTAs resident at once, each walking blocks of lines (measured: 512
// 0.729 -> 0.689 us, 1024 3.09 -> 2.77 us per position-slice with 8); the
// other lengths launch one CTA per block (the walking form measured slower
// at 256)
#ifndef QS_ROW_WALK
#define QS_ROW_WALK 8
#endif
constexpr int row_walk(int n) { return (n == 512 || n == 1024) ? QS_ROW_WALK : 0; }
template <int N, int MODE, bool PW>
__global__ void __launch_bounds__(line_threads(N) * row_lines(N), row_min_blocks(N))
    ms_rows(typename RowK<PW>::type a, long nblocks) {
    using Cfg = typename Line<N>::cfg;
    constexpr int T = Cfg::T, E = Cfg::E;
    extern __shared__ float2 dsm[];
    float2* s_tw = dsm;
    float2* s_line = dsm + N + threadIdx.y * Cfg::SMEM;
    const int tid = threadIdx.x + T * threadIdx.y;
    for (int i = tid; i < Cfg::TW; i += T * row_lines(N)) s_tw[i] = a.tw[i];
    __syncthreads();

    // one block of row_lines(N) lines, or (row_walk) blocks walked by the
    // grid: each line's threads reuse their own exchange line, whose last
    // read precedes the transform's closing warp barrier
    auto block_of_lines = [&](long blk) {
    const int t = threadIdx.x;
    const long line = blk * row_lines(N) + threadIdx.y;
    const int b = (int)(line / a.nx);
    const int x = (int)(line - (long)b * a.nx);
    const SmemRow<Cfg::R0> sm{s_line};
    int yA = a.yA, yB = a.yB;
    if constexpr (PW) {
        const int2 v = __ldg(a.band + b);
        yA = v.x;
        yB = v.y;
    }
    float2 reg[E];
    if constexpr (MODE == ROW_FIRST) {
        const float2* src = a.probe + b * a.probe_stride + (size_t)x * N;
#pragma unroll
        for (int e = 0; e < E; ++e) reg[e] = __ldg(src + t + T * e);
    } else {
        const float2* src = a.waves + ((size_t)b * a.nx + x) * N;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int y = t + T * e;
            reg[e] = (y <= yA || y >= yB) ? src[y] : make_float2(0.f, 0.f);
        }
        line_fft<Cfg, true>(reg, sm, s_tw, t);
#pragma unroll
        for (int e = 0; e < E; ++e) reg[e] = cscale(reg[e], a.norm);
    }
    if constexpr (MODE == ROW_LAST) {
        float2* dst = a.exit_waves + ((size_t)b * a.nx + x) * N;
#pragma unroll
        for (int e = 0; e < E; ++e) dst[t + T * e] = reg[e];
    } else {
        // transmit (stem3/stemlib.cpp:2867-2888): window at (posX, posY)
        const float2* tr = a.trans_slice + b * a.trans_stride + (size_t)(x + __ldg(a.posX + b)) * a.potNy +
                           __ldg(a.posY + b);
        if constexpr (PW) tr += (size_t)__ldg(a.step_slice + b) * a.potNx * a.potNy;
#pragma unroll
        for (int e = 0; e < E; ++e) reg[e] = cmul(reg[e], __ldg(tr + t + T * e));
        line_fft<Cfg, false>(reg, sm, s_tw, t);
        float2* dst = (a.waves_out ? a.waves_out : a.waves) + ((size_t)b * a.nx + x) * N;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int y = t + T * e;
            if (!always_out_of_band<N, T>(e) && (y <= yA || y >= yB)) dst[y] = reg[e];
        }
    }
    };
    if constexpr (row_walk(N) > 0) {
        for (long blk = blockIdx.x; blk < nblocks; blk += gridDim.x) block_of_lines(blk);
    } else {
        block_of_lines(blockIdx.x);
    }
}

template <int N>
static size_t row_smem(int lines = row_lines(N)) {
    return sizeof(float2) * (N + (size_t)lines * Line<N>::cfg::SMEM);
}
template <int N, int MODE, bool PW>
static int rows_n(const RowArgs& a, cudaStream_t s) {
    using Cfg = typename Line<N>::cfg;
    const size_t sm = row_smem<N>();
    QS_TRY(smem_attr((const void*)ms_rows<N, MODE, PW>, sm));
    const long lines = (long)a.nwaves * a.nx;
    if (lines % row_lines(N)) {
        set_error("row pass: nwaves*nx must be a multiple of " + std::to_string(row_lines(N)));
        return QS_ERR_ARG;
    }
    dim3 block(Cfg::T, row_lines(N));
    const long nblocks = lines / row_lines(N);
    long grid = nblocks;
    if (row_walk(N) > 0) {
        // row_walk times the CTAs that are resident at once, each walking blocks
        int resident = 0, sms = 0;
        QS_TRY(resident_ctas((const void*)ms_rows<N, MODE, PW>, Cfg::T * row_lines(N), sm, &resident, &sms));
        if (resident > 0) grid = std::min<long>(nblocks, (long)resident * sms * row_walk(N));
    }
    ms_rows<N, MODE, PW><<<(unsigned)grid, block, sm, s>>>(static_cast<const typename RowK<PW>::type&>(a),
                                                          nblocks);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

template <int MODE, bool PW>
static int rows_mode(const RowArgs& a, cudaStream_t s) {
    switch (a.ny) {
        case 64: return rows_n<64, MODE, PW>(a, s);
        case 128: return rows_n<128, MODE, PW>(a, s);
        case 256: return rows_n<256, MODE, PW>(a, s);
        case 384: return rows_n<384, MODE, PW>(a, s);
        case 512: return rows_n<512, MODE, PW>(a, s);
        case 768: return rows_n<768, MODE, PW>(a, s);
        case 1024: return rows_n<1024, MODE, PW>(a, s);
    }
    set_error("row pass: unsupported ny");
    return QS_ERR_UNSUPPORTED;
}

int launch_rows(const RowArgs& a, RowMode mode, cudaStream_t s) {
    if ((mode == ROW_FIRST ? !a.probe : !a.waves) || (mode == ROW_LAST ? !a.exit_waves : !(a.waves_out || a.waves))) {
        set_error("row pass given a null buffer");
        return QS_ERR_ARG;
    }
    const bool pw = a.band != nullptr;
    if (pw != (a.step_slice != nullptr) || (pw && mode == ROW_LAST)) {
        set_error("row pass: per-wave bands and step table go together, and not with exit waves");
        return QS_ERR_ARG;
    }
    if (mode == ROW_FIRST) return pw ? rows_mode<ROW_FIRST, true>(a, s) : rows_mode<ROW_FIRST, false>(a, s);
    if (mode == ROW_MID) return pw ? rows_mode<ROW_MID, true>(a, s) : rows_mode<ROW_MID, false>(a, s);
    return rows_mode<ROW_LAST, false>(a, s);
}

// Row passes of the transmission band limit (initSTEMSlices,
// stem3/stemlib.cpp:2305-2336), which bracket one column pass:
//   bl_rows_fwd  FFT_y of the transmission function, and only the in-band
//                ky (iy <= yA or iy >= yB) stored: the mask zeroes every
//                other column
//   bl_rows_inv  the in-band ky (the others read as the zeros the mask
//                gives them), IFFT_y, the whole line stored
// The values are those of the unpruned 2-D transform, mask and inverse; the
// out-of-band columns are never written or read in between.  (The phase
// grating stays a kernel of its own: its sincosf, fused into the transform,
// made the pass issue-bound at twice the time of the two kernels.)
template <int N>
__global__ void __launch_bounds__(line_threads(N) * ROW_LINES)
    bl_rows_fwd(float2* __restrict__ data, long nlines, int yA, int yB, const float2* tw) {
    using Cfg = typename Line<N>::cfg;
    constexpr int T = Cfg::T, E = Cfg::E;
    extern __shared__ float2 dsm[];
    float2* s_tw = dsm;
    float2* s_line = dsm + N + threadIdx.y * Cfg::SMEM;
    const int tid = threadIdx.x + T * threadIdx.y;
    for (int i = tid; i < Cfg::TW; i += T * ROW_LINES) s_tw[i] = tw[i];
    __syncthreads();
    const long line = (long)blockIdx.x * ROW_LINES + threadIdx.y;
    const bool ok = line < nlines;
    float2* p = data + (size_t)(ok ? line : 0) * N;
    const int t = threadIdx.x;
    float2 reg[E];
#pragma unroll
    for (int e = 0; e < E; ++e) reg[e] = ok ? p[t + T * e] : make_float2(0.f, 0.f);
    line_fft<Cfg, false>(reg, SmemRow<Cfg::R0>{s_line}, s_tw, t);
    if (ok) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int y = t + T * e;
            if (y <= yA || y >= yB) p[y] = reg[e];
        }
    }
}

template <int N>
__global__ void __launch_bounds__(line_threads(N) * ROW_LINES)
    bl_rows_inv(float2* __restrict__ data, long nlines, int yA, int yB, const float2* tw) {
    using Cfg = typename Line<N>::cfg;
    constexpr int T = Cfg::T, E = Cfg::E;
    extern __shared__ float2 dsm[];
    float2* s_tw = dsm;
    float2* s_line = dsm + N + threadIdx.y * Cfg::SMEM;
    const int tid = threadIdx.x + T * threadIdx.y;
    for (int i = tid; i < Cfg::TW; i += T * ROW_LINES) s_tw[i] = tw[i];
    __syncthreads();
    const long line = (long)blockIdx.x * ROW_LINES + threadIdx.y;
    const bool ok = line < nlines;
    float2* p = data + (size_t)(ok ? line : 0) * N;
    const int t = threadIdx.x;
    float2 reg[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int y = t + T * e;
        reg[e] = (ok && (y <= yA || y >= yB)) ? p[y] : make_float2(0.f, 0.f);
    }
    line_fft<Cfg, true>(reg, SmemRow<Cfg::R0>{s_line}, s_tw, t);
    if (ok) {
#pragma unroll
        for (int e = 0; e < E; ++e) p[t + T * e] = reg[e];
    }
}

template <int N>
static int bl_rows_n(float2* data, long nlines, int yA, int yB, bool inverse, cudaStream_t s) {
    const size_t sm = row_smem<N>(ROW_LINES);
    dim3 block(Line<N>::cfg::T, ROW_LINES);
    const unsigned grid = (unsigned)((nlines + ROW_LINES - 1) / ROW_LINES);
    if (inverse) {
        QS_TRY(smem_attr((const void*)bl_rows_inv<N>, sm));
        bl_rows_inv<N><<<grid, block, sm, s>>>(data, nlines, yA, yB, twiddles(N));
    } else {
        QS_TRY(smem_attr((const void*)bl_rows_fwd<N>, sm));
        bl_rows_fwd<N><<<grid, block, sm, s>>>(data, nlines, yA, yB, twiddles(N));
    }
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

int bandlimit_rows(float2* data, int n, long nlines, int yA, int yB, bool inverse, cudaStream_t s) {
    if (!twiddles(n)) {
        set_error("twiddle table allocation failed");
        return QS_ERR_NOMEM;
    }
    switch (n) {
        case 64: return bl_rows_n<64>(data, nlines, yA, yB, inverse, s);
        case 128: return bl_rows_n<128>(data, nlines, yA, yB, inverse, s);
        case 256: return bl_rows_n<256>(data, nlines, yA, yB, inverse, s);
        case 384: return bl_rows_n<384>(data, nlines, yA, yB, inverse, s);
        case 512: return bl_rows_n<512>(data, nlines, yA, yB, inverse, s);
        case 768: return bl_rows_n<768>(data, nlines, yA, yB, inverse, s);
        case 1024: return bl_rows_n<1024>(data, nlines, yA, yB, inverse, s);
    }
    set_error("band limit: unsupported row length " + std::to_string(n));
    return QS_ERR_UNSUPPORTED;
}

template <int N, bool INV>
__global__ void __launch_bounds__(line_threads(N) * ROW_LINES) fft_rows(float2* data, long nlines, const float2* tw) {
    using Cfg = typename Line<N>::cfg;
    constexpr int T = Cfg::T, E = Cfg::E;
    extern __shared__ float2 dsm[];
    float2* s_tw = dsm;
    float2* s_line = dsm + N + threadIdx.y * Cfg::SMEM;
    const int tid = threadIdx.x + T * threadIdx.y;
    for (int i = tid; i < Cfg::TW; i += T * ROW_LINES) s_tw[i] = tw[i];
    __syncthreads();
    const long line = (long)blockIdx.x * ROW_LINES + threadIdx.y;
    const bool ok = line < nlines;
    float2* p = data + (ok ? line : 0) * N;
    const int t = threadIdx.x;
    float2 reg[E];
#pragma unroll
    for (int e = 0; e < E; ++e) reg[e] = ok ? p[t + T * e] : make_float2(0.f, 0.f);
    line_fft<Cfg, INV>(reg, SmemRow<Cfg::R0>{s_line}, s_tw, t);
    if (ok) {
#pragma unroll
        for (int e = 0; e < E; ++e) p[t + T * e] = reg[e];
    }
}

template <int N, bool INV>
static int fft_rows_n(float2* data, long nlines, cudaStream_t s) {
    const size_t sm = row_smem<N>(ROW_LINES);
    QS_TRY(smem_attr((const void*)fft_rows<N, INV>, sm));
    dim3 block(Line<N>::cfg::T, ROW_LINES);
    fft_rows<N, INV><<<(unsigned)((nlines + ROW_LINES - 1) / ROW_LINES), block, sm, s>>>(data, nlines, twiddles(N));
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

template <bool INV>
static int fft_rows_any(float2* data, int n, long nlines, cudaStream_t s) {
    switch (n) {
        case 64: return fft_rows_n<64, INV>(data, nlines, s);
        case 128: return fft_rows_n<128, INV>(data, nlines, s);
        case 256: return fft_rows_n<256, INV>(data, nlines, s);
        case 384: return fft_rows_n<384, INV>(data, nlines, s);
        case 512: return fft_rows_n<512, INV>(data, nlines, s);
        case 768: return fft_rows_n<768, INV>(data, nlines, s);
        case 1024: return fft_rows_n<1024, INV>(data, nlines, s);
    }
    set_error("fft2d: unsupported row length " + std::to_string(n));
    return QS_ERR_UNSUPPORTED;
}

int line_fft_rows(float2* data, int n, long nlines, bool inverse, cudaStream_t s) {
    return inverse ? fft_rows_any<true>(data, n, nlines, s) : fft_rows_any<false>(data, n, nlines, s);
}

}  // namespace qs
