// qs_dft.cu -- 2-D DFTs of sizes the line FFTs do not cover (prime or other
// lengths of the potential grid), as batched complex FP32 matrix products.
//
// initSTEMSlices band-limits every slice of the transmission stack with a
// forward and an inverse 2-D transform on the potential grid
// (stem3/stemlib.cpp:2305-2336; FFTW plans of any size, stem3/stem3.cpp:1534-
// 1539).  Potential grids such as 307^2 (prime), 563^2 (prime) or 298^2
// (2 x 149) have no fast factorisation here; their transforms are the
// products  rows: Y = X F_ny,  columns: Z = F_nx Y  with the DFT matrix
// F_n[j][k] = exp(-+2 pi i jk/n) (symmetric), computed once per size in
// double with the angle reduced exactly (jk mod n) and stored as c64.
// A slice of 563^2 costs 4 * 563^3 complex multiply-adds per transform pair
// direction -- a few ms for a 40-slice stack, once per slice build.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "qs_internal.h"

namespace qs {

constexpr int DBM = 64, DBN = 64, DBK = 16, DTHREADS = 256;

// C[b] = A[b] * B[b]: A M x K, B K x N, C M x N, complex, row-major, batch
// strides in elements (0: the same matrix for every b).
__global__ void __launch_bounds__(DTHREADS) cgemm_batched(const float2* __restrict__ A, size_t strideA,
                                                          const float2* __restrict__ B, size_t strideB,
                                                          float2* __restrict__ C, size_t strideC, int M, int N,
                                                          int K) {
    __shared__ float2 As[DBK][DBM + 1];
    __shared__ float2 Bs[DBK][DBN + 1];
    const int b = blockIdx.z;
    A += b * strideA;
    B += b * strideB;
    C += b * strideC;
    const int m0 = blockIdx.y * DBM, n0 = blockIdx.x * DBN;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    float2 acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);
    for (int k0 = 0; k0 < K; k0 += DBK) {
        // A tile DBM x DBK (stored transposed), B tile DBK x DBN
#pragma unroll
        for (int r = 0; r < (DBM * DBK) / DTHREADS; ++r) {
            const int e = tid + DTHREADS * r;
            const int mm = e / DBK, kk = e % DBK;
            const int gm = m0 + mm, gk = k0 + kk;
            As[kk][mm] = (gm < M && gk < K) ? A[(size_t)gm * K + gk] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int r = 0; r < (DBK * DBN) / DTHREADS; ++r) {
            const int e = tid + DTHREADS * r;
            const int kk = e / DBN, nn = e % DBN;
            const int gk = k0 + kk, gn = n0 + nn;
            Bs[kk][nn] = (gk < K && gn < N) ? B[(size_t)gk * N + gn] : make_float2(0.f, 0.f);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < DBK; ++kk) {
            float2 a[4], bb[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bb[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    acc[i][j].x = fmaf(a[i].x, bb[j].x, fmaf(-a[i].y, bb[j].y, acc[i][j].x));
                    acc[i][j].y = fmaf(a[i].x, bb[j].y, fmaf(a[i].y, bb[j].x, acc[i][j].y));
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int gm = m0 + ty + 16 * i;
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gn = n0 + tx + 16 * j;
            if (gn < N) C[(size_t)gm * N + gn] = acc[i][j];
        }
    }
}

static int cgemm(const float2* A, size_t sA, const float2* B, size_t sB, float2* C, size_t sC, int M, int N, int K,
                 int batch, cudaStream_t s) {
    const dim3 grid((N + DBN - 1) / DBN, (M + DBM - 1) / DBM, batch);
    cgemm_batched<<<grid, DTHREADS, 0, s>>>(A, sA, B, sB, C, sC, M, N, K);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

// DFT matrix of length n, cached per (device, n, direction)
static const float2* dft_matrix(int n, bool inverse) {
    static std::mutex mu;
    static std::map<std::pair<int, int>, float2*> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    const std::pair<int, int> key(dev, inverse ? -n : n);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    std::vector<float2> h((size_t)n * n);
    const double sgn = inverse ? 1.0 : -1.0;
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k) {
            const long long r = ((long long)j * k) % n;
            const double ang = sgn * 2.0 * 3.14159265358979323846 * (double)r / (double)n;
            h[(size_t)j * n + k] = make_float2((float)std::cos(ang), (float)std::sin(ang));
        }
    float2* d = nullptr;
    if (cudaMalloc(&d, sizeof(float2) * h.size()) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    cache[key] = d;
    return d;
}

int dft2d(float2* data, int n0, int n1, int howmany, bool inverse, float2* scratch, int scratch_slices,
          cudaStream_t s) {
    if (n0 < 1 || n1 < 1 || howmany < 1 || scratch_slices < 1) {
        set_error("dft2d: bad sizes");
        return QS_ERR_ARG;
    }
    const float2* F0 = dft_matrix(n0, inverse);
    const float2* F1 = dft_matrix(n1, inverse);
    if (!F0 || !F1) {
        set_error("dft2d: DFT matrix allocation failed");
        return QS_ERR_NOMEM;
    }
    const size_t P = (size_t)n0 * n1;
    for (int b0 = 0; b0 < howmany; b0 += scratch_slices) {
        const int nb = std::min(scratch_slices, howmany - b0);
        float2* X = data + (size_t)b0 * P;
        // rows (along the contiguous index): Y = X F_n1
        QS_TRY(cgemm(X, P, F1, 0, scratch, P, n0, n1, n1, nb, s));
        // columns: X = F_n0 Y
        QS_TRY(cgemm(F0, 0, scratch, P, X, P, n0, n1, n0, nb, s));
    }
    return QS_OK;
}

}  // namespace qs
