// qs_tem.cu -- kernels of the TEM driver: the incident plane wave, exit-wave
// intensity sums and the objective-lens transfer function.
//
// doTEM (stem3/stem3.cpp:2354-2710) propagates an incident plane wave and
// averages exit-face intensities over frozen-phonon configurations; the CTF
// that turns an exit wave into an image lives in the reference's Matlab
// front end (GUI_Matlab/simImageFromWave.m:57-73).
#include <cuda_runtime.h>

#include <cmath>

#include "qs_internal.h"

namespace qs {

__global__ void fill_value(float2* __restrict__ w, size_t n, float2 v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        w[i] = v;
}

// acc[i] += scale * sum_b |w_b[i]|^2 (b < nwaves, arrays n apart)
__global__ void acc_intensity(const float2* __restrict__ w, int nwaves, size_t n, float scale,
                              float* __restrict__ acc) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nwaves; ++b) {
            const float2 v = w[(size_t)b * n + i];
            s += v.x * v.x + v.y * v.y;
        }
        acc[i] += scale * s;
    }
}

// out_b[i] = in_b[i] * H[i]
__global__ void mul_table(const float2* __restrict__ in, const float2* __restrict__ H, int nwaves, size_t n,
                          float2* __restrict__ out) {
    const size_t total = (size_t)nwaves * n;
    for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < total; j += (size_t)gridDim.x * blockDim.x) {
        const float2 a = in[j], h = H[j % n];
        out[j] = make_float2(a.x * h.x - a.y * h.y, a.x * h.y + a.y * h.x);
    }
}

// H(k) in FFT order, FP64 (the phase reaches 1e6 rad at large k without an
// aperture), stored as c64.  k = (i < n/2 ? i : i - n) / (n d) as the
// script's fftshifted [-n/2, n/2) grid.
__global__ void ctf_table(int nx, int ny, double dkx, double dky, double lambda, qs_ctf C, double df,
                          float2* __restrict__ H) {
    const size_t n = (size_t)nx * ny;
    const double pi = 3.14159265358979323846;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i / ny), iy = (int)(i % ny);
        const double kx = (ix < nx / 2 ? ix : ix - nx) * dkx;
        const double ky = (iy < ny / 2 ? iy : iy - ny) * dky;
        const double k2 = kx * kx + ky * ky, k = sqrt(k2);
        double A = 1.0;
        if (C.kmax > 0) {
            if (C.edge <= 0) {
                A = (k2 < C.kmax * C.kmax) ? 1.0 : 0.0;
            } else {
                const double lo = C.kmax - 0.5 * C.edge, hi = C.kmax + 0.5 * C.edge;
                A = k <= lo ? 1.0 : (k >= hi ? 0.0 : 0.5 * (1.0 + cos(pi * (k - lo) / C.edge)));
            }
        }
        if (A == 0.0) {
            H[i] = make_float2(0.f, 0.f);
            continue;
        }
        const double phi = atan2(ky, kx);
        const double Et = exp(-2.0 * (C.focalSpread * lambda * k2) * (C.focalSpread * lambda * k2));
        const double es = pi * C.alpha * df + pi * C.alpha * lambda * lambda * C.Cs * k2;
        const double Es = exp(-es * es * k2);
        double chi = pi * (lambda * (df + C.astig * cos(2.0 * (phi - C.astigPhi))) * k2 +
                           0.5 * lambda * lambda * lambda * C.Cs * k2 * k2);
        chi = fmod(chi, 2.0 * pi);
        const double m = A * Et * Es;
        H[i] = make_float2((float)(m * cos(chi)), (float)(-m * sin(chi)));
    }
}

static int grid_for(size_t n) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t want = (n + 255) / 256;
    return (int)(want < (size_t)sms * 8 ? (want ? want : 1) : (size_t)sms * 8);
}

int launch_fill(float2* w, size_t n, float re, float im, cudaStream_t s) {
    fill_value<<<grid_for(n), 256, 0, s>>>(w, n, make_float2(re, im));
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

int launch_acc_intensity(const float2* w, int nwaves, size_t n, float scale, float* acc, cudaStream_t s) {
    acc_intensity<<<grid_for(n), 256, 0, s>>>(w, nwaves, n, scale, acc);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

int launch_mul_table(const float2* in, const float2* H, int nwaves, size_t n, float2* out, cudaStream_t s) {
    mul_table<<<grid_for((size_t)nwaves * n), 256, 0, s>>>(in, H, nwaves, n, out);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

int launch_ctf_table(int nx, int ny, double dx, double dy, double lambda, const qs_ctf& C, double df, float2* H,
                     cudaStream_t s) {
    ctf_table<<<grid_for((size_t)nx * ny), 256, 0, s>>>(nx, ny, 1.0 / (nx * dx), 1.0 / (ny * dy), lambda, C, df, H);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

}  // namespace qs
