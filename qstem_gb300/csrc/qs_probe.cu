// qs_probe.cu -- the aberrated STEM/CBED probe (probe(),
// stem3/stemlib.cpp:1952-2191) and the single-wave detector reduction
// (collectIntensity, stem3/stemlib.cpp:2576-2687).
#include <cuda_runtime.h>

#include <cmath>

#include "qs_internal.h"

namespace qs {

struct ProbeK {
    int nx, ny, ismoth;
    double ax, by, rx, ry, rx2, ry2, wavlen, k2max, pixel, scale, dx, dy, pi;
    double df_delta, astigMag, astigAngle;
    double a33, a31, a44, a42, a55, a53, a51, a66, a64;
    double phi33, phi31, phi44, phi42, phi55, phi53, phi51, phi66, phi64;
    double Cs, C5;
};

// k-space aperture and aberration phase chi(k) (stem3/stemlib.cpp:2049-2104)
__global__ void probe_kspace(ProbeK P, float2* __restrict__ wave) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nx * P.ny) return;
    const int ix = i / P.ny, iy = i - ix * P.ny;
    const double ky = (iy > P.ny / 2) ? (double)(iy - P.ny) : (double)iy;
    const double kx = (ix > P.nx / 2) ? (double)(ix - P.nx) : (double)ix;
    const double k2 = kx * kx * P.rx2 + ky * ky * P.ry2;
    // outside the aperture and its smoothed edge the probe is zero: skip
    // the FP64 aberration phase there (most of k-space for small apertures)
    if (k2 > P.k2max && !(P.ismoth != 0 && fabs(k2 - P.k2max) <= P.pixel)) {
        wave[i] = make_float2(0.f, 0.f);
        return;
    }
    double kt2 = k2 * (P.wavlen * P.wavlen);
    const double kt = sqrt(kt2);
    const double phi = atan2(P.ry * ky, P.rx * kx);
    double chi = kt2 * (P.df_delta + P.astigMag * cos(2.0 * (phi - P.astigAngle))) / 2.0;
    kt2 *= kt;
    if (P.a33 > 0 || P.a31 > 0)
        chi += kt2 * (P.a33 * cos(3.0 * (phi - P.phi33)) + P.a31 * cos(phi - P.phi31)) / 3.0;
    kt2 *= kt;
    if (P.a44 > 0 || P.a42 > 0 || P.Cs != 0)
        chi += kt2 * (P.a44 * cos(4.0 * (phi - P.phi44)) + P.a42 * cos(2.0 * (phi - P.phi42)) + P.Cs) / 4.0;
    kt2 *= kt;
    if (P.a55 > 0 || P.a53 > 0 || P.a51 > 0)
        chi += kt2 * (P.a55 * cos(5.0 * (phi - P.phi55)) + P.a53 * cos(3.0 * (phi - P.phi53)) +
                      P.a51 * cos(phi - P.phi51)) / 5.0;
    kt2 *= kt;
    // the reference zeroes a62 inside this condition (:2082)
    if (P.a66 > 0 || P.a64 > 0 || P.C5 != 0)
        chi += kt2 * (P.a66 * cos(6.0 * (phi - P.phi66)) + P.a64 * cos(4.0 * (phi - P.phi64)) + P.C5) / 6.0;
    chi *= 2 * P.pi / P.wavlen;
    chi -= 2.0 * P.pi * ((P.dx * kx / P.ax) + (P.dy * ky / P.by));
    double sn, cs;
    sincos(chi, &sn, &cs);
    float2 w;
    if (P.ismoth != 0 && fabs(k2 - P.k2max) <= P.pixel) {
        w = make_float2((float)(0.5 * P.scale * cs), (float)(-0.5 * P.scale * sn));
    } else if (k2 <= P.k2max) {
        w = make_float2((float)((double)(float)P.scale * cs), (float)((double)(float)(-P.scale) * sn));
    } else {
        w = make_float2(0.f, 0.f);
    }
    wave[i] = w;
}

int launch_probe_kspace(const qs_params& p, double dx, double dy, float2* wave, cudaStream_t s) {
    ProbeK P;
    P.nx = p.nx;
    P.ny = p.ny;
    P.ismoth = p.ismoth;
    P.ax = (double)(float)(p.nx * p.resolutionX);
    P.by = (double)(float)(p.ny * p.resolutionY);
    P.dx = P.ax - dx;
    P.dy = P.by - dy;
    P.pi = 4.0 * std::atan(1.0);
    P.rx = 1.0 / P.ax;
    P.rx2 = P.rx * P.rx;
    P.ry = 1.0 / P.by;
    P.ry2 = P.ry * P.ry;
    const double v0 = p.v0;
    P.wavlen = 12.26 / std::sqrt(v0 * 1.e3 + v0 * v0 * 0.9788);  // the probe's own lambda (:2014)
    const double alpha = 0.001 * p.alpha;
    P.k2max = std::sin(alpha) / P.wavlen;
    P.k2max *= P.k2max;
    P.pixel = P.rx2 + P.ry2;
    P.scale = 1.0 / std::sqrt((double)p.nx * (double)p.ny);
    P.df_delta = p.df0 + (double)(p.Cc * p.dE_E);
    P.astigMag = p.astigMag;
    P.astigAngle = p.astigAngle;
    P.a33 = p.a33; P.a31 = p.a31; P.a44 = p.a44; P.a42 = p.a42; P.a55 = p.a55; P.a53 = p.a53;
    P.a51 = p.a51; P.a66 = p.a66; P.a64 = p.a64;
    P.phi33 = p.phi33; P.phi31 = p.phi31; P.phi44 = p.phi44; P.phi42 = p.phi42; P.phi55 = p.phi55;
    P.phi53 = p.phi53; P.phi51 = p.phi51; P.phi66 = p.phi66; P.phi64 = p.phi64;
    P.Cs = p.Cs;
    P.C5 = p.C5;
    const int n = p.nx * p.ny;
    probe_kspace<<<(n + 255) / 256, 256, 0, s>>>(P, wave);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

struct ProbeR {
    int nx, ny, gauss, ais;
    float gaussScale, rx, ry;
    double dx, dy, aAIS, edge, pi;
};

// real-space Gaussian and AIS masks, then sum |psi|^2 (:2118-2158)
__global__ void probe_realspace(ProbeR P, float2* __restrict__ wave, double* __restrict__ sum) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double local = 0;
    if (i < P.nx * P.ny) {
        const int ix = i / P.ny, iy = i - ix * P.ny;
        float2 w = wave[i];
        if (P.gauss) {
            const int num = (ix - P.nx / 2) * (ix - P.nx / 2) + (iy - P.ny / 2) * (iy - P.ny / 2);
            const float r = expf(-(float)num / ((float)(P.nx * P.nx) * P.gaussScale));
            w.x *= r;
            w.y *= r;
        }
        if (P.ais) {
            const double x = (double)((float)ix * P.rx) - P.dx;
            const double y = (double)((float)iy * P.ry) - P.dy;
            const double delta = sqrt(x * x + y * y) - 0.5 * P.aAIS + P.edge;
            if (delta > 0) {
                w = make_float2(0.f, 0.f);
            } else if (delta >= -P.edge) {
                const double sc = 0.5 * (1 - cos(P.pi * delta / P.edge));
                w = make_float2((float)(sc * w.x), (float)(sc * w.y));
            }
        }
        wave[i] = w;
        local = (double)(w.x * w.x + w.y * w.y);
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, local);
}

int launch_probe_realspace(const qs_params& p, double dx, double dy, float2* wave, double* d_sum, cudaStream_t s) {
    ProbeR P;
    P.nx = p.nx;
    P.ny = p.ny;
    P.gauss = p.gaussFlag;
    P.ais = p.aAIS > 0;
    P.gaussScale = p.gaussScale;
    P.rx = p.resolutionX;
    P.ry = p.resolutionY;
    const double ax = (double)(float)(p.nx * p.resolutionX), by = (double)(float)(p.ny * p.resolutionY);
    P.dx = ax - dx;
    P.dy = by - dy;
    P.aAIS = p.aAIS;
    const double avgRes =
        std::sqrt(0.5 * (double)(p.resolutionX * p.resolutionX + p.resolutionY * p.resolutionY));
    P.edge = 5 * avgRes;  // SMOOTH_EDGE (:1939)
    P.pi = 4.0 * std::atan(1.0);
    QS_CUDA_TRY(cudaMemsetAsync(d_sum, 0, sizeof(double), s));
    const int n = p.nx * p.ny;
    probe_realspace<<<(n + 255) / 256, 256, 0, s>>>(P, wave, d_sum);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

__global__ void scale_by_sum(float2* __restrict__ w, size_t n, const double* __restrict__ sum, double nxy) {
    const float sc = (float)sqrt(1.0 / *sum * nxy);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        w[i].x *= sc;
        w[i].y *= sc;
    }
}

int launch_scale_by_sum(float2* wave, size_t n, const double* d_sum, double nxy, cudaStream_t s) {
    scale_by_sum<<<(unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, s>>>(wave, n, d_sum, nxy);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

// ------------------------------------------------------- collectIntensity
struct CollectArgs {
    int nx, ny, ndet;
    float k2in[QS_MAX_DETECTORS], k2out[QS_MAX_DETECTORS];
    int sx[QS_MAX_DETECTORS], sy[QS_MAX_DETECTORS];
    double scaleDiff;
};

__global__ void collect_one(CollectArgs A, const float2* __restrict__ w, const float* __restrict__ kx2,
                            const float* __restrict__ ky2, double* __restrict__ sums, float* __restrict__ diffpat) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = i < A.nx * A.ny;
    const int ix = ok ? i / A.ny : 0, iy = ok ? i - ix * A.ny : 0;
    const float2 v = ok ? w[i] : make_float2(0.f, 0.f);
    const float I = v.x * v.x + v.y * v.y;
    if (ok && diffpat)
        diffpat[(size_t)((ix + A.nx / 2) % A.nx) * A.ny + (iy + A.ny / 2) % A.ny] = (float)((double)I * A.scaleDiff);
    const float k2 = ok ? kx2[ix] + ky2[iy] : -1.f;
    for (int d = 0; d < A.ndet; d++) {
        double c = 0;
        if (ok && k2 >= A.k2in[d] && k2 <= A.k2out[d]) {
            if (A.sx[d] == 0 && A.sy[d] == 0) {
                c = I;
            } else {
                const int ixs = (ix + A.sx[d] + A.nx) % A.nx, iys = (iy + A.sy[d] + A.ny) % A.ny;
                const float2 u = w[(size_t)ixs * A.ny + iys];
                c = (double)(u.x * u.x + u.y * u.y);
            }
        }
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if ((threadIdx.x & 31) == 0 && c != 0) atomicAdd(sums + d, c);
    }
}

int launch_collect(const qs_params& p, const float2* wave_k, const float* kx2, const float* ky2, double* d_sums,
                   float* diffpat, cudaStream_t s) {
    CollectArgs A;
    A.nx = p.nx;
    A.ny = p.ny;
    A.ndet = p.detectorNum;
    for (int d = 0; d < p.detectorNum; d++) {
        A.k2in[d] = p.detectors[d].k2Inside;
        A.k2out[d] = p.detectors[d].k2Outside;
        A.sx[d] = (int)p.detectors[d].shiftX;
        A.sy[d] = (int)p.detectors[d].shiftY;
    }
    A.scaleDiff = 1.0 / std::sqrt((double)(p.nx * p.ny));
    if (A.ndet > 0) QS_CUDA_TRY(cudaMemsetAsync(d_sums, 0, sizeof(double) * A.ndet, s));
    const int n = p.nx * p.ny;
    collect_one<<<(n + 255) / 256, 256, 0, s>>>(A, wave_k, kx2, ky2, d_sums, diffpat);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

}  // namespace qs
