// qs_potential.cu -- projected-potential lookup tables, the atom scatter-sum
// into the slice stack, and the phase grating.
//
//   LUT          getAtomPotential3D / getAtomPotentialOffset3D
//                (stem3/stemlib.cpp:1342-1541, :1548-1741), in FP64
//   scatter-sum  make3DSlices, default 3-D branch (stem3/stemlib.cpp:894-1036,
//                :1090-1213)
//   grating      initSTEMSlices (stem3/stemlib.cpp:2280-2336)
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "qs_internal.h"
#include "qs_rez_table.h"

namespace qs {

constexpr int NSF = QS_REZ_NSF;
constexpr int OVERSAMP = 2;

// --------------------------------------------------------------- spline
void akima_spline(const double* x, const double* y, double* b, double* c, double* d, int n) {
    // Akima local cubic with linearly extrapolated end secants
    // (same construction as stem3/stemutil.cpp:975-1041)
    const double tiny = 1.0e-25;
    double m5 = (y[3] - y[2]) / (x[3] - x[2]);
    double m4 = (y[2] - y[1]) / (x[2] - x[1]);
    double m3 = (y[1] - y[0]) / (x[1] - x[0]);
    double m2 = m3 + m3 - m4;
    double m1 = m2 + m2 - m3;
    double m54 = std::fabs(m5 - m4), m43 = std::fabs(m4 - m3), m32 = std::fabs(m3 - m2), m21 = std::fabs(m2 - m1);
    double t1 = ((m43 + m21) > tiny) ? (m43 * m2 + m21 * m3) / (m43 + m21) : 0.5 * (m2 + m3);
    for (int i = 0; i < n - 1; i++) {
        double t2 = ((m54 + m32) > tiny) ? (m54 * m3 + m32 * m4) / (m54 + m32) : 0.5 * (m3 + m4);
        double h = x[i + 1] - x[i];
        b[i] = t1;
        c[i] = (3.0 * m3 - t1 - t1 - t2) / h;
        d[i] = (t1 + t2 - m3 - m3) / (h * h);
        m1 = m2; m2 = m3; m3 = m4; m4 = m5;
        m5 = (i < n - 4) ? (y[i + 4] - y[i + 3]) / (x[i + 4] - x[i + 3]) : m4 + m4 - m3;
        m21 = m32; m32 = m43; m43 = m54; m54 = std::fabs(m5 - m4);
        t1 = t2;
    }
    (void)m1;
}

__device__ __forceinline__ double spline_eval(const double* __restrict__ x, const double* __restrict__ y,
                                              const double* __restrict__ b, const double* __restrict__ c,
                                              const double* __restrict__ d, double x0) {
    int i;
    if (x0 <= x[0]) i = 0;
    else if (x0 >= x[NSF - 2]) i = NSF - 2;
    else {
        int lo = 0, hi = NSF;
        do {
            int k = (lo + hi) >> 1;
            if (x0 < x[k]) hi = k;
            else lo = k;
        } while (hi - lo > 1);
        i = lo;
    }
    const double z = x0 - x[i];
    return y[i] + (b[i] + (c[i] + d[i] * z) * z) * z;
}

// tail truncation of the s-grid at the LUT's k_max (stem3/stemlib.cpp:1390-1413)
static void truncate_tail(double* grid, double* row, double kmax) {
    grid[NSF - 1] = 1.2 * kmax;
    grid[NSF - 2] = 1.1 * kmax;
    grid[NSF - 3] = kmax;
    if (grid[NSF - 4] > grid[NSF - 3]) {
        for (int ix = 0; ix < NSF - 10; ix++) {
            if (grid[NSF - 4 - ix] < grid[NSF - 3] - 0.001 * (ix + 1)) break;
            grid[NSF - 4 - ix] = grid[NSF - 3] - 0.001 * (ix + 1);
            row[NSF - 4 - ix] = 0;
        }
    }
}

struct LutGeom {
    int nx, nz, nzPer, izOffset;
    double dkx, dky, dkz, smax2, zPos;
};

static LutGeom lut_geom(const qs_params& p) {
    LutGeom g;
    const float rx = p.resolutionX, ry = p.resolutionY, dzs = p.sliceThickness, R = p.atomRadius;
    g.nx = 2 * OVERSAMP * (int)ceilf(R / rx);
    const int ny = 2 * OVERSAMP * (int)ceilf(R / ry);
    int nzPer = (int)floorf((float)OVERSAMP * dzs / rx);
    if (2.0 * (nzPer >> 1) == nzPer) nzPer += 1;
    g.nzPer = nzPer;
    g.nz = (2 * (int)ceilf(R / dzs)) * nzPer;
    g.dkx = 0.5 * OVERSAMP / (double)((float)g.nx * rx);
    g.dky = 0.5 * OVERSAMP / (double)((float)ny * ry);
    g.dkz = nzPer / (double)((float)g.nz * dzs);
    const double kmax = 0.5 * g.nx * g.dkx / (double)OVERSAMP;
    g.smax2 = kmax * kmax;
    g.izOffset = (nzPer - 1) / 2;
    // the reference's PI (stem3/stemlib.cpp:75) in zPos (:1438)
    g.zPos = -2.0 * 3.14159265358979 * (double)(dzs / (float)nzPer * (float)g.izOffset);
    return g;
}

// f(kx, kz) with the analytic qy sum (stem3/stemlib.cpp:1446-1480)
__global__ void lut_fgrid(const double* __restrict__ tab, int nx, int nz, double dkx, double dqy, double dkz,
                          double smax2, double B, double zPos, float2* __restrict__ temp) {
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = blockIdx.y;
    if (ix >= nx) return;
    const double* g1 = tab;
    const double* r1 = tab + NSF;
    const double* sb = tab + 2 * NSF;
    const double* sc = tab + 3 * NSF;
    const double* sd = tab + 4 * NSF;
    const double* g2 = tab + 5 * NSF;
    const double* r2 = tab + 6 * NSF;
    const double kz = dkz * (iz < nz / 2 ? iz : iz - nz);
    const double kx = dkx * (ix < nx / 2 ? ix : ix - nx);
    const double s2 = kx * kx + kz * kz;
    float2 out = make_float2(0.f, 0.f);
    if (s2 < smax2) {
        double f = spline_eval(g1, r1, sb, sc, sd, sqrt(s2)) * exp(-s2 * B * 0.25);
        for (int iy = 1; iy < nx; iy++) {
            double s3 = dqy * iy;
            s3 = s3 * s3 + s2;
            if (s3 < smax2) f += 2 * spline_eval(g2, r2, sb, sc, sd, sqrt(s3)) * exp(-s3 * B * 0.25);
            else break;
        }
        f *= dkx;
        const double phase = kz * zPos;  // the kx*xPos term is zero (:1437)
        double sn, cs;
        sincos(phase, &sn, &cs);
        out = make_float2((float)(f * cs), (float)(f * sn));
    }
    temp[(size_t)iz * nx + ix] = out;
}

// backward DFT along x, keeping outputs ix' < nx/2 (FP64)
// exp(2 pi i k/n), k < n, the same sincospi values the direct sums used to
// evaluate per term; the sums below read them from shared memory (FP64
// transcendentals run at a small fraction of the FP32 rate on this part).
__global__ void lut_twiddles(int n, double2* __restrict__ W) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double sn, cs;
    sincospi(2.0 * k / n, &sn, &cs);
    W[k] = make_double2(cs, sn);
}

// Inverse DFT along x of every z row, the kx < nx/2 half kept (FP64).
__global__ void lut_dft_x(const float2* __restrict__ temp, const double2* __restrict__ Wx, int nx, int nz,
                          double2* __restrict__ G) {
    extern __shared__ double2 lsm[];
    double2* w = lsm;
    double2* row = lsm + nx;
    const int iz = blockIdx.y;
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
        w[i] = Wx[i];
        const float2 v = temp[(size_t)iz * nx + i];
        row[i] = make_double2(v.x, v.y);
    }
    __syncthreads();
    const int kx = blockIdx.x * blockDim.x + threadIdx.x;
    if (kx >= nx / 2) return;
    double re = 0, im = 0;
    int k = 0;  // (ix * kx) mod nx
    for (int ix = 0; ix < nx; ix++) {
        const double2 v = row[ix];
        const double2 t = w[k];
        re += v.x * t.x - v.y * t.y;
        im += v.x * t.y + v.y * t.x;
        k += kx;
        if (k >= nx) k -= nx;
    }
    G[(size_t)iz * (nx / 2) + kx] = make_double2(re, im);
}

// Inverse DFT along z, real part (FP64).
__global__ void lut_dft_z(const double2* __restrict__ G, const double2* __restrict__ Wz, int nxh, int nz,
                          float* __restrict__ H) {
    extern __shared__ double2 lsm[];
    for (int i = threadIdx.x; i < nz; i += blockDim.x) lsm[i] = Wz[i];
    __syncthreads();
    const int kx = blockIdx.x * blockDim.x + threadIdx.x;
    const int kz = blockIdx.y;
    if (kx >= nxh) return;
    double re = 0;
    int k = 0;  // (iz * kz) mod nz
    for (int iz = 0; iz < nz; iz++) {
        const double2 v = G[(size_t)iz * nxh + kx];
        const double2 t = lsm[k];
        re += v.x * t.x - v.y * t.y;
        k += kz;
        if (k >= nz) k -= nz;
    }
    H[(size_t)kz * nxh + kx] = (float)re;
}

__global__ void lut_zsum(const float* __restrict__ H, int nxh, int nzh, int izOffset, double scale,
                         float* __restrict__ out) {
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = blockIdx.y;
    if (ix >= nxh) return;
    double z = 0;
    for (int iiz = -izOffset; iiz <= izOffset; iiz++)
        if (iz + izOffset + iiz < nzh) z += H[(size_t)(iz + izOffset + iiz) * nxh + ix];
    if (z < 0) z = 0;
    out[(size_t)iz * nxh + ix] = (float)(scale * z);
}

int build_lut(const qs_params& p, int Z, double B, int charged, float* d_out, int* Nz, int* Nr, int* nzSub,
              cudaStream_t s) {
    if (Z < 1 || Z >= QS_REZ_NELEM) {
        set_error("qs_lut_build: atomic number out of range");
        return QS_ERR_ARG;
    }
    const LutGeom g = lut_geom(p);
    if (Nz) *Nz = g.nz / 2;
    if (Nr) *Nr = g.nx / 2;
    if (nzSub) *nzSub = g.nzPer;
    if (!d_out) return QS_OK;
    const double kmax = std::sqrt(g.smax2);
    std::vector<double> tab(7 * NSF);
    double *g1 = tab.data(), *r1 = g1 + NSF, *sb = g1 + 2 * NSF, *sc = g1 + 3 * NSF, *sd = g1 + 4 * NSF,
           *g2 = g1 + 5 * NSF, *r2 = g1 + 6 * NSF;
    // neutral table, truncated (always applied first, as the reference does)
    std::memcpy(g2, QS_REZ_F[0], sizeof(double) * NSF);
    std::memcpy(r2, QS_REZ_F[Z], sizeof(double) * NSF);
    truncate_tail(g2, r2, kmax);
    if (charged) {
        std::memcpy(g1, QS_REZ_Q[0], sizeof(double) * NSF);
        std::memcpy(r1, QS_REZ_Q[Z], sizeof(double) * NSF);
        truncate_tail(g1, r1, kmax);
    } else {
        std::memcpy(g1, g2, sizeof(double) * NSF);
        std::memcpy(r1, r2, sizeof(double) * NSF);
    }
    akima_spline(g1, r1, sb, sc, sd, NSF);
    // the charged table's qy sum evaluates the neutral table with the charged
    // spline coefficients and the y step dky (stem3/stemlib.cpp:1668-1675)
    const double dqy = charged ? g.dky : g.dkx;

    double* d_tab = nullptr;
    double2* d_W = nullptr;
    float2* d_temp = nullptr;
    double2* d_G = nullptr;
    float* d_H = nullptr;
    const int nxh = g.nx / 2, nzh = g.nz / 2;
    int rc = QS_OK;
    auto fail = [&](cudaError_t e, const char* what) {
        set_error(std::string("qs_lut_build: ") + what + ": " + cudaGetErrorString(e));
        rc = QS_ERR_CUDA;
    };
    const size_t smx = sizeof(double2) * 2 * (size_t)g.nx, smz = sizeof(double2) * (size_t)g.nz;
    cudaError_t e;
    if ((e = cudaMallocAsync(&d_tab, sizeof(double) * 7 * NSF, s)) != cudaSuccess) { fail(e, "alloc"); return rc; }
    if ((e = cudaMallocAsync(&d_temp, sizeof(float2) * (size_t)g.nx * g.nz, s)) != cudaSuccess) fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_W, sizeof(double2) * (size_t)(g.nx + g.nz), s)) != cudaSuccess)
        fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_G, sizeof(double2) * (size_t)nxh * g.nz, s)) != cudaSuccess) fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_H, sizeof(float) * (size_t)nxh * nzh, s)) != cudaSuccess) fail(e, "alloc");
    if (!rc) {
        cudaMemcpyAsync(d_tab, tab.data(), sizeof(double) * 7 * NSF, cudaMemcpyHostToDevice, s);
        lut_fgrid<<<dim3((g.nx + 127) / 128, g.nz), 128, 0, s>>>(d_tab, g.nx, g.nz, g.dkx, dqy, g.dkz, g.smax2, B,
                                                              g.zPos, d_temp);
        lut_twiddles<<<(g.nx + 127) / 128, 128, 0, s>>>(g.nx, d_W);
        lut_twiddles<<<(g.nz + 127) / 128, 128, 0, s>>>(g.nz, d_W + g.nx);
        rc = smem_attr((const void*)lut_dft_x, smx);
        if (!rc) rc = smem_attr((const void*)lut_dft_z, smz);
    }
    if (!rc) {
        lut_dft_x<<<dim3((nxh + 127) / 128, g.nz), 128, smx, s>>>(d_temp, d_W, g.nx, g.nz, d_G);
        lut_dft_z<<<dim3((nxh + 127) / 128, nzh), 128, smz, s>>>(d_G, d_W + g.nx, nxh, g.nz, d_H);
        const double scale = 47.8658 * g.dkx * g.dkz / (g.nz);
        lut_zsum<<<dim3((nxh + 127) / 128, nzh), 128, 0, s>>>(d_H, nxh, nzh, g.izOffset, scale, d_out);
        if ((e = cudaGetLastError()) != cudaSuccess) fail(e, "launch");
        else count_launch(6);
    }
    cudaFreeAsync(d_W, s);
    cudaFreeAsync(d_H, s);
    cudaFreeAsync(d_G, s);
    cudaFreeAsync(d_temp, s);
    cudaFreeAsync(d_tab, s);
    return rc;
}

// --------------------------------------------------------- 2-D tables
// getAtomPotential2D (stem3/stemlib.cpp:1750-1857): f(k) e^{i phase} on the
// oversampled nx x ny k-grid (stored as float, as the reference stores it),
// the inverse 2-D DFT in FP64, the real part rounded to float and scaled by
// dkx*dky*OVERSAMP^2.
__global__ void lut2d_fgrid(const double* __restrict__ tab, int nx, int ny, double dkx, double dky, double kmax2,
                            double B, double sx, double sy, float2* __restrict__ temp) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iy >= ny) return;
    const double* g = tab;
    const double* r = tab + NSF;
    const double* sb = tab + 2 * NSF;
    const double* sc = tab + 3 * NSF;
    const double* sd = tab + 4 * NSF;
    const double kx = dkx * (ix < nx / 2 ? ix : nx - ix);
    const double ky = dky * (iy < ny / 2 ? iy : ny - iy);
    const double s2 = kx * kx + ky * ky;
    float2 out = make_float2(0.f, 0.f);
    if (s2 < kmax2) {
        const double f = spline_eval(g, r, sb, sc, sd, sqrt(s2)) * exp(-s2 * B * 0.25);
        // the reference's PI (stem3/stemlib.cpp:75) times (kx dx nx + ky dy ny)
        const double phase = 3.14159265358979 * (kx * sx + ky * sy);
        double sn, cs;
        sincos(phase, &sn, &cs);
        out = make_float2((float)(f * cs), (float)(f * sn));
    }
    temp[(size_t)ix * ny + iy] = out;
}

// inverse DFT of every row (length n, all n outputs, FP64)
__global__ void lut2d_dft_rows(const float2* __restrict__ in, const double2* __restrict__ W, int n,
                               double2* __restrict__ out) {
    extern __shared__ double2 lsm[];
    double2* w = lsm;
    double2* row = lsm + n;
    const int ix = blockIdx.y;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        w[i] = W[i];
        const float2 v = in[(size_t)ix * n + i];
        row[i] = make_double2(v.x, v.y);
    }
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double re = 0, im = 0;
    int m = 0;  // (iy * k) mod n
    for (int iy = 0; iy < n; iy++) {
        const double2 v = row[iy], t = w[m];
        re += v.x * t.x - v.y * t.y;
        im += v.x * t.y + v.y * t.x;
        m += k;
        if (m >= n) m -= n;
    }
    out[(size_t)ix * n + k] = make_double2(re, im);
}

// inverse DFT along x of the row transforms; the real part, rounded to float,
// times scale (rounded to float again)
__global__ void lut2d_dft_cols(const double2* __restrict__ G, const double2* __restrict__ W, int nx, int ny,
                               double scale, float* __restrict__ out) {
    extern __shared__ double2 lsm[];
    for (int i = threadIdx.x; i < nx; i += blockDim.x) lsm[i] = W[i];
    __syncthreads();
    const int ky = blockIdx.x * blockDim.x + threadIdx.x;
    const int kx = blockIdx.y;
    if (ky >= ny) return;
    double re = 0;
    int m = 0;  // (ix * kx) mod nx
    for (int ix = 0; ix < nx; ix++) {
        const double2 v = G[(size_t)ix * ny + ky], t = lsm[m];
        re += v.x * t.x - v.y * t.y;
        m += kx;
        if (m >= nx) m -= nx;
    }
    out[(size_t)kx * ny + ky] = (float)((double)(float)re * scale);
}

int build_lut2d(const qs_params& p, int Z, double B, float* d_out, int* nxO, int* nyO, cudaStream_t s) {
    if (Z < 1 || Z >= QS_REZ_NELEM) {
        set_error("2-D potential table: atomic number out of range");
        return QS_ERR_ARG;
    }
    const float rx = p.resolutionX, ry = p.resolutionY, R = p.atomRadius;
    const int nx = 2 * OVERSAMP * (int)ceilf(R / rx);
    const int ny = 2 * OVERSAMP * (int)ceilf(R / ry);
    if (nxO) *nxO = nx;
    if (nyO) *nyO = ny;
    if (!d_out) return QS_OK;
    const double dkx = 0.5 * OVERSAMP / (double)((float)nx * rx);
    const double dky = 0.5 * OVERSAMP / (double)((float)ny * ry);
    const double kmax = 0.5 * nx * dkx / (double)OVERSAMP;
    std::vector<double> tab(5 * NSF);
    double *g = tab.data(), *r = g + NSF, *sb = g + 2 * NSF, *sc = g + 3 * NSF, *sd = g + 4 * NSF;
    std::memcpy(g, QS_REZ_F[0], sizeof(double) * NSF);
    std::memcpy(r, QS_REZ_F[Z], sizeof(double) * NSF);
    truncate_tail(g, r, kmax);
    akima_spline(g, r, sb, sc, sd, NSF);
    double* d_tab = nullptr;
    float2* d_temp = nullptr;
    double2 *d_W = nullptr, *d_G = nullptr;
    int rc = QS_OK;
    auto fail = [&](cudaError_t e, const char* what) {
        set_error(std::string("2-D potential table: ") + what + ": " + cudaGetErrorString(e));
        rc = QS_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaMallocAsync(&d_tab, sizeof(double) * 5 * NSF, s)) != cudaSuccess) { fail(e, "alloc"); return rc; }
    if ((e = cudaMallocAsync(&d_temp, sizeof(float2) * (size_t)nx * ny, s)) != cudaSuccess) fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_W, sizeof(double2) * (size_t)(nx + ny), s)) != cudaSuccess) fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_G, sizeof(double2) * (size_t)nx * ny, s)) != cudaSuccess) fail(e, "alloc");
    const size_t smr = sizeof(double2) * 2 * (size_t)ny, smc = sizeof(double2) * (size_t)nx;
    if (!rc) rc = smem_attr((const void*)lut2d_dft_rows, smr);
    if (!rc) rc = smem_attr((const void*)lut2d_dft_cols, smc);
    if (!rc) {
        cudaMemcpyAsync(d_tab, tab.data(), sizeof(double) * 5 * NSF, cudaMemcpyHostToDevice, s);
        lut2d_fgrid<<<dim3((ny + 127) / 128, nx), 128, 0, s>>>(d_tab, nx, ny, dkx, dky, kmax * kmax, B,
                                                               (double)rx * nx, (double)ry * ny, d_temp);
        lut_twiddles<<<(ny + 127) / 128, 128, 0, s>>>(ny, d_W);
        lut_twiddles<<<(nx + 127) / 128, 128, 0, s>>>(nx, d_W + ny);
        lut2d_dft_rows<<<dim3((ny + 127) / 128, nx), 128, smr, s>>>(d_temp, d_W, ny, d_G);
        lut2d_dft_cols<<<dim3((ny + 127) / 128, nx), 128, smc, s>>>(d_G, d_W + ny, nx, ny,
                                                                   dkx * dky * (OVERSAMP * OVERSAMP), d_out);
        if ((e = cudaGetLastError()) != cudaSuccess) fail(e, "launch");
        else count_launch(5);
    }
    cudaFreeAsync(d_G, s);
    cudaFreeAsync(d_W, s);
    cudaFreeAsync(d_temp, s);
    cudaFreeAsync(d_tab, s);
    return rc;
}

// make3DSlices' periodic 2-D branch (stem3/stemlib.cpp:1215-1262): one CTA
// per atom; warp w takes box rows w, w + 8, ...; every pixel whose table
// position lies inside the table adds the bilinear interpolation of its
// element's 2-D table (the reference's weights, named against other corners
// than the ones they multiply) to the atom's slice, wrapped into the array.
// The interpolation is FP64 as in the reference; the sum a float reduction.
__global__ void __launch_bounds__(256) scatter2d(const Atom2DJob* __restrict__ jobs, const float* const* __restrict__ luts,
                                                 int nyAtBox, int boxX, int boxY, int potNx, int potNy,
                                                 float* __restrict__ V) {
    const Atom2DJob J = jobs[blockIdx.x];
    const float* L = luts[J.lut];
    float* const slice = V + (size_t)J.iAtomZ * potNx * potNy;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int qx = warp; qx < boxX; qx += nwarps) {
        const int atPosX = OVERSAMP * qx - J.iOffsX;
        if (atPosX < 0 || atPosX >= nyAtBox - 1) continue;
        const int iax = J.iax0 + qx;
        const int cx = ((iax % potNx) + potNx) % potNx;
        const float* row0 = L + (size_t)atPosX * nyAtBox;
        const float* row1 = row0 + nyAtBox;
        float* const dst = slice + (size_t)cx * potNy;
        for (int qy = lane; qy < boxY; qy += 32) {
            const int atPosY = OVERSAMP * qy - J.iOffsY;
            if (atPosY >= nyAtBox - 1 || atPosY < 0) continue;
            const double v = J.s11 * (double)__ldg(row0 + atPosY) + J.s12 * (double)__ldg(row0 + atPosY + 1) +
                             J.s21 * (double)__ldg(row1 + atPosY) + J.s22 * (double)__ldg(row1 + atPosY + 1);
            const int iay = J.iay0 + qy;
            atomicAdd(dst + ((iay % potNy) + potNy) % potNy, (float)v);
        }
    }
}

int launch_scatter2d(const Atom2DJob* d_jobs, int njobs, const float* const* d_luts, int nyAtBox, int boxX, int boxY,
                     const qs_params& p, float* V, cudaStream_t s) {
    if (njobs <= 0) return QS_OK;
    scatter2d<<<njobs, 256, 0, s>>>(d_jobs, d_luts, nyAtBox, boxX, boxY, p.potNx, p.potNy, V);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

// --------------------------------------------------------- scatter-sum
// One block per atom job; threads stride over the atom's pixel box.  The
// interpolation follows stem3/stemlib.cpp:935-1028 (radial linear
// interpolation at dr = dx/2, nearest sub-slice in z).  FP32 arithmetic
// (FP64 runs at a small fraction of the FP32 rate on this part): the
// reference forms s = x2 + y2, r = sqrt(s) and r/dr in double
// (stem3/stemlib.cpp:935-943); the float r/dr (reciprocal square root,
// within ~4e-7 relative of it) is off by less than 1e-4 of an interval
// anywhere in the box, so the radial interval is taken from it except within
// 2e-4 of a knot.  There the reference's own decision is reproduced without a
// double square root or division: its interval index floor(fl(sqrt(s))/dr)
// never decreases as s grows, so it reaches knot k exactly when s is at
// least the smallest double that reaches it (scatter_knots, found on the host
// by bisection), and s itself costs one double product and one double FMA.
// The interpolation weight and the sum run in float.
//
// The LUT rows an atom touches are the same for every pixel of its box: the
// CTA finds the contiguous run of reachable rows once (the reference's
// iOffsZ tests) and stages them in shared memory as (value, slope) pairs
// L[ir], L[ir+1] - L[ir], the charge-dependent table already added in with
// the atom's charge (the interpolation is linear in both), so that a slice
// costs one shared load, one FMA and one reduction per pixel.  The pixels are
// walked row by row (scatter_rows): a warp takes a box row, computes its x
// offset, wrapped index and the columns that can reach the table once, and
// its lanes take 32 consecutive columns at a time; the box corners beyond
// the table's radius are never visited, and the slice loop is unrolled for
// the atom's run length.  The sums go to a real array (unit stride: a warp's
// reductions cover consecutive words); the phase grating expands it.
void scatter_knots(double dr, int Nr, std::vector<double>& T) {
    // T[k] = min{s >= 0 : floor(fl(fl(sqrt(s)) / dr)) >= k}; non-negative
    // doubles order like their bit patterns, so bisect over those
    T.assign(Nr + 1, 0.0);
    auto reaches = [&](double v, int k) { return std::floor(std::sqrt(v) / dr) >= (double)k; };
    for (int k = 1; k <= Nr; k++) {
        const double hi0 = ((double)k + 1.0) * dr * ((double)k + 1.0) * dr;
        uint64_t lo, hi;
        const double zero = 0.0;
        std::memcpy(&lo, &zero, 8);
        std::memcpy(&hi, &hi0, 8);
        while (hi - lo > 1) {  // invariant: !reaches(lo), reaches(hi)
            const uint64_t mid = lo + (hi - lo) / 2;
            double v;
            std::memcpy(&v, &mid, 8);
            if (reaches(v, k)) hi = mid;
            else lo = mid;
        }
        std::memcpy(&T[k], &hi, 8);
    }
}

__device__ __forceinline__ int lut_row(int iOffsZ, int Nr, int limLo, int limHi) {
    if (iOffsZ < 0) return iOffsZ > limLo ? -iOffsZ + Nr : -1;
    return iOffsZ < limHi ? iOffsZ : -1;
}

// The reference's radial interval of a pixel at (ddx, ddy) from the atom
// (make3DSlices, stem3/stemlib.cpp:935-990): ir and the interpolation weight
// ddr; false when the pixel lies beyond the table (ir >= Nr - 1).
__device__ __forceinline__ bool lut_interval(float ddx, float ddy, float inv_dr, int Nr,
                                             const double* __restrict__ knots, int& ir, float& ddr) {
    const float r2 = fmaf(ddx, ddx, ddy * ddy);
    const float rr = r2 > 0.f ? r2 * rsqrtf(r2) * inv_dr : 0.f;
    ir = (int)rr;
    ddr = rr - (float)ir;
    if (ddr < 2e-4f || ddr > 1.f - 2e-4f) {
        // the knot k nearest to rr: the interval is k - 1 or k
        const int k = (int)(rr + 0.5f);
        if (k > 0 && k <= Nr) {
            const double s2 = fma((double)ddx, (double)ddx, (double)ddy * (double)ddy);
            ir = s2 < __ldg(knots + k) ? k - 1 : k;
        } else {
            ir = k;
        }
        ddr = fminf(fmaxf(rr - (float)ir, 0.f), 1.f);
    }
    return ir < Nr - 1;
}

// One pixel's contributions to the NR slices of its run (NR = 0: nr of them,
// a loop), from the staged (value, slope) rows.
template <int NR>
__device__ __forceinline__ void add_slices(float* dst, size_t step, const float2* pr, int prs, float ddr, int nr) {
    if constexpr (NR > 0) {
#pragma unroll
        for (int r = 0; r < NR; r++) {
            const float2 ls = pr[r * prs];
            atomicAdd(dst + r * step, fmaf(ddr, ls.y, ls.x));
        }
    } else {
#pragma unroll 4
        for (int r = 0; r < nr; r++, dst += step, pr += prs) {
            const float2 ls = *pr;
            atomicAdd(dst, fmaf(ddr, ls.y, ls.x));
        }
    }
}

// The staged scatter's pixel walk: warp w takes the box rows qx = w,
// w + 8, ...; in a row only the columns within Nr*dr of the atom (plus one
// pixel each side: the exact interval test still decides every pixel) are
// visited, 32 consecutive columns at a time, so that a row's x offset, its
// wrapped index and the cut-off are computed once per row and a warp's
// reductions cover consecutive words.
template <int NR>
__device__ __forceinline__ void scatter_rows(const AtomJob& J, float* base, size_t sliceStep, const float2* s_pair,
                                             int Nr, int nr, float dx, float dy, const double* __restrict__ knots,
                                             float inv_dr, int potNx, int potNy, int periodic) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int nxBox = J.iax1 - J.iax0 + 1;
    const bool wideY = periodic && (J.iay1 - J.iay0 + 1 > potNy);
    const float rcut = (float)Nr / inv_dr;
    const float rc2 = rcut * rcut;
    for (int qx = warp; qx < nxBox; qx += nwarps) {
        const int iax = J.iax0 + qx;
        // x2 = iax*dx - atomX in float as the reference forms it
        // (stem3/stemlib.cpp:935-938), rounded step by step (no FMA)
        const float ddx = __fsub_rn(__fmul_rn((float)iax, dx), J.atomX);
        const float rem = rc2 - ddx * ddx;
        if (rem < 0.f) continue;
        const float half = sqrtf(rem);
        const int y0 = max(J.iay0, (int)floorf((J.atomY - half) / dy) - 1);
        const int y1 = min(J.iay1, (int)floorf((J.atomY + half) / dy) + 2);
        const int cx = periodic ? ((iax % potNx) + potNx) % potNx : iax;
        const int cy0 = periodic ? ((y0 % potNy) + potNy) % potNy : y0;
        float* const row = base + (size_t)cx * potNy;
        for (int iay = y0 + lane, cy = cy0 + lane; iay <= y1; iay += 32, cy += 32) {
            const float ddy = __fsub_rn(__fmul_rn((float)iay, dy), J.atomY);
            int ir;
            float ddr;
            if (!lut_interval(ddx, ddy, inv_dr, Nr, knots, ir, ddr)) continue;
            int c = cy;
            if (wideY) c %= potNy;
            else if (periodic) c -= c >= potNy ? potNy : 0;
            add_slices<NR>(row + c, sliceStep, s_pair + ir, Nr - 1, ddr, nr);
        }
    }
}

// CTAs per SM the scatter is compiled for (its register budget): 4 measured
// fastest on the 512^2 STEM and the largest CBED stacks, within 1 % on TEM
#ifndef QS_SCATTER_MIN_BLOCKS
#define QS_SCATTER_MIN_BLOCKS 4
#endif
template <bool STAGED>
__global__ void __launch_bounds__(256, QS_SCATTER_MIN_BLOCKS) scatter_atoms(const AtomJob* __restrict__ jobs, const float* const* __restrict__ luts, int Nz,
                              int Nr, int nzSub, float dx, float dy, const double* __restrict__ knots, float inv_dr,
                              float dzs, int potNx, int potNy, int periodic, int maxRows, float* __restrict__ V) {
    extern __shared__ float2 s_pair[];  // STAGED: [maxRows][Nr - 1] (value, slope)
    __shared__ int s_run[2];            // first reachable row (relative to iaz0), count
    const AtomJob J = jobs[blockIdx.x];
    const float* lut = luts[J.lut];
    const float* lutq = J.lutq >= 0 ? luts[J.lutq] : nullptr;
    const float q = J.q;
    const int w = J.iay1 - J.iay0 + 1;
    const int npx = (J.iax1 - J.iax0 + 1) * w;
    const int nrows = J.iaz1 - J.iaz0 + 1;
    const size_t sliceStep = (size_t)potNx * potNy;
    const int limHi = Nr * (Nz - 1), limLo = -Nr * (Nz - 1), step = nzSub * Nr;
    const double dOffsZ = (double)(((float)(J.iAtomZ + J.iaz0) - J.atomZ / dzs) * (float)nzSub);
    const int iOffsZ0 = ((int)(dOffsZ + 0.5)) * Nr;
    if (threadIdx.x == 0) {
        // the reachable rows form one run: iOffsZ grows by `step` per slice
        // and the reachable ones lie strictly between limLo and limHi
        int first = -1, count = 0;
        for (int k = 0; k < nrows; k++)
            if (lut_row(iOffsZ0 + k * step, Nr, limLo, limHi) >= 0) {
                if (first < 0) first = k;
                count = k - first + 1;
            }
        s_run[0] = first;
        s_run[1] = first < 0 ? 0 : count;
    }
    __syncthreads();
    const int r0 = s_run[0], nr = s_run[1];
    if (nr == 0) return;
    if constexpr (STAGED) {
        const int P = Nr - 1;
        for (int i = threadIdx.x; i < nr * P; i += blockDim.x) {
            const int k = i / P, j = i - k * P;
            const float* L = lut + lut_row(iOffsZ0 + (r0 + k) * step, Nr, limLo, limHi) + j;
            float v0 = __ldg(L), v1 = __ldg(L + 1);
            if (lutq) {
                const float* Lq = lutq + (L - lut);
                v0 += q * __ldg(Lq);
                v1 += q * __ldg(Lq + 1);
            }
            s_pair[i] = make_float2(v0, v1 - v0);
        }
        __syncthreads();
    }
    float* const base = V + (size_t)(J.iAtomZ + J.iaz0 + r0) * sliceStep;
    if constexpr (STAGED) {
        switch (nr) {
            case 1: scatter_rows<1>(J, base, sliceStep, s_pair, Nr, nr, dx, dy, knots, inv_dr, potNx, potNy, periodic); break;
            case 2: scatter_rows<2>(J, base, sliceStep, s_pair, Nr, nr, dx, dy, knots, inv_dr, potNx, potNy, periodic); break;
            case 3: scatter_rows<3>(J, base, sliceStep, s_pair, Nr, nr, dx, dy, knots, inv_dr, potNx, potNy, periodic); break;
            case 4: scatter_rows<4>(J, base, sliceStep, s_pair, Nr, nr, dx, dy, knots, inv_dr, potNx, potNy, periodic); break;
            case 5: scatter_rows<5>(J, base, sliceStep, s_pair, Nr, nr, dx, dy, knots, inv_dr, potNx, potNy, periodic); break;
            case 6: scatter_rows<6>(J, base, sliceStep, s_pair, Nr, nr, dx, dy, knots, inv_dr, potNx, potNy, periodic); break;
            case 7: scatter_rows<7>(J, base, sliceStep, s_pair, Nr, nr, dx, dy, knots, inv_dr, potNx, potNy, periodic); break;
            case 8: scatter_rows<8>(J, base, sliceStep, s_pair, Nr, nr, dx, dy, knots, inv_dr, potNx, potNy, periodic); break;
            default: scatter_rows<0>(J, base, sliceStep, s_pair, Nr, nr, dx, dy, knots, inv_dr, potNx, potNy, periodic);
        }
        return;
    }
    const int sx = blockDim.x / w, sy = blockDim.x - sx * w;
    int qx = threadIdx.x / w, qy = threadIdx.x - qx * w;
    // periodic wrap: the box's first row and column are wrapped into the
    // cell once; while the box is no wider than the cell, a pixel's wrapped
    // index is then that offset plus its place in the box, less one period
    // at most (no integer division per pixel)
    const int wx0 = periodic ? ((J.iax0 % potNx) + potNx) % potNx : J.iax0;
    const int wy0 = periodic ? ((J.iay0 % potNy) + potNy) % potNy : J.iay0;
    const bool wide = periodic && (J.iax1 - J.iax0 + 1 > potNx || w > potNy);
    for (int k = threadIdx.x; k < npx; k += blockDim.x) {
        const int iax = J.iax0 + qx, iay = J.iay0 + qy;
        int cx = wx0 + qx, cy = wy0 + qy;
        qx += sx;
        qy += sy;
        if (qy >= w) {
            qy -= w;
            ++qx;
        }
        // x2 = iax*dx - atomX in float as the reference forms it
        // (stem3/stemlib.cpp:935-938), rounded step by step (no FMA)
        const float ddx = __fsub_rn(__fmul_rn((float)iax, dx), J.atomX);
        const float ddy = __fsub_rn(__fmul_rn((float)iay, dy), J.atomY);
        int ir;
        float ddr;
        if (!lut_interval(ddx, ddy, inv_dr, Nr, knots, ir, ddr)) continue;
        if (wide) {
            cx = ((iax % potNx) + potNx) % potNx;
            cy = ((iay % potNy) + potNy) % potNy;
        } else if (periodic) {
            cx -= cx >= potNx ? potNx : 0;
            cy -= cy >= potNy ? potNy : 0;
        }
        // LUT rows from global memory (tables too large to stage)
        float* dst = base + (size_t)cx * potNy + cy;
        const float w0 = 1.f - ddr;
        for (int r = 0; r < nr; r++, dst += sliceStep) {
            const int row = lut_row(iOffsZ0 + (r0 + r) * step, Nr, limLo, limHi);
            float v = w0 * __ldg(lut + row + ir) + ddr * __ldg(lut + row + ir + 1);
            if (lutq) v += q * (w0 * __ldg(lutq + row + ir) + ddr * __ldg(lutq + row + ir + 1));
            atomicAdd(dst, v);
        }
    }
}

int launch_scatter(const AtomJob* d_jobs, int njobs, bool charged, const float* const* d_luts, int Nz, int Nr,
                   int nzSub, const qs_params& p, const double* d_knots, float* V, cudaStream_t s) {
    if (njobs <= 0) return QS_OK;
    (void)charged;
    const double dr = p.resolutionX / OVERSAMP;
    // every atom's z range spans at most 2 iRadZ + 1 slices
    const int maxRows = 2 * (int)ceilf(p.atomRadius / p.sliceThickness) + 1;
    const size_t staged = sizeof(float2) * (size_t)maxRows * (Nr - 1);
    const int periodic = p.nonPeriod ? 0 : 1;
    const float inv_dr = (float)(1.0 / dr);
    if (staged <= 160 * 1024) {
        QS_TRY(smem_attr((const void*)scatter_atoms<true>, staged));
        scatter_atoms<true><<<njobs, 256, staged, s>>>(d_jobs, d_luts, Nz, Nr, nzSub, p.resolutionX, p.resolutionY,
                                                       d_knots, inv_dr, p.sliceThickness, p.potNx, p.potNy,
                                                       periodic, maxRows, V);
    } else {
        scatter_atoms<false><<<njobs, 256, 0, s>>>(d_jobs, d_luts, Nz, Nr, nzSub, p.resolutionX, p.resolutionY,
                                                   d_knots, inv_dr, p.sliceThickness, p.potNx, p.potNy, periodic,
                                                   maxRows, V);
    }
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

// ------------------------------------------------------- phase grating
// t = exp(i scale V).  The reference evaluates cos/sin in double
// (stem3/stemlib.cpp:2290-2299); here the phase is rounded to float once and
// sincosf (within 2 ulp) evaluates it: for the phases of real potentials
// (|scale V| of order 10 rad) the result differs by ~1e-6 absolute, and FP64
// transcendentals run at a small fraction of the FP32 rate on this part.
__global__ void grating_from_real(const float* __restrict__ V, float2* __restrict__ t, size_t n, float scale) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float sn, cs;
        sincosf(V[i] * scale, &sn, &cs);
        t[i] = make_float2(cs, sn);
    }
}

// trans = (V, 0): the potential itself in the complex stack's layout
__global__ void expand_real(const float* __restrict__ V, float2* __restrict__ t, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        t[i] = make_float2(V[i], 0.f);
}

int launch_expand_real(const float* V, float2* trans, size_t n, cudaStream_t s) {
    if (!n) return QS_OK;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    expand_real<<<sms * 8, 256, 0, s>>>(V, trans, n);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

int launch_grating_from_real(const float* V, float2* trans, size_t n, double scale, cudaStream_t s) {
    if (!n) return QS_OK;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    grating_from_real<<<sms * 8, 256, 0, s>>>(V, trans, n, (float)scale);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

// The reference scales by fftScale = 1/(potNx*potNy) in double and stores
// float (stem3/stemlib.cpp:2315-2329); the float product differs from that
// by at most one rounding of the scale (none for power-of-two grids).
__global__ void bandlimit_mask(float2* __restrict__ t, int slices, int potNx, int potNy,
                               const float* __restrict__ kx2, const float* __restrict__ ky2, float k2max,
                               float fftScale) {
    const size_t n = (size_t)slices * potNx * potNy;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int iy = (int)(i % potNy);
        const int ix = (int)((i / potNy) % potNx);
        const float k2 = ky2[iy] + kx2[ix];
        float2 v = t[i];
        if (k2 < k2max) v = make_float2(v.x * fftScale, v.y * fftScale);
        else v = make_float2(0.f, 0.f);
        t[i] = v;
    }
}

int launch_bandlimit_mask(float2* trans, int slices, int potNx, int potNy, const float* kx2, const float* ky2,
                          float k2max, double fftScale, cudaStream_t s) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    bandlimit_mask<<<sms * 8, 256, 0, s>>>(trans, slices, potNx, potNy, kx2, ky2, k2max, (float)fftScale);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

}  // namespace qs
