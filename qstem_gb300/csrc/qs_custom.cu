// qs_custom.cu -- the slice potential from custom scattering factors
// (make3DSlicesFT, stem3/customslice.cpp:56-317), the path stem3's doCBED and
// doNBED take for "Structure Factors: custom" (stem3/stem3.cpp:1411-1415,
// 2177-2197).
//
//   per element  f(s) from the custom table (sfLUT, stem3/stemutil.cpp:
//                1427-1467: Akima spline, 0 above the last k and where
//                negative) on the k-grid of a 40 A (z, r) box, inverse 2-D
//                DFT in FP64, the reference's scale and radial cut-off (the
//                first negative value in scan order shrinks it), then
//                reduceAndExpand's z sums and edge extrapolation
//                (:359-401) into a (z, r) table
//   per pixel    every atom within the cut-off adds the table's bicubic
//                interpolation (stem3/stemutil.cpp:1470-1520) at its (z, r)
//                distance, in the reference's atom order (z-sorted), FP64
//                arithmetic with the float running sum the reference keeps,
//                so the sums are the reference's to the bit
//
// The reference's brute force (every atom against every pixel of every slice
// it reaches, no lateral cut-off but the radial one) is kept: one thread per
// pixel and slice walks the atoms of the slice's z range.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "qs_internal.h"
#include "qs_zorder.h"

namespace qs {

namespace {

// seval (stem3/stemutil.cpp:1069-1092) over n knots
__device__ double ft_seval(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ b,
                           const double* __restrict__ c, const double* __restrict__ d, int n, double x0) {
    int i;
    if (x0 <= x[0]) i = 0;
    else if (x0 >= x[n - 2]) i = n - 2;
    else {
        int lo = 0, hi = n;
        do {
            const int k = (lo + hi) / 2;
            if (x0 < x[k]) hi = k;
            else lo = k;
        } while (hi - lo > 1);
        i = lo;
    }
    const double z = x0 - x[i];
    return y[i] + (b[i] + (c[i] + d[i] * z) * z) * z;
}

// sfLUT: 0 above the last k and where the spline is negative
__device__ double ft_sf(const double* tab, int n, double s) {
    const double* k = tab;
    if (s > k[n - 1]) return 0.0;
    const double v = ft_seval(k, tab + n, tab + 2 * n, tab + 3 * n, tab + 4 * n, n, s);
    return v < 0 ? 0.0 : v;
}

struct FtBox {
    int Nz, Nx, Nzm, Nxm, zOversample;
    double dZ, dX, dsZ, dsX, sz2max, sx2max, halfAx, halfCz, scale;
};

// f(s) e^{i arg} on the box's k-grid (stem3/customslice.cpp:168-190)
__global__ void ft_kgrid(const double* __restrict__ tab, int n, FtBox B, double2* __restrict__ pot) {
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = blockIdx.y;
    if (ix >= B.Nx) return;
    double2 v = make_double2(0.0, 0.0);
    const double sz = (iz < B.Nzm ? iz : iz - B.Nz) * B.dsZ, sz2 = sz * sz, sz2r = B.sz2max * sz2;
    if ((B.Nz < 2) || (sz2r <= 1.0)) {
        const double sx = (ix < B.Nxm ? ix : ix - B.Nx) * B.dsX, sx2 = sx * sx;
        if (sz2r + B.sx2max * sx2 <= 1.0) {
            const double s = sqrt(sz2 + sx2);
            const double arg = 6.28318530717959 * (sx * B.halfAx + sz * B.halfCz);
            const double f = ft_sf(tab, n, 0.5 * s);
            v = make_double2(f * cos(arg), f * sin(arg));
        }
    }
    pot[(size_t)iz * B.Nx + ix] = v;
}

// inverse DFT of every row (length n, FP64), e^{+2 pi i k/n} from W
__global__ void ft_dft_rows(const double2* __restrict__ in, const double2* __restrict__ W, int n,
                            double2* __restrict__ out) {
    extern __shared__ double2 lsm[];
    double2* w = lsm;
    double2* row = lsm + n;
    const int r = blockIdx.y;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        w[i] = W[i];
        row[i] = in[(size_t)r * n + i];
    }
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double re = 0, im = 0;
    int m = 0;
    for (int j = 0; j < n; j++) {
        const double2 v = row[j], t = w[m];
        re += v.x * t.x - v.y * t.y;
        im += v.x * t.y + v.y * t.x;
        m += k;
        if (m >= n) m -= n;
    }
    out[(size_t)r * n + k] = make_double2(re, im);
}

// inverse DFT of every column (length nz over rows of length nx, FP64)
__global__ void ft_dft_cols(const double2* __restrict__ in, const double2* __restrict__ W, int nz, int nx,
                            double2* __restrict__ out) {
    extern __shared__ double2 lsm[];
    for (int i = threadIdx.x; i < nz; i += blockDim.x) lsm[i] = W[i];
    __syncthreads();
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (ix >= nx) return;
    double re = 0, im = 0;
    int m = 0;
    for (int j = 0; j < nz; j++) {
        const double2 v = in[(size_t)j * nx + ix], t = lsm[m];
        re += v.x * t.x - v.y * t.y;
        im += v.x * t.y + v.y * t.x;
        m += k;
        if (m >= nz) m -= nz;
    }
    out[(size_t)k * nx + ix] = make_double2(re, im);
}

__global__ void ft_twiddles(int n, double2* __restrict__ W) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double sn, cs;
    sincospi(2.0 * k / n, &sn, &cs);
    W[k] = make_double2(cs, sn);
}

// The scale and the radial cut-off in the reference's scan order (each
// negative value within the current cut-off shrinks it), the zeroing beyond
// the final cut-off, and reduceAndExpand into ff (nz = Nzm + 2 rows of
// nx = Nxm, flat: the last column of a row lands on the next row's first
// element, as in the reference's row-major array).  One thread: the cut-off
// is a sequential scan.
__global__ void ft_reduce(double2* __restrict__ pot, FtBox B, double* __restrict__ ff, double* __restrict__ rcOut) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double rc = 50;
    for (int iz = 0; iz < B.Nz; iz++)
        for (int ix = 0; ix < B.Nx; ix++) {
            double2& v = pot[(size_t)iz * B.Nx + ix];
            const double a = B.dZ * (iz - B.Nzm), b = B.dX * (ix - B.Nxm);
            const double r = sqrt(a * a + b * b);
            if (r > rc) v = make_double2(0.0, 0.0);
            else if (v.x < 0) rc = r, v = make_double2(0.0, 0.0);
            else v = make_double2(v.x * B.scale, v.y * B.scale);
        }
    for (int iz = 0; iz < B.Nz; iz++)
        for (int ix = 0; ix < B.Nx; ix++) {
            const double a = B.dZ * (iz - B.Nzm), b = B.dX * (ix - B.Nxm);
            if (sqrt(a * a + b * b) > rc) pot[(size_t)iz * B.Nx + ix] = make_double2(0.0, 0.0);
        }
    *rcOut = rc;
    const int Nxm = B.Nxm, Nzm = B.Nzm, nx = Nxm, nz = Nzm + 2;
    for (size_t i = 0; i < (size_t)nz * nx; i++) ff[i] = 0.0;
    const int Ninteg = (B.zOversample - 1) / 2;
    for (int iz = 0; iz < Nzm; iz++)
        for (int ix = 0; ix < Nxm; ix++)
            for (int j = -Ninteg; j <= Ninteg; j++)
                if ((iz + j + Nzm >= 0) && (iz + j < Nzm))
                    ff[(size_t)(iz + 1) * nx + ix + 1] += pot[(size_t)(iz + Nzm + j) * B.Nx + ix + Nxm].x;
    for (int iz = 1; iz <= Nzm; iz++)
        ff[(size_t)iz * nx] = ff[(size_t)iz * nx + 1] + (ff[(size_t)iz * nx + 1] - ff[(size_t)iz * nx + 2]);
    for (int ix = 0; ix <= Nxm; ix++) ff[ix] = ff[nx + ix] + (ff[nx + ix] - ff[2 * (size_t)nx + ix]);
}

// bicubic (stem3/stemutil.cpp:1470-1520) on a flat nz x nx table
__device__ double ft_bicubic(const double* __restrict__ ff, int Nz, int Nx, double z, double x) {
    const int xi = (int)x, zi = (int)z;
    x = x - (double)xi;
    z = z - (double)zi;
    const double x0 = ((2.0 - x) * x - 1.0) * x;
    const double x1 = (3.0 * x - 5.0) * x * x + 2.0;
    const double x2 = ((4.0 - 3.0 * x) * x + 1.0) * x;
    x = (x - 1.0) * x * x;
    auto fx = [&](int r) {
        const double* p = ff + (size_t)r * Nx;
        return p[xi - 1] * x0 + p[xi] * x1 + p[xi + 1] * x2 + p[xi + 2] * x;
    };
    double f;
    if (Nz > 2) {
        if ((zi > Nz - 3) || (xi > Nx - 3)) return 0.0;
        if ((zi < 1) && (xi < 1)) return ff[0];
        if (zi < 1) return ff[xi];
        if (xi < 1) return ff[(size_t)zi * Nx];
        f = fx(zi - 1) * (((2.0 - z) * z - 1) * z);
        f += fx(zi) * ((3.0 * z - 5.0) * z * z + 2.0);
        f += fx(zi + 1) * (((4.0 - 3.0 * z) * z + 1.0) * z);
        f += fx(zi + 2) * ((z - 1.0) * z * z);
        f *= 0.25;
    } else {
        f = 0.5 * fx(0);
    }
    return f;
}

struct FtAtom {
    double x, y, z;  // the atom's x, y, z as the reference reads them (floats)
    int kind;
};

// every atom of the slice's z range added to one pixel, in z order
// (stem3/customslice.cpp:260-290): the running float sum of the reference
__global__ void ft_accumulate(const FtAtom* __restrict__ atoms, const int2* __restrict__ range,
                              const double* const* __restrict__ ffs, const double* __restrict__ rc, int Nzl, int Nxl,
                              int Nxp, int Nyp, double dXp, double dYp, double dZp, double dZ, double dX,
                              double zStart, double offX, double offY, float* __restrict__ V) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y, iz = blockIdx.z;
    if (iy >= Nyp) return;
    const int2 rg = range[iz];
    float acc = 0.f;
    for (int j = rg.x; j < rg.y; j++) {
        const FtAtom A = atoms[j];
        const double rck = rc[A.kind];
        const double z = fabs((iz + 0.5) * dZp - (A.z - zStart) + 0.0);
        if (!(z <= rck + dZp)) continue;
        const double x = ((ix + 0.5) * dXp - A.x + 0.0) + offX;
        const double y = ((iy + 0.5) * dYp - A.y + 0.0) + offY;
        const double rxy2 = x * x + y * y;
        const double r = sqrt(rxy2 + z * z);
        if (r <= rck + dZp + dXp)
            acc = (float)((double)acc + ft_bicubic(ffs[A.kind], Nzl, Nxl, z / dZ + 1.0, sqrt(rxy2) / dX + 1.0));
    }
    V[((size_t)iz * Nxp + ix) * Nyp + iy] = acc;
}

}  // namespace

int build_custom_potential(const qs_params& P, const qs_atom* atoms_in, int natom, const double* kIn, int nk,
                           const int* Zs, const double* sf, int nkinds, float* V, cudaStream_t s) {
    const int Nxp = P.potNx, Nyp = P.potNy, Nzp = P.slices;
    if (Nzp < 2) {
        set_error("custom scattering factors: the reference adds no atoms to a single slice");
        return QS_ERR_UNSUPPORTED;
    }
    if (nk < 4 || nkinds < 1 || !kIn || !Zs || !sf) {
        set_error("custom scattering factors: a table of at least 4 k values and one element is needed");
        return QS_ERR_ARG;
    }
    // the 40 A (z, r) box (stem3/customslice.cpp:114-160), in the
    // reference's float and double types
    const float czp = P.c / (float)P.cellDiv;
    const float axp = P.potSizeX, byp = P.potSizeY;
    const float dXp = (float)(axp / (double)Nxp), dYp = (float)(byp / (double)Nyp), dZp = (float)(czp / (double)Nzp);
    float ax = 40.0f, cz = 40.0f;
    double dZ = dZp;
    int zOversample = 1;
    while (dZ > 0.4) zOversample += 2, dZ = dZp / (double)(zOversample);
    int Nz = (int)(cz / dZ + 0.5);
    if (Nz / 2 < 0.5 * (double)Nz) Nz++;
    cz = (float)((double)Nz * dZ);
    double dX = (dXp < dYp ? dXp : dYp);
    int xOversample = 1;
    while (dX > 0.1) dX = dXp / (double)(++xOversample);
    int Nx = (int)(ax / dX);
    if (Nx / 2 < 0.5 * (double)Nx) Nx++;
    ax = (float)((double)Nx * dX);
    FtBox B;
    B.Nz = Nz;
    B.Nx = Nx;
    B.Nxm = Nx / 2;
    B.zOversample = zOversample;
    B.dZ = dZ;
    B.dX = dX;
    B.dsX = 1.0 / ax;
    B.dsZ = 1.0 / cz;
    B.sx2max = 10.8 * (B.Nxm * B.dsX);
    B.sx2max = 1.0 / (B.sx2max * B.sx2max);
    if (Nz > 1) {
        B.Nzm = Nz / 2;
        const double t = 10.8 * (B.Nzm * B.dsZ);
        B.sz2max = 1.0 / (t * t);
    } else {
        B.Nzm = 1;
        B.sz2max = 1.0;
    }
    B.halfAx = 0.5 * ax;
    B.halfCz = 0.5 * cz;
    B.scale = 2 * 47.87658 / (std::sqrt((double)(Nx * Nz) * ax * cz));
    const int Nzl = B.Nzm + 2, Nxl = B.Nxm;

    // atoms in the reference's order (atomCompare: by z; glibc's qsort keeps
    // ties in input order, as a stable sort does), each with its element's
    // table index; per slice the run of atoms whose z can reach it (the
    // per-atom test z <= rc + dZp still decides)
    std::vector<int> zo;
    z_order(natom, [&](int i) { return atoms_in[i].z; }, zo);
    std::vector<qs_atom> at(natom);
    for (int i = 0; i < natom; i++) at[i] = atoms_in[zo[i]];
    std::vector<FtAtom> fa(std::max(natom, 1));
    for (int j = 0; j < natom; j++) {
        int kind = 0;
        while (kind < nkinds && Zs[kind] != at[j].Znum) kind++;
        if (kind == nkinds) {
            set_error("custom scattering factors: no table for Z = " + std::to_string(at[j].Znum));
            return QS_ERR_ARG;
        }
        fa[j] = FtAtom{(double)at[j].x, (double)at[j].y, (double)at[j].z, kind};
    }

    // device work: per element the k-grid, two DFT passes and the reduction
    int rc = QS_OK;
    auto fail = [&](cudaError_t e, const char* what) {
        set_error(std::string("custom scattering factors: ") + what + ": " + cudaGetErrorString(e));
        rc = QS_ERR_CUDA;
    };
    const int n = nk + 1;
    std::vector<double> tabs((size_t)nkinds * 5 * n);
    for (int kind = 0; kind < nkinds; kind++) {
        double* t = tabs.data() + (size_t)kind * 5 * n;
        std::memcpy(t, kIn, sizeof(double) * nk);
        t[nk] = 2.0 * kIn[nk - 1];
        std::memcpy(t + n, sf + (size_t)kind * nk, sizeof(double) * nk);
        t[n + nk] = 0.0;
        akima_spline(t, t + n, t + 2 * n, t + 3 * n, t + 4 * n, n);
    }
    double *d_tab = nullptr, *d_ff = nullptr, *d_rc = nullptr;
    double2 *d_pot = nullptr, *d_tmp = nullptr, *d_W = nullptr;
    double** d_ffp = nullptr;
    FtAtom* d_atoms = nullptr;
    int2* d_range = nullptr;
    const size_t ffElems = (size_t)Nzl * Nxl;
    cudaError_t e;
    if ((e = cudaMallocAsync(&d_tab, sizeof(double) * tabs.size(), s)) != cudaSuccess) { fail(e, "alloc"); return rc; }
    if ((e = cudaMallocAsync(&d_pot, sizeof(double2) * (size_t)Nz * Nx, s)) != cudaSuccess) fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_tmp, sizeof(double2) * (size_t)Nz * Nx, s)) != cudaSuccess) fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_W, sizeof(double2) * (size_t)(Nx + Nz), s)) != cudaSuccess) fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_ff, sizeof(double) * ffElems * nkinds, s)) != cudaSuccess) fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_rc, sizeof(double) * nkinds, s)) != cudaSuccess) fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_ffp, sizeof(double*) * nkinds, s)) != cudaSuccess) fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_atoms, sizeof(FtAtom) * fa.size(), s)) != cudaSuccess) fail(e, "alloc");
    if (!rc && (e = cudaMallocAsync(&d_range, sizeof(int2) * Nzp, s)) != cudaSuccess) fail(e, "alloc");
    const size_t smr = sizeof(double2) * 2 * (size_t)Nx, smc = sizeof(double2) * (size_t)Nz;
    if (!rc && (e = cudaFuncSetAttribute(ft_dft_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr)) !=
                   cudaSuccess)
        fail(e, "shared memory");
    std::vector<double*> ffp(nkinds);
    std::vector<int2> range(Nzp);
    if (!rc) {
        for (int kind = 0; kind < nkinds; kind++) ffp[kind] = d_ff + (size_t)kind * ffElems;
        // the atoms whose z lies within rc_max + dZp of a slice centre; the
        // cut-off is at most 50 A (its start value)
        const double reach = 50.0 + (double)dZp + 1.0, zStart = P.czOffset;
        for (int iz = 0; iz < Nzp; iz++) {
            const double zc = (iz + 0.5) * dZp + zStart;
            const auto lo = std::lower_bound(fa.begin(), fa.begin() + natom, zc - reach,
                                             [](const FtAtom& a, double v) { return a.z < v; });
            const auto hi = std::upper_bound(fa.begin(), fa.begin() + natom, zc + reach,
                                             [](double v, const FtAtom& a) { return v < a.z; });
            range[iz] = make_int2((int)(lo - fa.begin()), (int)(hi - fa.begin()));
        }
        cudaMemcpyAsync(d_tab, tabs.data(), sizeof(double) * tabs.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_ffp, ffp.data(), sizeof(double*) * nkinds, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_atoms, fa.data(), sizeof(FtAtom) * fa.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_range, range.data(), sizeof(int2) * Nzp, cudaMemcpyHostToDevice, s);
        ft_twiddles<<<(Nx + 127) / 128, 128, 0, s>>>(Nx, d_W);
        ft_twiddles<<<(Nz + 127) / 128, 128, 0, s>>>(Nz, d_W + Nx);
        for (int kind = 0; kind < nkinds; kind++) {
            ft_kgrid<<<dim3((Nx + 127) / 128, Nz), 128, 0, s>>>(d_tab + (size_t)kind * 5 * n, n, B, d_pot);
            ft_dft_rows<<<dim3((Nx + 127) / 128, Nz), 128, smr, s>>>(d_pot, d_W, Nx, d_tmp);
            ft_dft_cols<<<dim3((Nx + 127) / 128, Nz), 128, smc, s>>>(d_tmp, d_W + Nx, Nz, Nx, d_pot);
            ft_reduce<<<1, 1, 0, s>>>(d_pot, B, ffp[kind], d_rc + kind);
        }
        ft_accumulate<<<dim3((Nyp + 127) / 128, Nxp, Nzp), 128, 0, s>>>(
            d_atoms, d_range, (const double* const*)d_ffp, d_rc, Nzl, Nxl, Nxp, Nyp, (double)dXp, (double)dYp,
            (double)dZp, dZ, dX, (double)P.czOffset, (double)P.potOffsetX, (double)P.potOffsetY, V);
        if ((e = cudaGetLastError()) != cudaSuccess) fail(e, "launch");
        else count_launch(3 + 4 * nkinds);
    }
    // the host tables above must outlive their copies
    const cudaError_t es = cudaStreamSynchronize(s);
    if (!rc && es != cudaSuccess) fail(es, "run");
    cudaFreeAsync(d_range, s);
    cudaFreeAsync(d_atoms, s);
    cudaFreeAsync(d_ffp, s);
    cudaFreeAsync(d_rc, s);
    cudaFreeAsync(d_ff, s);
    cudaFreeAsync(d_W, s);
    cudaFreeAsync(d_tmp, s);
    cudaFreeAsync(d_pot, s);
    cudaFreeAsync(d_tab, s);
    return rc;
}

}  // namespace qs
