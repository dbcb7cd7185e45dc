/*
 * qs_oracle.c -- C restatement of QSTEM's multislice hot path (CPU).
 *
 * TEST INFRASTRUCTURE ONLY (see qs_oracle.h).  Every function names the
 * reference function and lines it restates.  Where the reference mixes float
 * and double arithmetic, this code keeps the same types so that the results
 * agree with the reference to rounding; the 2-D FFTs go through qs_fft.c,
 * the same arithmetic the FFT shim supplies to the compiled reference.
 */
#include "qs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../qstem_gb300/csrc/qs_rez_table.h"
#include "qs_fft.h"

#define OVERSAMP_X 2
#define REF_PI 3.14159265358979 /* the PI of stem3/stemlib.cpp:75 */
#define NSF QS_REZ_NSF

/* ------------------------------------------------------------------ util */
double qso_wavelength(double kev) {
    /* stem3/stemutil.cpp:714-725: lambda = hc / sqrt(E (2 m c^2 + E)) */
    const double emass = 510.99906, hc = 12.3984244;
    return hc / sqrt(kev * (2 * emass + kev));
}

void qso_splinh(const double *x, const double *y, double *b, double *c, double *d, int n) {
    /* Akima's local cubic (stem3/stemutil.cpp:975-1041): node slopes from the
     * weighted neighbouring secant slopes, two secants extrapolated linearly
     * at each end. */
    const double tiny = 1.0e-25;
    if (n < 4) return;
    double m5 = (y[3] - y[2]) / (x[3] - x[2]);
    double m4 = (y[2] - y[1]) / (x[2] - x[1]);
    double m3 = (y[1] - y[0]) / (x[1] - x[0]);
    double m2 = m3 + m3 - m4;
    double m1 = m2 + m2 - m3;
    double m54 = fabs(m5 - m4), m43 = fabs(m4 - m3), m32 = fabs(m3 - m2), m21 = fabs(m2 - m1);
    double t1 = ((m43 + m21) > tiny) ? (m43 * m2 + m21 * m3) / (m43 + m21) : 0.5 * (m2 + m3);
    for (int i = 0; i < n - 1; i++) {
        double t2 = ((m54 + m32) > tiny) ? (m54 * m3 + m32 * m4) / (m54 + m32) : 0.5 * (m3 + m4);
        double h = x[i + 1] - x[i];
        b[i] = t1;
        c[i] = (3.0 * m3 - t1 - t1 - t2) / h;
        d[i] = (t1 + t2 - m3 - m3) / (h * h);
        m1 = m2; m2 = m3; m3 = m4; m4 = m5;
        m5 = (i < n - 4) ? (y[i + 4] - y[i + 3]) / (x[i + 4] - x[i + 3]) : m4 + m4 - m3;
        m21 = m32; m32 = m43; m43 = m54; m54 = fabs(m5 - m4);
        t1 = t2;
    }
    (void)m1;
}

double qso_seval(const double *x, const double *y, const double *b, const double *c,
                 const double *d, int n, double x0) {
    /* stem3/stemutil.cpp:1069-1092: bisection for the interval, clamped to
     * the first and the second-to-last interval. */
    int i;
    if (x0 <= x[0]) i = 0;
    else if (x0 >= x[n - 2]) i = n - 2;
    else {
        int lo = 0, hi = n;
        do {
            int k = (lo + hi) / 2;
            if (x0 < x[k]) hi = k;
            else lo = k;
        } while (hi - lo > 1);
        i = lo;
    }
    double z = x0 - x[i];
    return y[i] + (b[i] + (c[i] + d[i] * z) * z) * z;
}

int qso_thickness_count(const qs_params *p) {
    /* tCount = (slices*cellDiv)/outputInterval (integer division), plus the
     * final-thickness slot (stem3/stemlib.cpp:2589, stem3/stem3.cpp:1318) */
    return (p->slices * p->cellDiv) / p->outputInterval + 1;
}

void qso_params_finalize(qs_params *p) {
    double wl = qso_wavelength(p->v0);
    for (int i = 0; i < p->detectorNum; i++) {
        qs_detector *d = &p->detectors[i];
        /* stem3/stem3.cpp:1343-1350: float(sin(r/1000)/lambda), squared in float */
        d->k2Inside = (float)(sin(d->rInside * 0.001) / wl);
        d->k2Outside = (float)(sin(d->rOutside * 0.001) / wl);
        d->k2Inside *= d->k2Inside;
        d->k2Outside *= d->k2Outside;
    }
}

/* ------------------------------------------------------------------- LUT */
/* The reference truncates the s-grid tail at the LUT's k_max on first use
 * (stem3/stemlib.cpp:1390-1413, :1598-1620): the last three grid points
 * become 1.2, 1.1 and 1.0 k_max, and grid points above k_max are pulled down
 * to k_max - 0.001*j with their f values zeroed. */
static void truncate_tail(double *grid, double *row, double kmax) {
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

int qso_lut(const qs_params *p, int Z, double B, int charged, float *out, int *NzL, int *NrO,
            int *nzSubO) {
    if (Z < 1 || Z >= QS_REZ_NELEM) return QS_ERR_ARG;
    const float rx = p->resolutionX, ry = p->resolutionY, dzs = p->sliceThickness;
    const float R = p->atomRadius;
    const int nx = 2 * OVERSAMP_X * (int)ceilf(R / rx);
    const int ny = 2 * OVERSAMP_X * (int)ceilf(R / ry);
    int nzPer = (int)floorf((float)OVERSAMP_X * dzs / rx);
    if (2.0 * (nzPer >> 1) == nzPer) nzPer += 1;
    const int nz = (2 * (int)ceilf(R / dzs)) * nzPer;
    if (NzL) *NzL = nz / 2;
    if (NrO) *NrO = nx / 2;
    if (nzSubO) *nzSubO = nzPer;
    if (!out) return QS_OK;

    const double dkx = 0.5 * OVERSAMP_X / (double)((float)nx * rx);
    const double dky = charged ? 0.5 * OVERSAMP_X / (double)((float)ny * ry) : dkx;
    const double dkz = nzPer / (double)((float)nz * dzs);
    const double kmax = 0.5 * nx * dkx / (double)OVERSAMP_X;
    const double smax2 = kmax * kmax;

    /* f(s) tables after the reference's tail truncation */
    double fg[NSF], fr[NSF], qg[NSF], qr[NSF];
    memcpy(fg, QS_REZ_F[0], sizeof fg);
    memcpy(fr, QS_REZ_F[Z], sizeof fr);
    truncate_tail(fg, fr, kmax);
    const double *g1 = fg, *r1 = fr; /* spline table and the s=|k| term */
    if (charged) {
        memcpy(qg, QS_REZ_Q[0], sizeof qg);
        memcpy(qr, QS_REZ_Q[Z], sizeof qr);
        truncate_tail(qg, qr, kmax);
        g1 = qg;
        r1 = qr;
    }
    double sb[NSF], sc[NSF], sd[NSF];
    qso_splinh(g1, r1, sb, sc, sd, NSF);
    /* the qy-sum evaluates the neutral table with these coefficients in the
     * charged case too (stem3/stemlib.cpp:1672) */
    const double *g2 = charged ? fg : g1, *r2 = charged ? fr : r1;

    float *temp = (float *)calloc(2 * (size_t)nx * nz, sizeof(float));
    const int izOffset = (nzPer - 1) / 2;
    const double xPos = -2.0 * REF_PI * 0.0;
    const double zPos = -2.0 * REF_PI * (double)(dzs / (float)nzPer * (float)izOffset);
    for (int iz = 0; iz < nz; iz++) {
        const double kz = dkz * (iz < nz / 2 ? iz : iz - nz);
        for (int ix = 0; ix < nx; ix++) {
            const double kx = dkx * (ix < nx / 2 ? ix : ix - nx);
            const double s2 = kx * kx + kz * kz;
            if (s2 < smax2) {
                double f = qso_seval(g1, r1, sb, sc, sd, NSF, sqrt(s2)) * exp(-s2 * B * 0.25);
                for (int iy = 1; iy < nx; iy++) {
                    double s3 = (charged ? dky : dkx) * iy;
                    s3 = s3 * s3 + s2;
                    if (s3 < smax2)
                        f += 2 * qso_seval(g2, r2, sb, sc, sd, NSF, sqrt(s3)) * exp(-s3 * B * 0.25);
                    else
                        break;
                }
                f *= dkx;
                const double phase = kx * xPos + kz * zPos;
                temp[2 * (ix + (size_t)iz * nx)] = (float)(f * cos(phase));
                temp[2 * (ix + (size_t)iz * nx) + 1] = (float)(f * sin(phase));
            }
        }
    }
    qs_fft2d_c64(nz, nx, temp, +1);
    for (int ix = 0; ix < nx / 2; ix++)
        for (int iz = 0; iz < nz / 2; iz++) {
            double zScale = 0;
            for (int iiz = -izOffset; iiz <= izOffset; iiz++)
                if (iz + izOffset + iiz < nz / 2) zScale += temp[2 * (ix + (size_t)(iz + izOffset + iiz) * nx)];
            if (zScale < 0) zScale = 0;
            out[ix + (size_t)iz * (nx / 2)] = (float)(47.8658 * dkx * dkz / (nz)*zScale);
        }
    free(temp);
    return QS_OK;
}

/* getAtomPotential2D (stem3/stemlib.cpp:1750-1857): the oversampled 2-D
 * projected-potential table of element Z, nx x ny complex floats
 * (nx = 2*OVERSAMP_X*ceil(R/dx)), f(k) e^{i phase} on the k-grid (the
 * scattering-factor tail truncated at kmax as the reference truncates its
 * global table on the first call), inverse 2-D FFT, real part scaled by
 * dkx*dky*OVERSAMP_X^2 (the imaginary part left unscaled, as the reference
 * leaves it).  out may be NULL to query the size. */
int qso_lut2d(const qs_params *p, int Z, double B, float *out, int *nxO, int *nyO) {
    if (Z < 1 || Z >= QS_REZ_NELEM) return QS_ERR_ARG;
    const float rx = p->resolutionX, ry = p->resolutionY, R = p->atomRadius;
    const int nx = 2 * OVERSAMP_X * (int)ceilf(R / rx);
    const int ny = 2 * OVERSAMP_X * (int)ceilf(R / ry);
    if (nxO) *nxO = nx;
    if (nyO) *nyO = ny;
    if (!out) return QS_OK;
    const double dkx = 0.5 * OVERSAMP_X / (double)((float)nx * rx);
    const double dky = 0.5 * OVERSAMP_X / (double)((float)ny * ry);
    double kmax2 = 0.5 * nx * dkx / (double)OVERSAMP_X;
    double fg[NSF], fr[NSF], sb[NSF], sc[NSF], sd[NSF];
    memcpy(fg, QS_REZ_F[0], sizeof fg);
    memcpy(fr, QS_REZ_F[Z], sizeof fr);
    truncate_tail(fg, fr, kmax2);
    kmax2 *= kmax2;
    qso_splinh(fg, fr, sb, sc, sd, NSF);
    memset(out, 0, sizeof(float) * 2 * (size_t)nx * ny);
    for (int ix = 0; ix < nx; ix++) {
        const double kx = dkx * (ix < nx / 2 ? ix : nx - ix);
        for (int iy = 0; iy < ny; iy++) {
            const double ky = dky * (iy < ny / 2 ? iy : ny - iy);
            const double s2 = kx * kx + ky * ky;
            if (s2 < kmax2) {
                const double f = qso_seval(fg, fr, sb, sc, sd, NSF, sqrt(s2)) * exp(-s2 * B * 0.25);
                const double phase = REF_PI * (kx * (double)rx * nx + ky * (double)ry * ny);
                out[2 * (iy + (size_t)ix * ny)] = (float)(f * cos(phase));
                out[2 * (iy + (size_t)ix * ny) + 1] = (float)(f * sin(phase));
            }
        }
    }
    qs_fft2d_c64(nx, ny, out, +1);
    const double scale = dkx * dky * (OVERSAMP_X * OVERSAMP_X);
    for (size_t i = 0; i < (size_t)nx * ny; i++) out[2 * i] = (float)((double)out[2 * i] * scale);
    return QS_OK;
}

/* ------------------------------------------------------------- potential */
static int cmp_z(const void *a, const void *b) {
    /* atomCompare, stem3/stemutil.cpp:1524-1531: by z only */
    float za = ((const qs_atom *)a)->z, zb = ((const qs_atom *)b)->z;
    return (za == zb) ? 0 : ((za > zb) ? 1 : -1);
}

typedef struct {
    float *lut[QS_REZ_NELEM];
    float *lutq[QS_REZ_NELEM];
    int Nz, Nr, nzSub;
} lut_cache;

static const float *cache_get(lut_cache *c, const qs_params *p, int Z, double B, int charged) {
    float **slot = charged ? &c->lutq[Z] : &c->lut[Z];
    if (!*slot) {
        int Nz, Nr, ns;
        qso_lut(p, Z, B, charged, NULL, &Nz, &Nr, &ns);
        *slot = (float *)malloc(sizeof(float) * (size_t)Nz * Nr);
        qso_lut(p, Z, B, charged, *slot, &c->Nz, &c->Nr, &c->nzSub);
    }
    return *slot;
}

/* Add one atom's LUT over the slices [iAtomZ+iaz0, iAtomZ+iaz1] at pixel
 * column `col` (float* into slice iAtomZ+iaz0): the inner iaz loop of
 * stem3/stemlib.cpp:946-1028 / :1127-1204. */
static inline void add_column(float *col, size_t sliceStep, int iaz0, int iaz1, double ddr,
                              int ir, int iOffsZ, int Nr, int Nz, int nzSub, const float *lut,
                              const float *lutq, float q) {
    const int limHi = Nr * (Nz - 1), limLo = -Nr * (Nz - 1), step = nzSub * Nr;
    for (int iaz = iaz0; iaz <= iaz1; iaz++) {
        double potVal = 0;
        if (iOffsZ < 0) {
            if (iOffsZ > limLo) {
                potVal = (1 - ddr) * lut[ir - iOffsZ + Nr] + ddr * lut[ir + 1 - iOffsZ + Nr];
                if (lutq) potVal += q * ((1 - ddr) * lutq[ir - iOffsZ + Nr] + ddr * lutq[ir + 1 - iOffsZ + Nr]);
            }
        } else {
            if (iOffsZ < limHi) {
                potVal = (1 - ddr) * lut[ir + iOffsZ] + ddr * lut[ir + 1 + iOffsZ];
                if (lutq) potVal += q * ((1 - ddr) * lutq[ir + iOffsZ] + ddr * lutq[ir + 1 + iOffsZ]);
            }
        }
        *col = (float)((double)*col + potVal);
        col += sliceStep;
        iOffsZ += step;
    }
}

int qso_potential(const qs_params *p, const qs_atom *atoms_in, int natom, float *trans) {
    return qso_potential_slab(p, atoms_in, natom, 0, trans);
}

/* make3DSlices' call for slab `slab` of a cellDiv-divided cell: the atoms are
 * offset by -slab * c, c = slices * sliceThickness (stem3/stemlib.cpp:456-465,
 * :572, :709-713; divCount counts the slabs down from cellDiv - 1). */
static int potential2d_periodic(const qs_params *p, const qs_atom *atoms_in, int natom, int slab, float *trans);

int qso_potential_slab(const qs_params *p, const qs_atom *atoms_in, int natom, int slab, float *trans) {
    if (!p->fftpotential || slab < 0 || slab >= p->cellDiv) return QS_ERR_UNSUPPORTED;
    if (!p->potential3D) {
        /* only the periodic 2-D branch: the non-periodic one reads its table
         * outside the array for atoms near the edges */
        if (p->nonPeriod) return QS_ERR_UNSUPPORTED;
        return potential2d_periodic(p, atoms_in, natom, slab, trans);
    }
    const int potNx = p->potNx, potNy = p->potNy, slices = p->slices;
    const size_t sliceStep = 2 * (size_t)potNx * potNy; /* floats */
    memset(trans, 0, sizeof(float) * sliceStep * slices);
    if (natom < 1) return QS_OK;
    qs_atom *atoms = (qs_atom *)malloc(sizeof(qs_atom) * (size_t)natom);
    memcpy(atoms, atoms_in, sizeof(qs_atom) * (size_t)natom);
    qsort(atoms, natom, sizeof(qs_atom), cmp_z);

    /* stem3/stemlib.cpp:563-573 */
    const float c = p->sliceThickness * (float)slices;
    const float dx = p->resolutionX, dy = p->resolutionY, dzs = p->sliceThickness;
    const double dr = p->resolutionX / OVERSAMP_X;
    const int iRadX = (int)ceilf(p->atomRadius / dx);
    const int iRadY = (int)ceilf(p->atomRadius / dy);
    const int iRadZ = (int)ceilf(p->atomRadius / dzs);
    lut_cache cache;
    memset(&cache, 0, sizeof cache);

    for (int iatom = 0; iatom < natom; iatom++) {
        while (iatom < natom && atoms[iatom].Znum == 0) iatom++; /* vacancies, :680 */
        if (iatom >= natom) break;
        /* :709-713; c*(cellDiv-divCount-1) is c*slab */
        float atomZ = (float)((double)(atoms[iatom].z - c * (float)slab + p->czOffset) -
                              0.5 * p->sliceThickness * (1 - p->centerSlices));
        atomZ -= p->sliceThickness;
        if (p->nonPeriodZ) { /* :716-731 */
            if (atomZ - p->atomRadius > c) break;
            do {
                if (atomZ + p->atomRadius + p->sliceThickness >= 0) break;
                ++iatom;
                atomZ = (float)((double)(atoms[iatom].z - c * (float)slab + p->czOffset) -
                                0.5 * p->sliceThickness * (1 - p->centerSlices));
                atomZ -= p->sliceThickness;
            } while (iatom < natom - 1);
        }
        const float atomX = atoms[iatom].x - p->potOffsetX;
        const float atomY = atoms[iatom].y - p->potOffsetY;
        const int iAtomX = (int)floorf(atomX / dx);
        const int iAtomY = (int)floorf(atomY / dy);
        atomZ += p->sliceThickness; /* :886 */
        const int iAtomZ = (int)floor(atomZ / dzs + 0.5);
        const int Z = atoms[iatom].Znum;
        const double B = p->tds ? 0.0 : atoms[iatom].dw;
        const float q = atoms[iatom].q;
        int iax0, iax1, iay0, iay1;
        if (p->nonPeriod) { /* :894-1036 */
            iax0 = iAtomX - iRadX < 0 ? 0 : iAtomX - iRadX;
            iax1 = iAtomX + iRadX >= potNx ? potNx - 1 : iAtomX + iRadX;
            iay0 = iAtomY - iRadY < 0 ? 0 : iAtomY - iRadY;
            iay1 = iAtomY + iRadY >= potNy ? potNy - 1 : iAtomY + iRadY;
            if (!((iax0 < potNx) && (iax1 >= 0) && (iay0 < potNy) && (iay1 >= 0))) continue;
        } else { /* :1090-1213, exclusive upper bounds */
            iax0 = iAtomX - iRadX;
            iax1 = iAtomX + iRadX - 1;
            iay0 = iAtomY - iRadY;
            iay1 = iAtomY + iRadY - 1;
        }
        const int iaz0 = iAtomZ - iRadZ < 0 ? -iAtomZ : -iRadZ;
        const int iaz1 = iAtomZ + iRadZ >= slices ? slices - iAtomZ - 1 : iRadZ;
        if (!((iAtomZ + iaz0 < slices) && (iAtomZ + iaz1 >= 0))) continue;
        if (Z < 1 || Z >= QS_REZ_NELEM) continue;
        const float *lut = cache_get(&cache, p, Z, B, 0);
        const float *lutq = (q != 0) ? cache_get(&cache, p, Z, B, 1) : NULL;
        const int Nr = cache.Nr, Nz = cache.Nz, nzSub = cache.nzSub;
        /* :951-955 -- C truncation of the rounded sub-slice offset */
        const double dOffsZ = (double)(((float)(iAtomZ + iaz0) - atomZ / dzs) * (float)nzSub);
        const int iOffsZ0 = ((int)(dOffsZ + 0.5)) * Nr;
        float *slice0 = trans + (size_t)(iAtomZ + iaz0) * sliceStep;
        for (int iax = iax0; iax <= iax1; iax++) {
            const int cx = p->nonPeriod ? iax : (iax + 2 * potNx) % potNx;
            double x2 = (double)((float)iax * dx - atomX);
            x2 *= x2;
            for (int iay = iay0; iay <= iay1; iay++) {
                const int cy = p->nonPeriod ? iay : ((iay % potNy) + potNy) % potNy;
                double y2 = (double)((float)iay * dy - atomY);
                y2 *= y2;
                const double r = sqrt(x2 + y2);
                double ddr = r / dr;
                const int ir = (int)floor(ddr);
                if (ir < Nr - 1) {
                    ddr = ddr - (double)ir;
                    add_column(slice0 + 2 * ((size_t)cx * potNy + cy), sliceStep, iaz0, iaz1, ddr, ir,
                               iOffsZ0, Nr, Nz, nzSub, lut, lutq, q);
                }
            }
        }
    }
    for (int z = 0; z < QS_REZ_NELEM; z++) { free(cache.lut[z]); free(cache.lutq[z]); }
    free(atoms);
    return QS_OK;
}

/* make3DSlices' periodic 2-D branch (stem3/stemlib.cpp:709-731 for the atom
 * z, :1215-1262): each atom adds the bilinear interpolation of its element's
 * 2-D table (getAtomPotential2D; B of the element's first atom in z order)
 * into the one slice floor(atomZ/dz) it lies in, over a 2 iRadX x 2 iRadY box
 * wrapped into the array; the interpolation weights are the reference's,
 * whose names are swapped against the corners they multiply.  Atoms whose
 * slice falls outside the stack are skipped (the reference writes outside its
 * array there). */
static int potential2d_periodic(const qs_params *p, const qs_atom *atoms_in, int natom, int slab, float *trans) {
    const int potNx = p->potNx, potNy = p->potNy, slices = p->slices;
    const size_t sliceStep = 2 * (size_t)potNx * potNy; /* floats */
    memset(trans, 0, sizeof(float) * sliceStep * slices);
    if (natom < 1) return QS_OK;
    qs_atom *atoms = (qs_atom *)malloc(sizeof(qs_atom) * (size_t)natom);
    memcpy(atoms, atoms_in, sizeof(qs_atom) * (size_t)natom);
    qsort(atoms, natom, sizeof(qs_atom), cmp_z);
    const float c = p->sliceThickness * (float)slices;
    const float dx = p->resolutionX, dy = p->resolutionY, dzs = p->sliceThickness;
    const int iRadX = (int)ceilf(p->atomRadius / dx);
    const int iRadY = (int)ceilf(p->atomRadius / dy);
    const int nyAtBox = 2 * OVERSAMP_X * (int)ceilf(p->atomRadius / dy), nyAtBox2 = 2 * nyAtBox;
    float *tab[QS_REZ_NELEM];
    memset(tab, 0, sizeof tab);
    int nx2 = 0, ny2 = 0;
    qso_lut2d(p, 1, 0.0, NULL, &nx2, &ny2);
    for (int iatom = 0; iatom < natom; iatom++) {
        while (iatom < natom && atoms[iatom].Znum == 0) iatom++;
        if (iatom >= natom) break;
        float atomZ = (float)((double)(atoms[iatom].z - c * (float)slab + p->czOffset) -
                              0.5 * p->sliceThickness * (1 - p->centerSlices));
        atomZ = (float)((double)atomZ + 0.5 * p->sliceThickness);
        if (p->nonPeriodZ) {
            if (atomZ > c) break;
            do {
                if (atomZ >= 0) break;
                ++iatom;
                atomZ = (float)((double)(atoms[iatom].z - c * (float)slab + p->czOffset) -
                                0.5 * p->sliceThickness * (1 - p->centerSlices));
                atomZ = (float)((double)atomZ + 0.5 * p->sliceThickness);
            } while (iatom < natom - 1);
        }
        const float atomX = atoms[iatom].x - p->potOffsetX;
        const float atomY = atoms[iatom].y - p->potOffsetY;
        const int iAtomX = (int)floorf(atomX / dx);
        const int iAtomY = (int)floorf(atomY / dy);
        const int iAtomZ = (int)floor(atomZ / dzs);
        const int Z = atoms[iatom].Znum;
        if (Z < 1 || Z >= QS_REZ_NELEM) continue;
        if (iAtomZ < 0 || iAtomZ >= slices) continue;
        if (!tab[Z]) {
            tab[Z] = (float *)malloc(sizeof(float) * 2 * (size_t)nx2 * ny2);
            qso_lut2d(p, Z, p->tds ? 0.0 : atoms[iatom].dw, tab[Z], NULL, NULL);
        }
        const float *L = tab[Z];
        const int iax0 = iAtomX - iRadX + 2 * potNx, iax1 = iAtomX + iRadX + 2 * potNx;
        const int iay0 = iAtomY - iRadY + 2 * potNy, iay1 = iAtomY + iRadY + 2 * potNy;
        double ddx = (-(double)iax0 + (atomX / dx - (double)(iRadX - 2 * potNx))) * (double)OVERSAMP_X;
        double ddy = (-(double)iay0 + (atomY / dy - (double)(iRadY - 2 * potNy))) * (double)OVERSAMP_X;
        const int iOffsX = (int)floor(ddx), iOffsY = (int)floor(ddy);
        ddx -= (double)iOffsX;
        ddy -= (double)iOffsY;
        const double s22 = (1 - ddx) * (1 - ddy), s21 = (1 - ddx) * ddy, s12 = ddx * (1 - ddy), s11 = ddx * ddy;
        float *slice = trans + (size_t)iAtomZ * sliceStep;
        for (int iax = iax0; iax < iax1; iax++) {
            const int atPosX = OVERSAMP_X * (iax - iax0) - iOffsX;
            if (atPosX < 0 || atPosX >= nyAtBox - 1) continue;
            for (int iay = iay0; iay < iay1; iay++) {
                const int atPosY = (iay - iay0) * OVERSAMP_X - iOffsY;
                if (atPosY >= nyAtBox - 1 || atPosY < 0) continue;
                const float *ptr = L + 2 * ((size_t)atPosX * nyAtBox + atPosY);
                float *t = slice + 2 * ((size_t)(iax % potNx) * potNy + (iay % potNy));
                *t = (float)((double)*t + (s11 * ptr[0] + s12 * ptr[2] + s21 * ptr[nyAtBox2] + s22 * ptr[nyAtBox2 + 2]));
            }
        }
    }
    for (int z = 0; z < QS_REZ_NELEM; z++) free(tab[z]);
    free(atoms);
    return QS_OK;
}

/* ------------------------------------------ custom scattering factors */
/* make3DSlicesFT (stem3/customslice.cpp:56-317) with the custom table of
 * readSFactLUT (stem3/stem3.cpp:555-600): k[nk] and f[kind][nk] as read,
 * extended by k = 2 k[nk-1] with f = 0; sfLUT (stem3/stemutil.cpp:1427-1467)
 * evaluates them with the Akima spline, 0 above the last k and where
 * negative. */
typedef struct {
    int n;
    double *k, *f, *b, *c, *d;
} ft_sf;

static double ft_sfeval(const ft_sf *t, double s) {
    if (s > t->k[t->n - 1]) return 0.0;
    const double v = qso_seval(t->k, t->f, t->b, t->c, t->d, t->n, s);
    return v < 0 ? 0.0 : v;
}

/* reduceAndExpand (stem3/customslice.cpp:359-401) on a flat nz x nx array:
 * the real part summed over the z oversampling into rows 1..Nzm, columns
 * 1..Nxm (the last column landing on the next row's first element, as the
 * reference's row-major array places it), then row 0 and column 0
 * extrapolated. */
static double *ft_reduce(const double *fc, int Nz, int Nx, int zOversample, int *fNz, int *fNx) {
    const int Nxm = Nx / 2, Nzm = Nz / 2, nx = Nxm, nz = Nzm + 2;
    double *ff = (double *)calloc((size_t)nz * nx, sizeof(double));
    *fNx = nx;
    *fNz = nz;
    const int Ninteg = (zOversample - 1) / 2;
    for (int iz = 0; iz < Nzm; iz++)
        for (int ix = 0; ix < Nxm; ix++)
            for (int j = -Ninteg; j <= Ninteg; j++)
                if ((iz + j + Nzm >= 0) && (iz + j < Nzm))
                    ff[(size_t)(iz + 1) * nx + ix + 1] += fc[2 * ((size_t)(iz + Nzm + j) * Nx + ix + Nxm)];
    for (int iz = 1; iz <= Nzm; iz++)
        ff[(size_t)iz * nx] = ff[(size_t)iz * nx + 1] + (ff[(size_t)iz * nx + 1] - ff[(size_t)iz * nx + 2]);
    for (int ix = 0; ix <= Nxm; ix++) ff[ix] = ff[nx + ix] + (ff[nx + ix] - ff[2 * (size_t)nx + ix]);
    return ff;
}

/* bicubic (stem3/stemutil.cpp:1470-1520) on the flat table */
static double ft_bicubic(const double *ff, int Nz, int Nx, double z, double x) {
    const int xi = (int)x, zi = (int)z;
    x = x - (double)xi;
    z = z - (double)zi;
    const double x0 = ((2.0 - x) * x - 1.0) * x;
    const double x1 = (3.0 * x - 5.0) * x * x + 2.0;
    const double x2 = ((4.0 - 3.0 * x) * x + 1.0) * x;
    x = (x - 1.0) * x * x;
#define FTX(r) (ff[(size_t)(r) * Nx + xi - 1] * x0 + ff[(size_t)(r) * Nx + xi] * x1 + \
                ff[(size_t)(r) * Nx + xi + 1] * x2 + ff[(size_t)(r) * Nx + xi + 2] * x)
    double f;
    if (Nz > 2) {
        if ((zi > Nz - 3) || (xi > Nx - 3)) return 0.0;
        if ((zi < 1) && (xi < 1)) return ff[0];
        if (zi < 1) return ff[xi];
        if (xi < 1) return ff[(size_t)zi * Nx];
        f = FTX(zi - 1) * (((2.0 - z) * z - 1) * z);
        f += FTX(zi) * ((3.0 * z - 5.0) * z * z + 2.0);
        f += FTX(zi + 1) * (((4.0 - 3.0 * z) * z + 1.0) * z);
        f += FTX(zi + 2) * ((z - 1.0) * z * z);
        f *= 0.25;
    } else {
        f = 0.5 * FTX(0);
    }
#undef FTX
    return f;
}

int qso_potential_ft(const qs_params *p, const qs_atom *atoms_in, int natom, const double *k, int nk,
                     const int *Zs, const double *sf, int nkinds, float *trans) {
    const int Nxp = p->potNx, Nyp = p->potNy, Nzp = p->slices;
    if (Nzp < 2 || nk < 4 || nkinds < 1) return QS_ERR_UNSUPPORTED;
    const size_t sliceStep = 2 * (size_t)Nxp * Nyp;
    memset(trans, 0, sizeof(float) * sliceStep * Nzp);
    /* box geometry (stem3/customslice.cpp:114-160) */
    const float czp = p->c / (float)p->cellDiv;
    const float axp = p->potSizeX, byp = p->potSizeY;
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
    const int Nxm = Nx / 2;
    const double dsX = 1.0 / ax, dsZ = 1.0 / cz;
    double sx2max = 10.8 * (Nxm * dsX);
    sx2max = 1.0 / (sx2max * sx2max);
    int Nzm;
    double sz2max;
    if (Nz > 1) Nzm = Nz / 2, sz2max = 1.0 / ((10.8 * (Nzm * dsZ)) * (10.8 * (Nzm * dsZ)));
    else Nzm = 1, sz2max = 1.0;
    const double twopi = 6.28318530717959;
    double **lut = (double **)calloc(nkinds, sizeof(double *));
    double *rc = (double *)calloc(nkinds, sizeof(double));
    int Nzl = 0, Nxl = 0;
    double *pot = (double *)malloc(sizeof(double) * 2 * (size_t)Nz * Nx);
    ft_sf t;
    t.n = nk + 1;
    t.k = (double *)malloc(sizeof(double) * t.n);
    t.f = (double *)malloc(sizeof(double) * t.n);
    t.b = (double *)malloc(sizeof(double) * t.n);
    t.c = (double *)malloc(sizeof(double) * t.n);
    t.d = (double *)malloc(sizeof(double) * t.n);
    memcpy(t.k, k, sizeof(double) * nk);
    t.k[nk] = 2.0 * k[nk - 1];
    for (int kind = 0; kind < nkinds; kind++) {
        memcpy(t.f, sf + (size_t)kind * nk, sizeof(double) * nk);
        t.f[nk] = 0.0;
        qso_splinh(t.k, t.f, t.b, t.c, t.d, t.n);
        memset(pot, 0, sizeof(double) * 2 * (size_t)Nz * Nx);
        for (int iz = 0; iz < Nz; iz++) {
            const double sz = (iz < Nzm ? iz : iz - Nz) * dsZ, sz2 = sz * sz, sz2r = sz2max * sz2;
            if ((Nz < 2) || (sz2r <= 1.0)) {
                for (int ix = 0; ix < Nx; ix++) {
                    const double sx = (ix < Nxm ? ix : ix - Nx) * dsX, sx2 = sx * sx;
                    if (sz2r + sx2max * sx2 <= 1.0) {
                        const double s = sqrt(sz2 + sx2);
                        const double arg = twopi * (sx * (0.5 * ax) + sz * (0.5 * cz));
                        const double ffr = cos(arg), ffi = sin(arg);
                        pot[2 * ((size_t)iz * Nx + ix)] = ft_sfeval(&t, 0.5 * s) * ffr;
                        pot[2 * ((size_t)iz * Nx + ix) + 1] = ft_sfeval(&t, 0.5 * s) * ffi;
                    }
                }
            }
        }
        const int dims[2] = {Nz, Nx};
        qs_fftnd_c128(2, dims, 1, 0, pot, +1);
        const double scale = 2 * 47.87658 / (sqrt((double)(Nx * Nz) * ax * cz));
        double rcut = 50;
        for (int iz = 0; iz < Nz; iz++)
            for (int ix = 0; ix < Nx; ix++) {
                double *v = pot + 2 * ((size_t)iz * Nx + ix);
                const double r = sqrt((dZ * (iz - Nzm)) * (dZ * (iz - Nzm)) + (dX * (ix - Nxm)) * (dX * (ix - Nxm)));
                if (r > rcut) v[0] = 0.0, v[1] = 0.0;
                else if (v[0] < 0) rcut = r, v[0] = 0.0, v[1] = 0.0;
                else v[0] *= scale, v[1] *= scale;
            }
        for (int iz = 0; iz < Nz; iz++)
            for (int ix = 0; ix < Nx; ix++) {
                const double r = sqrt((dZ * (iz - Nzm)) * (dZ * (iz - Nzm)) + (dX * (ix - Nxm)) * (dX * (ix - Nxm)));
                if (r > rcut) pot[2 * ((size_t)iz * Nx + ix)] = 0.0, pot[2 * ((size_t)iz * Nx + ix) + 1] = 0.0;
            }
        rc[kind] = rcut;
        lut[kind] = ft_reduce(pot, Nz, Nx, zOversample, &Nzl, &Nxl);
    }
    /* the atoms, sorted by z (atomCompare), each added to every pixel of
     * every slice within the cut-off (stem3/customslice.cpp:260-290); divCount
     * is a local of the reference's function, so the z origin is czOffset */
    qs_atom *atoms = (qs_atom *)malloc(sizeof(qs_atom) * (size_t)(natom > 0 ? natom : 1));
    if (natom > 0) memcpy(atoms, atoms_in, sizeof(qs_atom) * (size_t)natom);
    qsort(atoms, natom, sizeof(qs_atom), cmp_z);
    const double zStart = p->czOffset;
    int rc_ok = QS_OK;
    for (int j = 0; j < natom && rc_ok == QS_OK; j++) {
        int kind = 0;
        while (kind < nkinds && Zs[kind] != atoms[j].Znum) kind++;
        if (kind == nkinds) { rc_ok = QS_ERR_ARG; break; }
        for (int iz = 0; iz < Nzp; iz++) {
            const double z = fabs((iz + 0.5) * dZp - (atoms[j].z - zStart) + 0 * czp);
            if (z <= rc[kind] + dZp) {
                for (int ix = 0; ix < Nxp; ix++) {
                    const double x = ((ix + 0.5) * dXp - atoms[j].x + 0 * axp) + p->potOffsetX;
                    for (int iy = 0; iy < Nyp; iy++) {
                        const double y = ((iy + 0.5) * dYp - atoms[j].y + 0 * byp) + p->potOffsetY;
                        const double rxy2 = x * x + y * y;
                        const double r = sqrt(rxy2 + z * z);
                        if (r <= rc[kind] + dZp + dXp) {
                            float *tp = trans + (size_t)iz * sliceStep + 2 * ((size_t)ix * Nyp + iy);
                            *tp = (float)((double)*tp + ft_bicubic(lut[kind], Nzl, Nxl, z / dZ + 1.0, sqrt(rxy2) / dX + 1.0));
                        }
                    }
                }
            }
        }
    }
    for (int kind = 0; kind < nkinds; kind++) free(lut[kind]);
    free(lut); free(rc); free(pot); free(atoms);
    free(t.k); free(t.f); free(t.b); free(t.c); free(t.d);
    return rc_ok;
}

/* ---------------------------------------------------------- transmission */
int qso_transmission(const qs_params *p, float *trans) {
    /* stem3/stemlib.cpp:2199-2357 */
    const int nx = p->potNx, ny = p->potNy;
    const double mm0 = (double)(1.0f + p->v0 / 511.0f);
    const double scale = mm0 * qso_wavelength(p->v0);
    const size_t n = (size_t)p->slices * nx * ny;
    for (size_t i = 0; i < n; i++) {
        double vz = trans[2 * i] * scale;
        trans[2 * i] = (float)cos(vz);
        trans[2 * i + 1] = (float)sin(vz);
    }
    if (p->bandlimittrans) {
        float *kx2 = (float *)malloc(sizeof(float) * nx);
        float *ky2 = (float *)malloc(sizeof(float) * ny);
        for (int ix = 0; ix < nx; ix++) {
            float kx = (ix > nx / 2) ? (float)(ix - nx) / p->potSizeX : (float)ix / p->potSizeX;
            kx2[ix] = kx * kx;
        }
        for (int iy = 0; iy < ny; iy++) {
            /* negative ky divided by `by`, positive by potSizeY (:2237-2238) */
            float ky = (iy > ny / 2) ? (float)(iy - ny) / p->by : (float)iy / p->potSizeY;
            ky2[iy] = ky * ky;
        }
        float k2max = nx / (2.0f * p->potSizeX);
        float t = ny / (2.0f * p->potSizeY);
        if (t < k2max) k2max = t;
        k2max = (float)((2.0f / 3.0f) * k2max);
        k2max = k2max * k2max;
        const double fftScale = 1.0 / (nx * ny);
        int dims[2] = {nx, ny};
        qs_fftnd_c64(2, dims, p->slices, (ptrdiff_t)nx * ny, trans, -1);
        for (int l = 0; l < p->slices; l++)
            for (int ix = 0; ix < nx; ix++)
                for (int iy = 0; iy < ny; iy++) {
                    float *v = trans + 2 * (((size_t)l * nx + ix) * ny + iy);
                    float k2 = ky2[iy] + kx2[ix];
                    if (k2 < k2max) {
                        v[0] = (float)(v[0] * fftScale);
                        v[1] = (float)(v[1] * fftScale);
                    } else {
                        v[0] = v[1] = 0.0f;
                    }
                }
        qs_fftnd_c64(2, dims, p->slices, (ptrdiff_t)nx * ny, trans, +1);
        free(kx2);
        free(ky2);
    }
    return QS_OK;
}

/* ----------------------------------------------------------------- probe */
int qso_probe(const qs_params *p, double dx, double dy, float *wave) {
    /* stem3/stemlib.cpp:1952-2191 */
    const int nx = p->nx, ny = p->ny;
    const double ax = (float)(nx * p->resolutionX), by = (float)(ny * p->resolutionY);
    dx = ax - dx;
    dy = by - dy;
    const double avgRes = sqrt(0.5 * (p->resolutionX * p->resolutionX + p->resolutionY * p->resolutionY));
    const double edge = 5 * avgRes; /* SMOOTH_EDGE, :1939 */
    double delta = (double)(p->Cc * p->dE_E);
    const double pi = 4.0 * atan(1.0);
    const double rx = 1.0 / ax, rx2 = rx * rx, ry = 1.0 / by, ry2 = ry * ry;
    const int ixmid = nx / 2, iymid = ny / 2;
    const double v0 = p->v0;
    const double wavlen = 12.26 / sqrt(v0 * 1.e3 + v0 * v0 * 0.9788);
    const double alpha = 0.001 * p->alpha;
    double k2max = sin(alpha) / wavlen;
    k2max = k2max * k2max;
    const double pixel = rx2 + ry2;
    double scale = 1.0 / sqrt((double)nx * (double)ny);
    for (int iy = 0; iy < ny; iy++) {
        double ky = (double)iy;
        if (iy > iymid) ky = (double)(iy - ny);
        const double ky2 = ky * ky * ry2;
        for (int ix = 0; ix < nx; ix++) {
            double kx = (double)ix;
            if (ix > ixmid) kx = (double)(ix - nx);
            const double k2 = kx * kx * rx2 + ky2;
            double ktheta2 = k2 * (wavlen * wavlen);
            const double ktheta = sqrt(ktheta2);
            const double phi = atan2(ry * ky, rx * kx);
            double chi = ktheta2 * (p->df0 + delta + p->astigMag * cos(2.0 * (phi - p->astigAngle))) / 2.0;
            ktheta2 *= ktheta;
            if ((p->a33 > 0) || (p->a31 > 0))
                chi += ktheta2 * (p->a33 * cos(3.0 * (phi - p->phi33)) + p->a31 * cos(phi - p->phi31)) / 3.0;
            ktheta2 *= ktheta;
            if ((p->a44 > 0) || (p->a42 > 0) || (p->Cs != 0))
                chi += ktheta2 * (p->a44 * cos(4.0 * (phi - p->phi44)) + p->a42 * cos(2.0 * (phi - p->phi42)) + p->Cs) / 4.0;
            ktheta2 *= ktheta;
            if ((p->a55 > 0) || (p->a53 > 0) || (p->a51 > 0))
                chi += ktheta2 * (p->a55 * cos(5.0 * (phi - p->phi55)) + p->a53 * cos(3.0 * (phi - p->phi53)) +
                                  p->a51 * cos(phi - p->phi51)) / 5.0;
            ktheta2 *= ktheta;
            /* the reference's condition assigns a62 = 0 (:2082), so the a62
             * term never contributes and the test is a66||a64||C5 */
            if ((p->a66 > 0) || (p->a64 > 0) || (p->C5 != 0))
                chi += ktheta2 * (p->a66 * cos(6.0 * (phi - p->phi66)) + p->a64 * cos(4.0 * (phi - p->phi64)) +
                                  0.0f * cos(2.0 * (phi - p->phi62)) + p->C5) / 6.0;
            chi *= 2 * pi / wavlen;
            chi -= 2.0 * pi * ((dx * kx / ax) + (dy * ky / by));
            float *w = wave + 2 * ((size_t)ix * ny + iy);
            if ((p->ismoth != 0) && (fabs(k2 - k2max) <= pixel)) {
                w[0] = (float)(0.5 * scale * cos(chi));
                w[1] = (float)(-0.5 * scale * sin(chi));
            } else if (k2 <= k2max) {
                w[0] = (float)((double)(float)scale * cos(chi));
                w[1] = (float)((double)(float)(-scale) * sin(chi));
            } else {
                w[0] = w[1] = 0.0f;
            }
        }
    }
    qs_fft2d_c64(nx, ny, wave, +1);
    if (p->gaussFlag) {
        for (int ix = 0; ix < nx; ix++)
            for (int iy = 0; iy < ny; iy++) {
                int num = (ix - nx / 2) * (ix - nx / 2) + (iy - ny / 2) * (iy - ny / 2);
                double r = expf(-(float)num / ((float)(nx * nx) * p->gaussScale));
                float *w = wave + 2 * ((size_t)ix * ny + iy);
                w[0] *= (float)r;
                w[1] *= (float)r;
            }
    }
    if (p->aAIS > 0) {
        for (int ix = 0; ix < nx; ix++)
            for (int iy = 0; iy < ny; iy++) {
                double x = (double)((float)ix * p->resolutionX) - dx;
                double y = (double)((float)iy * p->resolutionY) - dy;
                double r = sqrt(x * x + y * y);
                delta = r - 0.5 * p->aAIS + edge;
                float *w = wave + 2 * ((size_t)ix * ny + iy);
                if (delta > 0) {
                    w[0] = w[1] = 0;
                } else if (delta >= -edge) {
                    double s = 0.5 * (1 - cos(pi * delta / edge));
                    w[0] = (float)(s * w[0]);
                    w[1] = (float)(s * w[1]);
                }
            }
    }
    double sum = 0.0;
    for (size_t i = 0; i < (size_t)nx * ny; i++) sum += wave[2 * i] * wave[2 * i] + wave[2 * i + 1] * wave[2 * i + 1];
    scale = 1.0 / sum;
    scale = scale * ((double)nx) * ((double)ny);
    scale = sqrt(scale);
    for (size_t i = 0; i < 2 * (size_t)nx * ny; i++) wave[i] *= (float)scale;
    return QS_OK;
}

/* ------------------------------------------------------------ multislice */
typedef struct {
    int nx, ny;
    float *kx2, *ky2, *pxr, *pxi, *pyr, *pyi;
    float k2max;
} prop_tables;

static void prop_init(const qs_params *p, prop_tables *t) {
    /* the static tables of propagate_slow, stem3/stemlib.cpp:2783-2824 */
    const int nx = p->nx, ny = p->ny;
    t->nx = nx;
    t->ny = ny;
    t->kx2 = (float *)malloc(sizeof(float) * nx);
    t->pxr = (float *)malloc(sizeof(float) * nx);
    t->pxi = (float *)malloc(sizeof(float) * nx);
    t->ky2 = (float *)malloc(sizeof(float) * ny);
    t->pyr = (float *)malloc(sizeof(float) * ny);
    t->pyi = (float *)malloc(sizeof(float) * ny);
    const float ax = p->resolutionX * nx, by = p->resolutionY * ny;
    const float scale = (float)(p->sliceThickness * REF_PI);
    const float wavlen = (float)qso_wavelength(p->v0);
    for (int i = 0; i < nx; i++) {
        float k = (i > nx / 2) ? (float)(i - nx) / ax : (float)i / ax;
        t->kx2[i] = k * k;
        float a = scale * (t->kx2[i] * wavlen);
        t->pxr[i] = cosf(a);
        t->pxi[i] = -sinf(a);
    }
    for (int i = 0; i < ny; i++) {
        float k = (i > ny / 2) ? (float)(i - ny) / by : (float)i / by;
        t->ky2[i] = k * k;
        float a = scale * (t->ky2[i] * wavlen);
        t->pyr[i] = cosf(a);
        t->pyi[i] = -sinf(a);
    }
    float k2max = nx / (2.0f * ax);
    if (ny / (2.0f * by) < k2max) k2max = ny / (2.0f * by);
    k2max = (float)(2.0 / 3.0 * k2max);
    t->k2max = k2max * k2max;
}

static void prop_free(prop_tables *t) {
    free(t->kx2); free(t->ky2); free(t->pxr); free(t->pxi); free(t->pyr); free(t->pyi);
}

/* One runMulsSTEM call: the slices of one slab; slice0 = totalSliceCount,
 * the absolute index of its first slice (stem3/stemlib.cpp:2405). */
static void run_position(const qs_params *p, const prop_tables *pt, const float *trans, int iPosX,
                         int iPosY, float *w, float *det, float *diffpat, int slice0) {
    const int nx = p->nx, ny = p->ny, potNy = p->potNy;
    const size_t N = (size_t)nx * ny;
    const size_t sliceElems = (size_t)p->potNx * potNy;
    const int tCount = p->slices * p->cellDiv / p->outputInterval;
    const double scaleI = p->electronScale / ((double)(nx * ny) * (nx * ny));
    const double scaleDiff = 1.0 / sqrt((double)(nx * ny));
    const double fftScale = 1.0 / (double)(nx * ny);
    for (int islice = 0; islice < p->slices; islice++) {
        /* transmit, :2867-2888 */
        const float *t = trans + 2 * (size_t)islice * sliceElems;
        for (int ix = 0; ix < nx; ix++) {
            const float *trow = t + 2 * ((size_t)(ix + iPosX) * potNy + iPosY);
            float *wrow = w + 2 * (size_t)ix * ny;
            for (int iy = 0; iy < ny; iy++) {
                double wr = wrow[2 * iy], wi = wrow[2 * iy + 1];
                double tr = trow[2 * iy], ti = trow[2 * iy + 1];
                wrow[2 * iy] = (float)(wr * tr - wi * ti);
                wrow[2 * iy + 1] = (float)(wr * ti + wi * tr);
            }
        }
        qs_fft2d_c64(nx, ny, w, -1);
        /* propagate_slow, :2831-2849 */
        for (int ix = 0; ix < nx; ix++) {
            float *wrow = w + 2 * (size_t)ix * ny;
            if (pt->kx2[ix] < pt->k2max) {
                for (int iy = 0; iy < ny; iy++) {
                    if ((pt->kx2[ix] + pt->ky2[iy]) < pt->k2max) {
                        float wr = wrow[2 * iy], wi = wrow[2 * iy + 1];
                        float tr = wr * pt->pyr[iy] - wi * pt->pyi[iy];
                        float ti = wr * pt->pyi[iy] + wi * pt->pyr[iy];
                        wrow[2 * iy] = tr * pt->pxr[ix] - ti * pt->pxi[ix];
                        wrow[2 * iy + 1] = tr * pt->pxi[ix] + ti * pt->pxr[ix];
                    } else {
                        wrow[2 * iy] = wrow[2 * iy + 1] = 0.0f;
                    }
                }
            } else {
                memset(wrow, 0, sizeof(float) * 2 * ny);
            }
        }
        /* collectIntensity, :2576-2687, slice = absolute_slice */
        {
            const int aslice = slice0 + islice;
            int tt;
            if (p->outputInterval == 0) tt = 0;
            else if (aslice < p->slices * p->cellDiv - 1) tt = aslice / p->outputInterval;
            else tt = tCount;
            float img[QS_MAX_DETECTORS], err[QS_MAX_DETECTORS];
            for (int i = 0; i < p->detectorNum; i++) img[i] = err[i] = 0.0f;
            for (int ix = 0; ix < nx; ix++)
                for (int iy = 0; iy < ny; iy++) {
                    const float k2 = pt->kx2[ix] + pt->ky2[iy];
                    const float *v = w + 2 * ((size_t)ix * ny + iy);
                    double intensity = (double)(v[0] * v[0] + v[1] * v[1]);
                    if (diffpat)
                        diffpat[(size_t)((ix + nx / 2) % nx) * ny + (iy + ny / 2) % ny] = (float)(intensity * scaleDiff);
                    intensity *= scaleI;
                    for (int i = 0; i < p->detectorNum; i++) {
                        const qs_detector *d = &p->detectors[i];
                        if ((k2 >= d->k2Inside) && (k2 <= d->k2Outside)) {
                            if (d->shiftX == 0 && d->shiftY == 0) {
                                img[i] = (float)((double)img[i] + intensity);
                                err[i] = (float)((double)err[i] + intensity);
                            } else {
                                int ixs = (ix + (int)d->shiftX + nx) % nx;
                                int iys = (iy + (int)d->shiftY + ny) % ny;
                                const float *u = w + 2 * ((size_t)ixs * ny + iys);
                                double is = scaleI * (double)(u[0] * u[0] + u[1] * u[1]);
                                img[i] = (float)((double)img[i] + is);
                                err[i] = (float)((double)err[i] + is);
                            }
                        }
                    }
                }
            if (det)
                for (int i = 0; i < p->detectorNum; i++) det[tt * p->detectorNum + i] = img[i];
        }
        qs_fft2d_c64(nx, ny, w, +1);
        for (size_t i = 0; i < 2 * N; i++) w[i] = (float)(w[i] * fftScale);
    }
}

int qso_run_position(const qs_params *p, const float *trans, int iPosX, int iPosY, float *wave,
                     float *det, float *diffpat) {
    prop_tables pt;
    prop_init(p, &pt);
    run_position(p, &pt, trans, iPosX, iPosY, wave, det, diffpat, 0);
    prop_free(&pt);
    return QS_OK;
}

void qso_scan_offsets(const qs_params *p, int ix, int iy, int *iPosX, int *iPosY) {
    /* stem3/stem3.cpp:2860-2871: float arithmetic, truncation, clamp */
    int x = (int)((float)ix * (p->scanXStop - p->scanXStart) / ((float)p->scanXN * p->resolutionX));
    int y = (int)((float)iy * (p->scanYStop - p->scanYStart) / ((float)p->scanYN * p->resolutionY));
    if (x > p->potNx - p->nx) x = p->potNx - p->nx;
    if (y > p->potNy - p->ny) y = p->potNy - p->ny;
    *iPosX = x;
    *iPosY = y;
}

int qso_stem(const qs_params *p, const float *trans, const float *probe_in, int p0, int p1,
             float *det_images, float *diffpats, float *exit_waves, int nthreads) {
    return qso_stem_slabs(p, trans, 0, probe_in, p0, p1, det_images, diffpats, exit_waves, nthreads);
}

/* doSTEM's slab loop (stem3/stem3.cpp:2795-2949): cellDiv runMulsSTEM calls
 * per position, the wave carried from one slab to the next (through
 * mulswav files in the reference), totalSliceCount advancing by slices.
 * trans: one stack reused for every slab (equal divisions), or with
 * slab_stacks cellDiv stacks back to back. */
int qso_stem_slabs(const qs_params *p, const float *trans, int slab_stacks, const float *probe_in, int p0,
                   int p1, float *det_images, float *diffpats, float *exit_waves, int nthreads) {
    const size_t stackFloats = 2 * (size_t)p->slices * p->potNx * p->potNy;
    const int nx = p->nx, ny = p->ny;
    const size_t N = (size_t)nx * ny;
    const int nt = qso_thickness_count(p);
    const int ndet = p->detectorNum;
    const int npix = p->scanXN * p->scanYN;
    float *probe = (float *)malloc(sizeof(float) * 2 * N);
    if (probe_in) memcpy(probe, probe_in, sizeof(float) * 2 * N);
    else qso_probe(p, nx / 2 * p->resolutionX, ny / 2 * p->resolutionY, probe);
    prop_tables pt;
    prop_init(p, &pt);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        float *w = (float *)malloc(sizeof(float) * 2 * N);
        float *det = (float *)malloc(sizeof(float) * (size_t)nt * (ndet > 0 ? ndet : 1));
#pragma omp for schedule(dynamic, 1)
        for (int pos = p0; pos < p1; pos++) {
            const int ix = pos / p->scanYN, iy = pos % p->scanYN;
            int iPosX, iPosY;
            qso_scan_offsets(p, ix, iy, &iPosX, &iPosY);
            memcpy(w, probe, sizeof(float) * 2 * N);
            memset(det, 0, sizeof(float) * (size_t)nt * (ndet > 0 ? ndet : 1));
            float *dp = diffpats ? diffpats + (size_t)(pos - p0) * N : NULL;
            for (int k = 0; k < p->cellDiv; k++)
                run_position(p, &pt, trans + (slab_stacks ? stackFloats * k : 0), iPosX, iPosY, w, det, dp,
                             k * p->slices);
            if (det_images)
                for (int t = 0; t < nt; t++)
                    for (int i = 0; i < ndet; i++)
                        det_images[((size_t)t * ndet + i) * npix + (size_t)ix * p->scanYN + iy] = det[t * ndet + i];
            if (exit_waves) memcpy(exit_waves + 2 * (size_t)(pos - p0) * N, w, sizeof(float) * 2 * N);
        }
        free(w);
        free(det);
    }
    prop_free(&pt);
    free(probe);
    return QS_OK;
}
