/*
 * qs_oracle.h -- C restatement of QSTEM's multislice hot path (CPU).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library and the "port"
 * CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference arm call it.  Parity of this restatement with the
 * reference itself is pinned by tests/test_oracle_golden.py against fixtures
 * produced by the reference compiled from its sources (oracle/Makefile ref).
 *
 * Each function follows the cited reference function; float vs double
 * arithmetic follows the reference's declared types (MULS float_tt fields,
 * fftwf single-precision storage) so that results agree to rounding.
 */
#ifndef QS_ORACLE_H
#define QS_ORACLE_H

#include "../include/qstem_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* stem3/stemutil.cpp:714-725 */
double qso_wavelength(double kev);

/* stem3/stemutil.cpp:975-1041 (Akima spline) and :1069-1092 (evaluation) */
void qso_splinh(const double *x, const double *y, double *b, double *c, double *d, int n);
double qso_seval(const double *x, const double *y, const double *b, const double *c,
                 const double *d, int n, double x0);

/* getAtomPotential3D (charged=0, stem3/stemlib.cpp:1342-1541) or
 * getAtomPotentialOffset3D (charged=1, :1548-1741).  Writes Nz_lut*Nr floats
 * (real parts) into out when out != NULL. */
int qso_lut(const qs_params *p, int Znum, double B, int charged, float *out, int *Nz_lut,
            int *Nr, int *nzSub);

/* make3DSlices, default branch (fftpotential, potential3D; periodic and
 * non-periodic in x-y), stem3/stemlib.cpp:383-681, :884-1036, :1090-1213.
 * trans: slices*potNx*potNy c64, overwritten with V in .re and 0 in .im.
 * atoms is not modified (a sorted copy is used). */
int qso_potential(const qs_params *p, const qs_atom *atoms, int natom, float *trans);
/* make3DSlicesFT with a custom scattering-factor table: k[nk], f[kind][nk]
 * for the elements Zs[kind] */
int qso_potential_ft(const qs_params *p, const qs_atom *atoms, int natom, const double *k, int nk,
                     const int *Zs, const double *sf, int nkinds, float *trans);
/* getAtomPotential2D: nx x ny complex floats (out NULL: sizes only) */
int qso_lut2d(const qs_params *p, int Znum, double B, float *out, int *nx, int *ny);
/* the same for slab `slab` of a cell divided into cellDiv slabs along z */
int qso_potential_slab(const qs_params *p, const qs_atom *atoms, int natom, int slab, float *trans);

/* initSTEMSlices, stem3/stemlib.cpp:2199-2357: V -> exp(i lambda gamma V),
 * band limit when p->bandlimittrans. */
int qso_transmission(const qs_params *p, float *trans);

/* probe, stem3/stemlib.cpp:1952-2191. */
int qso_probe(const qs_params *p, double dx, double dy, float *wave);

/* runMulsSTEM for one position (stem3/stemlib.cpp:2375-2534) including
 * transmit (:2867), propagate_slow (:2760), collectIntensity (:2576) and
 * fft_normalize (:2890).  wave: nx*ny c64, in/out.  det: [tCount+1][ndet]
 * float detector values, overwritten per collectIntensity semantics (may be
 * NULL).  diffpat: nx*ny float of the last slice (may be NULL). */
int qso_run_position(const qs_params *p, const float *trans, int iPosX, int iPosY, float *wave,
                     float *det, float *diffpat);

/* The doSTEM position loop (stem3/stem3.cpp:2820-2946) for positions
 * [p0, p1) of the raster p = ix*scanYN + iy, OpenMP over positions.
 * det_images: [tCount+1][ndet][scanXN][scanYN] (may be NULL);
 * diffpats/exit_waves: per position in [p0,p1) (may be NULL). */
/* doSTEM's slab loop over cellDiv slabs; trans holds cellDiv stacks when
 * slab_stacks, else one stack reused for every slab. */
int qso_stem_slabs(const qs_params *p, const float *trans, int slab_stacks, const float *probe, int p0, int p1,
                   float *det_images, float *diffpats, float *exit_waves, int nthreads);
int qso_stem(const qs_params *p, const float *trans, const float *probe, int p0, int p1,
             float *det_images, float *diffpats, float *exit_waves, int nthreads);

/* iPosX/iPosY of raster index (ix, iy) as doSTEM computes them. */
void qso_scan_offsets(const qs_params *p, int ix, int iy, int *iPosX, int *iPosY);

/* detector k2 bounds (stem3/stem3.cpp:1343-1350) */
void qso_params_finalize(qs_params *p);
int qso_thickness_count(const qs_params *p);

#ifdef __cplusplus
}
#endif
#endif
