/*
 * fftw_shim.c -- the eleven FFTW3 entry points that the reference CPU path
 * links against, implemented over qs_fft.c.
 *
 * TEST INFRASTRUCTURE ONLY.  No Linux libfftw3f exists on the build machine,
 * so the reference (FFTW 3, single precision; call sites listed in
 * qs_fft.h) is linked against this shim to run as the oracle.  The behaviour
 * follows FFTW's documented interface (unnormalised, FFTW_FORWARD = -1,
 * row-major, plan_many_dft with unit stride and contiguous embedding, the
 * new-array execute).  Internally the transforms run in double precision, so
 * outputs differ from real FFTW by rounding only; every number produced with
 * it is labelled "reference + project FFT shim (not FFTW)".
 *
 * The plan records its precision, so a float plan handed to fftw_execute
 * (which the reference does in its TEM path, stem3/stem3.cpp:2648) still
 * transforms the float array it was planned for.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "qs_fft.h"

typedef struct qs_shim_plan {
    int is_double;
    int rank;
    int dims[3];
    int howmany;
    ptrdiff_t dist;
    void *in;
    void *out;
    int sign;
} qs_shim_plan;

static size_t plan_total(const qs_shim_plan *p) {
    size_t t = 1;
    for (int d = 0; d < p->rank; d++) t *= (size_t)p->dims[d];
    return t;
}

static void run(const qs_shim_plan *p, void *in, void *out) {
    size_t elem = p->is_double ? 2 * sizeof(double) : 2 * sizeof(float);
    size_t span = (size_t)(p->howmany - 1) * (size_t)p->dist + plan_total(p);
    if (in != out) memmove(out, in, span * elem);
    if (p->is_double)
        qs_fftnd_c128(p->rank, p->dims, p->howmany, p->dist, (double *)out, p->sign);
    else
        qs_fftnd_c64(p->rank, p->dims, p->howmany, p->dist, (float *)out, p->sign);
}

static qs_shim_plan *mk(int is_double, int rank, const int *n, int howmany, ptrdiff_t dist,
                        void *in, void *out, int sign) {
    qs_shim_plan *p = (qs_shim_plan *)calloc(1, sizeof(qs_shim_plan));
    p->is_double = is_double;
    p->rank = rank;
    for (int d = 0; d < rank; d++) p->dims[d] = n[d];
    p->howmany = howmany;
    p->dist = dist;
    p->in = in;
    p->out = out;
    p->sign = sign;
    return p;
}

void *fftwf_malloc(size_t n) {
    void *p = NULL;
    if (posix_memalign(&p, 64, n ? n : 1) != 0) return NULL;
    return p;
}
void *fftw_malloc(size_t n) { return fftwf_malloc(n); }
void fftwf_free(void *p) { free(p); }
void fftw_free(void *p) { free(p); }

void *fftwf_plan_dft_2d(int n0, int n1, void *in, void *out, int sign, unsigned flags) {
    int n[2] = {n0, n1};
    (void)flags;
    return mk(0, 2, n, 1, 0, in, out, sign);
}

void *fftwf_plan_dft_3d(int n0, int n1, int n2, void *in, void *out, int sign, unsigned flags) {
    int n[3] = {n0, n1, n2};
    (void)flags;
    return mk(0, 3, n, 1, 0, in, out, sign);
}

void *fftwf_plan_many_dft(int rank, const int *n, int howmany, void *in, const int *inembed,
                          int istride, int idist, void *out, const int *onembed, int ostride,
                          int odist, int sign, unsigned flags) {
    (void)flags;
    if (rank < 1 || rank > 3 || istride != 1 || ostride != 1 || idist != odist ||
        (inembed && inembed != n) || (onembed && onembed != n)) {
        fprintf(stderr, "fftw shim: unsupported plan_many_dft layout\n");
        abort();
    }
    return mk(0, rank, n, howmany, idist, in, out, sign);
}

void fftwf_execute(const void *plan) {
    const qs_shim_plan *p = (const qs_shim_plan *)plan;
    run(p, p->in, p->out);
}

void fftwf_execute_dft(const void *plan, void *in, void *out) {
    run((const qs_shim_plan *)plan, in, out);
}

void fftwf_destroy_plan(void *plan) { free(plan); }

void *fftw_plan_dft_2d(int n0, int n1, void *in, void *out, int sign, unsigned flags) {
    int n[2] = {n0, n1};
    (void)flags;
    return mk(1, 2, n, 1, 0, in, out, sign);
}

void fftw_execute(const void *plan) { fftwf_execute(plan); }

void fftw_destroy_plan(void *plan) { free(plan); }
