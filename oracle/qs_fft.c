/*
 * qs_fft.c -- CPU discrete Fourier transforms (double precision internally).
 *
 * TEST INFRASTRUCTURE ONLY: arithmetic for the FFTW entry-point shim that
 * links the reference CPU path, and for the C restatement in qs_oracle.c.
 *
 * Written from the mathematics of the DFT:
 *   - mixed-radix self-sorting (Stockham) passes: at the pass with radix R
 *     after radices whose product is Ns, butterfly j reads the R inputs
 *     in[j + r*n/R], multiplies input r by exp(s*2*pi*i*r*(j mod Ns)/(Ns*R)),
 *     applies an R-point DFT and writes out[(j/Ns)*Ns*R + (j mod Ns) + r*Ns];
 *   - Bluestein: jk = (j^2 + k^2 - (k-j)^2)/2 turns a length-n DFT into a
 *     cyclic convolution of length m >= 2n-1 (a power of two).
 */
#include "qs_fft.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define QS_MAX_STAGES 40
#define QS_GENERIC_MAX 61
#define QS_TWO_PI 6.283185307179586476925286766559

struct qs_fft1d {
    int n;
    int nstages;
    int radix[QS_MAX_STAGES];
    int ns[QS_MAX_STAGES];
    double *tw[QS_MAX_STAGES];   /* Ns*(R-1) complex, forward sign */
    double *roots[QS_MAX_STAGES];/* R complex roots exp(-2 pi i q/R) (generic radix) */
    /* Bluestein */
    int blue;
    int m;
    qs_fft1d *sub;
    double *chirp;   /* n complex: exp(-i pi (j^2 mod 2n)/n) */
    double *bhat_f;  /* m complex: DFT_m of b for the forward sign */
    double *bhat_b;  /* m complex: DFT_m of b for the backward sign */
};

static void cis(double turns_num, double turns_den, double *re, double *im) {
    /* exp(-2 pi i num/den) with the angle reduced to [-pi, pi] first */
    double a = turns_num / turns_den;
    a -= floor(a + 0.5);
    double ang = -QS_TWO_PI * a;
    *re = cos(ang);
    *im = sin(ang);
}

static int next_pow2(int v) {
    int m = 1;
    while (m < v) m <<= 1;
    return m;
}

static int factorize(int n, int *radix, int *count) {
    int k = 0;
    while (n % 4 == 0 && n > 4) { radix[k++] = 4; n /= 4; }
    while (n % 2 == 0) { radix[k++] = 2; n /= 2; }
    while (n % 4 == 0) { radix[k++] = 4; n /= 4; }
    for (int p = 3; p <= QS_GENERIC_MAX && n > 1; p += 2) {
        while (n % p == 0) { radix[k++] = p; n /= p; }
    }
    *count = k;
    return n; /* leftover (1 when fully factored) */
}

qs_fft1d *qs_fft1d_create(int n) {
    if (n < 1) return NULL;
    qs_fft1d *p = (qs_fft1d *)calloc(1, sizeof(qs_fft1d));
    p->n = n;
    int cnt = 0;
    int left = factorize(n, p->radix, &cnt);
    if (left != 1) {
        /* Bluestein */
        p->blue = 1;
        p->m = next_pow2(2 * n - 1);
        p->sub = qs_fft1d_create(p->m);
        p->chirp = (double *)malloc(sizeof(double) * 2 * n);
        for (int j = 0; j < n; j++) {
            long long q = ((long long)j * j) % (2LL * n);
            /* exp(-i pi q/n) = exp(-2 pi i q/(2n)) */
            cis((double)q, 2.0 * n, &p->chirp[2 * j], &p->chirp[2 * j + 1]);
        }
        int m = p->m;
        p->bhat_f = (double *)calloc(2 * (size_t)m, sizeof(double));
        p->bhat_b = (double *)calloc(2 * (size_t)m, sizeof(double));
        /* forward sign: c_j = chirp_j, b_t = conj(c_t) for |t| < n */
        for (int t = 0; t < n; t++) {
            double re = p->chirp[2 * t], im = -p->chirp[2 * t + 1];
            p->bhat_f[2 * t] = re; p->bhat_f[2 * t + 1] = im;
            p->bhat_b[2 * t] = re; p->bhat_b[2 * t + 1] = -im;
            if (t > 0) {
                p->bhat_f[2 * (m - t)] = re; p->bhat_f[2 * (m - t) + 1] = im;
                p->bhat_b[2 * (m - t)] = re; p->bhat_b[2 * (m - t) + 1] = -im;
            }
        }
        double *w = (double *)malloc(sizeof(double) * qs_fft1d_work_doubles(p->sub));
        qs_fft1d_exec(p->sub, p->bhat_f, -1, w);
        qs_fft1d_exec(p->sub, p->bhat_b, -1, w);
        free(w);
        return p;
    }
    p->nstages = cnt;
    int ns = 1;
    for (int s = 0; s < cnt; s++) {
        int R = p->radix[s];
        p->ns[s] = ns;
        p->tw[s] = (double *)malloc(sizeof(double) * 2 * (size_t)ns * (R - 1) + 16);
        for (int jm = 0; jm < ns; jm++)
            for (int r = 1; r < R; r++) {
                double *t = &p->tw[s][2 * ((size_t)jm * (R - 1) + (r - 1))];
                cis((double)((long long)r * jm), (double)ns * R, &t[0], &t[1]);
            }
        if (R != 2 && R != 3 && R != 4) {
            p->roots[s] = (double *)malloc(sizeof(double) * 2 * R);
            for (int q = 0; q < R; q++) cis((double)q, (double)R, &p->roots[s][2 * q], &p->roots[s][2 * q + 1]);
        }
        ns *= R;
    }
    return p;
}

void qs_fft1d_destroy(qs_fft1d *p) {
    if (!p) return;
    for (int s = 0; s < p->nstages; s++) { free(p->tw[s]); free(p->roots[s]); }
    if (p->blue) {
        qs_fft1d_destroy(p->sub);
        free(p->chirp); free(p->bhat_f); free(p->bhat_b);
    }
    free(p);
}

int qs_fft1d_len(const qs_fft1d *p) { return p->n; }

size_t qs_fft1d_work_doubles(const qs_fft1d *p) {
    if (p->blue) return 2 * (size_t)p->m + qs_fft1d_work_doubles(p->sub);
    return 2 * (size_t)p->n + 2 * QS_GENERIC_MAX;
}

/* One Stockham pass. */
static void stockham_pass(const qs_fft1d *p, int s, const double *in, double *out, int sign,
                          double *v) {
    const int n = p->n, R = p->radix[s], Ns = p->ns[s];
    const int stride = n / R;
    const double *tw = p->tw[s];
    const double sg = (double)sign; /* sign of the exponent: -1 forward */
    for (int j = 0; j < stride; j++) {
        const int jm = j % Ns;
        const double *t = tw + 2 * (size_t)jm * (R - 1);
        v[0] = in[2 * j];
        v[1] = in[2 * j + 1];
        for (int r = 1; r < R; r++) {
            double xr = in[2 * (j + r * stride)], xi = in[2 * (j + r * stride) + 1];
            double wr = t[2 * (r - 1)], wi = -sg * t[2 * (r - 1) + 1];
            v[2 * r] = xr * wr - xi * wi;
            v[2 * r + 1] = xr * wi + xi * wr;
        }
        const int idxD = (j / Ns) * Ns * R + jm;
        if (R == 2) {
            out[2 * idxD] = v[0] + v[2];
            out[2 * idxD + 1] = v[1] + v[3];
            out[2 * (idxD + Ns)] = v[0] - v[2];
            out[2 * (idxD + Ns) + 1] = v[1] - v[3];
        } else if (R == 4) {
            double t0r = v[0] + v[4], t0i = v[1] + v[5];
            double t1r = v[0] - v[4], t1i = v[1] - v[5];
            double t2r = v[2] + v[6], t2i = v[3] + v[7];
            double dr = v[2] - v[6], di = v[3] - v[7];
            /* t3 = (s i) * d */
            double t3r = -sg * di, t3i = sg * dr;
            out[2 * idxD] = t0r + t2r;
            out[2 * idxD + 1] = t0i + t2i;
            out[2 * (idxD + Ns)] = t1r + t3r;
            out[2 * (idxD + Ns) + 1] = t1i + t3i;
            out[2 * (idxD + 2 * Ns)] = t0r - t2r;
            out[2 * (idxD + 2 * Ns) + 1] = t0i - t2i;
            out[2 * (idxD + 3 * Ns)] = t1r - t3r;
            out[2 * (idxD + 3 * Ns) + 1] = t1i - t3i;
        } else if (R == 3) {
            const double h = 0.86602540378443864676372317075294; /* sqrt(3)/2 */
            double t1r = v[2] + v[4], t1i = v[3] + v[5];
            double t2r = v[2] - v[4], t2i = v[3] - v[5];
            double mr = v[0] - 0.5 * t1r, mi = v[1] - 0.5 * t1i;
            /* n = (s*h) * i * t2 */
            double nr = -sg * h * t2i, ni = sg * h * t2r;
            out[2 * idxD] = v[0] + t1r;
            out[2 * idxD + 1] = v[1] + t1i;
            out[2 * (idxD + Ns)] = mr + nr;
            out[2 * (idxD + Ns) + 1] = mi + ni;
            out[2 * (idxD + 2 * Ns)] = mr - nr;
            out[2 * (idxD + 2 * Ns) + 1] = mi - ni;
        } else {
            const double *rt = p->roots[s];
            for (int k = 0; k < R; k++) {
                double ar = 0, ai = 0;
                for (int r = 0; r < R; r++) {
                    int q = (int)(((long long)r * k) % R);
                    double wr = rt[2 * q], wi = -sg * rt[2 * q + 1];
                    ar += v[2 * r] * wr - v[2 * r + 1] * wi;
                    ai += v[2 * r] * wi + v[2 * r + 1] * wr;
                }
                out[2 * (idxD + k * Ns)] = ar;
                out[2 * (idxD + k * Ns) + 1] = ai;
            }
        }
    }
}

void qs_fft1d_exec(const qs_fft1d *p, double *x, int sign, double *work) {
    double *own = NULL;
    if (!work) {
        own = (double *)malloc(sizeof(double) * qs_fft1d_work_doubles(p));
        work = own;
    }
    const int n = p->n;
    if (p->blue) {
        const int m = p->m;
        double *a = work;
        double *subw = work + 2 * (size_t)m;
        const double sg = (double)sign;
        for (int j = 0; j < n; j++) {
            double cr = p->chirp[2 * j], ci = -sg * p->chirp[2 * j + 1];
            double xr = x[2 * j], xi = x[2 * j + 1];
            a[2 * j] = xr * cr - xi * ci;
            a[2 * j + 1] = xr * ci + xi * cr;
        }
        memset(a + 2 * (size_t)n, 0, sizeof(double) * 2 * (size_t)(m - n));
        qs_fft1d_exec(p->sub, a, -1, subw);
        const double *bh = (sign < 0) ? p->bhat_f : p->bhat_b;
        for (int k = 0; k < m; k++) {
            double ar = a[2 * k], ai = a[2 * k + 1];
            double br = bh[2 * k], bi = bh[2 * k + 1];
            a[2 * k] = ar * br - ai * bi;
            a[2 * k + 1] = ar * bi + ai * br;
        }
        qs_fft1d_exec(p->sub, a, +1, subw);
        const double inv = 1.0 / (double)m;
        for (int k = 0; k < n; k++) {
            double cr = p->chirp[2 * k], ci = -sg * p->chirp[2 * k + 1];
            double ar = a[2 * k] * inv, ai = a[2 * k + 1] * inv;
            x[2 * k] = ar * cr - ai * ci;
            x[2 * k + 1] = ar * ci + ai * cr;
        }
    } else if (p->nstages > 0) {
        double *buf = work;
        double *v = work + 2 * (size_t)n;
        double *src = x, *dst = buf;
        for (int s = 0; s < p->nstages; s++) {
            stockham_pass(p, s, src, dst, sign, v);
            double *t = src; src = dst; dst = t;
        }
        if (src != x) memcpy(x, src, sizeof(double) * 2 * (size_t)n);
    }
    free(own);
}

/* ---------------------------------------------------------------- cache */
#define QS_CACHE_MAX 256
static struct { int n; qs_fft1d *p; } g_cache[QS_CACHE_MAX];
static int g_cache_n = 0;
static pthread_mutex_t g_cache_mu = PTHREAD_MUTEX_INITIALIZER;

const qs_fft1d *qs_fft1d_get(int n) {
    pthread_mutex_lock(&g_cache_mu);
    for (int i = 0; i < g_cache_n; i++)
        if (g_cache[i].n == n) {
            qs_fft1d *p = g_cache[i].p;
            pthread_mutex_unlock(&g_cache_mu);
            return p;
        }
    qs_fft1d *p = qs_fft1d_create(n);
    if (g_cache_n < QS_CACHE_MAX) {
        g_cache[g_cache_n].n = n;
        g_cache[g_cache_n].p = p;
        g_cache_n++;
    }
    pthread_mutex_unlock(&g_cache_mu);
    return p;
}

/* ------------------------------------------------------------ n-d layer */
#define QS_BLOCK 8

static void fft_axis(double *data, int outer, int len, ptrdiff_t inner, int sign) {
    const qs_fft1d *p = qs_fft1d_get(len);
    size_t wd = qs_fft1d_work_doubles(p);
    double *work = (double *)malloc(sizeof(double) * wd);
    if (inner == 1) {
        for (int o = 0; o < outer; o++) qs_fft1d_exec(p, data + 2 * (size_t)o * len, sign, work);
        free(work);
        return;
    }
    double *buf = (double *)malloc(sizeof(double) * 2 * (size_t)len * QS_BLOCK);
    for (int o = 0; o < outer; o++) {
        double *base = data + 2 * (size_t)o * len * inner;
        for (ptrdiff_t s0 = 0; s0 < inner; s0 += QS_BLOCK) {
            int b = (int)((inner - s0) < QS_BLOCK ? (inner - s0) : QS_BLOCK);
            for (int l = 0; l < len; l++) {
                const double *src = base + 2 * ((size_t)l * inner + s0);
                for (int q = 0; q < b; q++) {
                    buf[2 * ((size_t)q * len + l)] = src[2 * q];
                    buf[2 * ((size_t)q * len + l) + 1] = src[2 * q + 1];
                }
            }
            for (int q = 0; q < b; q++) qs_fft1d_exec(p, buf + 2 * (size_t)q * len, sign, work);
            for (int l = 0; l < len; l++) {
                double *dst = base + 2 * ((size_t)l * inner + s0);
                for (int q = 0; q < b; q++) {
                    dst[2 * q] = buf[2 * ((size_t)q * len + l)];
                    dst[2 * q + 1] = buf[2 * ((size_t)q * len + l) + 1];
                }
            }
        }
    }
    free(buf);
    free(work);
}

void qs_fftnd_c128(int rank, const int *dims, int howmany, ptrdiff_t dist, double *data, int sign) {
    size_t total = 1;
    for (int d = 0; d < rank; d++) total *= (size_t)dims[d];
    for (int h = 0; h < howmany; h++) {
        double *x = data + 2 * (size_t)h * dist;
        for (int d = 0; d < rank; d++) {
            int outer = 1;
            ptrdiff_t inner = 1;
            for (int e = 0; e < d; e++) outer *= dims[e];
            for (int e = d + 1; e < rank; e++) inner *= dims[e];
            fft_axis(x, outer, dims[d], inner, sign);
        }
    }
    (void)total;
}

void qs_fftnd_c64(int rank, const int *dims, int howmany, ptrdiff_t dist, float *data, int sign) {
    size_t total = 1;
    for (int d = 0; d < rank; d++) total *= (size_t)dims[d];
    double *tmp = (double *)malloc(sizeof(double) * 2 * total);
    for (int h = 0; h < howmany; h++) {
        float *x = data + 2 * (size_t)h * dist;
        for (size_t i = 0; i < 2 * total; i++) tmp[i] = (double)x[i];
        qs_fftnd_c128(rank, dims, 1, 0, tmp, sign);
        for (size_t i = 0; i < 2 * total; i++) x[i] = (float)tmp[i];
    }
    free(tmp);
}

void qs_fft2d_c64(int n0, int n1, float *data, int sign) {
    int dims[2] = {n0, n1};
    qs_fftnd_c64(2, dims, 1, 0, data, sign);
}
