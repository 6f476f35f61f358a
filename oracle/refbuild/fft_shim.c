/* FFTW3f subset for the reference build -- TEST INFRASTRUCTURE ONLY.
 *
 * Implements the calls declared in shim/fftw3.h with the discrete Fourier
 * transform's definition X_k = sum_j x_j exp(sign 2 pi i jk/n) (unnormalised),
 * evaluated by a mixed-radix Cooley-Tukey decimation in time (radix 4, 2, 3,
 * 5 butterflies, any other prime factor by its direct DFT) in double
 * precision with twiddles exp(sign 2 pi i t/n) tabulated in double.  Inputs
 * are read as float, each whole 2-D transform runs in double and the result
 * is rounded to float once -- at least as accurate as FFTW's single
 * precision (whose last-bit results depend on the plan FFTW_MEASURE picks).
 * Plans are immutable after creation; execution uses per-thread scratch, so
 * one plan may run on different arrays from many threads at once, which is
 * how the reference's worker threads use theirs.  No FFTW source is used.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

typedef double _Complex cplx;

enum { KIND_C2C = 0, KIND_R2C = 1, KIND_C2R = 2, KIND_R2R = 3 };
enum { MAXFAC = 32 };

typedef struct {
    int n;
    int nfac;
    int fac[MAXFAC];
    cplx *tw; /* tw[t] = exp(sign 2 pi i t / n), t < n */
} fft1d;

struct refshim_fft_plan {
    int kind, n0, n1, sign;
    fftwf_r2r_kind k0, k1;
    fft1d f0, f1;   /* sign of the transform (c2c, r2c: -1; c2r: +1) */
    fft1d b0, b1;   /* r2r: forward (-1) and backward (+1) tables */
};

static void fft1d_init(fft1d *f, int n, int sign) {
    f->n = n;
    f->nfac = 0;
    int r = n;
    static const int pref[] = {4, 2, 3, 5};
    for (int q = 0; q < 4; q++)
        while (r % pref[q] == 0 && r > 1) {
            f->fac[f->nfac++] = pref[q];
            r /= pref[q];
        }
    for (int d = 7; r > 1; d += 2)
        while (r % d == 0) {
            f->fac[f->nfac++] = d;
            r /= d;
        }
    if (f->nfac == 0) f->fac[f->nfac++] = 1;
    f->tw = (cplx *)malloc(sizeof(cplx) * (size_t)(n > 0 ? n : 1));
    for (int t = 0; t < n; t++) {
        double a = sign * 2.0 * M_PI * (double)t / (double)n;
        f->tw[t] = cos(a) + I * sin(a);
    }
}

static void fft1d_free(fft1d *f) {
    free(f->tw);
    f->tw = NULL;
}

/* out[0..n) = DFT of in[0], in[s], in[2s], ...; `tws` = table stride (N/n). */
static void fft_rec(const cplx *in, size_t s, cplx *out, int n, const int *fac, const fft1d *f,
                    int tws) {
    int r = fac[0];
    int m = n / r;
    if (m == 1) {
        for (int q = 0; q < r; q++) out[q] = in[(size_t)q * s];
    } else {
        for (int q = 0; q < r; q++) fft_rec(in + (size_t)q * s, s * r, out + q * m, m, fac + 1, f, tws * r);
    }
    const cplx *tw = f->tw;
    int N = f->n;
    cplx t[64];
    for (int k = 0; k < m; k++) {
        /* twiddled inputs of this butterfly: out[q*m+k] * w_n^{qk} */
        for (int q = 0; q < r; q++) t[q] = q == 0 ? out[k] : out[q * m + k] * tw[(size_t)q * k * tws % N];
        if (r == 2) {
            out[k] = t[0] + t[1];
            out[m + k] = t[0] - t[1];
        } else if (r == 4) {
            cplx w4 = tw[(size_t)(N / 4)]; /* exp(sign i pi/2) = sign * i */
            cplx a = t[0] + t[2], b = t[0] - t[2], c = t[1] + t[3], d = (t[1] - t[3]) * w4;
            out[k] = a + c;
            out[m + k] = b + d;
            out[2 * m + k] = a - c;
            out[3 * m + k] = b - d;
        } else {
            /* direct DFT of length r: X_s = sum_q t_q w_r^{qs} */
            int step = N / r;
            for (int sidx = 0; sidx < r; sidx++) {
                cplx acc = t[0];
                for (int q = 1; q < r; q++) acc += t[q] * tw[(size_t)((q * sidx) % r) * step];
                out[sidx * m + k] = acc;
            }
        }
    }
}

static void fft1d_exec(const fft1d *f, const cplx *in, size_t stride, cplx *out) {
    if (f->n == 1) {
        out[0] = in[0];
        return;
    }
    fft_rec(in, stride, out, f->n, f->fac, f, 1);
}

/* per-thread scratch */
static __thread cplx *g_scr = NULL;
static __thread size_t g_scr_n = 0;

static cplx *scratch(size_t n) {
    if (n > g_scr_n) {
        free(g_scr);
        g_scr = (cplx *)malloc(sizeof(cplx) * n);
        g_scr_n = n;
    }
    return g_scr;
}

static fftwf_plan new_plan(int kind, int n0, int n1) {
    fftwf_plan p = (fftwf_plan)calloc(1, sizeof(*p));
    p->kind = kind;
    p->n0 = n0;
    p->n1 = n1;
    return p;
}

fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out, int sign,
                             unsigned flags) {
    (void)in, (void)out, (void)flags;
    fftwf_plan p = new_plan(KIND_C2C, n0, n1);
    p->sign = sign;
    fft1d_init(&p->f0, n0, sign);
    fft1d_init(&p->f1, n1, sign);
    return p;
}

fftwf_plan fftwf_plan_dft_r2c_2d(int n0, int n1, float *in, fftwf_complex *out, unsigned flags) {
    (void)in, (void)out, (void)flags;
    fftwf_plan p = new_plan(KIND_R2C, n0, n1);
    p->sign = FFTW_FORWARD;
    fft1d_init(&p->f0, n0, FFTW_FORWARD);
    fft1d_init(&p->f1, n1, FFTW_FORWARD);
    return p;
}

fftwf_plan fftwf_plan_dft_c2r_2d(int n0, int n1, fftwf_complex *in, float *out, unsigned flags) {
    (void)in, (void)out, (void)flags;
    fftwf_plan p = new_plan(KIND_C2R, n0, n1);
    p->sign = FFTW_BACKWARD;
    fft1d_init(&p->f0, n0, FFTW_BACKWARD);
    fft1d_init(&p->f1, n1, FFTW_BACKWARD);
    return p;
}

fftwf_plan fftwf_plan_r2r_2d(int n0, int n1, float *in, float *out, fftwf_r2r_kind kind0,
                             fftwf_r2r_kind kind1, unsigned flags) {
    (void)in, (void)out, (void)flags;
    fftwf_plan p = new_plan(KIND_R2R, n0, n1);
    p->k0 = kind0;
    p->k1 = kind1;
    fft1d_init(&p->f0, n0, FFTW_FORWARD);
    fft1d_init(&p->f1, n1, FFTW_FORWARD);
    fft1d_init(&p->b0, n0, FFTW_BACKWARD);
    fft1d_init(&p->b1, n1, FFTW_BACKWARD);
    return p;
}

void fftwf_destroy_plan(fftwf_plan p) {
    if (!p) return;
    fft1d_free(&p->f0);
    fft1d_free(&p->f1);
    if (p->kind == KIND_R2R) {
        fft1d_free(&p->b0);
        fft1d_free(&p->b1);
    }
    free(p);
}

void fftwf_plan_free(fftwf_plan p) { fftwf_destroy_plan(p); }

void *fftwf_malloc(size_t n) { return malloc(n ? n : 1); }
void fftwf_free(void *p) { free(p); }

/* column pass over a row-major n0 x w double array held in a[] */
static void columns(const fft1d *f, cplx *a, int n0, int w, cplx *tmp) {
    for (int j = 0; j < w; j++) {
        fft1d_exec(f, a + j, (size_t)w, tmp);
        for (int i = 0; i < n0; i++) a[(size_t)i * w + j] = tmp[i];
    }
}

void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out) {
    int n0 = p->n0, n1 = p->n1;
    size_t n = (size_t)n0 * n1;
    int mx = n0 > n1 ? n0 : n1;
    cplx *a = scratch(2 * n + 2 * (size_t)mx);
    cplx *row = a + n, *tmp = a + n + mx;
    for (int i = 0; i < n0; i++) {
        for (int j = 0; j < n1; j++) row[j] = (cplx)in[(size_t)i * n1 + j];
        fft1d_exec(&p->f1, row, 1, a + (size_t)i * n1);
    }
    columns(&p->f0, a, n0, n1, tmp);
    for (size_t t = 0; t < n; t++) out[t] = (fftwf_complex)a[t];
}

void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out) {
    int n0 = p->n0, n1 = p->n1, h = n1 / 2 + 1;
    int mx = n0 > n1 ? n0 : n1;
    size_t n = (size_t)n0 * h;
    cplx *a = scratch(n + 3 * (size_t)mx);
    cplx *row = a + n, *spec = row + mx, *tmp = spec + mx;
    for (int i = 0; i < n0; i++) {
        for (int j = 0; j < n1; j++) row[j] = (double)in[(size_t)i * n1 + j];
        fft1d_exec(&p->f1, row, 1, spec);
        for (int j = 0; j < h; j++) a[(size_t)i * h + j] = spec[j];
    }
    columns(&p->f0, a, n0, h, tmp);
    for (size_t t = 0; t < n; t++) out[t] = (fftwf_complex)a[t];
}

void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out) {
    int n0 = p->n0, n1 = p->n1, h = n1 / 2 + 1;
    int mx = n0 > n1 ? n0 : n1;
    size_t n = (size_t)n0 * h;
    cplx *a = scratch(n + 3 * (size_t)mx);
    cplx *row = a + n, *res = row + mx, *tmp = res + mx;
    for (size_t t = 0; t < n; t++) a[t] = (cplx)in[t];
    columns(&p->f0, a, n0, h, tmp);
    for (int i = 0; i < n0; i++) {
        /* Hermitian extension of the half row; imaginary parts of the
         * self-conjugate terms drop out of the real part taken below */
        for (int j = 0; j < h; j++) row[j] = a[(size_t)i * h + j];
        for (int j = h; j < n1; j++) row[j] = conj(a[(size_t)i * h + (n1 - j)]);
        fft1d_exec(&p->f1, row, 1, res);
        for (int j = 0; j < n1; j++) out[(size_t)i * n1 + j] = (float)creal(res[j]);
    }
}

/* 1-D real <-> half-complex along a strided line of a double array */
static void r2hc_line(const fft1d *fw, double *x, size_t s, int n, cplx *row, cplx *spec) {
    for (int j = 0; j < n; j++) row[j] = x[(size_t)j * s];
    fft1d_exec(fw, row, 1, spec);
    x[0] = creal(spec[0]);
    for (int k = 1; k <= n / 2; k++) x[(size_t)k * s] = creal(spec[k]);
    for (int k = 1; k < (n + 1) / 2; k++) x[(size_t)(n - k) * s] = cimag(spec[k]);
}

static void hc2r_line(const fft1d *bw, double *x, size_t s, int n, cplx *row, cplx *res) {
    row[0] = x[0];
    for (int k = 1; k < (n + 1) / 2; k++) {
        row[k] = x[(size_t)k * s] + I * x[(size_t)(n - k) * s];
        row[n - k] = conj(row[k]);
    }
    if (n % 2 == 0 && n > 1) row[n / 2] = x[(size_t)(n / 2) * s];
    fft1d_exec(bw, row, 1, res);
    for (int j = 0; j < n; j++) x[(size_t)j * s] = creal(res[j]);
}

void fftwf_execute_r2r(const fftwf_plan p, float *in, float *out) {
    int n0 = p->n0, n1 = p->n1;
    size_t n = (size_t)n0 * n1;
    int mx = n0 > n1 ? n0 : n1;
    /* double work array in the complex scratch (n doubles fit in n/2+1 cplx) */
    cplx *sc = scratch(n / 2 + 1 + 2 * (size_t)mx);
    double *x = (double *)sc;
    cplx *row = sc + n / 2 + 1, *tmp = row + mx;
    for (size_t t = 0; t < n; t++) x[t] = in[t];
    for (int i = 0; i < n0; i++) {
        if (p->k1 == FFTW_R2HC)
            r2hc_line(&p->f1, x + (size_t)i * n1, 1, n1, row, tmp);
        else
            hc2r_line(&p->b1, x + (size_t)i * n1, 1, n1, row, tmp);
    }
    for (int j = 0; j < n1; j++) {
        if (p->k0 == FFTW_R2HC)
            r2hc_line(&p->f0, x + j, (size_t)n1, n0, row, tmp);
        else
            hc2r_line(&p->b0, x + j, (size_t)n1, n0, row, tmp);
    }
    for (size_t t = 0; t < n; t++) out[t] = (float)x[t];
}
