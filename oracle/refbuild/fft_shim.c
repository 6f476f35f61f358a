/* FFTW3f subset for the reference build -- TEST INFRASTRUCTURE ONLY.
 *
 * Implements the calls declared in shim/fftw3.h with the discrete Fourier
 * transform's definition X_k = sum_j x_j exp(sign 2 pi i jk/n) (unnormalised),
 * evaluated by a mixed-radix Cooley-Tukey decimation in time: the input is
 * gathered in digit-reversed order, then stages of radix 4, 2, 3 and 5
 * butterflies (any other prime factor by its direct DFT) combine blocks,
 * with every stage's twiddles exp(sign 2 pi i qk/B) tabulated in double when
 * the plan is made.  Inputs are read as float, each whole 2-D transform runs
 * in double and the result is rounded to float once -- at least as accurate
 * as FFTW's single precision (whose last-bit results depend on the plan
 * FFTW_MEASURE picks).  Real 2-D transforms take two real rows per complex
 * row transform.  Plans are immutable after creation; execution uses
 * per-thread scratch, so one plan may run on different arrays from many
 * threads at once, which is how the reference's worker threads use theirs.
 * No FFTW source is used.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

typedef struct {
    double re, im;
} cpx;

enum { KIND_C2C = 0, KIND_R2C = 1, KIND_C2R = 2, KIND_R2R = 3 };
enum { MAXFAC = 32 };

typedef struct {
    int r, M, B; /* radix, butterflies per block, block size B = r * M */
    cpx *tw;     /* tw[k * r + q] = exp(sign 2 pi i q k / B), k < M, q < r */
    cpx *wr;     /* radix other than 1-5: exp(sign 2 pi i t / r), t < r */
} stage;

typedef struct {
    int n, sign, nst;
    int *perm; /* work[p] = in[perm[p]] */
    stage st[MAXFAC];
    cpx w3, w5a, w5b; /* exp(sign 2 pi i / 3), exp(sign 2 pi i / 5), exp(sign 4 pi i / 5) */
} fft1d;

struct refshim_fft_plan {
    int kind, n0, n1;
    fftwf_r2r_kind k0, k1;
    fft1d f0, f1; /* the transform's own sign (c2c, r2c: -1; c2r: +1) */
    fft1d b0, b1; /* r2r: backward (+1) tables */
};

static cpx cexpi(double a) {
    cpx c = {cos(a), sin(a)};
    return c;
}

static void build_perm(int *perm, int in0, int stride, int n, const int *fac, int pos0) {
    int r = fac[0], m = n / r;
    if (m == 1) {
        for (int q = 0; q < r; q++) perm[pos0 + q] = in0 + q * stride;
    } else {
        for (int q = 0; q < r; q++) build_perm(perm, in0 + q * stride, stride * r, m, fac + 1, pos0 + q * m);
    }
}

static void fft1d_init(fft1d *f, int n, int sign) {
    int fac[MAXFAC], nf = 0, rem = n;
    static const int pref[] = {4, 2, 3, 5};
    memset(f, 0, sizeof(*f));
    f->n = n;
    f->sign = sign;
    for (int q = 0; q < 4; q++)
        while (rem % pref[q] == 0 && rem > 1) {
            fac[nf++] = pref[q];
            rem /= pref[q];
        }
    for (int d = 7; rem > 1; d += 2)
        while (rem % d == 0) {
            fac[nf++] = d;
            rem /= d;
        }
    if (nf == 0) fac[nf++] = 1;
    for (int q = 0; q < nf; q++)
        if (fac[q] > 64) abort(); /* butterflies hold at most 64 terms */
    f->perm = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    build_perm(f->perm, 0, 1, n, fac, 0);
    /* combining stages run from the deepest recursion level up: level d has
     * block size n / (fac[0] ... fac[d-1]) and radix fac[d] */
    f->nst = nf;
    for (int d = nf - 1, s = 0; d >= 0; d--, s++) {
        int B = n;
        for (int e = 0; e < d; e++) B /= fac[e];
        stage *g = &f->st[s];
        g->r = fac[d];
        g->B = B;
        g->M = B / fac[d];
        g->tw = (cpx *)malloc(sizeof(cpx) * (size_t)g->M * g->r);
        for (int k = 0; k < g->M; k++)
            for (int q = 0; q < g->r; q++) g->tw[k * g->r + q] = cexpi(sign * 2.0 * M_PI * (double)q * k / B);
        if (g->r > 5) {
            g->wr = (cpx *)malloc(sizeof(cpx) * (size_t)g->r);
            for (int t = 0; t < g->r; t++) g->wr[t] = cexpi(sign * 2.0 * M_PI * t / g->r);
        }
    }
    f->w3 = cexpi(sign * 2.0 * M_PI / 3.0);
    f->w5a = cexpi(sign * 2.0 * M_PI / 5.0);
    f->w5b = cexpi(sign * 4.0 * M_PI / 5.0);
}

static void fft1d_free(fft1d *f) {
    free(f->perm);
    for (int s = 0; s < f->nst; s++) {
        free(f->st[s].tw);
        free(f->st[s].wr);
    }
    memset(f, 0, sizeof(*f));
}

/* in place on w[0..n) (already in digit-reversed order) */
static void run_stages(const fft1d *f, cpx *w) {
    const int n = f->n;
    for (int s = 0; s < f->nst; s++) {
        const stage *g = &f->st[s];
        const int r = g->r, M = g->M, B = g->B;
        for (int b = 0; b < n; b += B) {
            cpx *blk = w + b;
            for (int k = 0; k < M; k++) {
                const cpx *tw = g->tw + k * r;
                cpx t[64];
                t[0] = blk[k];
                for (int q = 1; q < r; q++) {
                    const cpx x = blk[q * M + k], c = tw[q];
                    t[q].re = x.re * c.re - x.im * c.im;
                    t[q].im = x.re * c.im + x.im * c.re;
                }
                if (r == 4) {
                    /* w4 = exp(sign i pi / 2) = sign * i */
                    const double sg = (double)f->sign;
                    cpx a = {t[0].re + t[2].re, t[0].im + t[2].im}, bb = {t[0].re - t[2].re, t[0].im - t[2].im};
                    cpx c = {t[1].re + t[3].re, t[1].im + t[3].im};
                    cpx d0 = {t[1].re - t[3].re, t[1].im - t[3].im};
                    cpx d = {-sg * d0.im, sg * d0.re};
                    blk[k].re = a.re + c.re;
                    blk[k].im = a.im + c.im;
                    blk[M + k].re = bb.re + d.re;
                    blk[M + k].im = bb.im + d.im;
                    blk[2 * M + k].re = a.re - c.re;
                    blk[2 * M + k].im = a.im - c.im;
                    blk[3 * M + k].re = bb.re - d.re;
                    blk[3 * M + k].im = bb.im - d.im;
                } else if (r == 2) {
                    blk[k].re = t[0].re + t[1].re;
                    blk[k].im = t[0].im + t[1].im;
                    blk[M + k].re = t[0].re - t[1].re;
                    blk[M + k].im = t[0].im - t[1].im;
                } else if (r == 3) {
                    /* X0 = t0 + s, X1,2 = t0 + c3 s -/+ i s3 (t1 - t2) with s = t1 + t2 */
                    const double c3 = f->w3.re, s3 = f->w3.im;
                    cpx sm = {t[1].re + t[2].re, t[1].im + t[2].im}, df = {t[1].re - t[2].re, t[1].im - t[2].im};
                    cpx m0 = {t[0].re + c3 * sm.re, t[0].im + c3 * sm.im};
                    blk[k].re = t[0].re + sm.re;
                    blk[k].im = t[0].im + sm.im;
                    blk[M + k].re = m0.re - s3 * df.im;
                    blk[M + k].im = m0.im + s3 * df.re;
                    blk[2 * M + k].re = m0.re + s3 * df.im;
                    blk[2 * M + k].im = m0.im - s3 * df.re;
                } else if (r == 5) {
                    const double c1 = f->w5a.re, s1 = f->w5a.im, c2 = f->w5b.re, s2 = f->w5b.im;
                    cpx a1 = {t[1].re + t[4].re, t[1].im + t[4].im}, b1 = {t[1].re - t[4].re, t[1].im - t[4].im};
                    cpx a2 = {t[2].re + t[3].re, t[2].im + t[3].im}, b2 = {t[2].re - t[3].re, t[2].im - t[3].im};
                    cpx p1 = {t[0].re + c1 * a1.re + c2 * a2.re, t[0].im + c1 * a1.im + c2 * a2.im};
                    cpx p2 = {t[0].re + c2 * a1.re + c1 * a2.re, t[0].im + c2 * a1.im + c1 * a2.im};
                    /* i (s1 b1 + s2 b2) and i (s2 b1 - s1 b2) */
                    cpx q1 = {-(s1 * b1.im + s2 * b2.im), s1 * b1.re + s2 * b2.re};
                    cpx q2 = {-(s2 * b1.im - s1 * b2.im), s2 * b1.re - s1 * b2.re};
                    blk[k].re = t[0].re + a1.re + a2.re;
                    blk[k].im = t[0].im + a1.im + a2.im;
                    blk[M + k].re = p1.re + q1.re;
                    blk[M + k].im = p1.im + q1.im;
                    blk[4 * M + k].re = p1.re - q1.re;
                    blk[4 * M + k].im = p1.im - q1.im;
                    blk[2 * M + k].re = p2.re + q2.re;
                    blk[2 * M + k].im = p2.im + q2.im;
                    blk[3 * M + k].re = p2.re - q2.re;
                    blk[3 * M + k].im = p2.im - q2.im;
                } else if (r == 1) {
                    blk[k] = t[0];
                } else {
                    /* direct DFT of length r: X_s = sum_q t_q exp(sign 2 pi i qs / r) */
                    for (int sidx = 0; sidx < r; sidx++) {
                        cpx acc = t[0];
                        for (int q = 1, e = sidx; q < r; q++, e = (e + sidx) % r) {
                            const cpx c = g->wr[e];
                            acc.re += t[q].re * c.re - t[q].im * c.im;
                            acc.im += t[q].re * c.im + t[q].im * c.re;
                        }
                        blk[sidx * M + k] = acc;
                    }
                }
            }
        }
    }
}

/* out[0..n) = DFT of x[0], x[s], x[2s], ... (out must not alias x) */
static void fft1d_exec(const fft1d *f, const cpx *x, size_t s, cpx *out) {
    const int n = f->n;
    for (int p = 0; p < n; p++) out[p] = x[(size_t)f->perm[p] * s];
    run_stages(f, out);
}

/* per-thread scratch */
static __thread cpx *g_scr = NULL;
static __thread size_t g_scr_n = 0;

static cpx *scratch(size_t n) {
    if (n > g_scr_n) {
        free(g_scr);
        g_scr = (cpx *)malloc(sizeof(cpx) * n);
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
    fft1d_init(&p->f0, n0, sign);
    fft1d_init(&p->f1, n1, sign);
    return p;
}

fftwf_plan fftwf_plan_dft_r2c_2d(int n0, int n1, float *in, fftwf_complex *out, unsigned flags) {
    (void)in, (void)out, (void)flags;
    fftwf_plan p = new_plan(KIND_R2C, n0, n1);
    fft1d_init(&p->f0, n0, FFTW_FORWARD);
    fft1d_init(&p->f1, n1, FFTW_FORWARD);
    return p;
}

fftwf_plan fftwf_plan_dft_c2r_2d(int n0, int n1, fftwf_complex *in, float *out, unsigned flags) {
    (void)in, (void)out, (void)flags;
    fftwf_plan p = new_plan(KIND_C2R, n0, n1);
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

/* column transforms of a row-major n0 x w array a[] */
static void columns(const fft1d *f, cpx *a, int n0, int w, cpx *tmp) {
    for (int j = 0; j < w; j++) {
        fft1d_exec(f, a + j, (size_t)w, tmp);
        for (int i = 0; i < n0; i++) a[(size_t)i * w + j] = tmp[i];
    }
}

static inline cpx ld(const fftwf_complex *z) {
    const float *f = (const float *)z;
    cpx c = {f[0], f[1]};
    return c;
}

static inline void st(fftwf_complex *z, cpx c) {
    float *f = (float *)z;
    f[0] = (float)c.re;
    f[1] = (float)c.im;
}

void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out) {
    const int n0 = p->n0, n1 = p->n1;
    const size_t n = (size_t)n0 * n1;
    const int mx = n0 > n1 ? n0 : n1;
    cpx *a = scratch(n + 2 * (size_t)mx);
    cpx *row = a + n, *tmp = row + mx;
    for (int i = 0; i < n0; i++) {
        for (int j = 0; j < n1; j++) row[j] = ld(in + (size_t)i * n1 + j);
        fft1d_exec(&p->f1, row, 1, a + (size_t)i * n1);
    }
    columns(&p->f0, a, n0, n1, tmp);
    for (size_t t = 0; t < n; t++) st(out + t, a[t]);
}

void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out) {
    const int n0 = p->n0, n1 = p->n1, h = n1 / 2 + 1;
    const int mx = n0 > n1 ? n0 : n1;
    const size_t n = (size_t)n0 * h;
    cpx *a = scratch(n + 3 * (size_t)mx);
    cpx *row = a + n, *z = row + mx, *tmp = z + mx;
    for (int i = 0; i < n0; i += 2) {
        /* rows i and i+1 as the real and imaginary parts of one transform:
         * X_i[k] = (Z[k] + conj Z[-k]) / 2, X_{i+1}[k] = (Z[k] - conj Z[-k]) / 2i */
        const int two = i + 1 < n0;
        for (int j = 0; j < n1; j++) {
            row[j].re = in[(size_t)i * n1 + j];
            row[j].im = two ? in[(size_t)(i + 1) * n1 + j] : 0.0;
        }
        fft1d_exec(&p->f1, row, 1, z);
        for (int k = 0; k < h; k++) {
            const cpx zk = z[k], zn = z[(n1 - k) % n1];
            cpx x0 = {0.5 * (zk.re + zn.re), 0.5 * (zk.im - zn.im)};
            a[(size_t)i * h + k] = two ? x0 : zk;
            if (two) {
                cpx x1 = {0.5 * (zk.im + zn.im), -0.5 * (zk.re - zn.re)};
                a[(size_t)(i + 1) * h + k] = x1;
            }
        }
    }
    columns(&p->f0, a, n0, h, tmp);
    for (size_t t = 0; t < n; t++) st(out + t, a[t]);
}

void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out) {
    const int n0 = p->n0, n1 = p->n1, h = n1 / 2 + 1;
    const int mx = n0 > n1 ? n0 : n1;
    const size_t n = (size_t)n0 * h;
    cpx *a = scratch(n + 3 * (size_t)mx);
    cpx *row = a + n, *res = row + mx, *tmp = res + mx;
    for (size_t t = 0; t < n; t++) a[t] = ld(in + t);
    columns(&p->f0, a, n0, h, tmp);
    for (int i = 0; i < n0; i += 2) {
        /* rows i and i+1: the Hermitian extensions A and B of the half rows,
         * transformed together as A + iB; the real and imaginary parts of
         * the result are rows i and i+1 (the imaginary parts of the
         * self-conjugate terms of A and B drop out, as in a c2r transform) */
        const int two = i + 1 < n0;
        const cpx *ha = a + (size_t)i * h, *hb = two ? a + (size_t)(i + 1) * h : NULL;
        for (int k = 0; k < n1; k++) {
            cpx A, Bv = {0.0, 0.0};
            if (k < h) {
                A = ha[k];
                if (two) Bv = hb[k];
            } else {
                A.re = ha[n1 - k].re;
                A.im = -ha[n1 - k].im;
                if (two) {
                    Bv.re = hb[n1 - k].re;
                    Bv.im = -hb[n1 - k].im;
                }
            }
            if (k == 0 || (n1 % 2 == 0 && k == n1 / 2)) {
                A.im = 0.0;
                Bv.im = 0.0;
            }
            row[k].re = A.re - Bv.im;
            row[k].im = A.im + Bv.re;
        }
        fft1d_exec(&p->f1, row, 1, res);
        for (int j = 0; j < n1; j++) {
            out[(size_t)i * n1 + j] = (float)res[j].re;
            if (two) out[(size_t)(i + 1) * n1 + j] = (float)res[j].im;
        }
    }
}

/* 1-D real <-> half-complex along a strided line of a double array */
static void r2hc_line(const fft1d *fw, double *x, size_t s, int n, cpx *row, cpx *spec) {
    for (int j = 0; j < n; j++) {
        row[j].re = x[(size_t)j * s];
        row[j].im = 0.0;
    }
    fft1d_exec(fw, row, 1, spec);
    for (int k = 0; k <= n / 2; k++) x[(size_t)k * s] = spec[k].re;
    for (int k = 1; k < (n + 1) / 2; k++) x[(size_t)(n - k) * s] = spec[k].im;
}

static void hc2r_line(const fft1d *bw, double *x, size_t s, int n, cpx *row, cpx *res) {
    row[0].re = x[0];
    row[0].im = 0.0;
    for (int k = 1; k < (n + 1) / 2; k++) {
        row[k].re = x[(size_t)k * s];
        row[k].im = x[(size_t)(n - k) * s];
        row[n - k].re = row[k].re;
        row[n - k].im = -row[k].im;
    }
    if (n % 2 == 0 && n > 1) {
        row[n / 2].re = x[(size_t)(n / 2) * s];
        row[n / 2].im = 0.0;
    }
    fft1d_exec(bw, row, 1, res);
    for (int j = 0; j < n; j++) x[(size_t)j * s] = res[j].re;
}

void fftwf_execute_r2r(const fftwf_plan p, float *in, float *out) {
    const int n0 = p->n0, n1 = p->n1;
    const size_t n = (size_t)n0 * n1;
    const int mx = n0 > n1 ? n0 : n1;
    cpx *sc = scratch(n / 2 + 1 + 2 * (size_t)mx);
    double *x = (double *)sc;
    cpx *row = sc + n / 2 + 1, *tmp = row + mx;
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
