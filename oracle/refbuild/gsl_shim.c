/* GSL subset for the reference build -- TEST INFRASTRUCTURE ONLY.
 * Written from the published algorithms named in shim/gsl/*.h; no GSL
 * source is used (GSL is not part of the reference tree). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "gsl/gsl_linalg.h"
#include "gsl/gsl_randist.h"
#include "gsl/gsl_rng.h"

/* ---------------- MT19937 ---------------- */
enum { MT_STATE = 624, MT_SHIFT = 397 };

struct refshim_gsl_rng {
    uint32_t s[MT_STATE];
    int pos;
};

static const gsl_rng_type mt_type = {"mt19937"};
const gsl_rng_type *gsl_rng_mt19937 = &mt_type;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) {
    (void)T;
    gsl_rng *r = (gsl_rng *)calloc(1, sizeof(gsl_rng));
    if (r) gsl_rng_set(r, 0);
    return r;
}

void gsl_rng_free(gsl_rng *r) { free(r); }

void gsl_rng_set(const gsl_rng *rc, unsigned long seed) {
    gsl_rng *r = (gsl_rng *)rc;
    uint32_t x = (uint32_t)((seed == 0 ? 4357UL : seed) & 0xffffffffUL);
    r->s[0] = x;
    for (int i = 1; i < MT_STATE; i++) {
        x = 1812433253u * (x ^ (x >> 30)) + (uint32_t)i;
        r->s[i] = x;
    }
    r->pos = MT_STATE;
}

static void mt_regenerate(gsl_rng *r) {
    /* twist: y = upper bit of s[k] | lower 31 bits of s[k+1];
     * s[k] = s[k+397] ^ (y >> 1) ^ (odd(y) ? 0x9908b0df : 0) */
    for (int k = 0; k < MT_STATE; k++) {
        uint32_t y = (r->s[k] & 0x80000000u) | (r->s[(k + 1) % MT_STATE] & 0x7fffffffu);
        uint32_t v = r->s[(k + MT_SHIFT) % MT_STATE] ^ (y >> 1);
        if (y & 1u) v ^= 0x9908b0dfu;
        r->s[k] = v;
    }
    r->pos = 0;
}

unsigned long gsl_rng_get(const gsl_rng *rc) {
    gsl_rng *r = (gsl_rng *)rc;
    if (r->pos >= MT_STATE) mt_regenerate(r);
    uint32_t y = r->s[r->pos++];
    /* tempering */
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return (unsigned long)y;
}

double gsl_rng_uniform(const gsl_rng *r) { return (double)gsl_rng_get(r) / 4294967296.0; }

double gsl_rng_uniform_pos(const gsl_rng *r) {
    double u;
    do {
        u = gsl_rng_uniform(r);
    } while (u == 0.0);
    return u;
}

double gsl_ran_gaussian(const gsl_rng *r, double sigma) {
    double x, y, r2;
    for (;;) {
        x = 2.0 * gsl_rng_uniform_pos(r) - 1.0;
        y = 2.0 * gsl_rng_uniform_pos(r) - 1.0;
        r2 = x * x + y * y;
        if (r2 <= 1.0 && r2 != 0.0) break;
    }
    return sigma * y * sqrt(-2.0 * log(r2) / r2);
}

/* ---------------- 6x6 LU inverse ---------------- */
gsl_matrix_view gsl_matrix_view_array(double *base, size_t n1, size_t n2) {
    gsl_matrix_view v;
    memset(&v, 0, sizeof(v));
    v.matrix.size1 = n1;
    v.matrix.size2 = n2;
    v.matrix.tda = n2;
    v.matrix.data = base;
    return v;
}

gsl_permutation *gsl_permutation_alloc(size_t n) {
    gsl_permutation *p = (gsl_permutation *)malloc(sizeof(gsl_permutation));
    if (!p) return NULL;
    p->size = n;
    p->data = (size_t *)malloc(sizeof(size_t) * (n ? n : 1));
    for (size_t i = 0; i < n; i++) p->data[i] = i;
    return p;
}

void gsl_permutation_free(gsl_permutation *p) {
    if (!p) return;
    free(p->data);
    free(p);
}

#define AT(m, i, j) ((m)->data[(i) * (m)->tda + (j)])

int gsl_linalg_LU_decomp(gsl_matrix *A, gsl_permutation *p, int *signum) {
    size_t n = A->size1;
    *signum = 1;
    for (size_t i = 0; i < n; i++) p->data[i] = i;
    for (size_t j = 0; j + 1 < n; j++) {
        /* pivot: largest magnitude in column j at or below the diagonal */
        size_t piv = j;
        double best = fabs(AT(A, j, j));
        for (size_t i = j + 1; i < n; i++) {
            double v = fabs(AT(A, i, j));
            if (v > best) {
                best = v;
                piv = i;
            }
        }
        if (piv != j) {
            for (size_t k = 0; k < n; k++) {
                double t = AT(A, j, k);
                AT(A, j, k) = AT(A, piv, k);
                AT(A, piv, k) = t;
            }
            size_t t = p->data[j];
            p->data[j] = p->data[piv];
            p->data[piv] = t;
            *signum = -*signum;
        }
        double d = AT(A, j, j);
        if (d != 0.0) {
            for (size_t i = j + 1; i < n; i++) {
                double l = AT(A, i, j) / d;
                AT(A, i, j) = l;
                for (size_t k = j + 1; k < n; k++) AT(A, i, k) -= l * AT(A, j, k);
            }
        }
    }
    return 0;
}

int gsl_linalg_LU_invert(const gsl_matrix *LU, const gsl_permutation *p, gsl_matrix *inv) {
    size_t n = LU->size1;
    double col[64];
    if (n > 64) return 1;
    for (size_t c = 0; c < n; c++) {
        /* b = P e_c, then L y = b (unit lower), U x = y */
        for (size_t i = 0; i < n; i++) col[i] = (p->data[i] == c) ? 1.0 : 0.0;
        for (size_t i = 0; i < n; i++) {
            double s = col[i];
            for (size_t k = 0; k < i; k++) s -= AT(LU, i, k) * col[k];
            col[i] = s;
        }
        for (size_t ii = n; ii-- > 0;) {
            double s = col[ii];
            for (size_t k = ii + 1; k < n; k++) s -= AT(LU, ii, k) * col[k];
            col[ii] = s / AT(LU, ii, ii);
        }
        for (size_t i = 0; i < n; i++) AT(inv, i, c) = col[i];
    }
    return 0;
}
