/*
 * Oracle noise streams -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the random-number streams that the reference's
 * Shack-Hartmann step draws from.  Only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline leg may load this library, and only as the checker.
 *
 *   PCG32 (state/inc, XSH-RR output)      cmod/src/centmodule.c:70-98
 *   rk_float / loggam / PTRS / mult.      cmod/src/centmodule.c:680-782
 *   per-thread seeding (seed+t, seq 1)    cmod/src/centmodule.c:2553-2556
 *   readCCD (read noise + threshold)      cmod/src/centmodule.c:785-817
 *   GSL mt19937 + gsl_ran_gaussian        third-party (GSL, unpinned system
 *     package); restated from the published algorithms: MT19937 with the
 *     1812433253 seeding recurrence (Matsumoto & Nishimura 1998/2002),
 *     uniform_pos = u32 / 2^32 rejecting 0, and the Marsaglia polar method
 *     returning sigma * y * sqrt(-2 ln r2 / r2).
 *
 * Float/double evaluation follows the C source expression by expression, so
 * this file must be compiled with -ffp-contract=off (no FMA contraction).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct { uint64_t state, inc; } orc_pcg32;

uint32_t orc_pcg32_next(orc_pcg32 *r) {
  uint64_t old = r->state;
  r->state = old * 6364136223846793005ULL + r->inc;
  uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  uint32_t rot = (uint32_t)(old >> 59u);
  return (xs >> rot) | (xs << ((-rot) & 31));
}

void orc_pcg32_seed(orc_pcg32 *r, uint64_t initstate, uint64_t initseq) {
  r->state = 0u;
  r->inc = (initseq << 1u) | 1u;
  orc_pcg32_next(r);
  r->state += initstate;
  orc_pcg32_next(r);
}

static inline float orc_rk_float(orc_pcg32 *r) {
  return orc_pcg32_next(r) * 2.3283064365386963e-10;
}

static double orc_loggam(double x) {
  float x0, x2, xp, gl, gl0;
  long k, n;
  /* double literals narrowed to float, as in the reference's table */
  static const float a[10] = {8.333333333333333e-02, -2.777777777777778e-03,
                              7.936507936507937e-04, -5.952380952380952e-04,
                              8.417508417508418e-04, -1.917526917526918e-03,
                              6.410256410256410e-03, -2.955065359477124e-02,
                              1.796443723688307e-01, -1.39243221690590e+00};
  x0 = x;
  n = 0;
  if ((x == 1.0) || (x == 2.0)) return 0.0;
  if (x <= 7.0) {
    n = (long)(7 - x);
    x0 = x + n;
  }
  x2 = 1.0 / (x0 * x0);
  xp = 2 * M_PI;
  gl0 = a[9];
  for (k = 8; k >= 0; k--) {
    gl0 *= x2;
    gl0 += a[k];
  }
  gl = gl0 / x0 + 0.5 * logf(xp) + (x0 - 0.5) * logf(x0) - x0;
  if (x <= 7.0) {
    for (k = 1; k <= n; k++) {
      gl -= logf(x0 - 1.0);
      x0 -= 1.0;
    }
  }
  return gl;
}

static long orc_poisson_ptrs(orc_pcg32 *st, float lam) {
  long k;
  float U, V, slam, loglam, a, b, invalpha, vr, us;
  slam = sqrtf(lam);
  loglam = logf(lam);
  b = 0.931 + 2.53 * slam;
  a = -0.059 + 0.02483 * b;
  invalpha = 1.1239 + 1.1328 / (b - 3.4);
  vr = 0.9277 - 3.6224 / (b - 2);
  for (;;) {
    U = orc_rk_float(st) - 0.5;
    V = orc_rk_float(st);
    us = 0.5 - fabsf(U);
    k = (long)floorf((2 * a / us + b) * U + lam + 0.43);
    if ((us >= 0.07) && (V <= vr)) return k;
    if ((k < 0) || ((us < 0.013) && (V > us))) continue;
    if ((logf(V) + logf(invalpha) - logf(a / (us * us) + b)) <=
        (-lam + k * loglam - orc_loggam(k + 1)))
      return k;
  }
}

long orc_poisson(orc_pcg32 *st, float lam) {
  if (lam >= 10) return orc_poisson_ptrs(st, lam);
  if (lam == 0) return 0;
  long X = 0;
  float prod = 1., enlam = expf(-lam);
  do {
    prod *= orc_rk_float(st);
    X++;
  } while (prod > enlam);
  return X - 1;
}

void orc_poissonise(orc_pcg32 *st, float *data, int n) {
  for (int i = 0; i < n; i++) data[i] = (float)orc_poisson(st, data[i]);
}

/* ---- MT19937 with GSL's seeding, uniform_pos and polar gaussian ---- */
#define MT_N 624
#define MT_M 397
typedef struct { uint32_t mt[MT_N]; int mti; } orc_mt;

void orc_mt_seed(orc_mt *s, unsigned long seed) {
  if (seed == 0) seed = 4357;
  s->mt[0] = (uint32_t)(seed & 0xffffffffUL);
  for (int i = 1; i < MT_N; i++)
    s->mt[i] = (uint32_t)(1812433253UL * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + i);
  s->mti = MT_N;
}

uint32_t orc_mt_next(orc_mt *s) {
  const uint32_t UPPER = 0x80000000UL, LOWER = 0x7fffffffUL;
  uint32_t y;
  if (s->mti >= MT_N) {
    int kk;
    for (kk = 0; kk < MT_N - MT_M; kk++) {
      y = (s->mt[kk] & UPPER) | (s->mt[kk + 1] & LOWER);
      s->mt[kk] = s->mt[kk + MT_M] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfUL : 0u);
    }
    for (; kk < MT_N - 1; kk++) {
      y = (s->mt[kk] & UPPER) | (s->mt[kk + 1] & LOWER);
      s->mt[kk] = s->mt[kk + (MT_M - MT_N)] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfUL : 0u);
    }
    y = (s->mt[MT_N - 1] & UPPER) | (s->mt[0] & LOWER);
    s->mt[MT_N - 1] = s->mt[MT_M - 1] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfUL : 0u);
    s->mti = 0;
  }
  y = s->mt[s->mti++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680UL;
  y ^= (y << 15) & 0xefc60000UL;
  y ^= (y >> 18);
  return y;
}

static double orc_mt_uniform_pos(orc_mt *s) {
  double x;
  do { x = orc_mt_next(s) / 4294967296.0; } while (x == 0);
  return x;
}

double orc_gaussian(orc_mt *s, double sigma) {
  double x, y, r2;
  do {
    x = -1 + 2 * orc_mt_uniform_pos(s);
    y = -1 + 2 * orc_mt_uniform_pos(s);
    r2 = x * x + y * y;
  } while (r2 > 1.0 || r2 == 0);
  return sigma * y * sqrt(-2.0 * log(r2) / r2);
}

/* readCCD: cmod/src/centmodule.c:785-817 */
void orc_readccd(orc_mt *s, float *data, int n, float noiseMean, float readNoise,
                 float floor_, int threshType) {
  int i;
  if (readNoise == 0) {
    if (threshType == 0) {
      for (i = 0; i < n; i++) {
        data[i] += noiseMean;
        data[i] = data[i] < floor_ ? 0. : data[i] - floor_;
      }
    } else if (threshType == 1) {
      for (i = 0; i < n; i++) {
        data[i] += noiseMean;
        data[i] = data[i] < floor_ ? 0. : data[i];
      }
    }
  } else {
    if (threshType == 0) {
      for (i = 0; i < n; i++) {
        data[i] += (float)orc_gaussian(s, (double)readNoise) + noiseMean;
        data[i] = data[i] < floor_ ? 0. : data[i] - floor_;
      }
    } else if (threshType == 1) {
      for (i = 0; i < n; i++) {
        data[i] += (float)orc_gaussian(s, (double)readNoise) + noiseMean;
        data[i] = data[i] < floor_ ? 0. : data[i];
      }
    }
  }
}

int orc_sizeof_pcg32(void) { return (int)sizeof(orc_pcg32); }
int orc_sizeof_mt(void) { return (int)sizeof(orc_mt); }
