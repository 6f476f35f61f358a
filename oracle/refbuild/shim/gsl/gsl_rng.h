/* Subset of GSL's random-number interface used by cmod/src/centmodule.c --
 * TEST INFRASTRUCTURE ONLY (the reference build of the oracle).
 *
 * GSL is a third-party system package the reference links but does not
 * vendor (cmod/src/Makefile, libgsl-dev; unpinned), absent from this image.
 * gsl_shim.c implements these calls from the published algorithms: MT19937
 * (Matsumoto & Nishimura 1998) seeded by the 2002 recurrence
 * x_i = 1812433253 (x_{i-1} xor (x_{i-1} >> 30)) + i with seed 0 replaced by
 * 4357 (GSL's documented default), uniform = u32 / 2^32, uniform_pos the same
 * with 0 rejected.  Call sites: cmod/src/centmodule.c:2552-2562, :2489.
 */
#ifndef DASP_REF_GSL_RNG_SHIM_H
#define DASP_REF_GSL_RNG_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    const char *name;
} gsl_rng_type;

typedef struct refshim_gsl_rng gsl_rng;

extern const gsl_rng_type *gsl_rng_mt19937;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long seed);
void gsl_rng_free(gsl_rng *r);
unsigned long gsl_rng_get(const gsl_rng *r);
double gsl_rng_uniform(const gsl_rng *r);
double gsl_rng_uniform_pos(const gsl_rng *r);

#ifdef __cplusplus
}
#endif
#endif
