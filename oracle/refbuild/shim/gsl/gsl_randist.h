/* gsl_ran_gaussian for the reference build -- TEST INFRASTRUCTURE ONLY.
 * GSL documents it as the Box-Muller (Marsaglia polar) method on two
 * uniform_pos draws per attempt: x, y uniform on (-1,1), retried until
 * 0 < r2 = x^2 + y^2 <= 1, returning sigma * y * sqrt(-2 ln r2 / r2).
 * Call sites: cmod/src/centmodule.c:805,810 (readCCD). */
#ifndef DASP_REF_GSL_RANDIST_SHIM_H
#define DASP_REF_GSL_RANDIST_SHIM_H
#include "gsl_rng.h"
#ifdef __cplusplus
extern "C" {
#endif
double gsl_ran_gaussian(const gsl_rng *r, double sigma);
#ifdef __cplusplus
}
#endif
#endif
