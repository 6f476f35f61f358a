/* Subset of the FFTW3 single-precision interface that cmod/src/centmodule.c
 * calls -- TEST INFRASTRUCTURE ONLY (the reference build of the oracle).
 *
 * FFTW3 is a third-party system package that the reference links but does
 * not vendor (cmod/src/Makefile, fftw3-dev; unpinned).  It is absent from
 * this image, so this header declares, and fft_shim.c implements, only the
 * calls the reference makes, with FFTW's documented conventions:
 *   - unnormalised transforms, forward sign -1 (FFTW_FORWARD), backward +1;
 *   - 2-D arrays row-major, n0 rows of n1 elements;
 *   - r2c output n0 x (n1/2+1) complex, c2r input of that shape, the
 *     imaginary parts of the self-conjugate elements ignored;
 *   - r2r_2d: the separable product of 1-D R2HC / HC2R transforms along
 *     each dimension, half-complex order r0,r1,..,r_{n/2},i_{(n+1)/2-1},..,i1;
 *   - plans may be executed on other arrays of the same shape from many
 *     threads at once (fftwf_execute_dft & co.).
 * Call sites: cmod/src/centmodule.c:498,532,540,1422,1481,2342-2345,
 * 2753-2756,3093-3094,3105,3172-3176,3301-3307.  The reference also calls
 * fftwf_plan_free (:2753-2754), a name FFTW does not export; it is provided
 * here as a synonym of fftwf_destroy_plan so the module links.
 */
#ifndef DASP_REF_FFTW3_SHIM_H
#define DASP_REF_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef float _Complex fftwf_complex;
typedef struct refshim_fft_plan *fftwf_plan;
typedef enum { FFTW_R2HC = 0, FFTW_HC2R = 1 } fftwf_r2r_kind;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out, int sign,
                             unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_2d(int n0, int n1, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_2d(int n0, int n1, fftwf_complex *in, float *out, unsigned flags);
fftwf_plan fftwf_plan_r2r_2d(int n0, int n1, float *in, float *out, fftwf_r2r_kind kind0,
                             fftwf_r2r_kind kind1, unsigned flags);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out);
void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out);
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out);
void fftwf_execute_r2r(const fftwf_plan p, float *in, float *out);
void fftwf_destroy_plan(fftwf_plan p);
void fftwf_plan_free(fftwf_plan p);
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
