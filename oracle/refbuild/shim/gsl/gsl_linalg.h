/* The GSL matrix/LU calls of the reference's parabolic-fit set-up
 * (cmod/src/centmodule.c:1046-1051, makeFitMx: invert a 6x6 double matrix)
 * -- TEST INFRASTRUCTURE ONLY.  gsl_shim.c implements LU decomposition with
 * partial pivoting (row of largest |a_ik| in the column, Golub & Van Loan
 * algorithm 3.4.1) and the inverse by forward/back substitution of the
 * identity's columns, as GSL documents gsl_linalg_LU_decomp/_invert. */
#ifndef DASP_REF_GSL_LINALG_SHIM_H
#define DASP_REF_GSL_LINALG_SHIM_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    size_t size1, size2, tda;
    double *data;
    void *block;
    int owner;
} gsl_matrix;

typedef struct {
    gsl_matrix matrix;
} gsl_matrix_view;

typedef struct {
    size_t size;
    size_t *data;
} gsl_permutation;

gsl_matrix_view gsl_matrix_view_array(double *base, size_t n1, size_t n2);
gsl_permutation *gsl_permutation_alloc(size_t n);
void gsl_permutation_free(gsl_permutation *p);
int gsl_linalg_LU_decomp(gsl_matrix *A, gsl_permutation *p, int *signum);
int gsl_linalg_LU_invert(const gsl_matrix *LU, const gsl_permutation *p, gsl_matrix *inverse);

#ifdef __cplusplus
}
#endif
#endif
