/* Test-only stand-in for GSL's symmetric eigensolver API (declarations
 * follow GSL's public documentation; the solver is a cyclic Jacobi). */
#ifndef MCX_GSL_SHIM_EIGEN_H_
#define MCX_GSL_SHIM_EIGEN_H_
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { size_t size; double data[3]; } gsl_vector;
typedef struct { size_t size1, size2; double data[9]; } gsl_matrix;
typedef struct { size_t size; } gsl_eigen_symmv_workspace;
typedef enum { GSL_EIGEN_SORT_VAL_ASC, GSL_EIGEN_SORT_VAL_DESC, GSL_EIGEN_SORT_ABS_ASC, GSL_EIGEN_SORT_ABS_DESC } gsl_eigen_sort_t;
gsl_vector *gsl_vector_alloc(size_t n);
gsl_matrix *gsl_matrix_alloc(size_t n1, size_t n2);
void gsl_matrix_set(gsl_matrix *m, size_t i, size_t j, double x);
double gsl_matrix_get(const gsl_matrix *m, size_t i, size_t j);
double gsl_vector_get(const gsl_vector *v, size_t i);
gsl_eigen_symmv_workspace *gsl_eigen_symmv_alloc(size_t n);
int gsl_eigen_symmv(gsl_matrix *A, gsl_vector *eval, gsl_matrix *evec, gsl_eigen_symmv_workspace *w);
int gsl_eigen_symmv_sort(gsl_vector *eval, gsl_matrix *evec, gsl_eigen_sort_t t);
#ifdef __cplusplus
}
#endif
#endif
