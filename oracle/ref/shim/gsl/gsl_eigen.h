/* GSL-API shim (symmetric eigenproblems, matrices, vectors) for the
 * reference's own sources (include/math/mat3.hh:25-185); oracle/_ref only. */
#ifndef MF_REF_GSL_EIGEN_H
#define MF_REF_GSL_EIGEN_H
#include <stddef.h>
#include "gsl_errno.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct {
  size_t size;
  size_t stride;
  double* data;
  void* block;
  int owner;
} gsl_vector;
typedef struct {
  size_t size1;
  size_t size2;
  size_t tda;
  double* data;
  void* block;
  int owner;
} gsl_matrix;
typedef struct { gsl_matrix matrix; } gsl_matrix_view;
typedef struct gsl_eigen_symmv_workspace gsl_eigen_symmv_workspace;
typedef enum { GSL_EIGEN_SORT_VAL_ASC, GSL_EIGEN_SORT_VAL_DESC, GSL_EIGEN_SORT_ABS_ASC,
               GSL_EIGEN_SORT_ABS_DESC } gsl_eigen_sort_t;
gsl_matrix_view gsl_matrix_view_array(double* base, size_t n1, size_t n2);
gsl_vector* gsl_vector_alloc(size_t n);
void gsl_vector_free(gsl_vector* v);
gsl_matrix* gsl_matrix_alloc(size_t n1, size_t n2);
void gsl_matrix_free(gsl_matrix* m);
double gsl_vector_get(const gsl_vector* v, size_t i);
double gsl_matrix_get(const gsl_matrix* m, size_t i, size_t j);
gsl_eigen_symmv_workspace* gsl_eigen_symmv_alloc(size_t n);
void gsl_eigen_symmv_free(gsl_eigen_symmv_workspace* w);
int gsl_eigen_symmv(gsl_matrix* A, gsl_vector* eval, gsl_matrix* evec, gsl_eigen_symmv_workspace* w);
int gsl_eigen_symmv_sort(gsl_vector* eval, gsl_matrix* evec, gsl_eigen_sort_t sort_type);
#ifdef __cplusplus
}
#endif
#endif
