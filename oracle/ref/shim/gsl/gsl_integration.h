/* GSL-API shim (adaptive quadrature, gsl_integration_qag) for the
 * reference's own sources (include/cosmology_calculator.hh:62-83);
 * oracle/_ref only.  The Gauss-Kronrod rules are computed, not tabulated
 * (gsl_shim.cc). */
#ifndef MF_REF_GSL_INTEGRATION_H
#define MF_REF_GSL_INTEGRATION_H
#include <stddef.h>
#include "gsl_errno.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct {
  double (*function)(double x, void* params);
  void* params;
} gsl_function;
typedef struct gsl_integration_workspace gsl_integration_workspace;
enum { GSL_INTEG_GAUSS15 = 1, GSL_INTEG_GAUSS21 = 2, GSL_INTEG_GAUSS31 = 3, GSL_INTEG_GAUSS41 = 4,
       GSL_INTEG_GAUSS51 = 5, GSL_INTEG_GAUSS61 = 6 };
gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace* w);
int gsl_integration_qag(const gsl_function* f, double a, double b, double epsabs, double epsrel, size_t limit,
                        int key, gsl_integration_workspace* workspace, double* result, double* abserr);
#ifdef __cplusplus
}
#endif
#endif
