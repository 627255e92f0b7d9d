/* GSL-API shim (cubic splines) for the reference's own sources
 * (include/math/interpolate.hh:87-101); oracle/_ref only. */
#ifndef MF_REF_GSL_SPLINE_H
#define MF_REF_GSL_SPLINE_H
#include <stddef.h>
#include "gsl_errno.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct gsl_interp_type { const char* name; int periodic; } gsl_interp_type;
extern const gsl_interp_type* gsl_interp_cspline;
extern const gsl_interp_type* gsl_interp_cspline_periodic;
typedef struct { size_t cache; } gsl_interp_accel;
typedef struct gsl_spline gsl_spline;
gsl_interp_accel* gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel* a);
gsl_spline* gsl_spline_alloc(const gsl_interp_type* T, size_t size);
int gsl_spline_init(gsl_spline* spline, const double xa[], const double ya[], size_t size);
double gsl_spline_eval(const gsl_spline* spline, double x, gsl_interp_accel* a);
void gsl_spline_free(gsl_spline* spline);
#ifdef __cplusplus
}
#endif
#endif
