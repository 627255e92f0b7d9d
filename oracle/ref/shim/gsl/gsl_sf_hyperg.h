/* GSL-API shim (Gauss hypergeometric function) for the reference's own
 * sources (include/particle_plt.hh:39-43); oracle/_ref only. */
#ifndef MF_REF_GSL_SF_HYPERG_H
#define MF_REF_GSL_SF_HYPERG_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_hyperg_2F1(double a, double b, double c, double x);
#ifdef __cplusplus
}
#endif
#endif
