/* GSL-API shim (error handling) for building the reference's own sources
 * without GSL; test infrastructure for oracle/_ref only (gsl_shim.cc). */
#ifndef MF_REF_GSL_ERRNO_H
#define MF_REF_GSL_ERRNO_H
#ifdef __cplusplus
extern "C" {
#endif
enum { GSL_SUCCESS = 0, GSL_FAILURE = -1, GSL_EDOM = 1, GSL_EINVAL = 4, GSL_EMAXITER = 11, GSL_EROUND = 18,
       GSL_ESING = 21, GSL_ENOMEM = 8 };
typedef void gsl_error_handler_t(const char* reason, const char* file, int line, int gsl_errno);
gsl_error_handler_t* gsl_set_error_handler(gsl_error_handler_t* new_handler);
gsl_error_handler_t* gsl_set_error_handler_off(void);
void gsl_error(const char* reason, const char* file, int line, int gsl_errno);
#ifdef __cplusplus
}
#endif
#endif
