/* GSL-API shim (constants) for the reference's own sources; oracle/_ref only. */
#ifndef MF_REF_GSL_MATH_H
#define MF_REF_GSL_MATH_H
#include <math.h>
#include "gsl_errno.h"
#endif
