/*
 * FFTW3-API shim for building the reference's own sources without FFTW.
 * Test infrastructure only (oracle/_ref): the reference's Grid_FFT calls
 * these entry points (src/grid_fft.cc:50-62,222,256; src/main.cc:159-229);
 * they are backed by the project CPU transform in fftw_shim.cc (mixed-radix,
 * double precision, OpenMP), with FFTW's conventions: unnormalised, sign -1
 * forward / +1 backward, r2c keeps kz in [0, n2/2], c2r reads only the real
 * parts of the kz = 0 and kz = n2/2 terms and transforms the leading
 * dimensions first.  Only the double-precision interface is provided.
 */
#ifndef MF_REF_FFTW3_SHIM_H
#define MF_REF_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fftw_plan_s* fftw_plan;

/* the reference names these types in precision branches it does not compile */
typedef float fftwf_complex[2];
typedef struct fftwf_plan_s* fftwf_plan;
typedef long double fftwl_complex[2];
typedef struct fftwl_plan_s* fftwl_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_PATIENT (1U << 5)

extern const char fftw_version[];

void* fftw_malloc(size_t n);
void fftw_free(void* p);
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double* in, fftw_complex* out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex* in, double* out, unsigned flags);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);

#ifdef __cplusplus
}
#endif
#endif
