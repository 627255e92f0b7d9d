/*
 * monofonic_gb300.h -- C ABI of libmfgpu, the GB300 (sm_103a) implementation
 * of monofonIC's nLPT field pipeline.
 *
 * Every entry point returns an int status (MF_OK = 0) and never traps on the
 * device; the message of the last failure on a context is available through
 * mf_last_error().  Handles own device memory.  A context is driven by one
 * host thread at a time; all work is queued on the context's CUDA stream.
 *
 * Each declaration names the reference interface it replaces (paths relative
 * to the monofonIC source tree).
 */
#ifndef MONOFONIC_GB300_H
#define MONOFONIC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes: the reference throws std::runtime_error or calls abort()
 * (src/main.cc:242-252, src/grid_fft.cc:145); here every failure is a code */
enum {
  MF_OK = 0,
  MF_ERR_ARG = 1,       /* invalid argument or unsupported option */
  MF_ERR_SHAPE = 2,     /* unsupported or mismatching grid size */
  MF_ERR_OOM = 3,       /* device or pinned host allocation failed */
  MF_ERR_CUDA = 4,      /* a CUDA call failed */
  MF_ERR_TIMEOUT = 5,   /* a bounded wait ran out */
  MF_ERR_CANCELLED = 6, /* request cancelled */
  MF_ERR_STATE = 7,     /* object in the wrong state for the call */
  MF_ERR_IO = 8         /* a file could not be created or written */
};

/* arithmetic of a grid: plain FP64, or the FP32-bulk form */
enum { MF_PREC_F64 = 0, MF_PREC_F32 = 1 };
/* space of a grid (include/grid_fft.hh:29 space_t) */
enum { MF_SPACE_R = 0, MF_SPACE_K = 1 };
/* convolver type (CMakeLists.txt:209-216 CONVOLVER_TYPE) */
enum { MF_CONV_ORSZAG = 0, MF_CONV_NAIVE = 1 };
/* operand k-space factors (include/convolution.hh:74-292) */
enum {
  MF_OPND_PLAIN = 0, /* f                                   multiply_field   */
  MF_OPND_HESS = 1,  /* (i g_a)(i g_b) f                    convolve_Hessians */
  MF_OPND_SUM = 2,   /* ((i g_a)(i g_b)+(i g_c)(i g_d)) f    SumOfHessians     */
  MF_OPND_DIFF = 3,  /* ((i g_a)(i g_b)-(i g_c)(i g_d)) f    DifferenceOfHessians */
  MF_OPND_GRAD = 4   /* (i g_a) f                           convolve_Gradients */
};
/* output operators (include/operators.hh:25-35) */
enum { MF_OP_ASSIGN = 0, MF_OP_ADD = 1, MF_OP_SUB = 2, MF_OP_AXPY = 3 };
/* particle loads (include/particle_generator.hh:31-39) */
enum { MF_LATTICE_SC = 0, MF_LATTICE_BCC = 1, MF_LATTICE_FCC = 2, MF_LATTICE_RSC = 3 };

typedef struct mf_ctx mf_ctx;
typedef struct mf_grid mf_grid;
typedef struct mf_conv mf_conv;

/* ---- context ----------------------------------------------------------- */
/* replaces the process-level set-up of src/main.cc:150-181 (FFTW/OpenMP init) */
int mf_ctx_create(int device, mf_ctx** out);
int mf_ctx_destroy(mf_ctx* ctx);
const char* mf_last_error(const mf_ctx* ctx);
int mf_ctx_synchronize(mf_ctx* ctx);
/* library version string */
const char* mf_version(void);
/* the context's CUDA stream (cudaStream_t), for event timing by callers */
int mf_ctx_stream(mf_ctx* ctx, void** stream);
/* kernel launches issued on the context so far, per kernel kind:
 * [conv x-inv, conv y-inv, conv z, conv y-fwd, conv x-fwd, fft z, fft col,
 *  pointwise]; the reference has no counterpart (measurement hook) */
int mf_ctx_launch_counts(const mf_ctx* ctx, int64_t* counts, int n);
/* record an event pair around every launch (per-kind device time); the
 * reference's per-stage get_wtime brackets (src/ic_generator.cc:459-546)
 * are the host-side analogue */
int mf_ctx_profile(mf_ctx* ctx, int enable);
/* sum of profiled device milliseconds and launch counts per kind; clears */
int mf_ctx_profile_read(mf_ctx* ctx, double* ms, int64_t* counts, int n);
/* measured FMA throughput of the device in TFLOP/s (prec MF_PREC_F64 or
 * MF_PREC_F32), the arithmetic ceiling of the FP64 path's roofline (no
 * reference counterpart) */
int mf_probe_fma_rate(mf_ctx* ctx, int prec, double* tflops);
/* page-locked host memory for streaming transfers (no reference
 * counterpart).  A buffer of at least one transparent huge page is backed by
 * huge pages (rounded up to whole pages) and registered with the driver,
 * which keeps copies over the host link at their full rate; smaller buffers
 * come from cudaHostAlloc.  Free with mf_host_free only. */
int mf_host_alloc(size_t bytes, void** out);
int mf_host_free(void* p);
/* the huge page size mf_host_alloc backs large buffers with (0: none) */
int mf_host_huge_page_bytes(size_t* bytes);
/* synchronous copy of device memory (e.g. particles of mf_ic_particles) to
 * host memory (no reference counterpart) */
int mf_copy_to_host(void* host, const void* device, size_t bytes);
/* autotuner (no reference counterpart; the reference's FFTW planning,
 * src/grid_fft.cc:50-62, plays the same role for its CPU transforms): times
 * the candidate schedules of the five convolution passes for grid size n in
 * precision prec (persistent CTAs per SM; z-pass kernel and radix plan) on a
 * scratch convolution and keeps the fastest in a process-wide table that every
 * later launch of those passes uses.  report (optional) receives one line per
 * pass kind.  Tune before recording graphs: the table is read at launch. */
int mf_autotune(mf_ctx* ctx, int n, int prec, char* report, size_t report_len);
/* back to the compiled default schedules */
int mf_autotune_reset(void);
/* set one entry of that table by hand: pass kind (0 conv_xinv, 1 conv_yinv,
 * 2 conv_z, 3 conv_yfwd, 4 conv_xfwd), transform length L (3N/2 for the
 * Orszag convolver), precision, persistent CTAs per SM (0: occupancy limit)
 * and, for conv_z, the kernel (0 TMA-pipelined radix-8 plan, 1 direct-load
 * radix-4 plan) */
int mf_schedule_set(int kind, int L, int prec, int occ, int variant);
/* self-test of the bounded-wait path (no reference counterpart): one CTA
 * waits on an mbarrier that nothing arrives on and no copy targets, polling
 * at most `polls` times (1 .. 2^24); the wait runs out, the kernel records
 * the error flag and returns, and the call reports it as MF_ERR_TIMEOUT the
 * way a stalled asynchronous copy of a pipeline kernel would be.  The
 * context stays usable afterwards. */
int mf_selftest_bounded_wait(mf_ctx* ctx, long polls);
/* self-test of the FP32-bulk form's float-pair arithmetic (no reference
 * counterpart; the reference evaluates the order sum of ic_generator.cc:835-845
 * and q + Psi of particle_generator.hh:524-541 in real_t): on `count`
 * pseudo-random inputs shaped like the pipeline's, the device helpers that
 * the order sum and the lattice readout use are compared with the FP64
 * evaluation rounded once; *mism_sum / *mism_q receive the numbers of stored
 * floats that differ.  Dplus sets the growth weights. */
int mf_selftest_float_pairs(mf_ctx* ctx, long long count, uint64_t seed, double Dplus, long long* mism_sum,
                            long long* mism_q);
/* 1 if grid size n is supported by the compiled kernels */
int mf_grid_size_supported(int n);

/* ---- Grid_FFT<real_t> (include/grid_fft.hh:40-914) --------------------- */
/* Grid_FFT ctor + allocate (grid_fft.hh:77-83, src/grid_fft.cc:40-112):
 * n^3 grid of box length boxlen, padded in-place layout of (n+2)*n*n reals */
int mf_grid_create(mf_ctx* ctx, int n, double boxlen, int prec, int space, mf_grid** out);
int mf_grid_destroy(mf_grid* g);
/* size(), space_, data_ and the byte size of the padded array */
int mf_grid_info(const mf_grid* g, int* n, int* prec, int* space, void** dptr, size_t* bytes);
/* copy the whole padded array (ntot_ reals of the grid's precision) from /
 * to host memory; upload sets the space flag (relem/kelem host access) */
int mf_grid_upload(mf_grid* g, const void* host, int space);
int mf_grid_download(mf_grid* g, void* host);
/* upload a real-space FP64 array of n^3 values (no padding), converting to
 * the grid's precision (RNG_plugin::Fill_Grid, include/random_plugin.hh:37) */
int mf_grid_fill_real64(mf_grid* g, const double* host_n3);
/* FourierTransformForward/Backward(do_transform) (src/grid_fft.cc:208-270) */
int mf_grid_fft_forward(mf_grid* g, int do_transform);
int mf_grid_fft_backward(mf_grid* g, int do_transform);
/* zero() (grid_fft.hh:150-155) */
int mf_grid_zero(mf_grid* g);
/* operator*= (grid_fft.hh:392-403) */
int mf_grid_scale(mf_grid* g, double x);
/* zero_DC_mode, k-space branch (grid_fft.hh:844-850) */
int mf_grid_zero_dc(mf_grid* g);
/* apply_InverseLaplacian (grid_fft.hh:440-449) */
int mf_grid_inverse_laplacian(mf_grid* g);
/* shift_field (grid_fft.hh:832-842) */
int mf_grid_shift(mf_grid* g, const double s[3], int transform_back);
/* Compute_PowerSpectrum (src/grid_fft.cc:1133-1210); arrays of nbins_cap,
 * *nbins receives int(kmax/kmin) */
int mf_grid_power_spectrum(mf_grid* g, double* bin_k, double* bin_P, double* bin_eP,
                           int64_t* bin_count, int nbins_cap, int* nbins);
/* Write_PowerSpectrum (src/grid_fft.cc:1104-1131): the same bins written as
 * text, a header line and one line per non-empty bin (k, P, err, #modes) */
int mf_grid_write_power_spectrum(mf_grid* g, const char* path);
/* Grid_FFT<ccomplex_t> transforms (src/grid_fft.cc:56-63, FFTW_FORWARD /
 * FFTW_BACKWARD, unitary): in place on an n^3 complex FP64 device array
 * [i][j][k] on the context's stream (asynchronous) */
int mf_cgrid_fft(mf_ctx* ctx, void* data, int n, int inverse);

/* ---- convolvers (include/convolution.hh) ------------------------------- */
typedef struct {
  mf_grid* grid; /* k-space input field */
  int kind;      /* MF_OPND_* */
  int d[4];      /* directions a, b, c, d */
} mf_operand;

/* OrszagConvolver / NaiveConvolver ctor (convolution.hh:463-495, 318-323) */
int mf_conv_create(mf_ctx* ctx, int n, double boxlen, int prec, int kind, mf_conv** out);
int mf_conv_destroy(mf_conv* cv);
/* convolve2 (convolution.hh:513-535 / 328-356) with output operator op
 * applied to out (x is the multiply_add_to factor) */
int mf_conv_convolve2(mf_conv* cv, const mf_operand* a, const mf_operand* b, mf_grid* out, int op, double x);
/* convolve3 (convolution.hh:543-549 / 359-402) */
int mf_conv_convolve3(mf_conv* cv, const mf_operand* a, const mf_operand* b, const mf_operand* c,
                      mf_grid* out, int op, double x);
/* convolve2 followed by apply_InverseLaplacian of out, fused (the last
 * source term of phi(2), phi(3), A(3); src/ic_generator.cc:488,528,545) */
int mf_conv_convolve2_invlap(mf_conv* cv, const mf_operand* a, const mf_operand* b, mf_grid* out, int op,
                             double x);

/* Orszag 3/2 convolve2 that allocates nothing -- no counterpart in the
 * reference.  For callers that cannot allocate device memory: a simulation
 * code embedding the generator whose memory pool already owns the device, or
 * host code that must not incur the implicit synchronisation of
 * cudaMalloc/cudaFree.  Inputs and output are caller-owned device arrays in
 * the k-space layout of an n-grid (n x n x (n/2+1) complex of the given
 * precision); the padded work buffers live in one static 48 MiB device array
 * that the library holds on every device it is loaded on, which limits this
 * call to n <= 128 (FP32) and n <= 96 (FP64); larger sizes return
 * MF_ERR_SHAPE.  All calls share the array, so calls that overlap on the
 * GPU race.  The call synchronises the stream and reads the device error flag
 * before it returns (the result is then complete; MF_ERR_TIMEOUT if a bounded
 * wait ran out), so it cannot be recorded into a CUDA graph.  kind_a /
 * kind_b are MF_OPND_* with directions dirs_a / dirs_b (4 ints each), op is
 * MF_OP_* applied to out with factor x. */
int mf_conv_convolve2_noalloc(void* stream, int n, double boxlen, int prec, const void* field_a, int kind_a,
                              const int* dirs_a, const void* field_b, int kind_b, const int* dirs_b, void* out,
                              int op, double x);

#ifdef __cplusplus
}
#endif
#endif /* MONOFONIC_GB300_H */
