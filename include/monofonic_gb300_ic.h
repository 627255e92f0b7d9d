/*
 * monofonic_gb300_ic.h -- C ABI of the initial-condition level of libmfgpu:
 * host cosmology scalars, the white-noise plugin, the LPT pipeline of
 * ic_generator::run and particle/field assembly.
 *
 * Each declaration names the reference interface it replaces (paths relative
 * to the monofonIC source tree).  Status codes are those of
 * monofonic_gb300.h.
 */
#ifndef MONOFONIC_GB300_IC_H
#define MONOFONIC_GB300_IC_H

#include <stddef.h>
#include <stdint.h>

#include "monofonic_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- cosmology (include/cosmology_parameters.hh:84-196,
 *      include/cosmology_calculator.hh:166-463) ---------------------------- */
typedef struct {
  double Omega_m, Omega_b, h, sigma_8, n_s;
  double Omega_L;    /* < 0: default set (Planck2018EE+BAO+SN) value      */
  double Tcmb;       /* <= 0: 2.7255                                       */
  double m_nu1;      /* < 0: 0.06 eV                                       */
  double N_ur;       /* < 0: 3.046 - number of massive species             */
  double w_0, w_a;   /* dark energy, -1 and 0 for a cosmological constant */
  int zero_radiation;
} mf_cosmo_params;

typedef struct {
  double Dplus;      /* get_growth_factor(a_start)          (:334-337) */
  double vfac;       /* get_vfact(a_start)                  (:360-363) */
  double f;          /* dlog D+ / dlog a at a_start                    */
  double pnorm;      /* (sigma_8 / sigma_8,measured)^2      (:458-463) */
  double sigma8_measured;
  double n_s, h, H0, Omega_m, Omega_b, Omega_r, Omega_DE, Tcmb;
} mf_cosmo_scalars;

/* fill every field of *p with the Planck2018EE+BAO+SN set
 * (src/cosmology_parameters.cc:89), the values ParameterSet = none gives the
 * keys a configuration leaves unset (include/cosmology_parameters.hh:84-150);
 * call it first, then set the keys the configuration holds */
void mf_cosmo_params_default(mf_cosmo_params* p);
/* cosmology::calculator ctor + scalars at z_start */
int mf_cosmology_compute(const mf_cosmo_params* p, double zstart, mf_cosmo_scalars* out);
/* TransferFunction_plugin::compute(k, delta_matter) of the eisenstein plugin
 * (src/plugins/transfer_eisenstein.cc:238-242), k in h/Mpc, n values */
int mf_eh_transfer(const mf_cosmo_params* p, const double* k, double* out, size_t n);

/* ---- white noise: RNG plugin (include/random_plugin.hh:26-39) ----------- */
/* i.i.d. N(0,1) float64 on an n^3 grid, cell (i*n+j)*n+k; Philox4x32-10 block
 * p = cell/2 at counter (p_lo, p_hi, 0, 0), key (seed_lo, seed_hi); the two
 * 53-bit integers b1, b2 of the block give u1 = (b1+1/2) 2^-53 and the angle
 * t = 2 pi (b2+1/2) 2^-53, and Box-Muller gives r cos t (even cell) and
 * r sin t (odd cell), r = sqrt(-2 ln u1).  ln, sin and cos are the library's
 * own (IEEE basic operations only), so the host and the device generator
 * (mf_grid_fill_white_noise, mf_ic_set_noise_seed) give the same bits.
 * Host, multithreaded (nthreads <= 0: all hardware threads). */
int mf_white_noise_host(int n, uint64_t seed, double* out, int nthreads);
/* RNG_plugin::Fill_Grid on the device: the same field written into a
 * real-space grid (values rounded to the grid precision); n even */
int mf_grid_fill_white_noise(mf_grid* g, uint64_t seed);

/* ---- LPT pipeline (src/ic_generator.cc:90-948) -------------------------- */
enum { MF_OUT_PARTICLES = 0, MF_OUT_FIELDS = 1 };
/* include/general.hh:71-76 (enum class cosmo_species) */
enum { MF_SPECIES_DM = 0, MF_SPECIES_BARYON, MF_SPECIES_NEUTRINO };
enum { MF_LOC_HOST = 0, MF_LOC_DEVICE = 1 };

typedef struct {
  int ngrid;          /* setup/GridRes                                     */
  double boxlen;      /* setup/BoxLength [Mpc/h]                           */
  double zstart;      /* setup/zstart                                      */
  int lpt_order;      /* setup/LPTorder, 1..3                              */
  int lattice;        /* setup/ParticleLoad, MF_LATTICE_*                  */
  int precision;      /* MF_PREC_F64 plain or MF_PREC_F32 bulk             */
  int convolver;      /* MF_CONV_ORSZAG or MF_CONV_NAIVE                   */
  int fixing;         /* setup/DoFixing                                    */
  int inversion;      /* setup/DoInversion                                 */
  int plt;            /* PLT corrected gradient and growth rate (ENABLE_PLT) */
  mf_cosmo_scalars cosmo; /* D+, vfac, pnorm, n_s, h, Omega_m, Omega_b, Tcmb */
  const double* tk_table; /* optional host table T(k) at k = sqrt(k2)*2pi/L,
                             k2 = 0..3(n/2)^2; NULL: device Eisenstein-Hu   */
  double lunit, vunit;    /* output_plugin::position_unit / velocity_unit   */
  int out_kind;           /* MF_OUT_PARTICLES or MF_OUT_FIELDS              */
  int pos64;              /* output_plugin::has_64bit_reals                 */
  int id64;               /* output_plugin::has_64bit_ids                   */
  int plt_ngrid;          /* PLT mesh size (lattice_gradient ngridself); 0: 64 */
  int per_term_conv;      /* 0: Orszag source terms through shared padded
                             real fields (each operand transformed once);
                             1: one convolution per term as the reference
                             orders them (less device memory) */
  /* two-species ICs (ic_generator.cc:153-166, :608-792): dark matter on the
   * lattice, baryons on the secondary lattice, perturbed particle masses */
  int baryons;            /* setup/DoBaryons (particle output only)          */
  int baryon_vrel;        /* setup/DoBaryonVrel: back-scaled decaying relative
                             velocity mode                                  */
  double munit;           /* output_plugin::mass_unit                       */
  const double* tk_dbc_table; /* optional host tables T_delta_bc(k) and      */
  const double* tk_tbc_table; /* T_theta_bc(k) at k = sqrt(k2)*2pi/L, k2 =
                             0..3(n/2)^2; NULL: zero, as the Eisenstein-Hu
                             plugin returns (transfer_eisenstein.cc:238-240) */
  double Dplus_target;    /* D+ at cosmology/ztarget; 0: 1 (ztarget = 0)     */
} mf_ic_params;

/* Particle container (include/particle_container.hh:29-139): positions and
 * velocities AoS [npart][3] in float or double, ids u32 or u64, particle
 * ip = ishift*n^3 + cell.  For MF_OUT_FIELDS, pos and vel each hold three
 * n^3 float64 grids (dx,dy,dz / vx,vy,vz, row-major i,j,k) and ids is unused. */
typedef struct {
  void* pos;
  void* vel;
  void* ids;
  int64_t npart;
  int location;       /* MF_LOC_HOST or MF_LOC_DEVICE */
  void* mass;         /* per-particle masses (float or double as pos) of a
                         two-species pipeline; unused otherwise          */
} mf_particles;

/* number of particles and output bytes for a parameter set */
int mf_ic_output_size(const mf_ic_params* p, int64_t* npart, size_t* pos_bytes, size_t* vel_bytes,
                      size_t* id_bytes);
/* device bytes the pipeline needs (fields, convolution buffers, particles) */
int mf_ic_device_footprint(const mf_ic_params* p, size_t* bytes);

typedef struct mf_ic mf_ic;
/* allocate the pipeline's device state for a parameter set */
int mf_ic_create(mf_ctx* ctx, const mf_ic_params* p, mf_ic** out);
int mf_ic_destroy(mf_ic* ic);
/* upload the real-space white noise (n^3 float64, host or device pointer);
 * an FP32 pipeline keeps an n^3-double staging buffer from its first host
 * upload on */
int mf_ic_set_noise(mf_ic* ic, const double* noise, int location);
/* generate the white noise on the device from a seed at the start of every
 * run (the generator of mf_white_noise_host; no host field, no upload) */
int mf_ic_set_noise_seed(mf_ic* ic, uint64_t seed);
/* new cosmology scalars for the next run (same grid, box and order): the
 * amplitude table, growth weights and velocity factors are recomputed on the
 * device from a parameter block copied at the start of each run.  Not
 * allowed when the pipeline was created with a tabulated T(k).  Call it only
 * when no run of this pipeline is in flight. */
int mf_ic_set_cosmology(mf_ic* ic, const mf_cosmo_scalars* cosmo);
/* run noise -> phi(1..3), A(3) -> particles or fields into out (device
 * buffers of the ic when out->location is MF_LOC_DEVICE and out->pos is
 * NULL; copies to host buffers when MF_LOC_HOST); synchronous */
int mf_ic_run(mf_ic* ic, mf_particles* out);
/* mf_ic_run into host buffers (out->location MF_LOC_HOST), returning without
 * waiting.  The particles are copied on the pipeline's copy stream as they
 * become final; the context's stream does not wait for those copies, so the
 * next run queued on the pipeline computes its fields while this run's
 * particles are still crossing to the host (the next run writes its particle
 * buffers only after them).  A host noise upload (mf_ic_set_noise) queued
 * after this call likewise overlaps this run.  The host buffers are complete,
 * and the host noise buffers of the queued runs may be reused, once
 * mf_ic_wait (or a synchronous run) returns.  Device errors of the queued
 * runs are reported there.  Runs into host buffers (this call, and
 * mf_ic_run with MF_LOC_HOST) are refused with MF_ERR_STATE while the
 * context's stream is being captured into a CUDA graph: record
 * mf_ic_enqueue instead. */
int mf_ic_run_async(mf_ic* ic, const mf_particles* out);
/* wait for every queued run of the pipeline, its host copies included */
int mf_ic_wait(mf_ic* ic);
/* enqueue the same pipeline on the context's stream and return without
 * waiting; the particles stay in the ic's device buffers (mf_ic_particles).
 * While the stream is being captured into a CUDA graph the work is recorded
 * (requires mf_ic_set_noise_seed); a replay of the graph reruns the pipeline
 * with the seed and cosmology set at replay time. */
int mf_ic_enqueue(mf_ic* ic);
/* device buffers of the particles (location MF_LOC_DEVICE) */
int mf_ic_particles(mf_ic* ic, mf_particles* out);
/* two-species pipelines (p.baryons): run and hand over out[0] = dark matter,
 * out[1] = baryons (nspecies = 2; each as mf_ic_run's out, with masses);
 * mf_ic_run refuses such a pipeline */
int mf_ic_run_species(mf_ic* ic, mf_particles* out, int nspecies);
/* device buffers of one species (MF_SPECIES_DM = 0, MF_SPECIES_BARYON = 1) */
int mf_ic_particles_species(mf_ic* ic, int species, mf_particles* out);
/* bytes of one species' masses (0 without baryons) */
int mf_ic_mass_bytes(const mf_ic_params* p, size_t* bytes);
/* the context (and so the stream) the pipeline runs on */
int mf_ic_context(mf_ic* ic, mf_ctx** out);
/* per-stage device times of the last run in milliseconds:
 * [noise r2c + phi1, phi2, phi3, A3, positions, velocities, ids, d2h] */
int mf_ic_stage_times(const mf_ic* ic, double* ms8);
/* access to the potentials of the last run (k-space grids, unscaled, i.e.
 * before the growth factors of ic_generator.cc:550-563): which = 0 phi,
 * 1 phi2, 2 phi3, 3..5 A3x..z */
int mf_ic_get_potential(mf_ic* ic, int which, mf_grid** out);
/* Grid of the k-space white noise after normalisation (ic_generator.cc:341-346);
 * after mf_ic_run it holds the velocity order sum of the assembly stage */
int mf_ic_get_noise(mf_ic* ic, mf_grid** out);

/* PLT tables of lattice_gradient (include/particle_plt.hh:68-549) on an
 * ng^3 mesh: real parts of D_r, D_theta, D_phi and the growth-rate
 * correction, each ng*ng*(ng/2+1) doubles in k-space order */
int mf_plt_tables(mf_ctx* ctx, int lattice, int ng, double* Dr, double* Dth, double* Dph, double* Dvf);

#ifdef __cplusplus
}
#endif
#endif /* MONOFONIC_GB300_IC_H */
