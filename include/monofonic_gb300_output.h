/* Output plugins of the field pipeline: the GRAFIC-2 / RAMSES field writer.
 *
 * Replaces src/plugins/output_grafic2.cc (class grafic2_output_plugin, registered
 * as "grafic2"), the one output format of the reference that needs no external
 * library (the HDF5 and GenericIO formats need the HDF5 and GenericIO
 * libraries, which this library does not link).  The writer takes a real-space field on the device, transposes it to
 * the file's plane order and converts it to float on the GPU, and streams the
 * planes through two page-locked staging buffers, so the copy of one chunk of
 * planes overlaps the file write of the previous one.
 *
 * File layout (output_grafic2.cc:186-236): one file per component,
 * `<dirname>/ic_{pos,vel}{c,b,n}{x,y,z}` / `ic_delta{c,b,n}` / `ic_mass{c,b,n}`,
 * holding Fortran unformatted records: the 44-byte header record
 * {n1,n2,n3 int32; dxini0, xoff10, xoff20, xoff30, astart0, omega_m0, omega_l0,
 * h00 float32}, then ngrid plane records of ngrid^2 float32, plane index = the
 * field's third index, in-plane offset = j*ngrid + i.  Every record is framed by
 * its byte count as uint32 before and after.
 */
#ifndef MONOFONIC_GB300_OUTPUT_H
#define MONOFONIC_GB300_OUTPUT_H

#include "monofonic_gb300.h"
#include "monofonic_gb300_ic.h"

#ifdef __cplusplus
extern "C" {
#endif

/* include/general.hh:60-70 (enum class fluid_component); the species enum
 * is in monofonic_gb300_ic.h */
enum {
  MF_FC_DENSITY = 0, MF_FC_VX, MF_FC_VY, MF_FC_VZ, MF_FC_DX, MF_FC_DY, MF_FC_DZ, MF_FC_MASS
};
/* include/output_plugin.hh:30 (enum class output_type) */
enum { MF_OUTTYPE_PARTICLES = 0, MF_OUTTYPE_FIELD_LAGRANGIAN, MF_OUTTYPE_FIELD_EULERIAN };

typedef struct {
  const char* dirname;  /* [output] filename: the output directory            */
  int ngrid;            /* setup/GridRes, a power of two                       */
  double boxlen;        /* setup/BoxLength [Mpc/h]                             */
  double zstart;        /* setup/zstart                                        */
  double H0;            /* cosmology H0 [km/s/Mpc]                             */
  double Omega_m, Omega_DE, Omega_b;
  int baryons;          /* setup/baryons: "hydro" in the RAMSES namelist       */
  int ramses_nml;       /* [output] ramses_nml (the reference's default is 1)  */
  int use_spt;          /* [output] grafic_use_SPT                             */
  int chunk_planes;     /* planes per staging chunk; 0 picks ~64 MiB chunks    */
} mf_grafic2_params;

typedef struct mf_grafic2 mf_grafic2;

/* constructor (output_grafic2.cc:60-115): checks ngrid is a power of two
 * (MF_ERR_ARG otherwise, where the reference aborts), removes an empty
 * directory of that name, creates the directory, writes ramses.nml */
int mf_grafic2_create(mf_ctx* ctx, const mf_grafic2_params* p, mf_grafic2** out);
int mf_grafic2_destroy(mf_grafic2* w);
/* write_species_as / has_64bit_reals / has_64bit_ids / position_unit /
 * velocity_unit / mass_unit (output_grafic2.cc:117-135) */
int mf_grafic2_info(const mf_grafic2* w, int species, int* write_as, int* has64reals, int* has64ids,
                    double* lunit, double* vunit, double* munit);
/* write_grid_data (output_grafic2.cc:186-246) of a real-space grid; a
 * component the plugin ignores (dm density; baryon dx/dy/dz/mass) writes
 * nothing and returns MF_OK */
int mf_grafic2_write_grid(mf_grafic2* w, mf_grid* g, int species, int component);
/* the same for a compact n^3 field (row-major i,j,k) of float64 or float32
 * (prec) at a device or page-locked/pageable host address (location) */
int mf_grafic2_write_field(mf_grafic2* w, const void* field, int prec, int location, int species,
                           int component);
/* ic_generator.cc:608-948 with this plugin: run the pipeline (created with
 * out_kind MF_OUT_FIELDS and the plugin's position/velocity units) and write
 * dx, dy, dz, vx, vy, vz of the dark matter (field_lagrangian); with baryons
 * (munit = the plugin's 1/Omega_m) also the dark matter's mass field and the
 * baryons' density and vx, vy, vz from the semiclassical Eulerian branch */
int mf_ic_write_grafic2(mf_ic* ic, mf_grafic2* w);
/* the last write call: bytes written to files, milliseconds of the device
 * plane-transpose launches (CUDA events on the context's stream) and of the
 * whole call on the host clock (for mf_ic_write_grafic2: the six writes after
 * the pipeline run) */
int mf_grafic2_last_write(const mf_grafic2* w, size_t* bytes, double* kernel_ms, double* wall_ms);

#ifdef __cplusplus
}
#endif

#endif
