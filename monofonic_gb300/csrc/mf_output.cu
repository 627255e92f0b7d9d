// GRAFIC-2 / RAMSES field writer (src/plugins/output_grafic2.cc).
//
// The reference fills one ngrid^2 float plane at a time on the host
// (output_grafic2.cc:219-236: plane index = the grid's third index, in-plane
// offset j*ngrid + i) and writes it as a Fortran record.  Here one kernel
// launch turns a chunk of planes of the device field into the exact bytes of
// the file — the transposed planes converted to float with their record
// markers — and the chunks stream to the file through two page-locked staging
// buffers: the copy of chunk c+1 runs while the host writes chunk c.
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/monofonic_gb300_output.h"
#include "mf_runtime.h"

namespace mf {
const mf_ic_params* ic_params(const mf_ic* ic);
}

namespace {

// output_grafic2.cc:38-43, written as one 44-byte record
struct GraficHeader {
  int32_t n1, n2, n3;
  float dxini0;
  float xoff10, xoff20, xoff30;
  float astart0, omega_m0, omega_l0, h00;
};
static_assert(sizeof(GraficHeader) == 44, "grafic header is 44 bytes");

// One chunk of nz planes starting at plane z0.  Record zl of the chunk is
// rec = n^2 + 2 words: [4 n^2][plane: word 1 + j*n + i = f(i, j, z0+zl)][4 n^2].
// Block (32 x 8 threads) = a 32 (i) x 32 (z) tile at one j, transposed through
// shared memory: loads run along z (contiguous in the field), stores along i
// (contiguous in the plane).
template <typename T>
__global__ void __launch_bounds__(256) k_grafic_planes(const T* __restrict__ f, size_t row_stride, int n, int z0,
                                                       int nz, uint32_t* __restrict__ out) {
  __shared__ float tile[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = blockIdx.x * 32, zt = blockIdx.y * 32, j = blockIdx.z;
  const size_t rec = (size_t)n * n + 2;
#pragma unroll
  for (int r = 0; r < 32; r += 8) {
    const int i = i0 + ty + r, zl = zt + tx;
    if (i < n && zl < nz) tile[ty + r][tx] = (float)f[((size_t)i * n + j) * row_stride + (size_t)(z0 + zl)];
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 32; r += 8) {
    const int zl = zt + ty + r, i = i0 + tx;
    if (zl < nz && i < n) out[(size_t)zl * rec + 1 + (size_t)j * n + i] = __float_as_uint(tile[tx][ty + r]);
  }
  if (blockIdx.x == 0 && j == 0 && ty == 0) {
    const int zl = zt + tx;
    if (zl < nz) {
      const uint32_t m = (uint32_t)(4ull * n * n);
      out[(size_t)zl * rec] = m;
      out[(size_t)zl * rec + rec - 1] = m;
    }
  }
}

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

bool write_all(int fd, const void* buf, size_t bytes) {
  const char* p = static_cast<const char*>(buf);
  while (bytes) {
    const ssize_t w = ::write(fd, p, bytes);
    if (w < 0) {
      if (errno == EINTR) continue;
      return false;
    }
    p += w;
    bytes -= (size_t)w;
  }
  return true;
}

}  // namespace

struct mf_grafic2 {
  mf_ctx* c = nullptr;
  mf_grafic2_params p{};
  std::string dir;
  GraficHeader hdr{};
  unsigned levelmin = 0;
  int planes = 1;      // planes per staging chunk
  size_t chunk_words = 0;
  uint32_t* dbuf[2] = {};
  uint32_t* hbuf[2] = {};
  cudaEvent_t done[2] = {}, k0[2] = {}, k1[2] = {};
  size_t last_bytes = 0;
  double last_kernel_ms = 0, last_wall_ms = 0;
};

namespace {

using mf::cuda_err;
using mf::set_err;

// file name of a component (output_grafic2.cc:139-184)
std::string grafic_file_name(const mf_grafic2* w, int species, int component) {
  static const char* sp[] = {"c", "b", "n"};
  const std::string s = sp[species];
  std::string f = w->dir + "/ic_";
  switch (component) {
    case MF_FC_DENSITY: return f + "delta" + s;
    case MF_FC_VX: return f + "vel" + s + "x";
    case MF_FC_VY: return f + "vel" + s + "y";
    case MF_FC_VZ: return f + "vel" + s + "z";
    case MF_FC_DX: return f + "pos" + s + "x";
    case MF_FC_DY: return f + "pos" + s + "y";
    case MF_FC_DZ: return f + "pos" + s + "z";
    default: return f + "mass" + s;
  }
}

// components the plugin does not write (output_grafic2.cc:189-193)
bool grafic_ignores(int species, int component) {
  if (species == MF_SPECIES_DM && component == MF_FC_DENSITY) return true;
  if (species == MF_SPECIES_BARYON && (component == MF_FC_DX || component == MF_FC_DY || component == MF_FC_DZ ||
                                       component == MF_FC_MASS))
    return true;
  return false;
}

// RAMSES namelist (output_grafic2.cc:249-320)
bool write_namelist(const mf_grafic2* w) {
  const std::string fn = w->dir + "/ramses.nml";
  FILE* fp = std::fopen(fn.c_str(), "w");
  if (!fp) return false;
  const unsigned naddref = 5;
  int ok = 1;
  ok &= std::fprintf(fp,
                     "&RUN_PARAMS\ncosmo=.true.\npic=.true.\npoisson=.true.\n%s\n"
                     "nrestart=0\nnremap=1\nnsubcycle=1,2\nncontrol=1\nverbose=.false.\n/\n\n",
                     w->p.baryons ? "hydro=.true." : "hydro=.false.") > 0;
  ok &= std::fprintf(fp, "&INIT_PARAMS\nfiletype='grafic'\nomega_b=%g\ninitfile(1)='%s'\n/\n\n", w->p.Omega_b,
                     w->dir.c_str()) > 0;
  ok &= std::fprintf(fp, "&AMR_PARAMS\nlevelmin=%u\nlevelmax=%u\nnexpand=1\nngridmax=2000000\nnpartmax=3000000\n/\n\n",
                     w->levelmin, w->levelmin + naddref) > 0;
  ok &= std::fprintf(fp, "&REFINE_PARAMS\nm_refine=%u*8.,\n/\n", 1 + naddref) > 0;
  ok &= std::fclose(fp) == 0;
  return ok != 0;
}

// one component file from a device field (row stride in elements: n for a
// compact field, n+2 for a real-space grid)
int write_component(mf_grafic2* w, const void* dfield, int prec, size_t row_stride, const std::string& fname,
                    size_t* bytes_out, double* kernel_ms) {
  mf_ctx* c = w->c;
  cudaStream_t s = c->stream;
  const int n = w->p.ngrid;
  const size_t rec = (size_t)n * n + 2;
  ::unlink(fname.c_str());
  const int fd = ::open(fname.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
  if (fd < 0) return set_err(c, MF_ERR_IO, "grafic2: cannot create " + fname + ": " + std::strerror(errno));
  unsigned char head[52];
  const uint32_t hb = sizeof(GraficHeader);
  std::memcpy(head, &hb, 4);
  std::memcpy(head + 4, &w->hdr, sizeof(GraficHeader));
  std::memcpy(head + 48, &hb, 4);
  bool ok = write_all(fd, head, sizeof head);
  size_t bytes = sizeof head;
  const int P = w->planes;
  const int nch = (n + P - 1) / P;
  cudaError_t e = cudaSuccess;
  auto issue = [&](int ch) -> cudaError_t {
    const int b = ch & 1, z0 = ch * P, nz = std::min(P, n - z0);
    cudaError_t e2 = cudaEventRecord(w->k0[b], s);
    if (e2 != cudaSuccess) return e2;
    {
      mf::LaunchScope ls(c, mf::KK_POINTWISE);
      const dim3 grid((unsigned)((n + 31) / 32), (unsigned)((nz + 31) / 32), (unsigned)n), block(32, 8);
      if (prec == MF_PREC_F64)
        k_grafic_planes<double><<<grid, block, 0, s>>>((const double*)dfield, row_stride, n, z0, nz, w->dbuf[b]);
      else
        k_grafic_planes<float><<<grid, block, 0, s>>>((const float*)dfield, row_stride, n, z0, nz, w->dbuf[b]);
      e2 = cudaGetLastError();
    }
    if (e2 == cudaSuccess) e2 = cudaEventRecord(w->k1[b], s);
    if (e2 == cudaSuccess)
      e2 = cudaMemcpyAsync(w->hbuf[b], w->dbuf[b], (size_t)nz * rec * 4, cudaMemcpyDeviceToHost, s);
    if (e2 == cudaSuccess) e2 = cudaEventRecord(w->done[b], s);
    return e2;
  };
  for (int ch = 0; ch < std::min(nch, 2) && ok && e == cudaSuccess; ++ch) e = issue(ch);
  for (int ch = 0; ch < nch && ok && e == cudaSuccess; ++ch) {
    const int b = ch & 1, nz = std::min(P, n - ch * P);
    e = cudaEventSynchronize(w->done[b]);
    if (e != cudaSuccess) break;
    float t = 0;
    if (cudaEventElapsedTime(&t, w->k0[b], w->k1[b]) == cudaSuccess) *kernel_ms += t;
    else cudaGetLastError();  // timing only: not an error of a later call
    ok = write_all(fd, w->hbuf[b], (size_t)nz * rec * 4);
    bytes += (size_t)nz * rec * 4;
    if (ok && ch + 2 < nch) e = issue(ch + 2);
  }
  // copies still in flight read the staging buffers: wait before returning
  const cudaError_t es = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = es;
  const int cl = ::close(fd);
  if (e != cudaSuccess) return cuda_err(c, e, "grafic2: plane transpose / copy");
  if (!ok || cl != 0) return set_err(c, MF_ERR_IO, "grafic2: write failed on " + fname + ": " + std::strerror(errno));
  *bytes_out += bytes;
  return MF_OK;
}

void release(mf_grafic2* w) {
  for (int b = 0; b < 2; ++b) {
    if (w->dbuf[b]) cudaFree(w->dbuf[b]);
    if (w->hbuf[b]) cudaFreeHost(w->hbuf[b]);
    for (cudaEvent_t ev : {w->done[b], w->k0[b], w->k1[b]})
      if (ev) cudaEventDestroy(ev);
  }
}

int check_target(mf_grafic2* w, int species, int component) {
  if (species < MF_SPECIES_DM || species > MF_SPECIES_NEUTRINO || component < MF_FC_DENSITY || component > MF_FC_MASS)
    return set_err(w->c, MF_ERR_ARG, "grafic2: bad species or component");
  return MF_OK;
}

}  // namespace

extern "C" int mf_grafic2_create(mf_ctx* c, const mf_grafic2_params* p, mf_grafic2** out) {
  if (!c || !p || !out) return MF_ERR_ARG;
  *out = nullptr;
  if (!p->dirname || !*p->dirname) return set_err(c, MF_ERR_ARG, "grafic2: no output directory");
  if (!is_pow2(p->ngrid) || p->ngrid < 2)
    return set_err(c, MF_ERR_ARG, "grafic2: RAMSES requires setup/GridRes to be power of 2");
  if (!(p->boxlen > 0) || !(p->H0 > 0) || !(p->zstart >= 0)) return set_err(c, MF_ERR_ARG, "grafic2: bad box or cosmology");
  if (p->chunk_planes < 0) return set_err(c, MF_ERR_ARG, "grafic2: negative chunk_planes");
  cudaSetDevice(c->device);
  mf_grafic2* w = new (std::nothrow) mf_grafic2();
  if (!w) return MF_ERR_OOM;
  w->c = c;
  w->p = *p;
  w->dir = p->dirname;
  w->p.dirname = nullptr;  // the string is owned by w->dir
  const int n = p->ngrid;
  w->levelmin = (unsigned)std::lround(std::log2((double)n));
  // output_grafic2.cc:88-98 (double expressions rounded to the float fields)
  w->hdr.n1 = w->hdr.n2 = w->hdr.n3 = n;
  w->hdr.dxini0 = (float)(p->boxlen / (p->H0 * 0.01) / n);
  w->hdr.xoff10 = w->hdr.xoff20 = w->hdr.xoff30 = 0.0f;
  w->hdr.astart0 = (float)(1.0 / (1.0 + p->zstart));
  w->hdr.omega_m0 = (float)p->Omega_m;
  w->hdr.omega_l0 = (float)p->Omega_DE;
  w->hdr.h00 = (float)p->H0;
  const size_t rec_bytes = ((size_t)n * n + 2) * 4;
  int P = p->chunk_planes;
  if (P == 0) P = (int)std::max<size_t>(1, ((size_t)64 << 20) / rec_bytes);
  w->planes = std::min(P, n);
  w->chunk_words = (size_t)w->planes * ((size_t)n * n + 2);
  for (int b = 0; b < 2; ++b) {
    if (cudaMalloc(&w->dbuf[b], w->chunk_words * 4) != cudaSuccess ||
        cudaHostAlloc(&w->hbuf[b], w->chunk_words * 4, cudaHostAllocPortable) != cudaSuccess ||
        cudaEventCreate(&w->done[b]) != cudaSuccess || cudaEventCreate(&w->k0[b]) != cudaSuccess ||
        cudaEventCreate(&w->k1[b]) != cudaSuccess) {
      cudaGetLastError();
      release(w);
      delete w;
      return set_err(c, MF_ERR_OOM, "grafic2: staging buffers");
    }
  }
  // output_grafic2.cc:106-109: remove an empty directory of that name, create it
  ::rmdir(w->dir.c_str());
  ::mkdir(w->dir.c_str(), 0777);
  struct stat st {};
  if (::stat(w->dir.c_str(), &st) != 0 || !S_ISDIR(st.st_mode)) {
    release(w);
    delete w;
    return set_err(c, MF_ERR_IO, "grafic2: cannot create directory " + std::string(p->dirname));
  }
  if (p->ramses_nml && !write_namelist(w)) {
    release(w);
    delete w;
    return set_err(c, MF_ERR_IO, "grafic2: cannot write ramses.nml");
  }
  ++c->children;
  *out = w;
  return MF_OK;
}

extern "C" int mf_grafic2_destroy(mf_grafic2* w) {
  if (!w) return MF_ERR_ARG;
  cudaSetDevice(w->c->device);
  cudaStreamSynchronize(w->c->stream);
  release(w);
  --w->c->children;
  delete w;
  return MF_OK;
}

extern "C" int mf_grafic2_info(const mf_grafic2* w, int species, int* write_as, int* has64reals, int* has64ids,
                               double* lunit, double* vunit, double* munit) {
  if (!w || species < MF_SPECIES_DM || species > MF_SPECIES_NEUTRINO) return MF_ERR_ARG;
  if (write_as)
    *write_as = (species == MF_SPECIES_BARYON && !w->p.use_spt) ? MF_OUTTYPE_FIELD_EULERIAN : MF_OUTTYPE_FIELD_LAGRANGIAN;
  if (has64reals) *has64reals = 0;
  if (has64ids) *has64ids = 0;
  if (lunit) *lunit = w->p.boxlen;
  if (vunit) *vunit = w->p.boxlen;
  if (munit) *munit = 1.0 / w->p.Omega_m;  // RAMSES wants mass in units of critical
  return MF_OK;
}

extern "C" int mf_grafic2_write_grid(mf_grafic2* w, mf_grid* g, int species, int component) {
  if (!w || !g) return MF_ERR_ARG;
  int rc = check_target(w, species, component);
  if (rc) return rc;
  if (g->n != w->p.ngrid) return set_err(w->c, MF_ERR_SHAPE, "grafic2: grid size differs from setup/GridRes");
  if (g->space != MF_SPACE_R) return set_err(w->c, MF_ERR_STATE, "grafic2: grid must be in real space");
  if (g->ctx != w->c) return set_err(w->c, MF_ERR_ARG, "grafic2: grid belongs to another context");
  const auto t0 = std::chrono::steady_clock::now();
  w->last_bytes = 0;
  w->last_kernel_ms = 0;
  if (!grafic_ignores(species, component)) {
    cudaSetDevice(w->c->device);
    rc = write_component(w, g->d, g->prec, (size_t)g->n + 2, grafic_file_name(w, species, component), &w->last_bytes,
                         &w->last_kernel_ms);
  }
  w->last_wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

extern "C" int mf_grafic2_write_field(mf_grafic2* w, const void* field, int prec, int location, int species,
                                      int component) {
  if (!w || !field) return MF_ERR_ARG;
  int rc = check_target(w, species, component);
  if (rc) return rc;
  if (prec != MF_PREC_F64 && prec != MF_PREC_F32) return set_err(w->c, MF_ERR_ARG, "grafic2: bad precision");
  if (location != MF_LOC_HOST && location != MF_LOC_DEVICE) return set_err(w->c, MF_ERR_ARG, "grafic2: bad location");
  const auto t0 = std::chrono::steady_clock::now();
  w->last_bytes = 0;
  w->last_kernel_ms = 0;
  if (!grafic_ignores(species, component)) {
    mf_ctx* c = w->c;
    cudaSetDevice(c->device);
    const int n = w->p.ngrid;
    const size_t bytes = (size_t)n * n * n * mf::prec_size(prec);
    void* d = const_cast<void*>(field);
    void* staged = nullptr;
    if (location == MF_LOC_HOST) {
      cudaError_t e = cudaMallocAsync(&staged, bytes, c->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(staged, field, bytes, cudaMemcpyHostToDevice, c->stream);
      if (e != cudaSuccess) {
        if (staged) cudaFreeAsync(staged, c->stream);
        return cuda_err(c, e, "grafic2: field upload");
      }
      d = staged;
    }
    rc = write_component(w, d, prec, (size_t)n, grafic_file_name(w, species, component), &w->last_bytes,
                         &w->last_kernel_ms);
    if (staged) {
      cudaFreeAsync(staged, c->stream);
      cudaStreamSynchronize(c->stream);
    }
  }
  w->last_wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

extern "C" int mf_ic_write_grafic2(mf_ic* ic, mf_grafic2* w) {
  if (!ic || !w) return MF_ERR_ARG;
  const mf_ic_params* p = mf::ic_params(ic);
  mf_ctx* c = w->c;
  mf_ctx* ic_ctx = nullptr;
  mf_ic_context(ic, &ic_ctx);
  if (ic_ctx != c) return set_err(c, MF_ERR_ARG, "mf_ic_write_grafic2: pipeline and writer use different contexts");
  if (p->out_kind != MF_OUT_FIELDS)
    return set_err(c, MF_ERR_ARG, "mf_ic_write_grafic2: the pipeline must be created with out_kind = MF_OUT_FIELDS");
  if (p->ngrid != w->p.ngrid) return set_err(c, MF_ERR_SHAPE, "mf_ic_write_grafic2: setup/GridRes differs");
  // the plugin's units enter the fields (ic_generator.cc:815, :872-873)
  auto same = [](double a, double b) { return std::fabs(a - b) <= 1e-12 * std::fabs(b); };
  if (!same(p->lunit, w->p.boxlen) || !same(p->vunit, w->p.boxlen))
    return set_err(c, MF_ERR_ARG, "mf_ic_write_grafic2: pipeline units differ from the plugin's position/velocity unit");
  if (p->baryons && w->p.use_spt)
    return set_err(c, MF_ERR_ARG, "mf_ic_write_grafic2: Lagrangian baryon fields (grafic_use_SPT) are not built");
  if (p->baryons && !same(p->munit, 1.0 / w->p.Omega_m))
    return set_err(c, MF_ERR_ARG, "mf_ic_write_grafic2: pipeline mass unit differs from the plugin's (1 / Omega_m)");
  mf_particles dev[2] = {};
  dev[0].location = dev[1].location = MF_LOC_DEVICE;
  int rc = p->baryons ? mf_ic_run_species(ic, dev, 2) : mf_ic_run(ic, &dev[0]);
  if (rc) return rc;
  const auto t0 = std::chrono::steady_clock::now();
  w->last_bytes = 0;
  w->last_kernel_ms = 0;
  const size_t n3 = (size_t)p->ngrid * p->ngrid * p->ngrid;
  // dark matter (field_lagrangian): dx, dy, dz, vx, vy, vz and, with baryons,
  // the mass field; baryons (field_eulerian, ic_generator.cc:766-789): the
  // density and vx, vy, vz
  struct Item { int species, comp; const double* src; };
  Item items[11];
  int ni = 0;
  static const int comp[6] = {MF_FC_DX, MF_FC_DY, MF_FC_DZ, MF_FC_VX, MF_FC_VY, MF_FC_VZ};
  for (int k = 0; k < 6; ++k)
    items[ni++] = {MF_SPECIES_DM, comp[k], (k < 3 ? (const double*)dev[0].pos : (const double*)dev[0].vel) + (size_t)(k % 3) * n3};
  if (p->baryons) {
    items[ni++] = {MF_SPECIES_DM, MF_FC_MASS, (const double*)dev[0].mass};
    items[ni++] = {MF_SPECIES_BARYON, MF_FC_DENSITY, (const double*)dev[1].pos};
    for (int k = 0; k < 3; ++k) items[ni++] = {MF_SPECIES_BARYON, comp[3 + k], (const double*)dev[1].vel + (size_t)k * n3};
  }
  for (int k = 0; k < ni && rc == MF_OK; ++k)
    if (!grafic_ignores(items[k].species, items[k].comp))
      rc = write_component(w, items[k].src, MF_PREC_F64, (size_t)p->ngrid,
                           grafic_file_name(w, items[k].species, items[k].comp), &w->last_bytes, &w->last_kernel_ms);
  w->last_wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

extern "C" int mf_grafic2_last_write(const mf_grafic2* w, size_t* bytes, double* kernel_ms, double* wall_ms) {
  if (!w) return MF_ERR_ARG;
  if (bytes) *bytes = w->last_bytes;
  if (kernel_ms) *kernel_ms = w->last_kernel_ms;
  if (wall_ms) *wall_ms = w->last_wall_ms;
  return MF_OK;
}
