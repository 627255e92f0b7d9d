// A host-memory fake of the grid / convolver part of the C ABI, for testing
// the C++ adapter (include/monofonic_gb300.hpp) without a GPU: grids are
// host arrays, transforms only flip the space flag, and the convolver
// records the operands, output operator and factor of its last call.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "monofonic_gb300.h"

struct mf_ctx {
  std::string err;
  int live = 0;
};
struct mf_grid {
  mf_ctx* ctx;
  int n, prec, space;
  double boxlen;
  std::vector<unsigned char> data;
  double scale = 1.0;
  int dc_zeroed = 0, invlap = 0, shifted = 0;
};
struct mf_conv {
  mf_ctx* ctx;
  int n, prec, kind;
};

extern "C" {
// the convolver's last call, read by the test program
mf_operand fake_last_opnd[3];
int fake_last_nopnd = 0, fake_last_op = -1, fake_last_invlap = 0;
double fake_last_x = 0;
mf_grid* fake_last_out = nullptr;

int mf_ctx_create(int device, mf_ctx** out) {
  if (device != 0) return MF_ERR_ARG;
  *out = new mf_ctx();
  return MF_OK;
}
int mf_ctx_destroy(mf_ctx* c) {
  if (!c) return MF_ERR_ARG;
  if (c->live) return MF_ERR_STATE;
  delete c;
  return MF_OK;
}
const char* mf_last_error(const mf_ctx* c) { return c ? c->err.c_str() : "null context"; }
int mf_ctx_synchronize(mf_ctx* c) { return c ? MF_OK : MF_ERR_ARG; }

int mf_grid_create(mf_ctx* c, int n, double boxlen, int prec, int space, mf_grid** out) {
  if (n != 16 && n != 32) {
    c->err = "mf_grid_create: unsupported grid size " + std::to_string(n);
    return MF_ERR_SHAPE;
  }
  mf_grid* g = new mf_grid();
  g->ctx = c;
  g->n = n;
  g->prec = prec;
  g->space = space;
  g->boxlen = boxlen;
  g->data.assign(size_t(n + 2) * n * n * (prec == MF_PREC_F64 ? 8 : 4), 0);
  ++c->live;
  *out = g;
  return MF_OK;
}
int mf_grid_destroy(mf_grid* g) {
  --g->ctx->live;
  delete g;
  return MF_OK;
}
int mf_grid_info(const mf_grid* g, int* n, int* prec, int* space, void** dptr, size_t* bytes) {
  if (n) *n = g->n;
  if (prec) *prec = g->prec;
  if (space) *space = g->space;
  if (dptr) *dptr = const_cast<unsigned char*>(g->data.data());
  if (bytes) *bytes = g->data.size();
  return MF_OK;
}
int mf_grid_upload(mf_grid* g, const void* host, int space) {
  std::memcpy(g->data.data(), host, g->data.size());
  g->space = space;
  return MF_OK;
}
int mf_grid_download(mf_grid* g, void* host) {
  std::memcpy(host, g->data.data(), g->data.size());
  return MF_OK;
}
int mf_grid_fill_real64(mf_grid* g, const double* x) {
  const int n = g->n;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k) {
        const size_t src = (size_t(i) * n + j) * n + k, dst = (size_t(i) * n + j) * (n + 2) + k;
        if (g->prec == MF_PREC_F64) reinterpret_cast<double*>(g->data.data())[dst] = x[src];
        else reinterpret_cast<float*>(g->data.data())[dst] = float(x[src]);
      }
  g->space = MF_SPACE_R;
  return MF_OK;
}
int mf_grid_fft_forward(mf_grid* g, int do_transform) {
  if (do_transform) g->space = MF_SPACE_K;
  return MF_OK;
}
int mf_grid_fft_backward(mf_grid* g, int do_transform) {
  if (do_transform) g->space = MF_SPACE_R;
  return MF_OK;
}
int mf_grid_zero(mf_grid* g) {
  std::fill(g->data.begin(), g->data.end(), 0);
  return MF_OK;
}
int mf_grid_scale(mf_grid* g, double x) {
  g->scale *= x;
  return MF_OK;
}
int mf_grid_zero_dc(mf_grid* g) {
  g->dc_zeroed = 1;
  return MF_OK;
}
int mf_grid_inverse_laplacian(mf_grid* g) {
  g->invlap = 1;
  return MF_OK;
}
int mf_grid_shift(mf_grid* g, const double s[3], int transform_back) {
  g->shifted = (s[0] == 0.5 && s[1] == 0.25 && s[2] == 0.0 && transform_back == 0) ? 1 : -1;
  return MF_OK;
}
int mf_grid_power_spectrum(mf_grid*, double* bk, double* bP, double* beP, int64_t* cnt, int cap, int* nb) {
  for (int i = 0; i < 3 && i < cap; ++i) {
    bk[i] = i + 1;
    bP[i] = 10.0 * (i + 1);
    beP[i] = 0.5;
    cnt[i] = 6 * (i + 1);
  }
  *nb = 3;
  return MF_OK;
}
int mf_grid_write_power_spectrum(mf_grid* g, const char* path) {
  if (!path || !*path) {
    g->ctx->err = "mf_grid_write_power_spectrum: cannot open ''";
    return MF_ERR_IO;
  }
  return MF_OK;
}
int mf_copy_to_host(void* host, const void* dev, size_t bytes) {
  std::memcpy(host, dev, bytes);
  return MF_OK;
}

int mf_conv_create(mf_ctx* c, int n, double, int prec, int kind, mf_conv** out) {
  *out = new mf_conv{c, n, prec, kind};
  return MF_OK;
}
int mf_conv_destroy(mf_conv* cv) {
  delete cv;
  return MF_OK;
}
static int record(const mf_operand* a, const mf_operand* b, const mf_operand* c, mf_grid* out, int op, double x,
                  int invlap) {
  fake_last_opnd[0] = *a;
  fake_last_opnd[1] = *b;
  if (c) fake_last_opnd[2] = *c;
  fake_last_nopnd = c ? 3 : 2;
  fake_last_out = out;
  fake_last_op = op;
  fake_last_x = x;
  fake_last_invlap = invlap;
  return MF_OK;
}
int mf_conv_convolve2(mf_conv*, const mf_operand* a, const mf_operand* b, mf_grid* out, int op, double x) {
  return record(a, b, nullptr, out, op, x, 0);
}
int mf_conv_convolve3(mf_conv*, const mf_operand* a, const mf_operand* b, const mf_operand* c, mf_grid* out, int op,
                      double x) {
  return record(a, b, c, out, op, x, 0);
}
int mf_conv_convolve2_invlap(mf_conv*, const mf_operand* a, const mf_operand* b, mf_grid* out, int op, double x) {
  return record(a, b, nullptr, out, op, x, 1);
}
}
