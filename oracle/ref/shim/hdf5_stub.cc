// Failing HDF5 entry points behind hdf5.h (oracle/_ref only; see the header).
#include "hdf5.h"

extern "C" {
hid_t H5Fopen(const char*, unsigned, hid_t) { return -1; }
hid_t H5Fcreate(const char*, unsigned, hid_t, hid_t) { return -1; }
herr_t H5Fclose(hid_t) { return -1; }
hid_t H5Dopen(hid_t, const char*) { return -1; }
hid_t H5Dcreate2(hid_t, const char*, hid_t, hid_t, hid_t, hid_t, hid_t) { return -1; }
herr_t H5Dread(hid_t, hid_t, hid_t, hid_t, hid_t, void*) { return -1; }
herr_t H5Dwrite(hid_t, hid_t, hid_t, hid_t, hid_t, const void*) { return -1; }
hid_t H5Dget_space(hid_t) { return -1; }
herr_t H5Dclose(hid_t) { return -1; }
hid_t H5Screate_simple(int, const hsize_t*, const hsize_t*) { return -1; }
herr_t H5Sselect_hyperslab(hid_t, H5S_seloper_t, const hsize_t*, const hsize_t*, const hsize_t*, const hsize_t*) {
  return -1;
}
int H5Sget_simple_extent_ndims(hid_t) { return -1; }
int H5Sget_simple_extent_dims(hid_t, hsize_t*, hsize_t*) { return -1; }
herr_t H5Sclose(hid_t) { return -1; }
hid_t H5Pcreate(hid_t) { return -1; }
herr_t H5Pclose(hid_t) { return -1; }
herr_t H5Eget_auto(herr_t (**func)(void*), void** client_data) {
  if (func) *func = nullptr;
  if (client_data) *client_data = nullptr;
  return 0;
}
herr_t H5Eset_auto(herr_t (*)(void*), void*) { return 0; }
}
