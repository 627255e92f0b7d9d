/*
 * HDF5-API stub for building the reference's own sources without HDF5;
 * test infrastructure for oracle/_ref only.  src/grid_fft.cc defines
 * Grid_FFT::Write_to_HDF5 / Read_from_HDF5 unconditionally; neither is on the
 * initial-condition path (constraints and diagnostic output only).  Every
 * stub call fails (negative return), so a configuration that would need
 * HDF5 stops with the reference's own error handling.
 */
#ifndef MF_REF_HDF5_STUB_H
#define MF_REF_HDF5_STUB_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef int64_t hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef long long hssize_t;
typedef enum { H5S_SELECT_SET = 0 } H5S_seloper_t;
#define H5P_DEFAULT ((hid_t)0)
#define H5S_ALL ((hid_t)0)
#define H5F_ACC_RDONLY 0x0000u
#define H5F_ACC_RDWR 0x0001u
#define H5F_ACC_TRUNC 0x0002u
#define H5P_DATASET_XFER ((hid_t)-10)
#define H5P_FILE_ACCESS ((hid_t)-11)
#define H5P_DATASET_CREATE ((hid_t)-12)
#define H5T_NATIVE_FLOAT ((hid_t)-20)
#define H5T_NATIVE_DOUBLE ((hid_t)-21)
#define H5T_NATIVE_LDOUBLE ((hid_t)-22)
#define H5T_NATIVE_INT ((hid_t)-23)
#define H5T_NATIVE_UINT ((hid_t)-24)
#define H5T_NATIVE_LLONG ((hid_t)-25)
#define H5T_NATIVE_ULLONG ((hid_t)-26)
hid_t H5Fopen(const char* name, unsigned flags, hid_t fapl);
hid_t H5Fcreate(const char* name, unsigned flags, hid_t fcpl, hid_t fapl);
herr_t H5Fclose(hid_t f);
hid_t H5Dopen(hid_t loc, const char* name);
hid_t H5Dcreate2(hid_t loc, const char* name, hid_t type, hid_t space, hid_t lcpl, hid_t dcpl, hid_t dapl);
herr_t H5Dread(hid_t d, hid_t mtype, hid_t mspace, hid_t fspace, hid_t xfer, void* buf);
herr_t H5Dwrite(hid_t d, hid_t mtype, hid_t mspace, hid_t fspace, hid_t xfer, const void* buf);
hid_t H5Dget_space(hid_t d);
herr_t H5Dclose(hid_t d);
hid_t H5Screate_simple(int rank, const hsize_t* dims, const hsize_t* maxdims);
herr_t H5Sselect_hyperslab(hid_t s, H5S_seloper_t op, const hsize_t* start, const hsize_t* stride,
                           const hsize_t* count, const hsize_t* block);
int H5Sget_simple_extent_ndims(hid_t s);
int H5Sget_simple_extent_dims(hid_t s, hsize_t* dims, hsize_t* maxdims);
herr_t H5Sclose(hid_t s);
hid_t H5Pcreate(hid_t cls);
herr_t H5Pclose(hid_t p);
herr_t H5Eget_auto(herr_t (**func)(void*), void** client_data);
herr_t H5Eset_auto(herr_t (*func)(void*), void* client_data);
#ifdef __cplusplus
}
#endif
#endif
