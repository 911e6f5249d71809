/* Declarations-only stand-in for hdf5.h so that the reference's source can be
 * compiled as a library for the oracle (oracle/build_ref.sh). The oracle
 * calls only the reference's tracing functions, never its file readers;
 * every function here fails if called. Not part of the product. */
#pragma once
#include <stdint.h>
typedef int64_t hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef enum { H5T_NO_CLASS = -1, H5T_ARRAY = 10 } H5T_class_t;
#define H5F_ACC_RDONLY 0u
#define H5P_DEFAULT ((hid_t)0)
#define H5S_ALL ((hid_t)0)
#define H5T_NATIVE_FLOAT ((hid_t)0)
static inline hid_t H5Fopen(const char*, unsigned, hid_t) { return -1; }
static inline herr_t H5Fclose(hid_t) { return -1; }
static inline hid_t H5Dopen2(hid_t, const char*, hid_t) { return -1; }
static inline herr_t H5Dclose(hid_t) { return -1; }
static inline hid_t H5Dget_space(hid_t) { return -1; }
static inline hid_t H5Dget_type(hid_t) { return -1; }
static inline herr_t H5Dread(hid_t, hid_t, hid_t, hid_t, hid_t, void*) { return -1; }
static inline int H5Sget_simple_extent_ndims(hid_t) { return -1; }
static inline int H5Sget_simple_extent_dims(hid_t, hsize_t*, hsize_t*) { return -1; }
static inline herr_t H5Sclose(hid_t) { return -1; }
static inline H5T_class_t H5Tget_class(hid_t) { return H5T_NO_CLASS; }
static inline int H5Tget_array_ndims(hid_t) { return -1; }
static inline int H5Tget_array_dims2(hid_t, hsize_t*) { return -1; }
static inline hid_t H5Tarray_create2(hid_t, unsigned, const hsize_t*) { return -1; }
static inline herr_t H5Tclose(hid_t) { return -1; }
