/* Type names from HDF5 that the EPREM reference headers mention, so that the
 * hot-path sources compile into the oracle library.  No HDF5 file is read by
 * the oracle.  Test infrastructure, not part of the product. */
#ifndef EPREM_REFSHIM_HDF5_H
#define EPREM_REFSHIM_HDF5_H
#include <stdint.h>
typedef long long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef long long hssize_t;
#define H5F_ACC_RDONLY 0
#define H5P_DEFAULT 0
#define H5S_ALL 0
#define H5T_NATIVE_FLOAT 1
#define H5T_NATIVE_DOUBLE 2
hid_t H5Fopen(const char *, unsigned, hid_t);
herr_t H5Fclose(hid_t);
hid_t H5Dopen2(hid_t, const char *, hid_t);
herr_t H5Dclose(hid_t);
hid_t H5Dget_type(hid_t);
hid_t H5Dget_space(hid_t);
int H5Tequal(hid_t, hid_t);
herr_t H5Tclose(hid_t);
herr_t H5Sclose(hid_t);
hssize_t H5Sget_simple_extent_npoints(hid_t);
herr_t H5Dread(hid_t, hid_t, hid_t, hid_t, hid_t, void *);
#endif
