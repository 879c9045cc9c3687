/* Minimal HDF5 declarations so that the chemtensor reference sources compile
 * without libhdf5. Every function is a stub that reports failure; the DMRG
 * path never calls them (only the MPS file save/load routines do). */
#pragma once
#include <stdint.h>

typedef int64_t hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef int htri_t;

#define H5P_DEFAULT        ((hid_t)0)
#define H5P_DATASET_CREATE ((hid_t)0)
#define H5S_ALL            ((hid_t)0)
#define H5S_SCALAR         0
#define H5F_ACC_RDONLY     0u
#define H5F_ACC_TRUNC      2u
#define H5T_COMPOUND       6
#define H5T_IEEE_F32LE     ((hid_t)0)
#define H5T_IEEE_F64LE     ((hid_t)0)
#define H5T_NATIVE_DOUBLE  ((hid_t)0)
#define H5T_NATIVE_FLOAT   ((hid_t)0)
#define H5T_NATIVE_INT     ((hid_t)0)
#define H5T_STD_I32LE      ((hid_t)0)

hid_t  H5Fcreate();
hid_t  H5Fopen();
herr_t H5Fclose();
hid_t  H5Acreate();
hid_t  H5Aopen();
herr_t H5Aclose();
hid_t  H5Aget_space();
herr_t H5Aread();
herr_t H5Awrite();
hid_t  H5Dcreate();
hid_t  H5Dopen();
herr_t H5Dclose();
hid_t  H5Dget_space();
hid_t  H5Dget_type();
herr_t H5Dread();
herr_t H5Dwrite();
hid_t  H5Pcreate();
herr_t H5Pclose();
herr_t H5Pset_obj_track_times();
hid_t  H5Screate();
hid_t  H5Screate_simple();
herr_t H5Sclose();
int    H5Sget_simple_extent_dims();
int    H5Sget_simple_extent_ndims();
hid_t  H5Tcreate();
herr_t H5Tclose();
htri_t H5Tequal();
herr_t H5Tinsert();
