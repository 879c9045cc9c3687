/* Failure-returning bodies for the HDF5 declarations in hdf5.h. */
#include "hdf5.h"
#define STUB(ret, name) ret name() { return (ret)-1; }
STUB(hid_t, H5Fcreate) STUB(hid_t, H5Fopen) STUB(herr_t, H5Fclose)
STUB(hid_t, H5Acreate) STUB(hid_t, H5Aopen) STUB(herr_t, H5Aclose) STUB(hid_t, H5Aget_space)
STUB(herr_t, H5Aread) STUB(herr_t, H5Awrite)
STUB(hid_t, H5Dcreate) STUB(hid_t, H5Dopen) STUB(herr_t, H5Dclose) STUB(hid_t, H5Dget_space)
STUB(hid_t, H5Dget_type) STUB(herr_t, H5Dread) STUB(herr_t, H5Dwrite)
STUB(hid_t, H5Pcreate) STUB(herr_t, H5Pclose) STUB(herr_t, H5Pset_obj_track_times)
STUB(hid_t, H5Screate) STUB(hid_t, H5Screate_simple) STUB(herr_t, H5Sclose)
STUB(int, H5Sget_simple_extent_dims) STUB(int, H5Sget_simple_extent_ndims)
STUB(hid_t, H5Tcreate) STUB(herr_t, H5Tclose) STUB(htri_t, H5Tequal) STUB(herr_t, H5Tinsert)
