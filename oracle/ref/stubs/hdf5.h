/* Declaration-only stand-in for <hdf5.h>, used only to compile the reference
 * unbinding sources into the oracle/_ref harness.  No HDF5 routine is reached
 * by Subhalo_t::Unbind; the inline helpers in the reference's hdf_wrapper.h
 * need these names to parse.  Test infrastructure only. */
#ifndef HBTU_STUB_HDF5_H
#define HBTU_STUB_HDF5_H
typedef long hid_t;
typedef unsigned long long hsize_t;
typedef int herr_t;
#define H5T_NATIVE_FLOAT 1
#define H5T_NATIVE_DOUBLE 2
#define H5T_NATIVE_INT 3
#define H5T_NATIVE_LONG 4
#define H5S_ALL 0
#define H5P_DEFAULT 0
hid_t H5Dget_space(hid_t);
int H5Sget_simple_extent_dims(hid_t, hsize_t *, hsize_t *);
herr_t H5Sclose(hid_t);
herr_t H5Dvlen_reclaim(hid_t, hid_t, hid_t, void *);
hid_t H5Dopen2(hid_t, const char *, hid_t);
herr_t H5Dread(hid_t, hid_t, hid_t, hid_t, hid_t, void *);
long H5Iget_name(hid_t, char *, unsigned long);
long H5Fget_name(hid_t, char *, unsigned long);
herr_t H5Dclose(hid_t);
hid_t H5Aopen_by_name(hid_t, const char *, const char *, hid_t, hid_t);
herr_t H5Aread(hid_t, hid_t, void *);
herr_t H5Aclose(hid_t);
herr_t H5Tclose(hid_t);
#endif
