/* Test infrastructure only: declarations of the HDF5 C API names that the
 * reference's src/file_io.cpp uses, so that file translation unit compiles
 * where libhdf5 is absent and its in-memory hand-off functions
 * (get_energy_spectrum_information_from_prerun_results,
 * get_lattice_from_prerun_results) can be called.  Nothing here reads or
 * writes files: the definitions (oracle/h5stub/h5stub.inc) only report
 * failure, and the file readers and writers that would call them are never
 * called.  Names and argument lists follow the public HDF5 1.14 C API. */
#ifndef WLG_TEST_HDF5_STUB_H_
#define WLG_TEST_HDF5_STUB_H_

#include <cstddef>
#include <sys/types.h>

typedef long long hid_t;
typedef int herr_t;
typedef int htri_t;
typedef bool hbool_t;
typedef unsigned long long hsize_t;

#define H5P_DEFAULT ((hid_t)0)
#define H5S_ALL ((hid_t)0)
#define H5F_ACC_RDONLY 0x0000u
#define H5F_ACC_TRUNC 0x0002u
#define H5P_FILE_ACCESS ((hid_t)1)
#define H5T_NATIVE_SCHAR ((hid_t)2)
#define H5T_NATIVE_UCHAR ((hid_t)3)
#define H5T_NATIVE_ULLONG ((hid_t)4)

extern "C" {
hid_t H5Fcreate(const char* name, unsigned flags, hid_t fcpl, hid_t fapl);
hid_t H5Fopen(const char* name, unsigned flags, hid_t fapl);
herr_t H5Fclose(hid_t file);
hid_t H5Gcreate2(hid_t loc, const char* name, hid_t lcpl, hid_t gcpl, hid_t gapl);
hid_t H5Gopen2(hid_t loc, const char* name, hid_t gapl);
herr_t H5Gclose(hid_t group);
herr_t H5Gget_num_objs(hid_t loc, hsize_t* num_objs);
ssize_t H5Gget_objname_by_idx(hid_t loc, hsize_t idx, char* name, size_t size);
hid_t H5Dcreate2(hid_t loc, const char* name, hid_t type, hid_t space, hid_t lcpl, hid_t dcpl, hid_t dapl);
hid_t H5Dopen2(hid_t loc, const char* name, hid_t dapl);
herr_t H5Dread(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t plist, void* buf);
herr_t H5Dwrite(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t plist, const void* buf);
hid_t H5Dget_space(hid_t dset);
herr_t H5Dclose(hid_t dset);
hid_t H5Screate_simple(int rank, const hsize_t* dims, const hsize_t* maxdims);
int H5Sget_simple_extent_ndims(hid_t space);
int H5Sget_simple_extent_dims(hid_t space, hsize_t* dims, hsize_t* maxdims);
herr_t H5Sclose(hid_t space);
hid_t H5Pcreate(hid_t cls);
herr_t H5Pset_fapl_core(hid_t fapl, size_t increment, hbool_t backing_store);
htri_t H5Lexists(hid_t loc, const char* name, hid_t lapl);
herr_t H5Ldelete(hid_t loc, const char* name, hid_t lapl);
}

/* the API's version-dispatch names */
#define H5Gopen H5Gopen2
#define H5Dopen H5Dopen2
#define H5Dcreate H5Dcreate2

#endif
