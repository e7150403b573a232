/*
 * TEST INFRASTRUCTURE ONLY.  Stand-in for the HDF5 1.8 C API so that the
 * reference's channel/*.c compiles as the CPU oracle.  HDF5 is not installed;
 * every call prints a message and fails (returns -1).  Only the reference's
 * restart/save code reaches these, and no oracle test uses it.
 */
#ifndef ORACLE_SHIM_HDF5_H
#define ORACLE_SHIM_HDF5_H

#include <stddef.h>
#include <stdlib.h> /* the real HDF5 headers pull this in too */

#ifdef __cplusplus
extern "C" {
#endif

typedef long long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef enum { H5T_COMPOUND = 6 } H5T_class_t;

#define H5P_DEFAULT        ((hid_t)0)
#define H5S_ALL            ((hid_t)0)
#define H5F_ACC_RDONLY     (0u)
#define H5F_ACC_TRUNC      (2u)
#define H5T_NATIVE_DOUBLE  ((hid_t)101)
#define H5T_NATIVE_INT     ((hid_t)102)
#define H5T_IEEE_F64LE     ((hid_t)103)
#define H5T_STD_I32LE      ((hid_t)104)
#define HOFFSET(S, M)      (offsetof(S, M))

hid_t H5Fcreate(const char *name, unsigned flags, hid_t fcpl, hid_t fapl);
hid_t H5Fopen(const char *name, unsigned flags, hid_t fapl);
herr_t H5Fclose(hid_t f);
hid_t H5Dcreate1(hid_t loc, const char *name, hid_t type, hid_t space, hid_t dcpl);
hid_t H5Dopen1(hid_t loc, const char *name);
herr_t H5Dread(hid_t d, hid_t mtype, hid_t mspace, hid_t fspace, hid_t xfer, void *buf);
herr_t H5Dwrite(hid_t d, hid_t mtype, hid_t mspace, hid_t fspace, hid_t xfer, const void *buf);
herr_t H5Dclose(hid_t d);
hid_t H5Screate_simple(int rank, const hsize_t *dims, const hsize_t *maxdims);
herr_t H5Sclose(hid_t s);
hid_t H5Tcreate(H5T_class_t cls, size_t size);
herr_t H5Tinsert(hid_t t, const char *name, size_t offset, hid_t member);

#ifdef __cplusplus
}
#endif
#endif
