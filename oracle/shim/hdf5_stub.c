/*
 * TEST INFRASTRUCTURE ONLY.  Failing HDF5 stand-ins; see hdf5.h.
 */
#include <stdio.h>

#include "hdf5.h"

static int unavailable(const char *fn)
{
    fprintf(stderr, "oracle: %s called but HDF5 is not available in this build\n", fn);
    return -1;
}

hid_t H5Fcreate(const char *n, unsigned f, hid_t a, hid_t b) { (void)n; (void)f; (void)a; (void)b; return unavailable("H5Fcreate"); }
hid_t H5Fopen(const char *n, unsigned f, hid_t a) { (void)n; (void)f; (void)a; return unavailable("H5Fopen"); }
herr_t H5Fclose(hid_t f) { (void)f; return -1; }
hid_t H5Dcreate1(hid_t l, const char *n, hid_t t, hid_t s, hid_t d) { (void)l; (void)n; (void)t; (void)s; (void)d; return unavailable("H5Dcreate1"); }
hid_t H5Dopen1(hid_t l, const char *n) { (void)l; (void)n; return unavailable("H5Dopen1"); }
herr_t H5Dread(hid_t d, hid_t m, hid_t ms, hid_t fs, hid_t x, void *b) { (void)d; (void)m; (void)ms; (void)fs; (void)x; (void)b; return unavailable("H5Dread"); }
herr_t H5Dwrite(hid_t d, hid_t m, hid_t ms, hid_t fs, hid_t x, const void *b) { (void)d; (void)m; (void)ms; (void)fs; (void)x; (void)b; return unavailable("H5Dwrite"); }
herr_t H5Dclose(hid_t d) { (void)d; return -1; }
hid_t H5Screate_simple(int r, const hsize_t *d, const hsize_t *m) { (void)r; (void)d; (void)m; return -1; }
herr_t H5Sclose(hid_t s) { (void)s; return -1; }
hid_t H5Tcreate(H5T_class_t c, size_t s) { (void)c; (void)s; return -1; }
herr_t H5Tinsert(hid_t t, const char *n, size_t o, hid_t m) { (void)t; (void)n; (void)o; (void)m; return -1; }
