/* Declarations of the netCDF calls made by the EPREM reference's output code.
 * Defined by oracle/ref_shims.c as an in-memory capture that writes each
 * closed dataset to <path>.cap.  Test infrastructure, not part of the
 * product. */
#ifndef EPREM_REFSHIM_NETCDF_H
#define EPREM_REFSHIM_NETCDF_H
#include <stddef.h>
typedef int nc_type;
#define NC_NOERR 0
#define NC_WRITE 1
#define NC_CLOBBER 0
#define NC_UNLIMITED 0L
#define NC_INT 4
#define NC_FLOAT 5
#define NC_DOUBLE 6
const char *nc_strerror(int);
int nc_create(const char *, int, int *);
int nc_open(const char *, int, int *);
int nc_close(int);
int nc_enddef(int);
int nc_def_dim(int, const char *, size_t, int *);
int nc_def_var(int, const char *, nc_type, int, const int *, int *);
int nc_inq_varid(int, const char *, int *);
int nc_put_att_text(int, int, const char *, size_t, const char *);
int nc_put_att_double(int, int, const char *, nc_type, size_t, const double *);
int nc_put_var(int, int, const void *);
int nc_put_var_double(int, int, const double *);
int nc_put_var1_double(int, int, const size_t *, const double *);
int nc_put_vara_double(int, int, const size_t *, const size_t *, const double *);
int nc_put_vara_int(int, int, const size_t *, const size_t *, const int *);
int nc_put_varm_double(int, int, const size_t *, const size_t *, const ptrdiff_t *, const ptrdiff_t *, const double *);
#endif
