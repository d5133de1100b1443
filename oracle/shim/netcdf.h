/*
 * netcdf.h (oracle shim) -- declares the netCDF C calls the reference makes
 * (src/netcdf_io.h:38-382).  In the oracle the writers return an error, so
 * the reference's output code prints its error and returns
 * (src/netcdf_io.h:16), and the readers read classic-format files (shim.c);
 * test infrastructure only.
 */
#ifndef QGW_SHIM_NETCDF_H
#define QGW_SHIM_NETCDF_H
#include <stddef.h>
typedef int nc_type;
#define NC_NOWRITE 0x0000
#define NC_WRITE 0x0001
#define NC_CLOBBER 0x0000
#define NC_UNLIMITED 0L
#define NC_FLOAT 5
#define NC_DOUBLE 6
#define NC_MAX_NAME 256
int nc_create(const char* path, int cmode, int* ncidp);
int nc_open(const char* path, int mode, int* ncidp);
int nc_def_dim(int ncid, const char* name, size_t len, int* idp);
int nc_def_var(int ncid, const char* name, nc_type xtype, int ndims, const int* dimidsp, int* varidp);
int nc_enddef(int ncid);
int nc_close(int ncid);
int nc_put_var_float(int ncid, int varid, const float* op);
int nc_put_vara_float(int ncid, int varid, const size_t* startp, const size_t* countp, const float* op);
int nc_get_vara_float(int ncid, int varid, const size_t* startp, const size_t* countp, float* ip);
int nc_inq(int ncid, int* ndimsp, int* nvarsp, int* nattsp, int* unlimdimidp);
int nc_inq_var(int ncid, int varid, char* name, nc_type* xtypep, int* ndimsp, int* dimidsp, int* nattsp);
const char* nc_strerror(int ncerr);
#endif
