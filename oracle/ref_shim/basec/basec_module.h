/*
 * Stand-in for the external "basec" base library that FV3D links against
 * (CMakeLists.txt:60,85 of the reference; the library itself is not part of
 * the reference tree).  TEST INFRASTRUCTURE ONLY: it exists so that the
 * reference's own hot-path C files compile unmodified into oracle/_ref/ and
 * can be run as the parity oracle.  The interface below is inferred from the
 * reference's call sites; every routine is written here from scratch.
 *
 *  - memory:      BM_ALLOCATE / BM_REALLOCATE / BM_DEALLOCATE -> calloc/realloc/free
 *  - checks:      BM_CHECK_EXPRESSION -> longjmp back into the harness entry
 *  - vectors:     copy_n, dot_n, len_n, sum_n, max_n, set_value_n, ...
 *  - parameters:  in-memory string-keyed store (BM_SET/GET_PARAMETER)
 *  - MPI:         serial (is_parallel() == 0, reductions copy)
 *  - HDF5:        unsupported (every call raises a check failure)
 *  - Krylov:      solve_gmres_n_m / solve_bicgstab_n_m restated in shim.c
 */
#ifndef BASEC_MODULE_H
#define BASEC_MODULE_H

#include <float.h>
#include <math.h>
#include <setjmp.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef char *string_t;
typedef const char *cstring_t;
typedef int bool_t;
typedef unsigned long long hsize_t;
typedef long hid_t;

#define BC_TRUE 1
#define BC_FALSE 0
#define BC_DMAX DBL_MAX

/* ---- error handling ---------------------------------------------------- */
extern jmp_buf *shim_jmp;
extern char shim_error[256];
void shim_fail(const char *expr, const char *file, int line);

#define BM_CHECK_EXPRESSION(e) \
    do { if (!(e)) shim_fail(#e, __FILE__, __LINE__); } while (0)
#define BM_UNUSED(x) ((void)(x))
#define BM_PRINT(...) shim_print(__VA_ARGS__)
void shim_print(const char *fmt, ...);

/* ---- memory ------------------------------------------------------------ */
#define BM_ALLOCATE(size) shim_allocate(size)
#define BM_REALLOCATE(ptr, size) shim_reallocate(ptr, size)
#define BM_DEALLOCATE(ptr) do { free((void *)(ptr)); (ptr) = NULL; } while (0)
void *shim_allocate(size_t size);
void *shim_reallocate(void *ptr, size_t size);

/* ---- math helpers ------------------------------------------------------ */
#define BM_MIN(a, b) (((a) < (b)) ? (a) : (b))
#define BM_MAX(a, b) (((a) > (b)) ? (a) : (b))
#define BM_ABS(a) (((a) < 0) ? -(a) : (a))

void set_value_n(double value, size_t n, double *x);
void set_value_int_n(int value, size_t n, int *x);
void copy_n(const double *x, size_t n, double *y);
double dot_n(const double *x, const double *y, size_t n);
double len_n(const double *x, size_t n);
double sum_n(const double *x, size_t n);
double max_n(const double *x, size_t n);
int is_nan_n(const double *x, size_t n);
int is_inf_n(const double *x, size_t n);

/* ---- strings ----------------------------------------------------------- */
int is_equal(cstring_t a, cstring_t b);
string_t allocate_strcat(cstring_t a, cstring_t b);
string_t allocate_strcpy(cstring_t a);

/* ---- parameters -------------------------------------------------------- */
enum { NumberParameter, DigitParameter, LogicalParameter, StringParameter };
void shim_set_parameter(cstring_t path, int type, const void *value);
void shim_get_parameter(cstring_t path, int type, void *value);
int shim_parameter_exists(cstring_t path);
void shim_clear_parameters(void);

#define BM_SET_PARAMETER(path, type, value, desc, opts, n_opts) \
    shim_set_parameter(path, type, value)
#define BM_GET_PARAMETER(path, type, value) shim_get_parameter(path, type, value)
#define BM_PARAMETER_EXISTS(path) shim_parameter_exists(path)
#define BM_REGISTER_INITIALIZE_ROUTINE(fn) ((void)(fn))
#define BM_REGISTER_FINALIZE_ROUTINE(fn) ((void)(fn))

/* ---- MPI (serial) -------------------------------------------------------- */
enum { MPIDouble, MPIInt };
enum { MPISum, MPIMin, MPIMax, MPILogAnd };
int is_parallel(void);
int get_rank_number(void);
int get_number_of_procs(void);
void check_abort(int flag);
void mpi_send(int type, int rank, void *data, int n);
void mpi_receive(int type, int rank, int n, void *data);
void mpi_all_reduce_n(int type, int op, void *in, int n, void *out);
#define BM_MPI_ALL_REDUCE(type, op, in, out) \
    memcpy((out), (in), sizeof(*(in)))

/* ---- HDF5 (unsupported here) ------------------------------------------- */
enum { HDF5Int, HDF5Double, HDF5String };
#define BM_GET_HDF5_ATTRIBUTE(...) shim_fail("HDF5 unsupported", __FILE__, __LINE__)
#define BM_GET_HDF5_DATASET_N(...) shim_fail("HDF5 unsupported", __FILE__, __LINE__)
#define BM_GET_HDF5_DATASET_N_M(...) shim_fail("HDF5 unsupported", __FILE__, __LINE__)
#define BM_GET_HDF5_DATASET_CHUNK_N(...) shim_fail("HDF5 unsupported", __FILE__, __LINE__)
#define BM_GET_HDF5_DATASET_CHUNK_N_M(...) shim_fail("HDF5 unsupported", __FILE__, __LINE__)
#define BM_GET_HDF5_DATASET_SELECT_N(...) shim_fail("HDF5 unsupported", __FILE__, __LINE__)
#define BM_GET_HDF5_DATASET_SELECT_N_M(...) shim_fail("HDF5 unsupported", __FILE__, __LINE__)
hid_t open_hdf5_file_read_only(cstring_t name);
hid_t open_hdf5_group(hid_t id, cstring_t name);
void close_hdf5_group(hid_t id);
void close_hdf5_file(hid_t id);
int get_hdf5_dataset_size(hid_t id, cstring_t name);
string_t *allocate_hdf5_string_buffer(int n, int max_length, string_t *init);
void deallocate_hdf5_string_buffer(string_t *buffer);

/* ---- Krylov solvers ---------------------------------------------------- */
typedef int (*shim_matvec_ft)(double *x, double *b, size_t n_var, size_t n_cells);
int get_gmres_n_m_work_size(int n_var, int n_cells, int max_krylov_dims);
int get_bicgstab_n_m_work_size(int n_var, int n_cells);
void solve_gmres_n_m(int n_var, int n_cells, double *rhs, double *x, double *work,
                     shim_matvec_ft matvec, int *n_iter, double *residual,
                     int max_krylov_dims, int max_krylov_restarts);
void solve_bicgstab_n_m(int n_var, int n_cells, double *rhs, double *x, double *work,
                        shim_matvec_ft matvec, int *n_iter, double *residual);

#endif /* BASEC_MODULE_H */
