/*
 * Implementation of the basec stand-in declared in basec/basec_module.h.
 * TEST INFRASTRUCTURE ONLY (links into oracle/_ref/libfv3d_ref.so together
 * with the reference's own, unmodified hot-path sources).
 *
 * The Krylov solvers are this repository's own restatement of textbook
 * restarted GMRES (Saad & Schultz 1986; modified Gram-Schmidt + Givens
 * rotations) and BiCGStab (van der Vorst 1992).  basec's own versions are not
 * available, so their arithmetic is NOT pinned: the reference calls them on a
 * block-diagonal system (implicit.c:362-384), whose converged answer is
 * unique, which is what the parity tests rely on.
 */
#include <stdarg.h>
#include "basec/basec_module.h"

jmp_buf *shim_jmp = NULL;
char shim_error[256] = {0};
static int shim_verbose = 0;

void shim_fail(const char *expr, const char *file, int line)
{
    snprintf(shim_error, sizeof(shim_error), "check failed: %s (%s:%d)", expr,
             file, line);
    if (shim_jmp != NULL)
        longjmp(*shim_jmp, 1);
    fprintf(stderr, "%s\n", shim_error);
    abort();
}

void shim_print(const char *fmt, ...)
{
    if (!shim_verbose)
        return;
    va_list ap;
    va_start(ap, fmt);
    vprintf(fmt, ap);
    va_end(ap);
}

void shim_set_verbose(int v) { shim_verbose = v; }

void *shim_allocate(size_t size)
{
    void *p = calloc(1, size > 0 ? size : 1);
    if (p == NULL)
        shim_fail("allocation", __FILE__, __LINE__);
    return p;
}

void *shim_reallocate(void *ptr, size_t size)
{
    void *p = realloc(ptr, size > 0 ? size : 1);
    if (p == NULL)
        shim_fail("reallocation", __FILE__, __LINE__);
    return p;
}

/* ---- vectors (plain left-to-right loops) ---------------------------------- */
void set_value_n(double value, size_t n, double *x)
{
    for (size_t i = 0; i < n; ++i)
        x[i] = value;
}

void set_value_int_n(int value, size_t n, int *x)
{
    for (size_t i = 0; i < n; ++i)
        x[i] = value;
}

void copy_n(const double *x, size_t n, double *y)
{
    for (size_t i = 0; i < n; ++i)
        y[i] = x[i];
}

double dot_n(const double *x, const double *y, size_t n)
{
    double s = 0.0;
    for (size_t i = 0; i < n; ++i)
        s += x[i] * y[i];
    return s;
}

double len_n(const double *x, size_t n) { return sqrt(dot_n(x, x, n)); }

double sum_n(const double *x, size_t n)
{
    double s = 0.0;
    for (size_t i = 0; i < n; ++i)
        s += x[i];
    return s;
}

double max_n(const double *x, size_t n)
{
    double m = -DBL_MAX;
    for (size_t i = 0; i < n; ++i)
        m = (x[i] > m) ? x[i] : m;
    return m;
}

int is_nan_n(const double *x, size_t n)
{
    for (size_t i = 0; i < n; ++i)
        if (isnan(x[i]))
            return 1;
    return 0;
}

int is_inf_n(const double *x, size_t n)
{
    for (size_t i = 0; i < n; ++i)
        if (isinf(x[i]))
            return 1;
    return 0;
}

/* ---- strings -------------------------------------------------------------- */
int is_equal(cstring_t a, cstring_t b) { return strcmp(a, b) == 0; }

string_t allocate_strcat(cstring_t a, cstring_t b)
{
    size_t la = strlen(a), lb = strlen(b);
    string_t s = shim_allocate(la + lb + 1);
    memcpy(s, a, la);
    memcpy(s + la, b, lb + 1);
    return s;
}

string_t allocate_strcpy(cstring_t a) { return allocate_strcat(a, ""); }

/* ---- parameters ------------------------------------------------------------ */
typedef struct
{
    char path[160];
    int type;
    double number;
    int digit;
    char string[96];
} shim_param_t;

#define SHIM_MAX_PARAMS 256
static shim_param_t shim_params[SHIM_MAX_PARAMS];
static int shim_n_params = 0;

static shim_param_t *find_param(cstring_t path)
{
    for (int i = 0; i < shim_n_params; ++i)
        if (strcmp(shim_params[i].path, path) == 0)
            return &shim_params[i];
    return NULL;
}

void shim_clear_parameters(void) { shim_n_params = 0; }

/* Registers a value.  Used both by the reference's *_define routines (where
 * the value is a default) and by the harness (which sets values first; a
 * later default then does not override them). */
static void put_param(cstring_t path, int type, const void *value, int overwrite)
{
    shim_param_t *p = find_param(path);
    if (p != NULL && !overwrite)
        return;
    if (p == NULL)
    {
        BM_CHECK_EXPRESSION(shim_n_params < SHIM_MAX_PARAMS);
        p = &shim_params[shim_n_params++];
        snprintf(p->path, sizeof(p->path), "%s", path);
    }
    p->type = type;
    switch (type)
    {
    case NumberParameter:
        p->number = *(const double *)value;
        break;
    case DigitParameter:
    case LogicalParameter:
        p->digit = *(const int *)value;
        break;
    case StringParameter:
        snprintf(p->string, sizeof(p->string), "%s", *(const cstring_t *)value);
        break;
    default:
        BM_CHECK_EXPRESSION(0);
    }
}

void shim_set_parameter(cstring_t path, int type, const void *value)
{
    put_param(path, type, value, 0);
}

void shim_put_parameter(cstring_t path, int type, const void *value)
{
    put_param(path, type, value, 1);
}

void shim_get_parameter(cstring_t path, int type, void *value)
{
    shim_param_t *p = find_param(path);
    BM_CHECK_EXPRESSION(p != NULL);
    switch (type)
    {
    case NumberParameter:
        *(double *)value = p->number;
        break;
    case DigitParameter:
    case LogicalParameter:
        *(int *)value = p->digit;
        break;
    case StringParameter:
        *(string_t *)value = allocate_strcpy(p->string);
        break;
    default:
        BM_CHECK_EXPRESSION(0);
    }
}

int shim_parameter_exists(cstring_t path)
{
    size_t n = strlen(path);
    for (int i = 0; i < shim_n_params; ++i)
    {
        /* a group path exists if any parameter lies below it */
        if (strncmp(shim_params[i].path, path, n) == 0 &&
            (shim_params[i].path[n] == '\0' || shim_params[i].path[n] == '/'))
            return 1;
    }
    return 0;
}

/* ---- MPI (serial) ------------------------------------------------------------ */
int is_parallel(void) { return 0; }
int get_rank_number(void) { return 0; }
int get_number_of_procs(void) { return 1; }
void check_abort(int flag) { (void)flag; }
void mpi_send(int type, int rank, void *data, int n)
{
    (void)type; (void)rank; (void)data; (void)n;
    shim_fail("MPI unsupported", __FILE__, __LINE__);
}
void mpi_receive(int type, int rank, int n, void *data)
{
    (void)type; (void)rank; (void)data; (void)n;
    shim_fail("MPI unsupported", __FILE__, __LINE__);
}
void mpi_all_reduce_n(int type, int op, void *in, int n, void *out)
{
    (void)op;
    memcpy(out, in, (size_t)n * (type == MPIDouble ? sizeof(double) : sizeof(int)));
}

/* ---- HDF5 ------------------------------------------------------------------ */
hid_t open_hdf5_file_read_only(cstring_t name)
{
    (void)name;
    shim_fail("HDF5 unsupported", __FILE__, __LINE__);
    return -1;
}
hid_t open_hdf5_group(hid_t id, cstring_t name)
{
    (void)id; (void)name;
    shim_fail("HDF5 unsupported", __FILE__, __LINE__);
    return -1;
}
void close_hdf5_group(hid_t id) { (void)id; }
void close_hdf5_file(hid_t id) { (void)id; }
int get_hdf5_dataset_size(hid_t id, cstring_t name)
{
    (void)id; (void)name;
    shim_fail("HDF5 unsupported", __FILE__, __LINE__);
    return 0;
}

string_t *allocate_hdf5_string_buffer(int n, int max_length, string_t *init)
{
    (void)init;
    string_t *buf = shim_allocate(sizeof(string_t) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i)
        buf[i] = shim_allocate((size_t)max_length + 1);
    return buf;
}

void deallocate_hdf5_string_buffer(string_t *buffer)
{
    (void)buffer; /* the harness owns region names; freed with the mesh */
}

/* ---- Krylov: shared with the restatement oracle ---------------------------- */
#include "../krylov.c"
