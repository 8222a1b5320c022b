/*
 * Harness that drives the reference's own (unmodified) FV3D C sources as the
 * parity oracle.  TEST INFRASTRUCTURE ONLY; compiled into
 * oracle/_ref/libfv3d_ref.so by oracle/Makefile.ref together with basec_shim.c.
 *
 * What it does instead of the reference's program start (fv3d.c:27-63):
 *  - builds Mesh_t in memory with the reference's allocators
 *    (mesh_data.c) instead of read_mesh_file (mesh.c:121), then calls the
 *    reference's calc_mesh_metrics (mesh.c:19-83); for periodic faces the
 *    caller supplies the minimum-image dist_cell_2, which overrides
 *    x_f - x_c1 (the reference has no periodic faces);
 *  - registers the parameters that navier_stokes.c:55-66, flux.c:273 and
 *    boundary.c:55-139 read, then runs their *_initialize routines;
 *  - initial conditions are written straight into phi_total followed by the
 *    registered update routine (the role of set_solution, finite_volume.c:189);
 *  - SSP-RK3 and the convective CFL time step are harness-level additions
 *    (no reference counterpart) built around the reference residual.
 */
#include <pthread.h>
#include "../fv3d_oracle.h"
#include "basec/basec_module.h"
#include "solver/solver_module.h"
#include "finite_volume/finite_volume_private.h"
#include "timedisc/timedisc_private.h"
#include "analyze/analyze_private.h"
#include "mesh/mesh_private.h"
#include "navier_stokes/navier_stokes_module.h"

/* globals the reference's timedisc.c expects from output/restart modules */
int solver_use_restart = 0;
int solver_iter_restart = 0;
double solver_t_restart = 0.0;
int solver_do_output_data = 0;
int solver_i_output_data = 0;
void write_output(int iter, double t) { (void)iter; (void)t; }

void shim_put_parameter(cstring_t path, int type, const void *value);
void calc_mesh_metrics(Mesh_t *mesh);
void deallocate_mesh(Mesh_t *mesh);
void flux_initialize(void);
void boundary_initialize(void);
void navier_stokes_initialize(void);

extern double *jac; /* implicit.c:54 */

static const char *bc_names[] = {"flow", "inflow", "outflow", "wall-adiabatic",
                                 "wall-isothermal", "wall-slip", "symmetry",
                                 "state", "function"};
static int g_ready = 0;
static int g_implicit_ready = 0;
static char g_region_names[64][16];

#define ENTER()                     \
    jmp_buf jb__;                   \
    shim_jmp = &jb__;               \
    if (setjmp(jb__) != 0)          \
    {                               \
        shim_jmp = NULL;            \
        return -1;                  \
    }
#define LEAVE() \
    shim_jmp = NULL; \
    return 0

const char *orc_error(void) { return shim_error; }

static void put_number(const char *path, double v) { shim_put_parameter(path, NumberParameter, &v); }
static void put_string(const char *path, const char *v) { shim_put_parameter(path, StringParameter, &v); }

void orc_free(void)
{
    if (!g_ready)
        return;
    if (g_implicit_ready)
        free_implicit();
    g_implicit_ready = 0;
    free_explicit();
    free_limiter();
    free_reconstruction();
    free_finite_volume();
    free_analyze();
    if (solver_mesh != NULL && solver_mesh->regions != NULL)
    {
        BM_DEALLOCATE(solver_mesh->regions->type);
        BM_DEALLOCATE(solver_mesh->regions->function_id);
        BM_DEALLOCATE(solver_mesh->regions->phi_total);
    }
    free_equation();
    free_mesh();
    shim_clear_parameters();
    g_ready = 0;
}

int orc_init(const orc_mesh *m, const orc_params *p, const int *region_type,
             const double *region_prim)
{
    orc_free();
    ENTER();
    BM_CHECK_EXPRESSION(m->n_regions <= 64);

    /* ---- parameters ---- */
    put_number("Equation/Navier-Stokes/cfl_scale", p->cfl_scale);
    put_number("Equation/Navier-Stokes/dfl_scale", p->dfl_scale);
    put_number("Equation/Navier-Stokes/mu_mix", p->mu_mix);
    put_number("Equation/Navier-Stokes/R_mix", p->R_mix);
    put_number("Equation/Navier-Stokes/Pr", p->Pr);
    put_number("Equation/Navier-Stokes/kappa", p->kappa);
    put_string("Equation/Navier-Stokes/Flux/flux_scheme",
               p->flux_scheme == 0 ? "AUSM" : "Rusanov");
    for (int r = 0; r < m->n_regions; ++r)
    {
        char path[160];
        snprintf(g_region_names[r], sizeof(g_region_names[r]), "r%d", r);
        BM_CHECK_EXPRESSION(region_type[r] >= 0 && region_type[r] <= 7);
        snprintf(path, sizeof(path), "Equation/Navier-Stokes/Boundary/r%d/type", r);
        put_string(path, bc_names[region_type[r]]);
        const char *keys[5] = {"u", "v", "w", "p", "T"};
        for (int k = 0; k < 5; ++k)
        {
            snprintf(path, sizeof(path), "Equation/Navier-Stokes/Boundary/r%d/%s", r, keys[k]);
            put_number(path, region_prim[r * 5 + k]);
        }
    }

    /* ---- mesh (the reference's allocators, filled from the arrays) ---- */
    Mesh_t *mesh = allocate_mesh();
    mesh->dimension = 3;
    mesh->is_partitioned = 0;
    allocate_vertices(mesh, 1);
    Cells_t *cells = allocate_cells(mesh, m->n_cells, 8, m->max_cell_faces);
    Boundaries_t *bnd = allocate_boundaries(mesh, m->n_boundaries, 4);
    Faces_t *faces = allocate_faces(mesh, m->n_faces, 4);
    Regions_t *regions = allocate_regions(mesh, m->n_regions, 15);
    for (int i = 0; i < m->n_cells; ++i)
    {
        cells->id[i] = 0;
        cells->n_faces[i] = m->cell_n_faces[i];
        cells->volume[i] = m->cell_volume[i];
        for (int d = 0; d < DIM; ++d)
        {
            cells->x[i * DIM + d] = m->cell_x[i * DIM + d];
            cells->dx[i * DIM + d] = m->cell_dx[i * DIM + d];
        }
        for (int k = 0; k < m->max_cell_faces; ++k)
            cells->faces[i * m->max_cell_faces + k] = m->cell_faces[i * m->max_cell_faces + k];
    }
    for (int i = 0; i < m->n_faces; ++i)
    {
        faces->cells[2 * i] = m->face_cells[2 * i];
        faces->cells[2 * i + 1] = m->face_cells[2 * i + 1];
        faces->boundary[i] = m->face_boundary[i];
        faces->area[i] = m->face_area[i];
        faces->lambda[i] = m->face_lambda[i];
        for (int d = 0; d < DIM; ++d)
        {
            faces->x[i * DIM + d] = m->face_x[i * DIM + d];
            faces->n[i * DIM + d] = m->face_n[i * DIM + d];
            faces->t1[i * DIM + d] = m->face_t1[i * DIM + d];
            faces->t2[i * DIM + d] = m->face_t2[i * DIM + d];
        }
    }
    for (int i = 0; i < m->n_boundaries; ++i)
    {
        bnd->id[i] = m->boundary_id[i];
        bnd->face[i] = m->boundary_face[i];
    }
    for (int r = 0; r < m->n_regions; ++r)
    {
        snprintf(regions->name[r], 16, "%s", g_region_names[r]);
        regions->is_boundary[r] = m->region_is_boundary[r];
    }
    solver_mesh = mesh;
    calc_mesh_metrics(mesh);
    if (m->face_dist_cell_2 != NULL)
        for (int i = 0; i < m->n_faces; ++i)
            if (m->face_cells[2 * i + 1] >= 0)
                for (int d = 0; d < DIM; ++d)
                    faces->dist_cell_2[i * DIM + d] = m->face_dist_cell_2[i * DIM + d];

    /* ---- physics + solver modules (registration order of fv3d.c:30-37) ---- */
    navier_stokes_initialize();
    boundary_initialize();
    flux_initialize();
    init_finite_volume();
    init_reconstruction(p->reconstruction == 0 ? FirstOrder : Linear);
    init_limiter(p->limiter == 0 ? BarthJespersenn : NoLimter);
    init_analyze();
    BM_CHECK_EXPRESSION(p->gradient == 0); /* LSQ has no reference counterpart */
    g_ready = 1;
    LEAVE();
}

int orc_set_conserved(const double *u)
{
    ENTER();
    const int nt = solver_variables->n_tot_variables;
    for (int i = 0; i < solver_mesh->cells->n_domain_cells; ++i)
        for (int j = 0; j < 5; ++j)
            solver_data->phi_total[i * nt + j] = u[i * 5 + j];
    update_function_pointer(0.0);
    LEAVE();
}

int orc_get_total(double *phi_total)
{
    ENTER();
    int n = (solver_mesh->cells->n_local_cells + solver_mesh->boundaries->n_boundaries) *
            solver_variables->n_tot_variables;
    copy_n(solver_data->phi_total, (size_t)n, phi_total);
    LEAVE();
}

int orc_time_derivative(double t, double *phi_dt)
{
    ENTER();
    finite_volume_time_derivative(t);
    copy_n(solver_data->phi_dt, (size_t)solver_mesh->cells->n_domain_cells * 5, phi_dt);
    LEAVE();
}

int orc_get_gradients(double *gx, double *gy, double *gz)
{
    ENTER();
    int n = (solver_mesh->cells->n_local_cells + solver_mesh->boundaries->n_boundaries) *
            solver_variables->n_tot_variables;
    copy_n(solver_data->grad_phi_total_x, (size_t)n, gx);
    copy_n(solver_data->grad_phi_total_y, (size_t)n, gy);
    copy_n(solver_data->grad_phi_total_z, (size_t)n, gz);
    LEAVE();
}

int orc_get_face_states(double *left, double *right)
{
    ENTER();
    int n = solver_mesh->faces->n_faces * solver_variables->n_tot_variables;
    copy_n(solver_data->phi_total_left, (size_t)n, left);
    copy_n(solver_data->phi_total_right, (size_t)n, right);
    LEAVE();
}

int orc_get_flux(double *flux)
{
    ENTER();
    copy_n(solver_data->flux, (size_t)solver_mesh->faces->n_faces * 5, flux);
    LEAVE();
}

/* Convective part of calc_ns_timestep (navier_stokes.c:171-187) with an
 * explicit CFL number: dt = cfl * min_i V_i / sum_d (|u_d| + c) dx_d. */
double orc_timestep_convective(double cfl)
{
    Cells_t *cells = solver_mesh->cells;
    const int nt = solver_variables->n_tot_variables;
    double lam = BC_DMAX;
    for (int i = 0; i < cells->n_domain_cells; ++i)
    {
        const double *phi = &solver_data->phi_total[i * nt];
        const double *dx = &cells->dx[i * DIM];
        double s_rho = 1.0 / phi[ic_rho];
        double c = sqrt(kappa * phi[ip_p] * s_rho);
        double ds = (BM_ABS(phi[ip_u]) + c) * dx[0] + (BM_ABS(phi[ip_v]) + c) * dx[1] +
                    (BM_ABS(phi[ip_w]) + c) * dx[2];
        lam = BM_MIN(lam, cells->volume[i] / ds);
    }
    return lam * cfl;
}

double orc_calc_ns_timestep(void) { return calc_ns_timestep(0.0); }

/* the reference's stage loop keeps a VLA of 5*N doubles on the stack
 * (explicit.c:107); run it on a thread with a large stack */
typedef struct
{
    int iter;
    double t, dt;
    int rc;
} lserk_args_t;

static void *lserk_thread(void *arg)
{
    lserk_args_t *a = (lserk_args_t *)arg;
    jmp_buf jb;
    shim_jmp = &jb;
    if (setjmp(jb) != 0)
    {
        a->rc = -1;
        shim_jmp = NULL;
        return NULL;
    }
    timestep_lserkw2(a->iter, a->t, a->dt);
    shim_jmp = NULL;
    a->rc = 0;
    return NULL;
}

int orc_step_lserkw2(int scheme, int iter, double t, double dt)
{
    {
        ENTER();
        init_explicit(scheme == 0 ? EulerExplicit : (scheme == 1 ? RungeKutta33 : RungeKutta45));
        shim_jmp = NULL;
    }
    lserk_args_t a = {iter, t, dt, 0};
    size_t stack = (size_t)solver_mesh->cells->n_domain_cells * 5 * sizeof(double) + (64u << 20);
    pthread_attr_t attr;
    pthread_attr_init(&attr);
    pthread_attr_setstacksize(&attr, stack);
    pthread_t th;
    if (pthread_create(&th, &attr, lserk_thread, &a) != 0)
    {
        snprintf(shim_error, sizeof(shim_error), "pthread_create failed");
        pthread_attr_destroy(&attr);
        return -1;
    }
    pthread_join(th, NULL);
    pthread_attr_destroy(&attr);
    return a.rc;
}

/* SSP-RK3 (Shu & Osher 1988), harness-level: no reference counterpart. */
int orc_step_ssprk3(double t, double dt)
{
    ENTER();
    const int n = solver_mesh->cells->n_domain_cells;
    const int nt = solver_variables->n_tot_variables;
    double *u0 = BM_ALLOCATE(sizeof(double) * 5 * (size_t)n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 5; ++j)
            u0[i * 5 + j] = solver_data->phi_total[i * nt + j];
    /* stage 1: u1 = u0 + dt R(u0) */
    finite_volume_time_derivative(t);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 5; ++j)
            solver_data->phi_total[i * nt + j] = u0[i * 5 + j] + dt * solver_data->phi_dt[i * 5 + j];
    /* stage 2: u2 = 3/4 u0 + 1/4 (u1 + dt R(u1)) */
    finite_volume_time_derivative(t + dt);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 5; ++j)
        {
            double u1 = solver_data->phi_total[i * nt + j];
            solver_data->phi_total[i * nt + j] =
                0.75 * u0[i * 5 + j] + 0.25 * (u1 + dt * solver_data->phi_dt[i * 5 + j]);
        }
    /* stage 3: u = 1/3 u0 + 2/3 (u2 + dt R(u2)) */
    finite_volume_time_derivative(t + 0.5 * dt);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 5; ++j)
        {
            double u2 = solver_data->phi_total[i * nt + j];
            solver_data->phi_total[i * nt + j] =
                (1.0 / 3.0) * u0[i * 5 + j] + (2.0 / 3.0) * (u2 + dt * solver_data->phi_dt[i * 5 + j]);
        }
    BM_DEALLOCATE(u0);
    update_function_pointer(t + dt);
    LEAVE();
}

int orc_global_residual(double dt, double *res)
{
    ENTER();
    calc_global_residual(dt);
    copy_n(solver_residual, 5, res);
    LEAVE();
}

int orc_step_newton(int scheme, int solver, int max_iter_inner, double tolerance_lsoe,
                    int max_iter_lsoe, int krylov_dims, int krylov_restarts,
                    int is_transient, int iter, double t, double dt, int *n_inner,
                    int *n_lsoe)
{
    ENTER();
    if (!g_implicit_ready || iter == 0)
    {
        /* (re)initialise only at the start so BDF2 keeps its phi_old history */
        if (g_implicit_ready)
            free_implicit();
        init_timedisc(Implicit, 1 << 30, is_transient, 0.0, 0.0, 1e300);
        init_implicit(scheme == 0 ? EulerImplicit : BDF2, solver == 0 ? BiCGStab : GMRes,
                      max_iter_inner, tolerance_lsoe, max_iter_lsoe, krylov_dims,
                      krylov_restarts);
        g_implicit_ready = 1;
    }
    if (iter == 0)
        finite_volume_time_derivative(t); /* timedisc.c:537-538 */
    timestep_newton(iter, t, dt);
    *n_inner = n_iter_inner;
    *n_lsoe = n_iter_lsoe;
    LEAVE();
}

int orc_get_jacobian(double *out)
{
    ENTER();
    BM_CHECK_EXPRESSION(jac != NULL);
    copy_n(jac, (size_t)solver_mesh->cells->n_domain_cells * 25, out);
    LEAVE();
}
