/*
 * fv3d_gpu_shim.c - drops the GB300 library into FV3D's own program.
 *
 * Compiled next to FV3D against its headers (it uses Mesh_t, data_t and the
 * solver globals), with the include paths <repo>/include, src/Solver/include,
 * src/Solver/src, src/FV3D/include and src/FV3D/src of the FV3D tree, and
 * linked ahead of the solver library so that FV3D's calls of
 * finite_volume_time_derivative, timedisc and calc_global_residual resolve
 * to the GPU versions below:
 *
 *   gcc -std=gnu99 -c fv3d_gpu_shim.c -I<repo>/include -I<fv3d>/src/... \
 *   && link: fv3d_gpu_shim.o ... -lsolver -L<repo>/fv3d_gb300 -lfv3d_gb300
 *
 * Mesh reading, parameters, output and restart stay FV3D's.
 */
#include <stdio.h>
#include <stdlib.h>
#include "fv3d_gpu.h"
#include "solver/solver_module.h"
#include "navier_stokes/navier_stokes_module.h" /* kappa, R_mix, ..., ip_u */
#include "timedisc/timedisc_private.h"          /* n_bdf_stages, phi_old */
#include "analyze/analyze_private.h"            /* solver_residual */
#include "output/output_private.h"              /* solver_i_output_data */
#include "restart/restart_private.h"            /* solver_use_restart, ... */

extern string_t flux_scheme_name;               /* flux.c:15 */
extern int solver_max_iter;                     /* timedisc.c:21-25 */
extern double solver_abort_residual, solver_t_start, solver_t_end;

static fv3d_ctx *gpu = NULL;

/* the five conserved columns of phi_total, one row per cell (caller frees) */
static double *conserved_rows(void)
{
    int n = solver_mesh->cells->n_domain_cells;
    double *u = malloc(sizeof(double) * 5 * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 5; ++j)
            u[5 * i + j] = solver_data->phi_total[10 * i + j];
    return u;
}

static void upload_state(void)
{
    double *u = conserved_rows();
    fv3d_set_state(gpu, u);
    free(u);
}

void gpu_initialize(void)      /* after init_mesh / navier_stokes_initialize */
{
    Mesh_t *m = solver_mesh;
    Faces_t *f = m->faces;
    int *fc = malloc(sizeof(int) * 2 * f->n_faces);
    for (int i = 0; i < f->n_faces; ++i) {
        fc[2 * i] = f->cells[2 * i];
        fc[2 * i + 1] = (f->boundary[i] >= 0) ? -1 : f->cells[2 * i + 1];
    }
    fv3d_config cfg = {kappa, R_mix, mu_mix, Pr, cfl_scale, dfl_scale,
                       /* flux */ is_equal(flux_scheme_name, "Rusanov") ? FV3D_FLUX_RUSANOV
                                                                       : FV3D_FLUX_AUSM,
                       FV3D_RECON_LINEAR, FV3D_LIMITER_BARTH_JESPERSEN,
                       FV3D_GRADIENT_GREEN_GAUSS, FV3D_PRECISION_MIXED,
                       FV3D_RENUMBER_MORTON, /* device */ 0};
    fv3d_mesh_arrays a = {
        m->cells->n_local_cells, f->n_faces, m->boundaries->n_boundaries,
        m->cells->max_cell_faces, m->regions->n_regions,
        m->cells->x, m->cells->volume, m->cells->dx, m->cells->n_faces,
        m->cells->faces, fc, f->boundary, f->area, f->lambda, f->x, f->n,
        f->t1, f->t2, f->dist_cell_2, m->boundaries->id, m->boundaries->face,
        m->regions->is_boundary};
    if (fv3d_create(&cfg, &gpu) != FV3D_OK ||
        fv3d_mesh_from_arrays(gpu, &a) != FV3D_OK)
        BM_CHECK_EXPRESSION(0);
    for (int r = 0; r < m->regions->n_regions; ++r) {
        double *q = &m->regions->phi_total[r * 10];
        double prim[5] = {q[ip_u], q[ip_v], q[ip_w], q[ip_p], q[ip_T]};
        fv3d_set_region(gpu, r, m->regions->type[r], prim);
    }
    free(fc);
}

/* drop-in for finite_volume_time_derivative(t) */
void gpu_time_derivative(double t)
{
    upload_state();
    fv3d_time_derivative(gpu, t, solver_data->phi_dt);
}

static void on_iter(void *user, int iter, double t, double dt, const double res[5], int n_inner)
{
    (void)user;
    printf("%09d %12.5e %12.5e %6d:", iter, t, dt, n_inner);
    for (int i = 0; i < 5; ++i) printf(" %12.5e", res[i]);
    printf("\n");
}

static void on_output(void *user, int iter, double t)
{
    (void)user;
    int n = 0;
    fv3d_get_state(gpu, solver_data->phi_total);
    fv3d_get_time_derivative(gpu, solver_data->phi_dt);
    fv3d_get_bdf_history(gpu, 0, NULL, &n);
    for (int k = 0; k < n; ++k) fv3d_get_bdf_history(gpu, k, phi_old[k], NULL);
    write_output(iter, t);                   /* output.c:92-191, unchanged */
}

void gpu_timedisc(void)
{
    fv3d_timedisc_opts o = {0};
    o.implicit = !is_explicit();            /* init_timedisc's timedisc_type */
    o.scheme = o.implicit ? FV3D_NEWTON_BDF2 : FV3D_RK_33;
    o.max_iter = solver_max_iter;
    o.is_transient = solver_is_transient;
    o.abort_residual = solver_abort_residual;
    o.t_start = solver_t_start;
    o.t_end = solver_t_end;
    o.cfl = 0.0;                             /* calc_ns_timestep as written (cfl_scale, dfl_scale) */
    o.max_iter_inner = 100;
    o.on_iteration = on_iter;
    o.i_output_data = solver_i_output_data;
    o.on_output = on_output;
    if (solver_use_restart) {                /* after read_restart_data */
        o.iter_start = solver_iter_restart;
        o.t_start = solver_t_restart;
        upload_state();
        if (o.implicit) {                    /* the phi_old stages, stage-major */
            int n = solver_mesh->cells->n_domain_cells;
            double *h = malloc(sizeof(double) * 5 * n * n_bdf_stages);
            for (int k = 0; k < n_bdf_stages; ++k)
                for (int i = 0; i < 5 * n; ++i) h[(size_t)k * 5 * n + i] = phi_old[k][i];
            fv3d_set_bdf_history(gpu, o.scheme, n_bdf_stages, h);
            free(h);
        }
    }
    fv3d_timedisc_stats st;
    if (fv3d_timedisc(gpu, &o, &st) != FV3D_OK)
        BM_CHECK_EXPRESSION(0);
    fv3d_get_state(gpu, solver_data->phi_total);
}

/* a steady implicit run solved to a relative residual instead (the
 * pseudo-transient Newton-Krylov solver, not the reference's scheme) */
void gpu_solve_steady(double abort_residual, int max_iter)
{
    fv3d_implicit_opts o;
    fv3d_implicit_default_opts(&o);
    o.tol_rel = abort_residual;          /* relative FP64 residual target */
    o.max_newton = max_iter;
    o.preconditioner = FV3D_PC_COUPLED;  /* couples cells; FV3D_PC_LUMPED = reference blocks */
    fv3d_implicit_stats st;
    fv3d_status s = fv3d_solve_implicit(gpu, &o, &st);   /* FV3D_ERR_NOT_CONVERGED: stats still filled */
    if (s != FV3D_OK && s != FV3D_ERR_NOT_CONVERGED)
        BM_CHECK_EXPRESSION(0);
    fv3d_get_state(gpu, solver_data->phi_total);
}

/* ---- the reference-named entry points: link this file before -lsolver ---- */
void finite_volume_time_derivative(double t)   /* finite_volume.c:81-124 */
{
    if (gpu == NULL) gpu_initialize();
    gpu_time_derivative(t);
}

void timedisc(void)                              /* timedisc.c:134-222 */
{
    if (gpu == NULL) gpu_initialize();
    upload_state();                              /* fv3d_set_state from solver_data */
    gpu_timedisc();
}

void calc_global_residual(double dt)           /* analyze.c:37-61 */
{
    fv3d_global_residual(gpu, dt, solver_residual);
}
