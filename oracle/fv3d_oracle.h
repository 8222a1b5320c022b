/*
 * CPU oracle API for the FV3D residual / explicit-RK / implicit hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Two libraries implement this header:
 *   - oracle/liboracle.so          this repository's FP64 C restatement of the
 *                                  reference algorithm (fv3d_oracle.c); builds
 *                                  anywhere gcc exists;
 *   - oracle/_ref/libfv3d_ref.so   the reference's own unmodified C sources
 *                                  compiled against a basec stand-in
 *                                  (ref_shim/), built only where the reference
 *                                  tree is present.
 * Only tests/, the smoke check and bench.py's CPU-baseline leg use them.
 *
 * Layouts are the reference's: AoS, phi_total[(n_cells + n_boundaries) * 10]
 * with variables (rho, rho_u, rho_v, rho_w, rho_e, u, v, w, p, T)
 * (navier_stokes.c:107-117), phi_dt[n_cells * 5].  Both libraries hold one
 * global instance, as the reference does.
 */
#ifndef FV3D_ORACLE_H
#define FV3D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Mesh in the reference's HDF5/Mesh_t layout (solver_type.h:22-168).
 * face_cells[2*i+1] is -1 for boundary faces (as written by pyMeshFV3D).
 * face_dist_cell_2 (optional, may be NULL) overrides x_f - x_c1 for faces
 * whose second cell is a periodic image. */
typedef struct orc_mesh
{
    int n_cells;
    int n_faces;
    int n_boundaries;
    int max_cell_faces;
    int n_regions;
    const double *cell_x;
    const double *cell_volume;
    const double *cell_dx;
    const int *cell_n_faces;
    const int *cell_faces;
    const int *face_cells;
    const int *face_boundary;
    const double *face_area;
    const double *face_lambda;
    const double *face_x;
    const double *face_n;
    const double *face_t1;
    const double *face_t2;
    const double *face_dist_cell_2;
    const int *boundary_id;
    const int *boundary_face;
    const int *region_is_boundary;
} orc_mesh;

typedef struct orc_params
{
    double kappa;
    double R_mix;
    double mu_mix;
    double Pr;
    double cfl_scale;
    double dfl_scale;
    int flux_scheme;    /* 0 AUSM, 1 Rusanov (flux.c:273 option order) */
    int reconstruction; /* 0 FirstOrder, 1 Linear (solver_type.h:222-226) */
    int limiter;        /* 0 BarthJespersenn, 1 None (solver_type.h:212-216) */
    int gradient;       /* 0 Green-Gauss (reference), 1 least squares (new) */
} orc_params;

/* Region (boundary-condition) types: the reference's enum BoundaryType
 * (navier_stokes_module.h:47-59) plus ORC_BC_PRESSURE_OUTLET (new). */
enum
{
    ORC_BC_FLOW = 0,
    ORC_BC_INFLOW = 1,
    ORC_BC_OUTFLOW = 2,
    ORC_BC_WALL_ADIABATIC = 3,
    ORC_BC_WALL_ISOTHERMAL = 4,
    ORC_BC_WALL_SLIP = 5,
    ORC_BC_SYMMETRY = 6,
    ORC_BC_STATE = 7,
    ORC_BC_FUNCTION = 8,
    ORC_BC_PRESSURE_OUTLET = 9
};

/* region_prim[n_regions * 5] = (u, v, w, p, T) per region. */
int orc_init(const orc_mesh *mesh, const orc_params *params,
             const int *region_type, const double *region_prim);
void orc_free(void);
const char *orc_error(void);

int orc_set_conserved(const double *u_con);   /* [n_cells*5], then update */
int orc_get_total(double *phi_total);         /* [(n_cells+n_b)*10] */
int orc_time_derivative(double t, double *phi_dt); /* [n_cells*5] */
int orc_get_gradients(double *gx, double *gy, double *gz); /* [(n_cells+n_b)*10] */
int orc_get_face_states(double *left, double *right);      /* [n_faces*10] */
int orc_get_flux(double *flux);                            /* [n_faces*5] */

double orc_timestep_convective(double cfl);
double orc_calc_ns_timestep(void);
int orc_step_lserkw2(int scheme, int iter, double t, double dt);
int orc_step_ssprk3(double t, double dt);
int orc_global_residual(double dt, double *res);

/* Reference-style implicit step (implicit.c:224-351): lumped block-diagonal
 * FD Jacobian, Krylov solve of the block system.  solver: 0 BiCGStab,
 * 1 GMRes; scheme: 0 Euler, 1 BDF2.  Returns inner/lsoe iteration counts. */
int orc_step_newton(int scheme, int solver, int max_iter_inner,
                    double tolerance_lsoe, int max_iter_lsoe,
                    int krylov_dims, int krylov_restarts, int is_transient,
                    int iter, double t, double dt, int *n_inner, int *n_lsoe);
int orc_get_jacobian(double *jac); /* [n_cells*25], column-major blocks */

#ifdef __cplusplus
}
#endif

#endif /* FV3D_ORACLE_H */
