/*
 * fv3d_gpu.h - C ABI of the GB300 (sm_103a) FV3D residual / explicit-RK /
 * implicit-solve path.
 *
 * Drop-in boundary for the reference solver library's hot path
 * (src/Solver/include/solver/solver_module.h:16-273 and the Navier-Stokes
 * plug-in registered in src/FV3D/src/navier_stokes/navier_stokes.c:85-124):
 * plain pointers and sizes, no CUDA or C++ types, every call returns a status
 * instead of aborting (the reference aborts through BM_CHECK_EXPRESSION).
 *
 * Ownership: the context owns all device memory.  Host arrays passed in are
 * read during the call only; outputs go to caller-provided host buffers.
 * Arrays are in the reference's order and AoS layouts; the context renumbers
 * internally and maps back.  One host thread per context; all work runs on
 * the context's CUDA stream.
 */
#ifndef FV3D_GPU_H
#define FV3D_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fv3d_ctx fv3d_ctx;

typedef enum fv3d_status {
    FV3D_OK = 0,
    FV3D_ERR_INVALID_ARG = 1,      /* bad argument or inconsistent mesh */
    FV3D_ERR_UNSUPPORTED = 2,      /* feature not available in this build */
    FV3D_ERR_NONFINITE = 3,        /* NaN/Inf residual (timedisc.c:179-181) */
    FV3D_ERR_NOT_CONVERGED = 4,    /* Newton did not converge (implicit.c:350-351) */
    FV3D_ERR_STAGNATED_FALLBACK = 5, /* learned preconditioner stagnated, fell back */
    FV3D_ERR_DEVICE = 6,           /* CUDA error */
    FV3D_ERR_TIMEOUT = 7,          /* a bounded device wait ran out */
    FV3D_ERR_BOUNDS = 8,           /* an index outside its array */
    FV3D_ERR_STATE = 9             /* call out of order (e.g. no mesh yet) */
} fv3d_status;

/* Option codes follow the reference's option order:
 * flux (flux.c:273), reconstruction / limiter (solver_type.h:212-226),
 * explicit scheme (solver_type.h:236-241; SSP-RK3 is new). */
enum { FV3D_FLUX_AUSM = 0, FV3D_FLUX_RUSANOV = 1 };
enum { FV3D_RECON_FIRST_ORDER = 0, FV3D_RECON_LINEAR = 1 };
enum { FV3D_LIMITER_BARTH_JESPERSEN = 0, FV3D_LIMITER_NONE = 1 };
enum { FV3D_GRADIENT_GREEN_GAUSS = 0, FV3D_GRADIENT_LEAST_SQUARES = 1 };
enum { FV3D_PRECISION_FP64 = 0, FV3D_PRECISION_MIXED = 1 };
enum { FV3D_RENUMBER_NONE = 0, FV3D_RENUMBER_MORTON = 1, FV3D_RENUMBER_RCM = 2 };
enum { FV3D_RK_EULER = 0, FV3D_RK_33 = 1, FV3D_RK_45 = 2, FV3D_SSP_RK3 = 3 };
/* boundary (region) types: navier_stokes_module.h:47-59 + pressure outlet */
enum {
    FV3D_BC_FLOW = 0, FV3D_BC_INFLOW = 1, FV3D_BC_OUTFLOW = 2,
    FV3D_BC_WALL_ADIABATIC = 3, FV3D_BC_WALL_ISOTHERMAL = 4,
    FV3D_BC_WALL_SLIP = 5, FV3D_BC_SYMMETRY = 6, FV3D_BC_STATE = 7,
    FV3D_BC_FUNCTION = 8, FV3D_BC_PRESSURE_OUTLET = 9
};

/* Physics and discretisation (parameter keys Equation/Navier-Stokes/...,
 * navier_stokes.c:55-66; FV/Reconstruction, FV/Limiter, .../Flux/flux_scheme) */
typedef struct fv3d_config {
    double kappa;
    double R_mix;
    double mu_mix;
    double Pr;
    double cfl_scale;
    double dfl_scale;
    int flux_scheme;
    int reconstruction;
    int limiter;
    int gradient;
    int precision;
    int renumber;
    int device;
} fv3d_config;

/* Mesh in the reference's processed layout (Mesh_t, solver_type.h:22-168, as
 * read by read_mesh_file mesh.c:121-630).  face_cells[2i+1] = -1 on boundary
 * faces.  face_dist_cell_2 may be NULL; when given it replaces x_f - x_c1 for
 * interior faces (periodic images). */
typedef struct fv3d_mesh_arrays {
    int n_cells;
    int n_faces;
    int n_boundaries;
    int max_cell_faces;
    int n_regions;
    const double *cell_x;       /* [n_cells*3] */
    const double *cell_volume;  /* [n_cells] */
    const double *cell_dx;      /* [n_cells*3] */
    const int *cell_n_faces;    /* [n_cells] */
    const int *cell_faces;      /* [n_cells*max_cell_faces], -1 padded */
    const int *face_cells;      /* [n_faces*2] */
    const int *face_boundary;   /* [n_faces], -1 interior */
    const double *face_area;    /* [n_faces] */
    const double *face_lambda;  /* [n_faces] */
    const double *face_x;       /* [n_faces*3] */
    const double *face_n;       /* [n_faces*3] */
    const double *face_t1;      /* [n_faces*3] */
    const double *face_t2;      /* [n_faces*3] */
    const double *face_dist_cell_2; /* [n_faces*3] or NULL */
    const int *boundary_id;     /* [n_boundaries] region id */
    const int *boundary_face;   /* [n_boundaries] */
    const int *region_is_boundary; /* [n_regions] */
} fv3d_mesh_arrays;

typedef struct fv3d_step_stats {
    double t;           /* time after the steps */
    double dt;          /* last time step used */
    int steps;          /* steps taken */
    double elapsed_ms;  /* device time of the steps (CUDA events) */
} fv3d_step_stats;

/* ---- lifecycle ---------------------------------------------------------- */
/* replaces navier_stokes_initialize + init_reconstruction/init_limiter
 * (navier_stokes.c:85-124, reconstruction.c:110-137, limiter.c:27-41) */
fv3d_status fv3d_create(const fv3d_config *config, fv3d_ctx **ctx);
/* replaces the free_* routines (solver_module.h:61-115) */
fv3d_status fv3d_destroy(fv3d_ctx *ctx);
const char *fv3d_last_error(const fv3d_ctx *ctx);
/* version string and the compiled device architecture */
const char *fv3d_version(void);

/* ---- mesh ------------------------------------------------------------------ */
/* replaces init_mesh(mesh_file) (mesh.c:98-106): takes the arrays that
 * read_mesh_file would load, runs calc_mesh_metrics (mesh.c:19-83),
 * validates indices, renumbers and uploads structure-of-arrays.
 * FV3D_ERR_UNSUPPORTED for a mesh of 2^30 faces or more, or whose face
 * slots (4, 6 or 8 per cell as max_cell_faces rounds up, cells rounded up
 * to a multiple of 128) plus boundaries reach 2^30: face-side indices are
 * carried with the side bit in an int (2^30 slots = 268 million tetrahedra) */
fv3d_status fv3d_mesh_from_arrays(fv3d_ctx *ctx, const fv3d_mesh_arrays *mesh);
/* replaces read_mesh_file (mesh.c:121-630); FV3D_ERR_UNSUPPORTED when this
 * build has no HDF5 library */
fv3d_status fv3d_mesh_load_h5(fv3d_ctx *ctx, const char *path);
/* cell permutation chosen by renumbering: perm[new] = reference index */
fv3d_status fv3d_get_permutation(const fv3d_ctx *ctx, int *perm);

/* replaces boundary_initialize / parse_primitive_state (boundary.c:55-183):
 * prim = (u, v, w, p, T); rho = p / (R T) */
fv3d_status fv3d_set_region(fv3d_ctx *ctx, int region, int bc_type, const double prim[5]);

/* ---- state ---------------------------------------------------------------- */
/* conserved state [n_cells*5] in reference order (set_solution,
 * finite_volume.c:189-201, followed by the update routine) */
fv3d_status fv3d_set_state(fv3d_ctx *ctx, const double *u_con);
/* set_exact_function + set_solution (finite_volume.c:162-200): the initial
 * state from a host function evaluated at every cell centre in reference
 * order, fn(user, id, t, x[3], phi[10]) filling the reference's phi_total row
 * (conserved entries 0..4 used, the primitives recomputed as ns_update does);
 * the reference calls it with id 0 and t 0. */
typedef void (*fv3d_exact_fn)(void *user, int id, double t, const double *x, double *phi);
fv3d_status fv3d_set_exact_function(fv3d_ctx *ctx, fv3d_exact_fn fn, void *user, int id, double t);
/* reference phi_total layout [n_cells*10]: rho, rho_u, rho_v, rho_w, rho_e,
 * u, v, w, p, T (navier_stokes.c:107-117) */
fv3d_status fv3d_get_state(fv3d_ctx *ctx, double *phi_total);
fv3d_status fv3d_get_conserved(fv3d_ctx *ctx, double *u_con);
/* phi_dt [n_cells*5] of the last residual evaluation, in reference order:
 * the time derivative write_output stores (output.c:92-191) */
fv3d_status fv3d_get_time_derivative(fv3d_ctx *ctx, double *phi_dt);

/* ---- hot path ---------------------------------------------------------------- */
/* finite_volume_time_derivative (finite_volume.c:81-124): phi_dt [n_cells*5] */
fv3d_status fv3d_time_derivative(fv3d_ctx *ctx, double t, double *phi_dt);
/* time step.  cfl > 0: cfl * min_i V_i / sum_d (|u_d| + c) dx_d (the
 * convective part of calc_ns_timestep, navier_stokes.c:171-187);
 * cfl <= 0: calc_ns_timestep as written (navier_stokes.c:159-193) */
fv3d_status fv3d_timestep(fv3d_ctx *ctx, double cfl, double *dt);
/* n_steps explicit steps (timestep_lserkw2, explicit.c:96-140, or SSP-RK3),
 * dt recomputed on the device each step from cfl (cfl > 0) or fixed dt_fixed,
 * replayed as one CUDA graph per step.  stats may be NULL. */
fv3d_status fv3d_step_explicit(fv3d_ctx *ctx, int scheme, int n_steps, double cfl,
                               double dt_fixed, fv3d_step_stats *stats);
/* fv3d_set_state(u_in) + fv3d_step_explicit + fv3d_get_conserved(u_out) in
 * one call with one synchronisation: the host-state form of a time step
 * (u_in / u_out [n_cells*5] in reference order, may be the same array;
 * either may be NULL to keep the state on the device). */
fv3d_status fv3d_step_explicit_io(fv3d_ctx *ctx, int scheme, int n_steps, double cfl,
                                  double dt_fixed, const double *u_in, double *u_out,
                                  fv3d_step_stats *stats);
/* calc_global_residual (analyze.c:37-61) of the last residual evaluation */
fv3d_status fv3d_global_residual(fv3d_ctx *ctx, double dt, double res[5]);
/* No counterpart in the reference.  fv3d_global_residual for callers that
 * must not allocate device memory when they call (code running under a fixed
 * device-memory budget or in a section where allocation calls are not
 * allowed): the reduction scratch is one static device array of fixed size
 * (320 KiB per device), so meshes of at most FV3D_NOALLOC_MAX_CELLS cells;
 * larger meshes get FV3D_ERR_UNSUPPORTED.  Results are bitwise those of
 * fv3d_global_residual.  The first call on a device looks up the array's
 * address (cudaGetSymbolAddress).  The address is kept for the rest of the
 * process: after a
 * cudaDeviceReset of that device (which also ends every context of this
 * library on it) do not call this function on the device again.  Each call
 * waits for the context's stream before it returns, as the result is
 * copied into res on the host.  Nothing in the array needs to start at zero.
 * Calls that overlap on one device (other threads, other contexts) race on
 * the one array: serialise them. */
#define FV3D_NOALLOC_MAX_CELLS 2097152
fv3d_status fv3d_global_residual_noalloc(fv3d_ctx *ctx, double dt, double res[5]);

/* ---- implicit steady solve ---------------------------------------------------- */
/* Pseudo-transient Newton-Krylov replacing timestep_newton / calc_jacobian_
 * numerical / the basec Krylov call (implicit.c:61-351): backward Euler with
 * local time steps and a CFL ramp, matrix-free finite-difference J v,
 * FGMRES(krylov_dim) with FP64 Arnoldi, batched 5x5 block-Jacobi
 * preconditioning.  Iterates until ||R||_2 / ||R_0||_2 <= tol_rel. */
enum {
    FV3D_PC_BLOCK_JACOBI = 0,  /* first-order diagonal blocks (FD, FP64 build, FP32 apply) */
    FV3D_PC_LUMPED = 1,        /* the reference's lumped blocks (implicit.c:61-119) */
    FV3D_PC_LEARNED = 2,       /* per-cell MLP; a stagnating cycle is redone with `fallback` */
    FV3D_PC_NONE = 3,
    FV3D_PC_COUPLED = 4        /* couples cells: inner GMRES(inner_dim) on I/dt - dR1/dU, R1 the
                                  first-order inviscid residual with the case's flux (applied
                                  matrix-free: each face flux's exact derivative), right-
                                  preconditioned by inner_sweeps damped block-Jacobi sweeps of the
                                  first-order Rusanov Jacobian (analytic, wave speed frozen) */
};
typedef struct fv3d_implicit_opts {
    double cfl_start;      /* initial CFL (100) */
    double cfl_max;        /* CFL cap of the ramp (1e4) */
    double tol_rel;        /* stop at ||R|| / ||R_0|| <= tol_rel (1e-8) */
    int max_newton;        /* Newton step limit (500) */
    int krylov_dim;        /* FGMRES restart length, 1..31 (30) */
    double eta;            /* linear relative tolerance per Newton step (1e-2) */
    double fd_eps;         /* relative finite-difference step of FP64 J v (1e-7) */
    int jv_precision;      /* 0: J v from the FP64 residual, FP64 Krylov basis; 1: J v from the
                              FP32 residual, FP32 basis and Gram-Schmidt products (FP64 sums and
                              coefficients); 2: J v from the FP32 residual, FP64 basis,
                              Gram-Schmidt and Givens rotations */
    int preconditioner;    /* FV3D_PC_* */
    int pc_refresh;        /* rebuild the preconditioner every pc_refresh Newton steps (and after a
                              CFL back-off); 0: 3 for FV3D_PC_COUPLED, 1 for the others */
    int max_restarts;      /* FGMRES restarts per Newton step (0: one cycle) */
    int sync_every;        /* Arnoldi steps launched between host synchronisations (0: 3 for
                              FV3D_PC_COUPLED, 10 for the others): the Givens rotations of a chunk
                              run after it, so a cycle that meets eta inside a chunk computes up
                              to sync_every - 1 unused steps */
    int inner_dim;         /* FV3D_PC_COUPLED: inner GMRES iterations per application, 1..30 (10) */
    int inner_sweeps;      /* FV3D_PC_COUPLED: Rusanov block-Jacobi sweeps per inner
                              preconditioning, 1..8 (2) */
    double inner_omega;    /* FV3D_PC_COUPLED: damping of those sweeps, (0, 2] (0.7) */
    int fallback;          /* FV3D_PC_LEARNED: the preconditioner a stagnating cycle is redone
                              with, FV3D_PC_BLOCK_JACOBI (default) or FV3D_PC_COUPLED */
} fv3d_implicit_opts;
typedef struct fv3d_implicit_stats {
    int newton_steps;
    int gmres_iterations;
    int jv_evaluations;
    int rejected_steps;    /* Newton updates refused (non-positive state) and retried */
    int fallbacks;         /* learned-preconditioner solves redone with block Jacobi */
    int converged;
    double res0, res_final, rel_res;
    double wall_ms;
    double cfl_final;
} fv3d_implicit_stats;
fv3d_status fv3d_implicit_default_opts(fv3d_implicit_opts *opts);
fv3d_status fv3d_solve_implicit(fv3d_ctx *ctx, const fv3d_implicit_opts *opts,
                                fv3d_implicit_stats *stats);
/* ||R||_2 after each Newton step of the last solve; *count = steps recorded */
fv3d_status fv3d_implicit_history(const fv3d_ctx *ctx, double *res, int max, int *count);
/* 5x5 blocks of the last preconditioner build, [n_cells][25] column-major,
 * reference cell order (lumped blocks: compare with calc_jacobian_numerical) */
fv3d_status fv3d_get_blocks(fv3d_ctx *ctx, double *blocks);
/* Blocks of the operators of the last FV3D_PC_COUPLED build (no reference
 * counterpart: the reference's preconditioner is its lumped diagonal,
 * implicit.c:61-119).  The solve applies them matrix-free; this call writes
 * them out by the same arithmetic, in reference cell order, row-major 5x5:
 * which 0 gives P_A = I/dt - dR1/dU (diagonal blocks and one block per face
 * slot), which 1 the Rusanov matrix P_R (its inverted diagonal blocks and
 * its slot blocks).  diag [n_cells*25],
 * slots [n_cells*max_slots*25], neighbour [n_cells*max_slots] (the slot's
 * other cell, -1 for a boundary face or an unused slot); *max_slots is set
 * first, and NULL arrays are skipped. */
fv3d_status fv3d_get_coupled_blocks(fv3d_ctx *ctx, int which, double *diag, double *slots,
                                    int *neighbour, int *max_slots);
/* The implicit solve's matrix-free Jacobian-vector product at the current
 * state, J z = (R(U + eps z) - R(U)) / eps (the product the reference forms
 * from its lumped blocks in matrix_vector_numerical, implicit.c:362-384,
 * here of the full residual): jv_precision 1 takes FP32 residuals and
 * eps = 5e-4 (1 + |U|) / |z|, 0 FP64 residuals and eps = fd_eps (1 + |U|) / |z|.
 * z and jz are [n_cells][5] rows in reference cell order. */
fv3d_status fv3d_jacobian_vector(fv3d_ctx *ctx, int jv_precision, double fd_eps, const double *z,
                                 double *jz);

/* ---- the reference's implicit time step -------------------------------------- */
/* timestep_newton (implicit.c:224-351) with the lumped Jacobian of
 * calc_jacobian_numerical (implicit.c:61-119: every cell perturbed at once by
 * +-eps/2, eps = 1e-4 ||Y_v||_2, ten FP64 residuals per Newton iteration).
 * The reference solves the block-diagonal system J dY = f_Y with basec's
 * GMRES / BiCGStab to tolerance_lsoe; here each cell's 5x5 block is solved
 * directly (Gaussian elimination with partial pivoting, FP64), which is the
 * converged Krylov answer.  iter is the time-step index (0 starts BDF2 with
 * backward Euler and evaluates the time derivative at t, as timedisc.c does). */
typedef enum { FV3D_NEWTON_EULER = 0, FV3D_NEWTON_BDF2 = 1 } fv3d_newton_scheme;
typedef struct {
    int scheme;          /* a fv3d_newton_scheme value; coefficients of implicit.c:37-38 */
    int max_iter_inner;  /* Newton iterations per step (reference default 100) */
    int is_transient;    /* 0: stop after the first Newton iteration */
} fv3d_newton_opts;
typedef struct {
    int n_inner;         /* Newton iterations taken (the reference's n_inner) */
    double err0, err;    /* ||f_Y|| before and after */
} fv3d_newton_stats;
/* FV3D_ERR_NOT_CONVERGED when it reaches max_iter_inner, as the reference.
 * A BDF2 step with iter >= 1 needs the history of the steps before it (a
 * run started at iter 0, or fv3d_set_bdf_history): FV3D_ERR_STATE otherwise. */
fv3d_status fv3d_step_newton(fv3d_ctx *ctx, const fv3d_newton_opts *opts, int iter, double t,
                             double dt, fv3d_newton_stats *stats);
/* The implicit step's history phi_old (implicit.c:241-250), write_output's
 * phi_old:<stage> datasets: *n_stages = 1 (backward Euler) or 2 (BDF2), 0
 * before the first implicit step; phi_old [n_cells*5] of stage < *n_stages in
 * reference order (phi_old NULL: the count only). */
fv3d_status fv3d_get_bdf_history(fv3d_ctx *ctx, int stage, double *phi_old, int *n_stages);
/* read_restart_data's history (restart.c:50-178): n_stages (1 for backward
 * Euler, 2 for BDF2) arrays phi_old [n_stages*n_cells*5], stage-major, for a
 * run that fv3d_timedisc continues with iter_start > 0.  Call after
 * fv3d_set_state with the restart state: the next step's dY/dt, which the
 * reference takes from the file's phi_dt, is evaluated from that state. */
fv3d_status fv3d_set_bdf_history(fv3d_ctx *ctx, int scheme, int n_stages, const double *phi_old);

/* ---- time loop ----------------------------------------------------------------- */
/* timedisc (timedisc.c:134-222) with init_timedisc's options (timedisc.c:45-66):
 * each iteration takes dt (cfl > 0: the convective CFL step, for explicit
 * schemes computed on the device inside the previous step as the reference
 * computes it on its stage-input primitives; cfl <= 0: calc_ns_timestep as
 * written), clips it to t_end, takes one explicit step (one CUDA graph) or
 * one fv3d_step_newton step, evaluates calc_global_residual(dt) of the step's
 * time derivative, and stops at t_end (transient), when the largest residual
 * falls below abort_residual (steady) or after max_iter iterations.
 * on_iteration (may be NULL) receives what print_residual prints.  A zero
 * time step (calc_ns_timestep's inviscid branch, navier_stokes.c:188-192) is
 * FV3D_ERR_NONFINITE here; the reference loops on without advancing. */
typedef void (*fv3d_iteration_fn)(void *user, int iter, double t, double dt, const double res[5],
                                  int n_inner);
/* called where timedisc calls write_output (timedisc.c:155-156, 210-216):
 * before the first iteration of a run that is not a restart, and after each
 * iteration that print_residual marks ('*': the last one, and every
 * i_output_data-th when i_output_data > 0).  It may read the datasets
 * write_output stores from the same context: fv3d_get_state (phi_total),
 * fv3d_get_time_derivative (phi_dt), fv3d_get_bdf_history (phi_old:<k>). */
typedef void (*fv3d_output_fn)(void *user, int iter, double t);
typedef struct {
    int implicit;           /* 0: explicit (timestep_lserkw2 / SSP-RK3), 1: implicit (timestep_newton) */
    int scheme;             /* explicit: FV3D_RK_*, FV3D_SSP_RK3; implicit: a fv3d_newton_scheme value */
    int max_iter;
    int is_transient;
    double abort_residual;
    double t_start, t_end;
    double cfl;             /* see above */
    int max_iter_inner;     /* implicit */
    fv3d_iteration_fn on_iteration;
    void *user;             /* passed to on_iteration and on_output */
    int iter_start;         /* read_restart_data's iter for a restart (t_start its t), else 0 */
    int i_output_data;      /* Output/i_output_data: -1 first and last, 0 none, k > 0 also every k-th */
    fv3d_output_fn on_output;  /* may be NULL */
} fv3d_timedisc_opts;
typedef struct {
    int iter;               /* iterations taken */
    double t, dt;           /* final time, last step */
    double res[5];          /* last calc_global_residual */
    int stop_reason;        /* 0: t_end, 1: abort_residual, 2: max_iter */
} fv3d_timedisc_stats;
fv3d_status fv3d_timedisc(fv3d_ctx *ctx, const fv3d_timedisc_opts *opts, fv3d_timedisc_stats *stats);

/* ---- learned preconditioner (per-cell MLP 36-64-64-64-5, GELU) -------------------- */
/* BF16 weights / FP32 accumulation on tensor cores, trained on (residual,
 * Newton-correction) pairs that the plain implicit solver harvests; used only
 * inside FGMRES (preconditioner FV3D_PC_LEARNED) with a block-Jacobi redo
 * whenever a linear solve stagnates.  No reference counterpart. */
typedef struct fv3d_mlp_train_opts {
    int epochs;
    int batch;                 /* samples per Adam step (multiple of 64) */
    double lr;
    unsigned long long seed;   /* shuffling */
} fv3d_mlp_train_opts;
typedef struct fv3d_mlp_train_stats {
    double loss_first, loss_last;
    int samples;
    int steps;
    double wall_ms;
} fv3d_mlp_train_stats;
int fv3d_mlp_num_params(void);
fv3d_status fv3d_mlp_init(fv3d_ctx *ctx, unsigned long long seed);
/* packed FP32 parameters: W0[64][36] b0[64] W1[64][64] b1 W2[64][64] b2 W3[5][64] b3[5] */
fv3d_status fv3d_mlp_get_params(fv3d_ctx *ctx, float *params);
fv3d_status fv3d_mlp_set_params(fv3d_ctx *ctx, const float *params);
/* forward of n samples X[n][36] -> Y[n][5] (host buffers) */
fv3d_status fv3d_mlp_forward(fv3d_ctx *ctx, const float *X, int n, float *Y);
/* loss = mean_n sum_j (y - t)^2 and its parameter gradient (host buffers) */
fv3d_status fv3d_mlp_grad(fv3d_ctx *ctx, const float *X, const float *T, int n, double *loss,
                          float *grad);
/* harvest per_step sampled cells per Newton step in later implicit solves,
 * up to max_samples pairs kept on the device (0 disables) */
fv3d_status fv3d_mlp_harvest(fv3d_ctx *ctx, int per_step, int max_samples);
fv3d_status fv3d_mlp_dataset(const fv3d_ctx *ctx, int *n_samples);
/* Adam training on the harvested pairs (forward/backward/Adam kernels) */
fv3d_status fv3d_mlp_train(fv3d_ctx *ctx, const fv3d_mlp_train_opts *opts,
                           fv3d_mlp_train_stats *stats);
/* one Adam step (beta1 0.9, beta2 0.999, eps 1e-8) of the parameters with a
 * caller-given gradient [fv3d_mlp_num_params()], the device step each batch
 * of fv3d_mlp_train takes; moments and step count carry over between calls
 * and training (fv3d_mlp_init resets them) */
fv3d_status fv3d_mlp_adam_step(fv3d_ctx *ctx, const float *grad, double lr);
/* the network's inference kernels (forward and the preconditioner's
 * application): 1 (default) the tcgen05 ones, accumulators in tensor memory,
 * 128-cell tiles; 0 the warp-level mma.sync ones.  Same BF16 roundings. */
fv3d_status fv3d_mlp_set_kernel(fv3d_ctx *ctx, int tensor_core);
/* average device time (ms, CUDA events on the context's stream) of one
 * application of the network to a vector field on the mesh, over n_reps
 * back-to-back applications with the current inference kernels (needs the
 * cell features of a learned or harvesting solve) */
fv3d_status fv3d_profile_mlp(fv3d_ctx *ctx, int n_reps, double *ms);

/* ---- measurement helpers ------------------------------------------------------ */
/* average device time (ms) per launch of each kernel of one explicit stage
 * repeated n_reps times, each bracketed by CUDA events on the context
 * stream: a step's first stage (its RK register written, not read) with
 * dt = 0, so the state does not change; cfl > 0 selects the variant that
 * also computes the next dt.  ms[0] gradients, ms[1] face flux (mixed
 * path: flux + update), ms[2] gather+update (mixed path: 0) */
fv3d_status fv3d_profile_stage(fv3d_ctx *ctx, int n_reps, double cfl, double *ms);
/* the kernels of n_steps real explicit steps of scheme (the launches a step
 * replays, dt on the device from cfl > 0), each launch bracketed by CUDA
 * events: ms[0] gradient pass and ms[1] flux + update pass, each averaged
 * over every stage; ms[2] the last stage's flux pass.  Advances the state. */
fv3d_status fv3d_profile_step(fv3d_ctx *ctx, int scheme, int n_steps, double cfl, double *ms);
/* CUDA stream (cudaStream_t) the context launches on, for event timing */
fv3d_status fv3d_get_stream(const fv3d_ctx *ctx, void **stream);
/* device pointer of the conserved state, [5][n_cells] SoA in renumbered order */
fv3d_status fv3d_device_state(const fv3d_ctx *ctx, double **u_dev);
/* No counterpart in the reference.  Self-test of the bounded device waits
 * (the staged gradient pass's mbarrier waits, which report FV3D_ERR_TIMEOUT
 * instead of hanging): one wait on a phase that no copy completes, limited
 * to limit_us (1 .. 1,000,000); *timed_out = 1 when the kernel gave up and
 * said so, *elapsed_ms the kernel's device time (may be NULL).  Nothing is
 * left pending: no copy was issued. */
fv3d_status fv3d_selftest_bounded_wait(fv3d_ctx *ctx, int limit_us, int *timed_out, double *elapsed_ms);

#ifdef __cplusplus
}
#endif

#endif /* FV3D_GPU_H */
