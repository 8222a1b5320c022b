/*
 * FP64 CPU restatement of the FV3D hot path: residual evaluation, explicit
 * low-storage RK and the reference-style implicit Newton step.
 *
 * TEST INFRASTRUCTURE ONLY (the parity oracle).  Only tests/, the smoke check
 * and bench.py's CPU-baseline leg load it (as oracle/liboracle.so); nothing in
 * the product links it.
 *
 * Parity pin: tests/test_oracle_pin.py runs this file and the reference's own
 * unmodified C sources (oracle/_ref, built from the reference tree where it is
 * present) on the same meshes and requires bit-identical results; the
 * committed fixtures in tests/golden/ were produced by the reference build and
 * are checked against this file everywhere else.  To make that possible every
 * expression keeps the reference's operation order (left-to-right sums,
 * reciprocal-multiply vs divide exactly where the reference uses them) and the
 * build disables floating-point contraction.
 *
 * Citations are to files of the reference tree.  Pieces with no reference
 * counterpart (least-squares gradients, SSP-RK3, pressure outlet, convective
 * CFL step) are marked NEW.
 */
#include <math.h>
#include <float.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "fv3d_oracle.h"

#define NV 10 /* total variables per element */
#define NS 5  /* conserved variables */
enum { RHO = 0, MX = 1, MY = 2, MZ = 3, EN = 4, U = 5, V = 6, W = 7, P = 8, T = 9 };

typedef struct
{
    /* mesh (Mesh_t, after calc_mesh_metrics) */
    int nc, nf, nb, mcf, nr;
    double *cx, *vol, *dx;
    int *cnf, *cf;
    int *fcell;            /* second cell = ghost index nc+b on boundary faces */
    int *fbnd;
    double *area, *lam, *fx, *fn, *ft1, *ft2, *d1, *d2;
    int *internal, n_internal, *bfaces, n_bfaces;
    int *bid, *bface;
    double vol_total;
    /* least-squares weights (NEW), per face and side: [nf][2][3] */
    double *lsq;
    /* physics */
    orc_params p;
    double km1, kp1, s_km1, s_kp1, cp, kappa_pr, heat_lambda;
    int *rtype;
    double *rphi; /* [nr][NV] region states (prim given, converted to con) */
    /* solution data (data_t, finite_volume.c:23-55) */
    double *phi, *gx, *gy, *gz, *left, *right, *flux, *dphi;
    /* implicit */
    int imp_ready, n_bdf;
    double *phi_old[2], *Y, *fY, *dY, *dYdt, *jac, *work;
    double dt_loc, tpdt_loc, bdf_b_loc;
    int n_inner, n_lsoe;
} oracle_t;

static oracle_t G;
static char g_err[256];
static int g_ready = 0;

const char *orc_error(void) { return g_err; }

static void *zalloc(size_t n) { return calloc(1, n > 0 ? n : 1); }

/* ---- vector helpers with the stand-in's loop order ------------------------ */
static double dot3(const double *a, const double *b)
{
    double s = 0.0;
    s += a[0] * b[0];
    s += a[1] * b[1];
    s += a[2] * b[2];
    return s;
}

static double dotn(const double *a, const double *b, size_t n)
{
    double s = 0.0;
    for (size_t i = 0; i < n; ++i)
        s += a[i] * b[i];
    return s;
}
#define dot_n dotn
static double len_n(const double *a, size_t n) { return sqrt(dotn(a, a, n)); }
typedef int (*shim_matvec_ft)(double *x, double *b, size_t n_var, size_t n_cells);
#include "krylov.c"

static double dmin(double a, double b) { return (a < b) ? a : b; }
static double dmax(double a, double b) { return (a > b) ? a : b; }
static double dabs(double a) { return (a < 0) ? -a : a; }

/* ---- equation of state (eos.c) ---------------------------------------------- */
/* eos.c:81-92 */
static void cons_to_prims(double *q)
{
    q[U] = q[MX] / q[RHO];
    q[V] = q[MY] / q[RHO];
    q[W] = q[MZ] / q[RHO];
    q[P] = G.km1 * (q[EN] - 0.5 * dot3(&q[MX], &q[U]));
    q[P] = dmax(1.00E-10, q[P]);
    q[T] = q[P] / (q[RHO] * G.p.R_mix);
}

/* eos.c:120-127 */
static void prims_to_cons(double *q)
{
    q[MX] = q[U] * q[RHO];
    q[MY] = q[V] * q[RHO];
    q[MZ] = q[W] * q[RHO];
    q[EN] = G.s_km1 * q[P] + 0.5 * dot3(&q[U], &q[MX]);
}

/* eos.c:55-75: pressure behind a wave for the face-normal velocity q[U] */
static double wall_pressure(const double *q)
{
    const double k = G.p.kappa;
    if (q[U] <= 0.0)
    {
        double c = sqrt(k * q[P] / q[RHO]);
        return q[P] * pow(dmax(1e-4, 1. + 0.5 * G.km1 * q[U] / c), 2 * k * G.s_km1);
    }
    double ar = 2 * G.s_kp1 / q[U];
    double br = G.km1 * G.s_kp1 * q[P];
    return q[P] + q[U] / ar * 0.5 * (q[U] + sqrt(q[U] * q[U] + 4. * ar * (q[P] + br)));
}

/* ---- boundary ghost states (boundary.c:188-320) ---------------------------- */
static void rotate_back(double *g, const double *n, const double *t1, const double *t2)
{
    double a = g[U] * n[0] + g[V] * t1[0] + g[W] * t2[0];
    double b = g[U] * n[1] + g[V] * t1[1] + g[W] * t2[1];
    double c = g[U] * n[2] + g[V] * t1[2] + g[W] * t2[2];
    g[U] = a;
    g[V] = b;
    g[W] = c;
}

static void ghost_states(void)
{
    for (int b = 0; b < G.nb; ++b)
    {
        int f = G.bface[b];
        int c = G.fcell[2 * f];
        int r = G.bid[b];
        const double *n = &G.fn[3 * f], *t1 = &G.ft1[3 * f], *t2 = &G.ft2[3 * f];
        const double *in = &G.phi[(size_t)c * NV];
        double *g = &G.phi[(size_t)(G.nc + b) * NV];
        memcpy(g, in, sizeof(double) * NV);
        switch (G.rtype[r])
        {
        case ORC_BC_INFLOW:
        case ORC_BC_STATE:
            memcpy(g, &G.rphi[r * NV], sizeof(double) * NV);
            break;
        case ORC_BC_OUTFLOW:
            break;
        case ORC_BC_PRESSURE_OUTLET: /* NEW: interior state at the region's pressure */
            g[P] = G.rphi[r * NV + P];
            g[T] = g[P] / (g[RHO] * G.p.R_mix);
            break;
        case ORC_BC_WALL_ADIABATIC:
        case ORC_BC_WALL_ISOTHERMAL:
            g[U] = dot3(&in[U], n);
            g[V] = dot3(&in[U], t1);
            g[W] = dot3(&in[U], t2);
            g[P] = wall_pressure(g);
            g[U] = 0.0;
            g[V] = 0.0;
            g[W] = 0.0;
            if (G.rtype[r] == ORC_BC_WALL_ISOTHERMAL)
                g[T] = G.rphi[r * NV + T];
            g[RHO] = g[P] / (G.p.R_mix * g[T]);
            rotate_back(g, n, t1, t2);
            break;
        case ORC_BC_WALL_SLIP:
        case ORC_BC_SYMMETRY:
            g[U] = dot3(&in[U], n);
            g[V] = dot3(&in[U], t1);
            g[W] = dot3(&in[U], t2);
            g[P] = wall_pressure(g);
            g[U] = 0.0;
            g[T] = g[P] / (g[RHO] * G.p.R_mix);
            rotate_back(g, n, t1, t2);
            break;
        default:
            break;
        }
        prims_to_cons(g);
    }
}

/* ns_update (navier_stokes.c:199-209) */
static void update(void)
{
    for (int i = 0; i < G.nc; ++i)
        cons_to_prims(&G.phi[(size_t)i * NV]);
    ghost_states();
}

/* boundary.c:325-412 */
static void ghost_gradients(void)
{
    for (int b = 0; b < G.nb; ++b)
    {
        int f = G.bface[b];
        int c = G.fcell[2 * f];
        int r = G.bid[b];
        const double *n = &G.fn[3 * f], *t1 = &G.ft1[3 * f], *t2 = &G.ft2[3 * f];
        double *x = &G.gx[(size_t)(G.nc + b) * NV];
        double *y = &G.gy[(size_t)(G.nc + b) * NV];
        double *z = &G.gz[(size_t)(G.nc + b) * NV];
        memcpy(x, &G.gx[(size_t)c * NV], sizeof(double) * NV);
        memcpy(y, &G.gy[(size_t)c * NV], sizeof(double) * NV);
        memcpy(z, &G.gz[(size_t)c * NV], sizeof(double) * NV);
        if (G.rtype[r] == ORC_BC_WALL_SLIP || G.rtype[r] == ORC_BC_SYMMETRY)
        {
            for (int j = 0; j < NV; ++j)
            {
                /* normal component removed, tangential kept */
                double a1 = x[j] * t1[0] + y[j] * t1[1] + z[j] * t1[2];
                double a2 = x[j] * t2[0] + y[j] * t2[1] + z[j] * t2[2];
                double a0 = 0.0;
                x[j] = a0 * n[0] + a1 * t1[0] + a2 * t2[0];
                y[j] = a0 * n[1] + a1 * t1[1] + a2 * t2[1];
                z[j] = a0 * n[2] + a1 * t1[2] + a2 * t2[2];
            }
        }
    }
}

/* ---- gradients ------------------------------------------------------------- */
/* Green-Gauss, reconstruction.c:20-93 */
static void gradients_green_gauss(void)
{
    size_t ne = (size_t)(G.nc + G.nb) * NV;
    memset(G.gx, 0, sizeof(double) * ne);
    memset(G.gy, 0, sizeof(double) * ne);
    memset(G.gz, 0, sizeof(double) * ne);
    for (int f = 0; f < G.nf; ++f)
    {
        const int a = G.fcell[2 * f], b = G.fcell[2 * f + 1];
        const double *n = &G.fn[3 * f];
        const double A = G.area[f];
        for (int j = 0; j < NV; ++j)
        {
            double q0 = G.phi[(size_t)a * NV + j];
            double mean = q0 + G.lam[f] * (G.phi[(size_t)b * NV + j] - q0);
            G.gx[(size_t)a * NV + j] += mean * n[0] * A;
            G.gy[(size_t)a * NV + j] += mean * n[1] * A;
            G.gz[(size_t)a * NV + j] += mean * n[2] * A;
            G.gx[(size_t)b * NV + j] -= mean * n[0] * A;
            G.gy[(size_t)b * NV + j] -= mean * n[1] * A;
            G.gz[(size_t)b * NV + j] -= mean * n[2] * A;
        }
    }
    for (int i = 0; i < G.nc; ++i)
    {
        double s = 1.0 / G.vol[i];
        for (int j = 0; j < NV; ++j)
        {
            G.gx[(size_t)i * NV + j] *= s;
            G.gy[(size_t)i * NV + j] *= s;
            G.gz[(size_t)i * NV + j] *= s;
        }
    }
    ghost_gradients();
}

/* NEW: unweighted least squares.  For cell i with neighbour offsets d_k
 * (x_k - x_i, periodic image; for a boundary face the face centre with the
 * ghost value) grad = M^{-1} sum_k d_k (phi_k - phi_i), M = sum_k d_k d_k^T.
 * The per-face vectors w = M^{-1} d are precomputed in G.lsq. */
static void lsq_setup(void)
{
    G.lsq = zalloc(sizeof(double) * 6 * (size_t)G.nf);
    for (int i = 0; i < G.nc; ++i)
    {
        double M[6] = {0, 0, 0, 0, 0, 0}; /* xx xy xz yy yz zz */
        double d[8][3];
        int nf = G.cnf[i];
        for (int k = 0; k < nf; ++k)
        {
            int f = G.cf[i * G.mcf + k];
            if (G.fcell[2 * f] == i)
            {
                if (G.fbnd[f] >= 0)
                    for (int q = 0; q < 3; ++q)
                        d[k][q] = G.d1[3 * f + q];
                else
                    for (int q = 0; q < 3; ++q)
                        d[k][q] = G.d1[3 * f + q] - G.d2[3 * f + q];
            }
            else
                for (int q = 0; q < 3; ++q)
                    d[k][q] = G.d2[3 * f + q] - G.d1[3 * f + q];
            M[0] += d[k][0] * d[k][0];
            M[1] += d[k][0] * d[k][1];
            M[2] += d[k][0] * d[k][2];
            M[3] += d[k][1] * d[k][1];
            M[4] += d[k][1] * d[k][2];
            M[5] += d[k][2] * d[k][2];
        }
        /* inverse of the symmetric 3x3 by cofactors */
        double c00 = M[3] * M[5] - M[4] * M[4];
        double c01 = M[2] * M[4] - M[1] * M[5];
        double c02 = M[1] * M[4] - M[2] * M[3];
        double c11 = M[0] * M[5] - M[2] * M[2];
        double c12 = M[1] * M[2] - M[0] * M[4];
        double c22 = M[0] * M[3] - M[1] * M[1];
        double det = M[0] * c00 + M[1] * c01 + M[2] * c02;
        double s = 1.0 / det;
        for (int k = 0; k < nf; ++k)
        {
            int f = G.cf[i * G.mcf + k];
            int side = (G.fcell[2 * f] == i) ? 0 : 1;
            double *w = &G.lsq[6 * (size_t)f + 3 * side];
            w[0] = s * (c00 * d[k][0] + c01 * d[k][1] + c02 * d[k][2]);
            w[1] = s * (c01 * d[k][0] + c11 * d[k][1] + c12 * d[k][2]);
            w[2] = s * (c02 * d[k][0] + c12 * d[k][1] + c22 * d[k][2]);
        }
    }
}

static void gradients_least_squares(void)
{
    size_t ne = (size_t)(G.nc + G.nb) * NV;
    memset(G.gx, 0, sizeof(double) * ne);
    memset(G.gy, 0, sizeof(double) * ne);
    memset(G.gz, 0, sizeof(double) * ne);
    for (int i = 0; i < G.nc; ++i)
    {
        for (int k = 0; k < G.cnf[i]; ++k)
        {
            int f = G.cf[i * G.mcf + k];
            int side = (G.fcell[2 * f] == i) ? 0 : 1;
            int o = G.fcell[2 * f + (1 - side)];
            const double *w = &G.lsq[6 * (size_t)f + 3 * side];
            for (int j = 0; j < NV; ++j)
            {
                double dq = G.phi[(size_t)o * NV + j] - G.phi[(size_t)i * NV + j];
                G.gx[(size_t)i * NV + j] += w[0] * dq;
                G.gy[(size_t)i * NV + j] += w[1] * dq;
                G.gz[(size_t)i * NV + j] += w[2] * dq;
            }
        }
    }
    ghost_gradients();
}

/* ---- limiter (limiter.c:49-122) ----------------------------------------------- */
static double limit(int c, int j, double slope)
{
    if (G.p.limiter != 0)
        return 1.0;
    const double q = G.phi[(size_t)c * NV + j];
    double lo = q, hi = q;
    for (int k = 0; k < G.cnf[c]; ++k)
    {
        int f = G.cf[c * G.mcf + k];
        int o = (G.fcell[2 * f] == c) ? G.fcell[2 * f + 1] : G.fcell[2 * f];
        double qo = G.phi[(size_t)o * NV + j];
        lo = dmin(lo, qo);
        hi = dmax(hi, qo);
    }
    /* the factor depends only on this face's slope (limiter.c:86-103) */
    double y = 1.0;
    if (slope > 0)
        y = (hi - q) / slope;
    else if (slope < 0)
        y = (lo - q) / slope;
    return dmin(1.0, y);
}

/* ---- reconstruction (reconstruction.c:142-255) ------------------------------------ */
static void reconstruct_side(int f, int c, const double *r, double *out)
{
    const double *gx = &G.gx[(size_t)c * NV], *gy = &G.gy[(size_t)c * NV],
                 *gz = &G.gz[(size_t)c * NV];
    for (int j = 0; j < NV; ++j)
    {
        double slope = r[0] * gx[j] + r[1] * gy[j] + r[2] * gz[j];
        double l = limit(c, j, slope);
        out[j] = G.phi[(size_t)c * NV + j] + l * slope;
    }
    (void)f;
}

static void reconstruct(void)
{
    update();
    if (G.p.gradient == 0)
        gradients_green_gauss();
    else
        gradients_least_squares();
    if (G.p.reconstruction == 0)
    {
        for (int f = 0; f < G.nf; ++f)
        {
            memcpy(&G.left[(size_t)f * NV], &G.phi[(size_t)G.fcell[2 * f] * NV], sizeof(double) * NV);
            memcpy(&G.right[(size_t)f * NV], &G.phi[(size_t)G.fcell[2 * f + 1] * NV], sizeof(double) * NV);
        }
        return;
    }
    for (int ii = 0; ii < G.n_internal; ++ii)
    {
        int f = G.internal[ii];
        reconstruct_side(f, G.fcell[2 * f], &G.d1[3 * f], &G.left[(size_t)f * NV]);
        reconstruct_side(f, G.fcell[2 * f + 1], &G.d2[3 * f], &G.right[(size_t)f * NV]);
    }
    for (int ii = 0; ii < G.n_bfaces; ++ii)
    {
        int f = G.bfaces[ii];
        reconstruct_side(f, G.fcell[2 * f], &G.d1[3 * f], &G.left[(size_t)f * NV]);
        memcpy(&G.right[(size_t)f * NV], &G.phi[(size_t)G.fcell[2 * f + 1] * NV], sizeof(double) * NV);
    }
}

/* ---- fluxes (flux.c) -------------------------------------------------------------- */
/* flux.c:203-210 */
static void euler_flux_1d(const double *q, double *f)
{
    f[0] = q[MX];
    f[1] = q[MX] * q[U] + q[P];
    f[2] = q[MX] * q[V];
    f[3] = q[MX] * q[W];
    f[4] = (q[EN] + q[P]) * q[U];
}

/* flux.c:320-336 */
static void flux_rusanov(const double *l, const double *r, double *f)
{
    double cl = sqrt(G.p.kappa * l[P] / l[RHO]);
    double cr = sqrt(G.p.kappa * r[P] / r[RHO]);
    double lam = dmax(dabs(l[U]) + cl, dabs(r[U]) + cr);
    double fl[NS], fr[NS];
    euler_flux_1d(l, fl);
    euler_flux_1d(r, fr);
    for (int j = 0; j < NS; ++j)
        f[j] = 0.5 * (fl[j] + fr[j]) - 0.5 * lam * (r[j] - l[j]);
}

/* flux.c:344-406 */
static void flux_ausm(const double *l, const double *r, double *f)
{
    double cl = sqrt(G.p.kappa * l[P] / l[RHO]);
    double cr = sqrt(G.p.kappa * r[P] / r[RHO]);
    double ml = l[U] / cl, mr = r[U] / cr;
    double hl = (l[EN] + l[P]) / l[RHO];
    double hr = (r[EN] + r[P]) / r[RHO];
    double mp, pp, mm, pm;
    if (ml <= -1.0)
    {
        mp = 0.0;
        pp = 0.0;
    }
    else if (ml < 1.0)
    {
        mp = 0.25 * (ml + 1.0) * (ml + 1.0);
        pp = 0.25 * l[P] * (1.0 + ml) * (1.0 + ml) * (2.0 - ml);
    }
    else
    {
        mp = ml;
        pp = l[P];
    }
    if (mr <= -1.0)
    {
        mm = mr;
        pm = r[P];
    }
    else if (mr < 1.0)
    {
        mm = -0.25 * (mr - 1.0) * (mr - 1.0);
        pm = 0.25 * r[P] * (1.0 - mr) * (1.0 - mr) * (2.0 + mr);
    }
    else
    {
        mm = 0.0;
        pm = 0.0;
    }
    double up = dmax(0.0, mp + mm), um = dmin(0.0, mp + mm);
    f[0] = up * cl * l[RHO];
    f[1] = up * cl * l[RHO] * l[U] + pp;
    f[2] = up * cl * l[RHO] * l[V];
    f[3] = up * cl * l[RHO] * l[W];
    f[4] = up * cl * l[RHO] * hl;
    f[0] += um * cr * r[RHO];
    f[1] += um * cr * r[RHO] * r[U] + pm;
    f[2] += um * cr * r[RHO] * r[V];
    f[3] += um * cr * r[RHO] * r[W];
    f[4] += um * cr * r[RHO] * hr;
}

/* flux.c:215-263: stresses use gradients of the conserved momenta (as the
 * reference does), heat flux the temperature gradient */
static void viscous_flux_1d(const double *q, const double *gx, const double *gy,
                            const double *gz, double *f, double *g, double *h)
{
    const double s23 = 2.0 / 3.0, s43 = 4.0 / 3.0, mu = G.p.mu_mix;
    double txx = mu * (s43 * gx[1] - s23 * gy[2] - s23 * gz[3]);
    double tyy = mu * (-s23 * gx[1] + s43 * gy[2] - s23 * gz[3]);
    double tzz = mu * (-s23 * gx[1] - s23 * gy[2] + s43 * gz[3]);
    double txy = mu * (gy[1] + gx[2]);
    double txz = mu * (gz[1] + gx[3]);
    double tyz = mu * (gz[2] + gy[3]);
    const double k = G.heat_lambda;
    f[0] = 0.0;
    f[1] = -txx;
    f[2] = -txy;
    f[3] = -txz;
    f[4] = -txx * q[U] - txy * q[V] - txz * q[W] - k * gx[T];
    g[0] = 0.0;
    g[1] = -txy;
    g[2] = -tyy;
    g[3] = -tyz;
    g[4] = -txy * q[U] - tyy * q[V] - tyz * q[W] - k * gy[T];
    h[0] = 0.0;
    h[1] = -txz;
    h[2] = -tyz;
    h[3] = -tzz;
    h[4] = -txz * q[U] - tyz * q[V] - tzz * q[W] - k * gz[T];
}

static void rotate_in(const double *q, const double *n, const double *t1,
                      const double *t2, double *out)
{
    out[RHO] = q[RHO];
    out[MX] = dot3(&q[MX], n);
    out[MY] = dot3(&q[MX], t1);
    out[MZ] = dot3(&q[MX], t2);
    out[EN] = q[EN];
    cons_to_prims(out);
}

/* calc_ns_flux, flux.c:23-198 (same arithmetic for interior and boundary faces) */
static void face_fluxes(void)
{
    for (int f = 0; f < G.nf; ++f)
    {
        const int a = G.fcell[2 * f], b = G.fcell[2 * f + 1];
        const double *n = &G.fn[3 * f], *t1 = &G.ft1[3 * f], *t2 = &G.ft2[3 * f];
        const double *ql = &G.left[(size_t)f * NV], *qr = &G.right[(size_t)f * NV];
        double lr[NV], rr[NV], fc[NS];
        rotate_in(ql, n, t1, t2, lr);
        rotate_in(qr, n, t1, t2, rr);
        if (G.p.flux_scheme == 1)
            flux_rusanov(lr, rr, fc);
        else
            flux_ausm(lr, rr, fc);
        double *out = &G.flux[(size_t)f * NS];
        out[0] = fc[0];
        out[1] = fc[1] * n[0] + fc[2] * t1[0] + fc[3] * t2[0];
        out[2] = fc[1] * n[1] + fc[2] * t1[1] + fc[3] * t2[1];
        out[3] = fc[1] * n[2] + fc[2] * t1[2] + fc[3] * t2[2];
        out[4] = fc[4];
        double fl[NS], gl[NS], hl[NS], fr[NS], gr[NS], hr[NS];
        viscous_flux_1d(ql, &G.gx[(size_t)a * NV], &G.gy[(size_t)a * NV], &G.gz[(size_t)a * NV], fl, gl, hl);
        viscous_flux_1d(qr, &G.gx[(size_t)b * NV], &G.gy[(size_t)b * NV], &G.gz[(size_t)b * NV], fr, gr, hr);
        for (int j = 0; j < NS; ++j)
        {
            double fv = 0.5 * (fl[j] + fr[j]);
            double gv = 0.5 * (gl[j] + gr[j]);
            double hv = 0.5 * (hl[j] + hr[j]);
            out[j] += fv * n[0] + gv * n[1] + hv * n[2];
        }
    }
}

/* ---- residual (finite_volume.c:81-124) ----------------------------------------------- */
static void time_derivative(double t)
{
    (void)t;
    reconstruct();
    face_fluxes();
    memset(G.dphi, 0, sizeof(double) * NS * (size_t)(G.nc + G.nb));
    for (int f = 0; f < G.nf; ++f)
    {
        const int a = G.fcell[2 * f], b = G.fcell[2 * f + 1];
        const double A = G.area[f];
        for (int j = 0; j < NS; ++j)
        {
            G.dphi[(size_t)a * NS + j] += G.flux[(size_t)f * NS + j] * A;
            G.dphi[(size_t)b * NS + j] -= G.flux[(size_t)f * NS + j] * A;
        }
    }
    for (int i = 0; i < G.nc; ++i)
        for (int j = 0; j < NS; ++j)
            G.dphi[(size_t)i * NS + j] = -G.dphi[(size_t)i * NS + j] / G.vol[i];
}

/* ---- set-up ------------------------------------------------------------------------ */
void orc_free(void)
{
    if (!g_ready)
        return;
    void *ptrs[] = {G.cx, G.vol, G.dx, G.cnf, G.cf, G.fcell, G.fbnd, G.area, G.lam,
                    G.fx, G.fn, G.ft1, G.ft2, G.d1, G.d2, G.internal, G.bfaces, G.bid,
                    G.bface, G.lsq, G.rtype, G.rphi, G.phi, G.gx, G.gy, G.gz, G.left,
                    G.right, G.flux, G.dphi, G.phi_old[0], G.phi_old[1], G.Y, G.fY,
                    G.dY, G.dYdt, G.jac, G.work};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i)
        free(ptrs[i]);
    memset(&G, 0, sizeof(G));
    g_ready = 0;
}

#define COPY(dst, src, type, n)                              \
    do                                                       \
    {                                                        \
        (dst) = zalloc(sizeof(type) * (size_t)(n));          \
        memcpy((dst), (src), sizeof(type) * (size_t)(n));    \
    } while (0)

int orc_init(const orc_mesh *m, const orc_params *p, const int *region_type,
             const double *region_prim)
{
    orc_free();
    memset(&G, 0, sizeof(G));
    G.nc = m->n_cells;
    G.nf = m->n_faces;
    G.nb = m->n_boundaries;
    G.mcf = m->max_cell_faces;
    G.nr = m->n_regions;
    if (G.mcf > 8)
    {
        snprintf(g_err, sizeof(g_err), "max_cell_faces > 8 unsupported");
        return -1;
    }
    COPY(G.cx, m->cell_x, double, 3 * G.nc);
    COPY(G.vol, m->cell_volume, double, G.nc);
    COPY(G.dx, m->cell_dx, double, 3 * G.nc);
    COPY(G.cnf, m->cell_n_faces, int, G.nc);
    COPY(G.cf, m->cell_faces, int, G.mcf * G.nc);
    COPY(G.fcell, m->face_cells, int, 2 * G.nf);
    COPY(G.fbnd, m->face_boundary, int, G.nf);
    COPY(G.area, m->face_area, double, G.nf);
    COPY(G.lam, m->face_lambda, double, G.nf);
    COPY(G.fx, m->face_x, double, 3 * G.nf);
    COPY(G.fn, m->face_n, double, 3 * G.nf);
    COPY(G.ft1, m->face_t1, double, 3 * G.nf);
    COPY(G.ft2, m->face_t2, double, 3 * G.nf);
    COPY(G.bid, m->boundary_id, int, G.nb);
    COPY(G.bface, m->boundary_face, int, G.nb);
    G.p = *p;
    g_ready = 1;

    /* calc_mesh_metrics, mesh.c:19-83 */
    G.vol_total = 0.0;
    for (int i = 0; i < G.nc; ++i)
        G.vol_total += G.vol[i];
    G.d1 = zalloc(sizeof(double) * 3 * (size_t)G.nf);
    G.d2 = zalloc(sizeof(double) * 3 * (size_t)G.nf);
    G.internal = zalloc(sizeof(int) * (size_t)G.nf);
    G.bfaces = zalloc(sizeof(int) * (size_t)G.nf);
    for (int f = 0; f < G.nf; ++f)
    {
        int *fc = &G.fcell[2 * f];
        for (int d = 0; d < 3; ++d)
            G.d1[3 * f + d] = G.fx[3 * f + d] - G.cx[3 * fc[0] + d];
        if (fc[1] >= 0)
        {
            for (int d = 0; d < 3; ++d)
                G.d2[3 * f + d] = (m->face_dist_cell_2 != NULL)
                                      ? m->face_dist_cell_2[3 * f + d]
                                      : G.fx[3 * f + d] - G.cx[3 * fc[1] + d];
            G.internal[G.n_internal++] = f;
        }
        else
        {
            if (G.fbnd[f] < 0 || G.fbnd[f] >= G.nb)
            {
                snprintf(g_err, sizeof(g_err), "face %d: bad boundary index", f);
                orc_free();
                return -1;
            }
            fc[1] = G.nc + G.fbnd[f];
            G.bfaces[G.n_bfaces++] = f;
        }
    }

    /* navier_stokes.c:85-124 derived constants */
    G.km1 = p->kappa - 1.0;
    G.kp1 = p->kappa + 1.0;
    G.s_km1 = 1.0 / G.km1;
    G.s_kp1 = 1.0 / G.kp1;
    double cv = p->R_mix * G.s_km1;
    G.cp = p->kappa * cv;
    G.kappa_pr = p->kappa / p->Pr;
    G.heat_lambda = p->mu_mix * G.cp / p->Pr;

    /* regions (boundary.c:55-183): primitive state -> rho, then conserved */
    G.rtype = zalloc(sizeof(int) * (size_t)G.nr);
    G.rphi = zalloc(sizeof(double) * NV * (size_t)G.nr);
    for (int r = 0; r < G.nr; ++r)
    {
        G.rtype[r] = region_type[r];
        double *q = &G.rphi[r * NV];
        q[U] = region_prim[5 * r + 0];
        q[V] = region_prim[5 * r + 1];
        q[W] = region_prim[5 * r + 2];
        q[P] = region_prim[5 * r + 3];
        q[T] = region_prim[5 * r + 4];
        q[RHO] = q[P] / (p->R_mix * q[T]);
        prims_to_cons(q);
    }

    size_t ne = (size_t)(G.nc + G.nb);
    G.phi = zalloc(sizeof(double) * NV * ne);
    G.gx = zalloc(sizeof(double) * NV * ne);
    G.gy = zalloc(sizeof(double) * NV * ne);
    G.gz = zalloc(sizeof(double) * NV * ne);
    G.left = zalloc(sizeof(double) * NV * (size_t)G.nf);
    G.right = zalloc(sizeof(double) * NV * (size_t)G.nf);
    G.flux = zalloc(sizeof(double) * NS * (size_t)G.nf);
    G.dphi = zalloc(sizeof(double) * NS * ne);
    if (p->gradient == 1)
        lsq_setup();
    /* initial state = flow region (finite_volume.c:189-201 with
     * calc_ns_exact_function, navier_stokes.c:133-152) */
    int flow = 0;
    for (int r = 0; r < G.nr; ++r)
        if (m->region_is_boundary[r] == 0)
        {
            flow = r;
            break;
        }
    for (int i = 0; i < G.nc; ++i)
        memcpy(&G.phi[(size_t)i * NV], &G.rphi[flow * NV], sizeof(double) * NV);
    update();
    return 0;
}

int orc_set_conserved(const double *u)
{
    for (int i = 0; i < G.nc; ++i)
        for (int j = 0; j < NS; ++j)
            G.phi[(size_t)i * NV + j] = u[(size_t)i * NS + j];
    update();
    return 0;
}

int orc_get_total(double *out)
{
    memcpy(out, G.phi, sizeof(double) * NV * (size_t)(G.nc + G.nb));
    return 0;
}

int orc_time_derivative(double t, double *out)
{
    time_derivative(t);
    memcpy(out, G.dphi, sizeof(double) * NS * (size_t)G.nc);
    return 0;
}

int orc_get_gradients(double *x, double *y, double *z)
{
    size_t n = sizeof(double) * NV * (size_t)(G.nc + G.nb);
    memcpy(x, G.gx, n);
    memcpy(y, G.gy, n);
    memcpy(z, G.gz, n);
    return 0;
}

int orc_get_face_states(double *l, double *r)
{
    memcpy(l, G.left, sizeof(double) * NV * (size_t)G.nf);
    memcpy(r, G.right, sizeof(double) * NV * (size_t)G.nf);
    return 0;
}

int orc_get_flux(double *out)
{
    memcpy(out, G.flux, sizeof(double) * NS * (size_t)G.nf);
    return 0;
}

/* NEW: convective part of calc_ns_timestep with an explicit CFL number */
double orc_timestep_convective(double cfl)
{
    double lc = DBL_MAX;
    for (int i = 0; i < G.nc; ++i)
    {
        const double *q = &G.phi[(size_t)i * NV];
        const double *d = &G.dx[3 * (size_t)i];
        double s_rho = 1.0 / q[RHO];
        double c = sqrt(G.p.kappa * q[P] * s_rho);
        double ds = (dabs(q[U]) + c) * d[0] + (dabs(q[V]) + c) * d[1] + (dabs(q[W]) + c) * d[2];
        lc = dmin(lc, G.vol[i] / ds);
    }
    return lc * cfl;
}

/* navier_stokes.c:159-193, including its viscous branch as written */
double orc_calc_ns_timestep(void)
{
    double lc = DBL_MAX, lv = DBL_MAX;
    for (int i = 0; i < G.nc; ++i)
    {
        const double *q = &G.phi[(size_t)i * NV];
        const double *d = &G.dx[3 * (size_t)i];
        double s_rho = 1.0 / q[RHO];
        double c = sqrt(G.p.kappa * q[P] * s_rho);
        double ds = (dabs(q[U]) + c) * d[0] + (dabs(q[V]) + c) * d[1] + (dabs(q[W]) + c) * d[2];
        lc = dmin(lc, G.vol[i] / ds);
        double ds2 = dot3(d, d);
        lv = dmin(lv, s_rho * ds2 / G.vol[i]);
    }
    lc *= G.p.cfl_scale;
    lv *= G.p.dfl_scale * G.p.mu_mix * G.kappa_pr * lv;
    return dmin(lc, lv);
}

/* ---- explicit stepping (explicit.c) --------------------------------------------------- */
/* Williamson 2N low-storage tables, explicit.c:19-39 (coefficients of the
 * published schemes: forward Euler, Williamson RK3, Carpenter-Kennedy RK4(5)) */
static const double RK_A[3][5] = {
    {0.0},
    {0., -5. / 9., -153. / 128.},
    {0., -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
     -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0}};
static const double RK_G[3][5] = {
    {1.0},
    {1. / 3., 15. / 16., 8. / 15.},
    {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
     1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
     2277821191437.0 / 14882151754819.0}};
static const double RK_B[3][5] = {
    {0.0},
    {0., 1. / 3., 3. / 4.},
    {0., 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
     2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0}};
static const int RK_S[3] = {1, 3, 5};

/* explicit.c:96-140 */
int orc_step_lserkw2(int scheme, int iter, double t, double dt)
{
    (void)iter;
    if (scheme < 0 || scheme > 2)
    {
        snprintf(g_err, sizeof(g_err), "bad explicit scheme");
        return -1;
    }
    double *k = zalloc(sizeof(double) * NS * (size_t)G.nc);
    for (int s = 0; s < RK_S[scheme]; ++s)
    {
        time_derivative(t + dt * RK_B[scheme][s]);
        for (size_t i = 0; i < (size_t)G.nc * NS; ++i)
            k[i] = (s == 0) ? G.dphi[i] : G.dphi[i] + k[i] * RK_A[scheme][s];
        for (int i = 0; i < G.nc; ++i)
            for (int j = 0; j < NS; ++j)
                G.phi[(size_t)i * NV + j] += k[(size_t)i * NS + j] * dt * RK_G[scheme][s];
    }
    free(k);
    return 0;
}

/* NEW: SSP-RK3 (Shu & Osher 1988) in Shu-Osher form */
int orc_step_ssprk3(double t, double dt)
{
    double *u0 = zalloc(sizeof(double) * NS * (size_t)G.nc);
    for (int i = 0; i < G.nc; ++i)
        for (int j = 0; j < NS; ++j)
            u0[(size_t)i * NS + j] = G.phi[(size_t)i * NV + j];
    time_derivative(t);
    for (int i = 0; i < G.nc; ++i)
        for (int j = 0; j < NS; ++j)
            G.phi[(size_t)i * NV + j] = u0[(size_t)i * NS + j] + dt * G.dphi[(size_t)i * NS + j];
    time_derivative(t + dt);
    for (int i = 0; i < G.nc; ++i)
        for (int j = 0; j < NS; ++j)
        {
            double u1 = G.phi[(size_t)i * NV + j];
            G.phi[(size_t)i * NV + j] = 0.75 * u0[(size_t)i * NS + j] + 0.25 * (u1 + dt * G.dphi[(size_t)i * NS + j]);
        }
    time_derivative(t + 0.5 * dt);
    for (int i = 0; i < G.nc; ++i)
        for (int j = 0; j < NS; ++j)
        {
            double u2 = G.phi[(size_t)i * NV + j];
            G.phi[(size_t)i * NV + j] = (1.0 / 3.0) * u0[(size_t)i * NS + j] + (2.0 / 3.0) * (u2 + dt * G.dphi[(size_t)i * NS + j]);
        }
    free(u0);
    update();
    return 0;
}

/* analyze.c:37-61 */
int orc_global_residual(double dt, double *res)
{
    double tmp[NS] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = 0; i < G.nc; ++i)
        for (int j = 0; j < NS; ++j)
            tmp[j] += dabs(G.dphi[(size_t)i * NS + j]) * G.vol[i];
    for (int j = 0; j < NS; ++j)
        res[j] = tmp[j] * (dt / G.vol_total);
    return 0;
}

/* ---- implicit (implicit.c) ------------------------------------------------------------- */
/* implicit.c:61-119: lumped per-cell 5x5 blocks from central differences with
 * every cell perturbed at once; blocks column-major (jac[i*25 + col*5 + row]) */
static void jacobian(void)
{
    const size_t n = (size_t)G.nc;
    for (int v = 0; v < NS; ++v)
    {
        double eps = 0.0;
        for (size_t i = 0; i < n; ++i)
            eps += G.Y[i * NS + v] * G.Y[i * NS + v];
        eps = sqrt(eps) * 1e-4;
        for (size_t i = 0; i < n; ++i)
        {
            for (int j = 0; j < NS; ++j)
                G.phi[i * NV + j] = G.Y[i * NS + j];
            G.phi[i * NV + v] += 0.5 * eps;
        }
        time_derivative(G.tpdt_loc);
        for (size_t i = 0; i < n; ++i)
            for (int j = 0; j < NS; ++j)
                G.jac[i * 25 + v * 5 + j] = -G.dphi[i * NS + j];
        for (size_t i = 0; i < n; ++i)
        {
            for (int j = 0; j < NS; ++j)
                G.phi[i * NV + j] = G.Y[i * NS + j];
            G.phi[i * NV + v] -= 0.5 * eps;
        }
        time_derivative(G.tpdt_loc);
        for (size_t i = 0; i < n; ++i)
        {
            for (int j = 0; j < NS; ++j)
            {
                G.jac[i * 25 + v * 5 + j] += G.dphi[i * NS + j];
                G.jac[i * 25 + v * 5 + j] *= G.bdf_b_loc / (eps + 1e-16);
            }
            G.jac[i * 25 + v * 5 + v] += 1.0 / G.dt_loc;
        }
    }
}

/* implicit.c:362-384 */
static int block_matvec(double *x, double *b, size_t nv, size_t nc)
{
    for (size_t i = 0; i < nc; ++i)
    {
        const double *J = &G.jac[i * nv * nv];
        double *bi = &b[i * nv];
        const double *xi = &x[i * nv];
        for (size_t j = 0; j < nv; ++j)
            bi[j] = J[j] * xi[0];
        for (size_t c = 1; c < nv; ++c)
            for (size_t j = 0; j < nv; ++j)
                bi[j] += J[c * nv + j] * xi[c];
    }
    return 0;
}

static void newton_rhs(const double *bdf_a, int n_stages)
{
    const size_t n = (size_t)G.nc * NS;
    for (size_t i = 0; i < n; ++i)
        G.fY[i] = -(G.Y[i] - G.phi_old[0][i]) / G.dt_loc + G.bdf_b_loc * G.dYdt[i];
    for (int s = 0; s < n_stages; ++s)
        for (size_t i = 0; i < n; ++i)
            G.fY[i] -= bdf_a[s] / G.dt_loc * G.phi_old[s][i];
}

/* implicit.c:224-351 */
int orc_step_newton(int scheme, int solver, int max_iter_inner, double tolerance_lsoe,
                    int max_iter_lsoe, int krylov_dims, int krylov_restarts,
                    int is_transient, int iter, double t, double dt, int *n_inner,
                    int *n_lsoe)
{
    static const double a_euler[1] = {0.0};
    static const double a_bdf2[2] = {-1. / 3., 1 / 3.};
    const size_t n = (size_t)G.nc * NS;
    if (!G.imp_ready || iter == 0)
    {
        free(G.phi_old[0]); free(G.phi_old[1]); free(G.Y); free(G.fY); free(G.dY);
        free(G.dYdt); free(G.jac); free(G.work);
        G.n_bdf = (scheme == 0) ? 1 : 2;
        G.phi_old[0] = zalloc(sizeof(double) * n);
        G.phi_old[1] = zalloc(sizeof(double) * n);
        G.Y = zalloc(sizeof(double) * n);
        G.fY = zalloc(sizeof(double) * n);
        G.dY = zalloc(sizeof(double) * n);
        G.dYdt = zalloc(sizeof(double) * n);
        G.jac = zalloc(sizeof(double) * 25 * (size_t)G.nc);
        int ws = (solver == 0) ? get_bicgstab_n_m_work_size(NS, G.nc)
                               : get_gmres_n_m_work_size(NS, G.nc, krylov_dims);
        G.work = zalloc(sizeof(double) * (size_t)ws);
        G.imp_ready = 1;
        if (iter == 0)
            time_derivative(t); /* timedisc.c:537-538 */
    }
    int stages = (iter < G.n_bdf) ? 1 : G.n_bdf;
    const double *bdf_a = (iter < G.n_bdf) ? a_euler : (scheme == 0 ? a_euler : a_bdf2);
    G.bdf_b_loc = (iter < G.n_bdf) ? 1.0 : (scheme == 0 ? 1.0 : 2. / 3.);
    G.dt_loc = dt;
    G.tpdt_loc = t + dt;
    if (stages > 1)
        memcpy(G.phi_old[1], G.phi_old[0], sizeof(double) * n);
    for (int i = 0; i < G.nc; ++i)
        for (int j = 0; j < NS; ++j)
            G.phi_old[0][(size_t)i * NS + j] = G.phi[(size_t)i * NV + j];
    memcpy(G.Y, G.phi_old[0], sizeof(double) * n);
    memcpy(G.dYdt, G.dphi, sizeof(double) * n);
    newton_rhs(bdf_a, stages);
    const double err0 = len_n(G.fY, n);
    double err = err0;
    int it;
    for (it = 1; it <= max_iter_inner; ++it)
    {
        jacobian();
        if (err >= err0)
        {
            int nl = max_iter_lsoe;
            double res = tolerance_lsoe * err;
            if (solver == 0)
                solve_bicgstab_n_m(NS, G.nc, G.fY, G.dY, G.work, block_matvec, &nl, &res);
            else
                solve_gmres_n_m(NS, G.nc, G.fY, G.dY, G.work, block_matvec, &nl, &res,
                                krylov_dims, krylov_restarts);
            G.n_lsoe = nl;
            for (int i = 0; i < G.nc; ++i)
                for (int j = 0; j < NS; ++j)
                {
                    size_t idx = (size_t)i * NS + j;
                    G.Y[idx] += G.dY[idx];
                    G.phi[(size_t)i * NV + j] = G.Y[idx];
                }
            time_derivative(G.tpdt_loc);
            memcpy(G.dYdt, G.dphi, sizeof(double) * n);
            newton_rhs(bdf_a, stages);
            err = len_n(G.fY, n);
        }
        else
            time_derivative(G.tpdt_loc);
        if (err < err0)
            break;
        if (!is_transient)
            break;
    }
    G.n_inner = it;
    *n_inner = it;
    *n_lsoe = G.n_lsoe;
    if (it >= max_iter_inner)
    {
        snprintf(g_err, sizeof(g_err), "newton: no convergence in %d iterations", max_iter_inner);
        return -1;
    }
    return 0;
}

int orc_get_jacobian(double *out)
{
    if (G.jac == NULL)
        return -1;
    memcpy(out, G.jac, sizeof(double) * 25 * (size_t)G.nc);
    return 0;
}
