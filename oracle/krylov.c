/*
 * Krylov solvers shared by both CPU oracles (test infrastructure only).
 * This repository's own restatement of textbook restarted GMRES (Saad &
 * Schultz 1986; modified Gram-Schmidt + Givens rotations) and BiCGStab (van
 * der Vorst 1992), with the call signature of basec's solve_gmres_n_m /
 * solve_bicgstab_n_m as used at implicit.c:289,295 of the reference.  basec's
 * own versions are not available, so this arithmetic is NOT pinned to the
 * reference; the reference applies them to a block-diagonal system
 * (implicit.c:362-384) whose converged answer is unique.
 * Included (not linked) by basec_shim.c and fv3d_oracle.c; expects
 * dot_n/len_n and the shim_matvec_ft type to be declared before inclusion.
 */
int get_gmres_n_m_work_size(int n_var, int n_cells, int max_krylov_dims)
{
    int n = n_var * n_cells;
    int m = max_krylov_dims;
    return n * (m + 3) + (m + 1) * (m + 1) + 4 * (m + 1);
}

int get_bicgstab_n_m_work_size(int n_var, int n_cells)
{
    return 8 * n_var * n_cells;
}

/* Restarted GMRES(m), right-unpreconditioned, absolute stopping tolerance
 * *residual on ||b - A x||_2.  On return *n_iter holds the number of inner
 * iterations taken and *residual the last residual estimate. */
void solve_gmres_n_m(int n_var, int n_cells, double *rhs, double *x, double *work,
                     shim_matvec_ft matvec, int *n_iter, double *residual,
                     int max_krylov_dims, int max_krylov_restarts)
{
    const size_t n = (size_t)n_var * (size_t)n_cells;
    const int m = max_krylov_dims;
    const double tol = *residual;
    const int max_iter = *n_iter;
    double *V = work;                     /* (m+1) basis vectors */
    double *w = V + n * (size_t)(m + 1);  /* scratch vector */
    double *H = w + n;                    /* (m+1) x m Hessenberg, column-major */
    double *cs = H + (size_t)(m + 1) * (m + 1);
    double *sn = cs + (m + 1);
    double *g = sn + (m + 1);
    double *y = g + (m + 1);
    int iters = 0;
    double beta = 0.0;

    for (int restart = 0; restart <= max_krylov_restarts; ++restart)
    {
        matvec(x, w, (size_t)n_var, (size_t)n_cells);
        for (size_t i = 0; i < n; ++i)
            V[i] = rhs[i] - w[i];
        beta = len_n(V, n);
        if (beta <= tol || iters >= max_iter)
            break;
        for (size_t i = 0; i < n; ++i)
            V[i] /= beta;
        for (int i = 0; i <= m; ++i)
            g[i] = 0.0;
        g[0] = beta;

        int k = 0;
        for (; k < m && iters < max_iter; ++k)
        {
            double *vk = V + n * (size_t)k;
            double *vk1 = V + n * (size_t)(k + 1);
            matvec(vk, vk1, (size_t)n_var, (size_t)n_cells);
            for (int j = 0; j <= k; ++j)
            {
                double *vj = V + n * (size_t)j;
                double h = dot_n(vk1, vj, n);
                H[(size_t)k * (m + 1) + j] = h;
                for (size_t i = 0; i < n; ++i)
                    vk1[i] -= h * vj[i];
            }
            double hk1 = len_n(vk1, n);
            H[(size_t)k * (m + 1) + k + 1] = hk1;
            if (hk1 > 0.0)
                for (size_t i = 0; i < n; ++i)
                    vk1[i] /= hk1;
            for (int j = 0; j < k; ++j)
            {
                double a = H[(size_t)k * (m + 1) + j];
                double b = H[(size_t)k * (m + 1) + j + 1];
                H[(size_t)k * (m + 1) + j] = cs[j] * a + sn[j] * b;
                H[(size_t)k * (m + 1) + j + 1] = -sn[j] * a + cs[j] * b;
            }
            double a = H[(size_t)k * (m + 1) + k];
            double b = H[(size_t)k * (m + 1) + k + 1];
            double r = sqrt(a * a + b * b);
            cs[k] = (r > 0.0) ? a / r : 1.0;
            sn[k] = (r > 0.0) ? b / r : 0.0;
            H[(size_t)k * (m + 1) + k] = r;
            H[(size_t)k * (m + 1) + k + 1] = 0.0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = cs[k] * g[k];
            iters += 1;
            beta = fabs(g[k + 1]);
            if (beta <= tol)
            {
                k += 1;
                break;
            }
        }
        for (int i = k - 1; i >= 0; --i)
        {
            double s = g[i];
            for (int j = i + 1; j < k; ++j)
                s -= H[(size_t)j * (m + 1) + i] * y[j];
            y[i] = s / H[(size_t)i * (m + 1) + i];
        }
        for (int j = 0; j < k; ++j)
            for (size_t i = 0; i < n; ++i)
                x[i] += y[j] * V[n * (size_t)j + i];
        if (beta <= tol || iters >= max_iter)
            break;
    }
    *n_iter = iters;
    *residual = beta;
}

void solve_bicgstab_n_m(int n_var, int n_cells, double *rhs, double *x, double *work,
                        shim_matvec_ft matvec, int *n_iter, double *residual)
{
    const size_t n = (size_t)n_var * (size_t)n_cells;
    const double tol = *residual;
    const int max_iter = *n_iter;
    double *r = work, *r0 = r + n, *p = r0 + n, *v = p + n, *s = v + n, *t = s + n;
    matvec(x, v, (size_t)n_var, (size_t)n_cells);
    for (size_t i = 0; i < n; ++i)
    {
        r[i] = rhs[i] - v[i];
        r0[i] = r[i];
        p[i] = 0.0;
        v[i] = 0.0;
    }
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    double res = len_n(r, n);
    int it = 0;
    while (res > tol && it < max_iter)
    {
        double rho_new = dot_n(r0, r, n);
        double beta = (rho_new / rho) * (alpha / omega);
        rho = rho_new;
        for (size_t i = 0; i < n; ++i)
            p[i] = r[i] + beta * (p[i] - omega * v[i]);
        matvec(p, v, (size_t)n_var, (size_t)n_cells);
        alpha = rho / dot_n(r0, v, n);
        for (size_t i = 0; i < n; ++i)
            s[i] = r[i] - alpha * v[i];
        matvec(s, t, (size_t)n_var, (size_t)n_cells);
        double tt = dot_n(t, t, n);
        omega = (tt > 0.0) ? dot_n(t, s, n) / tt : 0.0;
        for (size_t i = 0; i < n; ++i)
        {
            x[i] += alpha * p[i] + omega * s[i];
            r[i] = s[i] - omega * t[i];
        }
        res = len_n(r, n);
        it += 1;
        if (omega == 0.0)
            break;
    }
    *n_iter = it;
    *residual = res;
}
