/*
 * kron.c -- oracle restatement of the Kronecker operator, the Kronecker
 * preconditioner and the restarted GMRES of src/kronecker.f90, plus the
 * SPARSKIT CSR product and triangular solves they call (src/ilut.f).
 *
 * TEST INFRASTRUCTURE ONLY (the checker); see xt_oracle.h.
 */
#include "xt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Host threads for the Kronecker apply, the preconditioner and the Krylov
 * vector operations.  1 (the default) runs the reference's serial code
 * order; above 1 the same arithmetic per entry runs under OpenMP (rows of
 * each amux pass, the q independent lusol calls, rows of the block mixing
 * and of every vector update), and only the dot products and norms change
 * their summation order (per-thread partial sums).  This is the threaded
 * CPU baseline; the reference itself has no threading on this path. */
static int g_threads = 1;

void orc_set_threads(int n) { g_threads = n > 1 ? n : 1; }

int orc_get_threads(void) { return g_threads; }

/* src/ilut.f:3-44.  Row-by-row CSR product, 1-based ia/ja. */
void orc_amux(int n, const double *x, double *y, const double *a,
              const int *ja, const int *ia)
{
    const int nt = g_threads;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int r = 0; r < n; ++r) {
        double acc = 0.0;
        for (int k = ia[r] - 1; k < ia[r + 1] - 1; ++k)
            acc = acc + a[k] * x[ja[k] - 1];
        y[r] = acc;
    }
}

/* y_blk(i) += sum_j c(i,j) * u_blk(j), the vector additions of
 * src/kronecker.f90:67-72 and :78-82 (c column-major q x q). */
static void block_mix_add(const double *c, int q, int p, const double *u,
                          double *y)
{
    const int nt = g_threads;
    if (nt > 1) {
        /* the same q*q updates of each entry, in the same order */
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int r = 0; r < p; ++r)
            for (int i = 0; i < q; ++i)
                for (int j = 0; j < q; ++j)
                    y[(size_t)i * p + r] = y[(size_t)i * p + r] +
                                           c[j * q + i] * u[(size_t)j * p + r];
        return;
    }
    for (int i = 0; i < q; ++i)
        for (int j = 0; j < q; ++j) {
            const double cij = c[j * q + i];
            double *yi = y + (size_t)i * p;
            const double *uj = u + (size_t)j * p;
            for (int r = 0; r < p; ++r)
                yi[r] = yi[r] + cij * uj[r];
        }
}

/* src/kronecker.f90:19-85.  q SpMVs with K, mixing with A, then q SpMVs
 * with M, mixing with B, accumulated into y in that order. */
void orc_kronspmv(const double *a, const double *b, int q,
                  const int *ki, const int *kj, const double *kv,
                  const int *mi, const int *mj, const double *mv,
                  int p, const double *x, double *y)
{
    const size_t n = (size_t)p * q;
    double *u = (double *)calloc(n, sizeof(double));
    memset(y, 0, n * sizeof(double));
    for (int i = 0; i < q; ++i)
        orc_amux(p, x + (size_t)i * p, u + (size_t)i * p, kv, kj, ki);
    block_mix_add(a, q, p, u, y);
    for (int i = 0; i < q; ++i)
        orc_amux(p, x + (size_t)i * p, u + (size_t)i * p, mv, mj, mi);
    block_mix_add(b, q, p, u, y);
    free(u);
}

/* src/kronecker.f90:88-127. */
void orc_kronspgemv(const double *a, const double *b, double alpha,
                    double beta, int q, const int *ki, const int *kj,
                    const double *kv, const int *mi, const int *mj,
                    const double *mv, int p, const double *x, double *y)
{
    const size_t n = (size_t)p * q;
    double *z = (double *)malloc(n * sizeof(double));
    orc_kronspmv(a, b, q, ki, kj, kv, mi, mj, mv, p, x, z);
    const int nt = g_threads;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (long long r = 0; r < (long long)n; ++r)
        y[r] = alpha * z[r] + beta * y[r];
    free(z);
}

/* src/kronecker.f90:368-395 (LAPACK dgetrf + dgetri).  Restated as an LU
 * factorisation with partial pivoting followed by n forward/back solves
 * against the unit vectors; the same mathematical inverse, not LAPACK's
 * operation order. */
int orc_inverse(int n, const double *A, double *Ainv)
{
    double *lu = (double *)malloc((size_t)n * n * sizeof(double));
    int *piv = (int *)malloc((size_t)n * sizeof(int));
    memcpy(lu, A, (size_t)n * n * sizeof(double));
#define LU(i, j) lu[(size_t)(j) * n + (i)]
    for (int c = 0; c < n; ++c) {
        int pr = c;
        double best = fabs(LU(c, c));
        for (int r = c + 1; r < n; ++r)
            if (fabs(LU(r, c)) > best) { best = fabs(LU(r, c)); pr = r; }
        piv[c] = pr;
        if (best == 0.0) { free(lu); free(piv); return 1; }
        if (pr != c)
            for (int j = 0; j < n; ++j) {
                double t = LU(c, j); LU(c, j) = LU(pr, j); LU(pr, j) = t;
            }
        for (int r = c + 1; r < n; ++r) {
            LU(r, c) /= LU(c, c);
            for (int j = c + 1; j < n; ++j)
                LU(r, j) -= LU(r, c) * LU(c, j);
        }
    }
    for (int col = 0; col < n; ++col) {
        double *e = Ainv + (size_t)col * n;
        for (int r = 0; r < n; ++r) e[r] = (r == col) ? 1.0 : 0.0;
        for (int c = 0; c < n; ++c)
            if (piv[c] != c) { double t = e[c]; e[c] = e[piv[c]]; e[piv[c]] = t; }
        for (int r = 1; r < n; ++r)
            for (int c = 0; c < r; ++c) e[r] -= LU(r, c) * e[c];
        for (int r = n - 1; r >= 0; --r) {
            for (int c = r + 1; c < n; ++c) e[r] -= LU(r, c) * e[c];
            e[r] /= LU(r, r);
        }
    }
#undef LU
    free(lu);
    free(piv);
    return 0;
}

/* src/ilut.f:2383-2432.  Forward sweep with the unit-lower L part of each
 * MSR row (jlu(i) .. ju(i)-1), then backward sweep with the U part
 * (ju(i) .. jlu(i+1)-1) and the inverted diagonal alu(i).  1-based MSR. */
void orc_lusol(int n, const double *y, double *x, const double *alu,
               const int *jlu, const int *ju)
{
    for (int i = 1; i <= n; ++i) {
        double xi = y[i - 1];
        for (int k = jlu[i - 1]; k <= ju[i - 1] - 1; ++k)
            xi = xi - alu[k - 1] * x[jlu[k - 1] - 1];
        x[i - 1] = xi;
    }
    for (int i = n; i >= 1; --i) {
        double xi = x[i - 1];
        for (int k = ju[i - 1]; k <= jlu[i] - 1; ++k)
            xi = xi - alu[k - 1] * x[jlu[k - 1] - 1];
        x[i - 1] = alu[i - 1] * xi;
    }
}

/* src/kronecker.f90:130-178.  x and y may alias (the reference calls it in
 * place at :335). */
int orc_kronlusol(const double *a, int q, const double *alu, const int *jlu,
                  const int *ju, int p, const double *x, double *y)
{
    const size_t n = (size_t)p * q;
    double inva[64 * 64];
    if (q > 64 || orc_inverse(q, a, inva) != 0) return 1;
    double *w = (double *)calloc(n, sizeof(double));
    const int nt = g_threads < q ? g_threads : q;
#pragma omp parallel for schedule(static, 1) num_threads(nt) if (nt > 1)
    for (int i = 0; i < q; ++i)
        orc_lusol(p, x + (size_t)i * p, w + (size_t)i * p, alu, jlu, ju);
    memset(y, 0, n * sizeof(double));
    block_mix_add(inva, q, p, w, y);
    free(w);
    return 0;
}

static double ddot(size_t n, const double *x, const double *y)
{
    const int nt = g_threads < 64 ? g_threads : 64;
    double s = 0.0;
    if (nt > 1) {
        /* each thread sums its contiguous share; the shares are added in
         * thread order, so a given thread count repeats bit for bit (an
         * OpenMP reduction may combine them in any order) */
        double part[64];
        int used = 1;
#pragma omp parallel num_threads(nt)
        {
#ifdef _OPENMP
            const int t = omp_get_thread_num(), T = omp_get_num_threads();
#else
            const int t = 0, T = 1;
#endif
            const size_t b = n * (size_t)t / (size_t)T, e = n * (size_t)(t + 1) / (size_t)T;
            double acc = 0.0;
            for (size_t i = b; i < e; ++i) acc += x[i] * y[i];
            part[t] = acc;
            if (t == 0) used = T;
        }
        for (int t = 0; t < used; ++t) s += part[t];
        return s;
    }
    for (size_t i = 0; i < n; ++i) s += x[i] * y[i];
    return s;
}

static double dnrm2(size_t n, const double *x)
{
    /* Plain two-norm; BLAS dnrm2 scales to avoid overflow, which changes
     * nothing at the magnitudes of this path. */
    return sqrt(ddot(n, x, x));
}

/* The vector updates of kronpgmres, one expression per entry as in the
 * reference; rows in parallel when threaded. */
static void vscal(size_t n, double *y, double t)          /* y = y*t */
{
    const int nt = g_threads;
    const long long nn = (long long)n;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (long long i = 0; i < nn; ++i) y[i] *= t;
}

static void vaxpy(size_t n, double *y, double t, const double *x)  /* y += t*x */
{
    const int nt = g_threads;
    const long long nn = (long long)n;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (long long i = 0; i < nn; ++i) y[i] += t * x[i];
}

static void vcopy_scaled(size_t n, double *y, const double *x, double t)  /* y = x*t */
{
    const int nt = g_threads;
    const long long nn = (long long)n;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (long long i = 0; i < nn; ++i) y[i] = x[i] * t;
}

/* src/kronecker.f90:181-365.  The control flow (labels 20, 4, 58, 121,
 * 990/991/999 of the reference) is kept: the correction of a cycle is
 * applied before a restart, the residual of the restart is rebuilt from the
 * Givens data, and maxits is only tested at the end of a cycle. */
int orc_kronpgmres(const double *a, const double *b, int q,
                   const int *ki, const int *kj, const double *kv,
                   const int *mi, const int *mj, const double *mv, int p,
                   const double *alu, const int *jlu, const int *ju,
                   double *rhs, double *sol, int im, double eps, int maxits,
                   int *its_out, double *hist, int hist_len)
{
    const size_t n = (size_t)p * q;
    const double epsmac = 1.0e-16;
    double *vv = (double *)calloc(n * (size_t)(im + 1), sizeof(double));
    double *hh = (double *)calloc((size_t)(im + 1) * im, sizeof(double));
    double *c = (double *)calloc(im, sizeof(double));
    double *s = (double *)calloc(im, sizeof(double));
    double *rs = (double *)calloc(im + 1, sizeof(double));
#define V(j) (vv + (size_t)(j) * n)           /* 0-based column j */
#define HH(r, col) hh[(size_t)(col) * (im + 1) + (r)]  /* 0-based */
    int ierr = 0, its = 0, i = 0;
    double ro, eps1 = 0.0, t;
    const double ro0 = dnrm2(n, rhs);

    orc_kronspmv(a, b, q, ki, kj, kv, mi, mj, mv, p, sol, V(0));
    {
        const int nt = g_threads;
        const long long nn = (long long)n;
        double *v0 = V(0);
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
        for (long long r = 0; r < nn; ++r) v0[r] = rhs[r] - v0[r];
    }

    for (;;) {                                   /* label 20 */
        ro = dnrm2(n, V(0));
        if (ro == 0.0) { ierr = -1; break; }
        t = 1.0 / ro;
        vscal(n, V(0), t);
        if (its == 0) eps1 = eps * ro;
        rs[0] = ro;
        i = 0;
        for (;;) {                               /* label 4 */
            i = i + 1;
            its = its + 1;
            const int i1 = i + 1;
            if (orc_kronlusol(a, q, alu, jlu, ju, p, V(i - 1), rhs)) {
                ierr = 2; goto done;
            }
            orc_kronspmv(a, b, q, ki, kj, kv, mi, mj, mv, p, rhs, V(i1 - 1));
            for (int j = 1; j <= i; ++j) {       /* modified Gram-Schmidt */
                t = ddot(n, V(j - 1), V(i1 - 1));
                HH(j - 1, i - 1) = t;
                vaxpy(n, V(i1 - 1), -t, V(j - 1));
            }
            t = dnrm2(n, V(i1 - 1));
            HH(i1 - 1, i - 1) = t;
            if (t != 0.0) {
                t = 1.0 / t;
                vscal(n, V(i1 - 1), t);
            }
            for (int k = 2; k <= i; ++k) {       /* label 58 */
                const int k1 = k - 1;
                t = HH(k1 - 1, i - 1);
                HH(k1 - 1, i - 1) = c[k1 - 1] * t + s[k1 - 1] * HH(k - 1, i - 1);
                HH(k - 1, i - 1) = -s[k1 - 1] * t + c[k1 - 1] * HH(k - 1, i - 1);
            }
            /* label 121 */
            double gam = sqrt(HH(i - 1, i - 1) * HH(i - 1, i - 1) +
                              HH(i1 - 1, i - 1) * HH(i1 - 1, i - 1));
            if (gam == 0.0) gam = epsmac;
            c[i - 1] = HH(i - 1, i - 1) / gam;
            s[i - 1] = HH(i1 - 1, i - 1) / gam;
            rs[i1 - 1] = -s[i - 1] * rs[i - 1];
            rs[i - 1] = c[i - 1] * rs[i - 1];
            HH(i - 1, i - 1) = c[i - 1] * HH(i - 1, i - 1) + s[i - 1] * HH(i1 - 1, i - 1);
            ro = fabs(rs[i1 - 1]);
            if (hist && its - 1 < hist_len) hist[its - 1] = ro / ro0;
            if (i < im && ro > eps1) continue;
            break;
        }
        /* solve the upper triangular system */
        rs[i - 1] = rs[i - 1] / HH(i - 1, i - 1);
        for (int ii = 2; ii <= i; ++ii) {
            const int k = i - ii + 1, k1 = k + 1;
            t = rs[k - 1];
            for (int j = k1; j <= i; ++j) t = t - HH(k - 1, j - 1) * rs[j - 1];
            rs[k - 1] = t / HH(k - 1, k - 1);
        }
        /* linear combination of the basis, preconditioner, update */
        t = rs[0];
        vcopy_scaled(n, rhs, V(0), t);
        for (int j = 2; j <= i; ++j) {
            t = rs[j - 1];
            vaxpy(n, rhs, t, V(j - 1));
        }
        if (orc_kronlusol(a, q, alu, jlu, ju, p, rhs, rhs)) { ierr = 2; break; }
        vaxpy(n, sol, 1.0, rhs);
        if (ro <= eps1) { ierr = 0; break; }
        if (its >= maxits) { ierr = 1; break; }
        /* residual of the restart from the Givens data */
        {
            const int i1 = i + 1;
            for (int j = 1; j <= i; ++j) {
                const int jj = i1 - j + 1;
                rs[jj - 2] = -s[jj - 2] * rs[jj - 1];
                rs[jj - 1] = c[jj - 2] * rs[jj - 1];
            }
            for (int j = 1; j <= i1; ++j) {
                t = rs[j - 1];
                if (j == 1) t = t - 1.0;
                vaxpy(n, V(0), t, V(j - 1));
            }
        }
    }
done:
#undef V
#undef HH
    if (its_out) *its_out = its;
    free(vv); free(hh); free(c); free(s); free(rs);
    return ierr;
}
