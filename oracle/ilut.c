/*
 * ilut.c -- oracle restatement of SPARSKIT ILUT (src/ilut.f:152-495) and its
 * quick-split partial sort qsplit (src/ilut.f:2487-2545).
 *
 * TEST INFRASTRUCTURE ONLY (the checker); see xt_oracle.h.
 *
 * Arrays are addressed 1-based through the macros below so that every index
 * expression can be compared with the Fortran line by line.
 */
#include "xt_oracle.h"

#include <math.h>
#include <stdlib.h>

/* src/ilut.f:2487-2545.  Partial quick-sort so that |a(k)| >= |a(ncut)| for
 * k < ncut and <= for k > ncut; ind is permuted alongside.  0-based
 * pointers, 1-based logic. */
void orc_qsplit(double *a0, int *ind0, int n, int ncut)
{
    double *a = a0 - 1;
    int *ind = ind0 - 1;
    int first = 1, last = n;
    if (ncut < first || ncut > last) return;
    for (;;) {
        int mid = first;
        const double abskey = fabs(a[mid]);
        for (int j = first + 1; j <= last; ++j) {
            if (fabs(a[j]) > abskey) {
                mid = mid + 1;
                double tmp = a[mid]; a[mid] = a[j]; a[j] = tmp;
                int itmp = ind[mid]; ind[mid] = ind[j]; ind[j] = itmp;
            }
        }
        double tmp = a[mid]; a[mid] = a[first]; a[first] = tmp;
        int itmp = ind[mid]; ind[mid] = ind[first]; ind[first] = itmp;
        if (mid == ncut) return;
        if (mid > ncut) last = mid - 1;
        else first = mid + 1;
    }
}

/* src/ilut.f:152-495.  Dual-threshold ILU: the multiplier test is the
 * absolute |fact| <= droptol (:292), the U test the row-relative
 * droptol*tnorm (:431); L keeps lfil entries, U keeps lfil-1 off-diagonal
 * entries (:436-448).  A zero pivot becomes (0.0001 + droptol)*tnorm where
 * 0.0001 is a single-precision literal in the reference (:455). */
int orc_ilut(int n, const double *a0, const int *ja0, const int *ia0,
             int lfil, double droptol, double *alu0, int *jlu0, int *ju0_,
             int iwk)
{
    const double *a = a0 - 1;
    const int *ja = ja0 - 1, *ia = ia0 - 1;
    double *alu = alu0 - 1;
    int *jlu = jlu0 - 1, *ju = ju0_ - 1;
    double *w = (double *)malloc((size_t)(n + 2) * sizeof(double)) ;
    int *jw = (int *)malloc((size_t)(2 * n + 2) * sizeof(int));
    int ierr = 0;
    if (lfil < 0) { ierr = -4; goto out; }

    int ju0 = n + 2;
    jlu[1] = ju0;
    for (int j = 1; j <= n; ++j) jw[n + j] = 0;

    for (int ii = 1; ii <= n; ++ii) {
        const int j1 = ia[ii], j2 = ia[ii + 1] - 1;
        double tnorm = 0.0;
        for (int k = j1; k <= j2; ++k) tnorm = tnorm + fabs(a[k]);
        if (tnorm == 0.0) { ierr = -5; goto out; }
        tnorm = tnorm / (double)(float)(j2 - j1 + 1);

        int lenu = 1, lenl = 0;
        jw[ii] = ii;
        w[ii] = 0.0;
        jw[n + ii] = ii;
        for (int j = j1; j <= j2; ++j) {
            const int k = ja[j];
            const double t = a[j];
            if (k < ii) {
                lenl = lenl + 1;
                jw[lenl] = k;
                w[lenl] = t;
                jw[n + k] = lenl;
            } else if (k == ii) {
                w[ii] = t;
            } else {
                lenu = lenu + 1;
                const int jpos = ii + lenu - 1;
                jw[jpos] = k;
                w[jpos] = t;
                jw[n + k] = jpos;
            }
        }
        int jj = 0, len = 0;
        for (;;) {                                  /* label 150 */
            jj = jj + 1;
            if (jj > lenl) break;
            int jrow = jw[jj], k = jj;
            for (int j = jj + 1; j <= lenl; ++j)
                if (jw[j] < jrow) { jrow = jw[j]; k = j; }
            if (k != jj) {
                int j = jw[jj];
                jw[jj] = jw[k];
                jw[k] = j;
                jw[n + jrow] = jj;
                jw[n + j] = k;
                double s = w[jj];
                w[jj] = w[k];
                w[k] = s;
            }
            jw[n + jrow] = 0;
            const double fact = w[jj] * alu[jrow];
            if (fabs(fact) <= droptol) continue;
            for (int kk = ju[jrow]; kk <= jlu[jrow + 1] - 1; ++kk) {
                const double s = fact * alu[kk];
                const int j = jlu[kk];
                const int jpos = jw[n + j];
                if (j >= ii) {
                    if (jpos == 0) {
                        lenu = lenu + 1;
                        if (lenu > n) { ierr = -1; goto out; }
                        const int i = ii + lenu - 1;
                        jw[i] = j;
                        jw[n + j] = i;
                        w[i] = -s;
                    } else {
                        w[jpos] = w[jpos] - s;
                    }
                } else {
                    if (jpos == 0) {
                        lenl = lenl + 1;
                        if (lenl > n) { ierr = -1; goto out; }
                        jw[lenl] = j;
                        jw[n + j] = lenl;
                        w[lenl] = -s;
                    } else {
                        w[jpos] = w[jpos] - s;
                    }
                }
            }
            len = len + 1;
            w[len] = fact;
            jw[len] = jrow;
        }
        /* label 160 */
        for (int k = 1; k <= lenu; ++k) jw[n + jw[ii + k - 1]] = 0;
        lenl = len;
        len = lenl < lfil ? lenl : lfil;
        orc_qsplit(&w[1], &jw[1], lenl, len);
        for (int k = 1; k <= len; ++k) {
            if (ju0 > iwk) { ierr = -2; goto out; }
            alu[ju0] = w[k];
            jlu[ju0] = jw[k];
            ju0 = ju0 + 1;
        }
        ju[ii] = ju0;
        len = 0;
        for (int k = 1; k <= lenu - 1; ++k) {
            if (fabs(w[ii + k]) > droptol * tnorm) {
                len = len + 1;
                w[ii + len] = w[ii + k];
                jw[ii + len] = jw[ii + k];
            }
        }
        lenu = len + 1;
        len = lenu < lfil ? lenu : lfil;
        orc_qsplit(&w[ii + 1], &jw[ii + 1], lenu - 1, len);
        if (len + ju0 > iwk) { ierr = -3; goto out; }
        for (int k = ii + 1; k <= ii + len - 1; ++k) {
            jlu[ju0] = jw[k];
            alu[ju0] = w[k];
            ju0 = ju0 + 1;
        }
        if (w[ii] == 0.0) w[ii] = ((double)0.0001f + droptol) * tnorm;
        alu[ii] = 1.0 / w[ii];
        jlu[ii + 1] = ju0;
    }
    ierr = 0;
out:
    free(w);
    free(jw);
    return ierr;
}
