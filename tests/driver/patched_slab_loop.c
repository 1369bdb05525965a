/*
 * patched_slab_loop.c -- the call sequence of the reference driver's
 * mechanical slab loop (src/main3d.f90:579-937) after the GMRES-route patch
 * of INTEGRATION.md, written in C against the library's C ABI.
 *
 * TEST PROGRAM (tests/test_driver_patch.py).  The patched Fortran driver
 * makes these calls; here the set-up the Fortran code keeps doing itself
 * (mesh, assembly, boundary conditions, SPARSKIT ilut, the deletion
 * surgery) is taken from the library's host entry points, which restate
 * the same routines:
 *
 *   set-up      xth_problem_rod, xth_problem_apply_bc          (:212-530)
 *   patch 1     ilut after the boundary conditions, in place of
 *               mumps_solver(..., 0)                           (:549-550)
 *   per slab    the deletion check: chkelesta_, the surgery,
 *               patch 2 a new ilut in place of mumps_solver(..., 1),
 *               xt_invalidate_ for the cached device copies    (:625-691)
 *               load blocks; patch 3 kronspgemv_ in place of
 *               mpikronspgemv for the jump term                (:804-818)
 *               patch 4 kronpgmres_ (with its log) in place of
 *               mpipgmres(..., mumps_par_m, ...)                (:831-832)
 *               kokkos_host_ through kokkos_damage's arguments  (:880)
 * Every solver call passes its scalars by reference, as the iso_c_binding
 * shim does.
 *
 * Usage: patched_slab_loop nx ny nz amplitude Dc ws0 nipc n1 n2 im eps nslab out.bin
 * Writes, per slab: deleted count, then after the last slab the
 * displacement (6p), D (8 ne) and elesta (ne).  Exit codes: 0 done, 2 bad
 * arguments or host set-up failure, 3 a library call reported an error
 * (the message is printed; on a machine without a GPU the first device
 * call ends the run here).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "xtfem_gb300.h"
#include "xtfem_gb300_host.h"

static int fail(const char* what)
{
    fprintf(stderr, "%s: %s\n", what, xt_last_error());
    return 3;
}

static int check_device(const char* what)
{
    const char* e = xt_last_error();
    if (e && e[0]) {
        fprintf(stderr, "%s: %s\n", what, e);
        return 3;
    }
    return 0;
}

typedef struct {
    int n, nnz;
    int *ia, *ja;
    double* a;
} csr;

static void csr_get(xth_problem pr, int which, csr* m)
{
    int nn, ne, nk, nm;
    xth_problem_sizes(pr, &nn, &ne, &nk, &nm);
    m->n = 3 * nn;
    m->nnz = which ? nm : nk;
    m->ia = realloc(m->ia, sizeof(int) * (m->n + 1));
    m->ja = realloc(m->ja, sizeof(int) * m->nnz);
    m->a = realloc(m->a, sizeof(double) * m->nnz);
    if (which) xth_problem_m(pr, m->ia, m->ja, m->a);
    else xth_problem_k(pr, m->ia, m->ja, m->a);
}

int main(int argc, char** argv)
{
    if (argc != 14) {
        fprintf(stderr, "usage: %s nx ny nz amplitude Dc ws0 nipc n1 n2 im eps nslab out\n", argv[0]);
        return 2;
    }
    const int nx = atoi(argv[1]), ny = atoi(argv[2]), nz = atoi(argv[3]);
    const double amp = atof(argv[4]), Dc = atof(argv[5]), ws0 = atof(argv[6]);
    const int nipc = atoi(argv[7]), n1 = atoi(argv[8]), n2 = atoi(argv[9]);
    int im = atoi(argv[10]);
    double eps = atof(argv[11]);
    const int nslab = atoi(argv[12]);
    FILE* out = fopen(argv[13], "wb");
    if (!out) return 2;
    const double lx = 3.0, E = 2.0e5, nu0 = 0.3, rho = 7.8e-9, freq = 20.0, dt0 = 0.005;
    const int lfil = 20, q = 6, ngpe = 8, nnse = 8, nnte = 3, ndofn = 3, ncmp = 6;
    const double droptol = 1e-4;

    xth_problem pr;
    if (xth_problem_rod(nx, ny, nz, lx, 1.0, 1.0, E, nu0, rho, &pr)) return 2;
    int nn, ne, nk, nm;
    xth_problem_sizes(pr, &nn, &ne, &nk, &nm);
    int p = 3 * nn;
    const int ngp = ngpe * ne;
    double* xyz = malloc(sizeof(double) * 3 * nn);
    int* conn = malloc(sizeof(int) * 8 * ne);
    xth_problem_mesh(pr, xyz, conn);
    /* clamped face x = 0, traction on x = lx shared per element-node incidence */
    int* bc = calloc(p, sizeof(int));
    for (int i = 0; i < nn; ++i)
        if (xyz[3 * i] == 0.0) bc[3 * i] = bc[3 * i + 1] = bc[3 * i + 2] = 1;
    xth_problem_apply_bc(pr, bc);
    double ntele = 0.0;
    for (int k = 0; k < 8 * ne; ++k) ntele += xyz[3 * (conn[k] - 1)] == lx;
    double* rext = calloc(p, sizeof(double));
    for (int k = 0; k < 8 * ne; ++k)
        if (xyz[3 * (conn[k] - 1)] == lx) rext[3 * (conn[k] - 1)] += amp * 1.0 / ntele;
    /* damage inputs: kokkos_damage's flattened arrays */
    double *Nx = malloc(sizeof(double) * 64 * ne), *Ny = malloc(sizeof(double) * 64 * ne),
           *Nz = malloc(sizeof(double) * 64 * ne);
    xth_problem_strain_rows(pr, Nx, Ny, Nz);
    int* nodes = malloc(sizeof(int) * 64 * ne);
    for (int g = 0; g < ngp; ++g)
        for (int i = 0; i < 8; ++i) nodes[g * 8 + i] = conn[(g / 8) * 8 + i];
    double *ym = malloc(sizeof(double) * ngp), *nuv = malloc(sizeof(double) * ngp);
    for (int g = 0; g < ngp; ++g) { ym[g] = E; nuv[g] = nu0; }
    double *eps_old = calloc((size_t)6 * ngp, 8), *eps_pl = calloc((size_t)6 * ngp, 8),
           *sig_eff = calloc((size_t)6 * ngp, 8), *sig_back = calloc((size_t)6 * ngp, 8);
    double *pp = calloc((size_t)ngp, 8), *D = calloc((size_t)ngp, 8), *ws = calloc((size_t)ngp, 8),
           *del_po = calloc((size_t)ngp, 8), *sig_d = calloc((size_t)ngp, 8);
    for (int g = 0; g < ngp; ++g) ws[g] = ws0;
    int *elesta = malloc(sizeof(int) * ne), *gpsta = malloc(sizeof(int) * ngp),
        *nefail = malloc(sizeof(int) * ne);
    for (int e = 0; e < ne; ++e) elesta[e] = 1;
    for (int g = 0; g < ngp; ++g) gpsta[g] = 1;

    /* patch 1: ILUT of the boundary-conditioned K (iwk = p (2 lfil + 1)) */
    csr K = {0}, M = {0};
    csr_get(pr, 0, &K);
    csr_get(pr, 1, &M);
    const int iwk = p * (2 * lfil + 1) + 1;
    double* alu = malloc(sizeof(double) * iwk);
    int *jlu = malloc(sizeof(int) * iwk), *ju = malloc(sizeof(int) * p);
    if (xth_ilut(p, K.ia, K.ja, K.a, lfil, droptol, iwk, alu, jlu, ju) != 0) return 2;
    kokkos_init_();
    if (check_device("kokkos_init_")) return 3;
    const int on = 1;
    xt_set_cache_(&on);

    double dt = dt0 * n1, tc[3] = {0.0, 0.0, 0.0};
    int nip = nipc * n1;
    const double w = 2.0 * 3.14159265358979323846 * freq;
    const size_t nst = (size_t)p * q;
    double *disp = calloc(nst, 8), *fext = malloc(sizeof(double) * nst);
    double *Nt = NULL, ck[36], cm[36], ckt[36], cmt[36], ck1[36], cm1[36], A[36], B[36];
    const double one = 1.0;
    const int iout = 0, maxits = 20000;
    for (int slab = 1; slab <= nslab; ++slab) {
        const double t3 = tc[2];
        for (int j = 0; j < 3; ++j) tc[j] = t3 + j * dt / 2.0;
        /* deletion check (:625-691) */
        int deleted = 0, any = 0;
        for (int g = 0; g < ngp; ++g) any |= D[g] >= Dc;
        if (slab > 1 && any) {
            int nef = 0;
            chkelesta_(&nn, &ne, &nnse, &ngpe, &Dc, D, elesta, gpsta, &nef, nefail);
            if (check_device("chkelesta_")) return 3;
            int ndf = 0;
            if (xth_problem_delete(pr, nef, nefail, bc, &ndf)) return fail("delete");
            csr_get(pr, 0, &K);
            csr_get(pr, 1, &M);
            /* patch 2: a new factor in place of the MUMPS refactorisation */
            if (xth_ilut(p, K.ia, K.ja, K.a, lfil, droptol, iwk, alu, jlu, ju) != 0)
                return fail("ilut");
            xt_invalidate_();
            dt = dt0 * n2;
            nip = nipc * n2;
            deleted = nef;
        }
        /* load blocks and jump term (:804-823) */
        double fextc[6], fint[6];
        xth_getfextc_m(tc[0], w, dt, fextc, fint);
        for (int j = 0; j < q; ++j)
            for (int r = 0; r < p; ++r) fext[(size_t)j * p + r] = fextc[j] * rext[r];
        xth_stcoeff_m(tc[0], dt, w, ck, cm, ckt, cmt, ck1, cm1);
        for (int k = 0; k < 36; ++k) { A[k] = ck[k] + ckt[k]; B[k] = cm[k] + cmt[k]; }
        /* patch 3 */
        kronspgemv_(ck1, cm1, &one, &one, &q, K.ia, K.ja, K.a, M.ia, M.ja, M.a, &p, disp, fext);
        if (check_device("kronspgemv_")) return 3;
        for (size_t k = 0; k < nst; ++k)
            if (bc[k % p]) fext[k] = 0.0;
        memset(disp, 0, sizeof(double) * nst);
        /* patch 4 (the shim's kronpgmres_logged writes gmres.log from xt_gmres_log) */
        int ierr = 0;
        kronpgmres_(A, B, &q, K.ia, K.ja, K.a, M.ia, M.ja, M.a, &p, alu, jlu, ju, fext, disp, &im,
                    &eps, &maxits, &iout, &ierr);
        if (ierr != 0) {
            fprintf(stderr, "kronpgmres_ ierr %d: %s\n", ierr, xt_last_error());
            return 3;
        }
        double rel0 = 0.0;
        if (xt_gmres_log(&rel0, 1) < 1) return fail("xt_gmres_log");
        for (size_t k = 0; k < nst; ++k)
            if (bc[k % p]) disp[k] = 0.0;
        /* damage (kokkos_damage, :880): temporal shape table, kernel, clean-up */
        Nt = realloc(Nt, sizeof(double) * 6 * nip);
        xth_nt_table(nip, tc, w, Nt);
        kokkos_host_(0, ne, nn, ndofn, nnse, nnte, ngpe, ncmp, nip, nodes, Nx, Ny, Nz, Nt, disp,
                     ym, nuv, eps_old, eps_pl, sig_eff, sig_back, pp, D, ws, del_po, sig_d);
        if (check_device("kokkos_host_")) return 3;
        for (int g = 0; g < ngp; ++g)
            if (gpsta[g] == 0) { D[g] = 0.0; ws[g] = 0.0; }
        fwrite(&deleted, sizeof(int), 1, out);
    }
    fwrite(disp, sizeof(double), nst, out);
    fwrite(D, sizeof(double), ngp, out);
    fwrite(elesta, sizeof(int), ne, out);
    fclose(out);
    kokkos_finish_();
    xth_problem_destroy(pr);
    return 0;
}
