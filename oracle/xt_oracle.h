/*
 * xt_oracle.h -- CPU oracle for the XTFEM space-time solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C on the host,
 * the reference routines of the hot path so that the GPU library can be
 * checked against them and so that the reference's CPU path can be timed as
 * a baseline.  Nothing in the product (xtfem_gb300/) links or calls it; only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do.
 *
 * Conventions follow the Fortran reference: CSR and MSR index arrays are
 * 1-based, q x q temporal matrices are column-major, and a space-time vector
 * of length p*q stores temporal block i at [(i-1)*p, i*p).
 *
 * Parity pinning: the reference ships no tests, golden vectors or known-answer
 * cases for this path, and it cannot be built here (no Fortran compiler, MPI,
 * Kokkos or MUMPS).  Each routine is therefore checked against mathematical
 * invariants and independent statements (explicit Kronecker products, exact
 * LU limits, quadrature of the temporal integrals, hand-built strain
 * histories) in tests/.  Parity is unpinned by the reference's own tests.
 */
#ifndef XT_ORACLE_H
#define XT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Host threads for amux, kronspmv/kronspgemv, kronlusol and kronpgmres
 * (default 1: the reference's serial order, bit for bit).  Above 1 the
 * per-entry arithmetic is unchanged and only the dot products and norms of
 * kronpgmres sum in another order; this is the threaded CPU baseline. */
void orc_set_threads(int n);
int orc_get_threads(void);

/* src/ilut.f:3-44  amux: y = A x for CSR A (1-based). */
void orc_amux(int n, const double *x, double *y, const double *a,
              const int *ja, const int *ia);

/* src/kronecker.f90:19-85  kronspmv: y = (A (x) K + B (x) M) x. */
void orc_kronspmv(const double *a, const double *b, int q,
                  const int *ki, const int *kj, const double *kv,
                  const int *mi, const int *mj, const double *mv,
                  int p, const double *x, double *y);

/* src/kronecker.f90:88-127  kronspgemv: y = alpha (A(x)K + B(x)M) x + beta y. */
void orc_kronspgemv(const double *a, const double *b, double alpha,
                    double beta, int q, const int *ki, const int *kj,
                    const double *kv, const int *mi, const int *mj,
                    const double *mv, int p, const double *x, double *y);

/* src/kronecker.f90:368-395  inverse of an n x n column-major matrix by LU
 * with partial pivoting.  Returns 0, or 1 when the matrix is singular. */
int orc_inverse(int n, const double *A, double *Ainv);

/* src/ilut.f:2383-2432  lusol: solve (LU) x = y with the MSR factor. */
void orc_lusol(int n, const double *y, double *x, const double *alu,
               const int *jlu, const int *ju);

/* src/kronecker.f90:130-178  kronlusol: y = (A^-1 (x) (LU)^-1) x.
 * Returns 0, or 1 when A is singular (the reference STOPs there). */
int orc_kronlusol(const double *a, int q, const double *alu, const int *jlu,
                  const int *ju, int p, const double *x, double *y);

/* src/ilut.f:152-495 (+ qsplit 2487-2545)  SPARSKIT ILUT(lfil, droptol).
 * alu/jlu must hold iwk entries, ju n entries.  Returns SPARSKIT's ierr. */
int orc_ilut(int n, const double *a, const int *ja, const int *ia, int lfil,
             double droptol, double *alu, int *jlu, int *ju, int iwk);

/* src/ilut.f:2487-2545  qsplit on a[0..n-1] with companion ind. */
void orc_qsplit(double *a, int *ind, int n, int ncut);

/* src/kronecker.f90:181-365  kronpgmres: right-preconditioned restarted
 * GMRES(im) with modified Gram-Schmidt and Givens rotations.  rhs is used as
 * scratch (destroyed), as in the reference.  Returns ierr (0 converged,
 * 1 maxits reached, -1 zero initial residual, 2 singular A).  *its_out gets
 * the iteration count; hist (may be NULL, length hist_len) gets |rs(i+1)|/ro0
 * per iteration. */
int orc_kronpgmres(const double *a, const double *b, int q,
                   const int *ki, const int *kj, const double *kv,
                   const int *mi, const int *mj, const double *mv, int p,
                   const double *alu, const int *jlu, const int *ju,
                   double *rhs, double *sol, int im, double eps, int maxits,
                   int *its_out, double *hist, int hist_len);

/* src/kokkos_damage.f90:36-47  temporal shape table Nt[jj*6+k], nip rows,
 * over the slab with node times tcoorde[0..2] and load frequency w. */
void orc_nt_table(int nip, const double *tcoorde, double w, double *Nt);

/* src/kokkos_host.cpp:37-41 signature; src/kokkos_kernel.h:45-344 math.
 * Two-scale fatigue-damage update of every Gauss point over nip temporal
 * points.  nthreads <= 1 runs serially. */
void orc_damage(int ne, int nn, int ndofn, int nnse, int nnte, int ngpe,
                int ncmp, int nip, const int *nodes, const double *Nx,
                const double *Ny, const double *Nz, const double *Nt,
                const double *sol, const double *ym, const double *nu,
                double *eps_old, double *eps_pl, double *sig_eff,
                double *sig_back, double *p, double *D, double *ws,
                double *del_po, double *sig_d, int nthreads);

/* src/getdfinal.f:10-397: the reference's stand-alone statement of the
 * same two-scale law, driven over a prescribed global strain history eps
 * (nsteps x 6, Voigt, engineering shear) for ONE point whose state (the six
 * -component eps_old, eps_pl, sig_eff, sig_back and the scalars) is updated
 * in place; E and nu replace the reference's hard-coded 1.97e5 and 0.3.
 * Written independently of orc_damage, to cross-check it. */
void orc_getdfinal_history(int nsteps, const double *eps, double *eps_old,
                           double *eps_pl, double *sig_eff, double *sig_back,
                           double *p, double *D, double *ws, double *del_po,
                           double *sig_d, double E, double nu);

/* Same as orc_damage but applies the failed-point clean-up of
 * src/kokkos_damage.f90:102-107 (D = ws = 0 where gpsta == 0). */
void orc_damage_cleanup(int ngp, const int *gpsta, double *D, double *ws);

/* src/delelement.f90:109-136  chkelesta: element failed when any of its
 * ngpe Gauss points has D >= Dc.  Returns nef; nefail gets 1-based element
 * numbers in ascending order. */
int orc_chkelesta(int ne, int ngpe, double Dc, const double *D, int *elesta,
                  int *gpsta, int *nefail);

/* src/stcoeff.f90:62-356 by definition: k, m, ktn, mtn, ktn1, mtn1 (6x6,
 * column-major) as integrals of the enriched temporal basis over the slab
 * [t1, t1+dt], evaluated by composite Gauss-Legendre quadrature. */
void orc_stcoeff_m_quad(double t1, double dt, double w, double *k, double *m,
                        double *ktn, double *mtn, double *ktn1, double *mtn1);

/* src/getfextc.f90:22-58 by definition (quadrature): fextc[6] = integral of
 * dN_j/dt * sin(w t) over the slab. */
void orc_getfextc_m_quad(double t1, double w, double dt, double *fextc);

/* src/stcoeff.f90:1-60 by definition (quadrature of the quadratic Lagrange
 * products): the thermal k, m, ktn, mtn, ktn1, mtn1 (3x3, column-major). */
void orc_stcoeff_t_quad(double dt, double *k, double *m, double *ktn,
                        double *mtn, double *ktn1, double *mtn1);

/* By definition: fint[j] = integral of dN_j/dt over the slab for the six
 * mechanical basis functions (the thermal-stress load weights whose closed
 * forms are src/getfextc.f90:53-58). */
void orc_fint_m_def(double t1, double w, double dt, double *fint);

#ifdef __cplusplus
}
#endif
#endif
