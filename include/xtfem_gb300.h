/*
 * xtfem_gb300.h -- C ABI of the GB300 space-time solve library
 * (xtfem_gb300/libxtfem_gb300.so).
 *
 * Drop-in for the iterative solve path of the XTFEM extended space-time
 * finite-element code: the Kronecker operator apply, the ILUT-preconditioned
 * restarted GMRES built on it, the per-Gauss-point fatigue-damage update and
 * the element-deletion test.  Every entry point takes plain pointers and
 * sizes.  Arrays are host memory owned by the caller unless the name says
 * "_device".
 *
 * Conventions of the Fortran entry points (trailing underscore, gfortran
 * name mangling): scalars by reference, CSR/MSR index arrays 1-based, q x q
 * temporal matrices column-major, a space-time vector of length p*q holds
 * temporal block i at [(i-1)*p, i*p).  They return nothing, as the
 * reference's subroutines do; the last error is available from
 * xt_last_error() and the status-returning xt_* variants.
 *
 * Status codes: 0 success; the GMRES codes 1 (maxits) and -1 (zero initial
 * residual) as in the reference; negative codes <= -10 for library errors.
 */
#ifndef XTFEM_GB300_H
#define XTFEM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define XT_OK 0
#define XT_ERR_ARG (-10)
#define XT_ERR_CUDA (-11)
#define XT_ERR_ALLOC (-12)
#define XT_ERR_NONFINITE (-13)
#define XT_ERR_SINGULAR (-14)
#define XT_ERR_STATE (-15)
#define XT_ERR_TIMEOUT (-16)
#define XT_ERR_HOST (-17)

/* ------------------------------------------------------------ lifetime */

/* Replaces kokkos_init_ (src/kokkos_host.cpp:14-20): selects device 0 and
 * creates the library's stream. */
void kokkos_init_(void);
/* Replaces kokkos_finish_ (src/kokkos_host.cpp:22-24): frees every cached
 * device object. */
void kokkos_finish_(void);

int xt_init(int device);
int xt_finalize(void);
/* Message of the last error on the calling thread ("" when none). */
const char *xt_last_error(void);
void xt_clear_error(void);
const char *xt_version(void);

/* Operator and factor caching of the Fortran entry points.  With caching
 * off (default) every call uploads K, M and the factor.  With caching on,
 * device copies are kept and reused for calls with the same array addresses
 * and sizes; the caller must call xt_invalidate_() after changing K, M or
 * the factor in place (after element deletion, reassembly or refactoring).
 */
void xt_set_cache_(const int *on);
void xt_invalidate_(void);

/* ------------------------------------- Fortran solver entry points */

/* src/kronecker.f90:19-85  kronspmv: y = (A (x) K + B (x) M) x. */
void kronspmv_(const double *a, const double *b, const int *q, const int *ki,
               const int *kj, const double *kv, const int *mi, const int *mj,
               const double *mv, const int *p, const double *x, double *y);

/* src/kronecker.f90:88-127  kronspgemv: y = alpha (A(x)K + B(x)M) x + beta y. */
void kronspgemv_(const double *a, const double *b, const double *alpha,
                 const double *beta, const int *q, const int *ki, const int *kj,
                 const double *kv, const int *mi, const int *mj,
                 const double *mv, const int *p, const double *x, double *y);

/* src/kronecker.f90:130-178  kronlusol: y = (A^-1 (x) (LU)^-1) x with the
 * SPARSKIT MSR factor alu/jlu/ju of src/ilut.f:152-495. */
void kronlusol_(const double *a, const int *q, const double *alu,
                const int *jlu, const int *ju, const int *p, const double *x,
                double *y);

/* src/kronecker.f90:181-365  kronpgmres: solve (A(x)K + B(x)M) sol = rhs by
 * ILUT-right-preconditioned GMRES(im), FP64, with the reference's restart,
 * convergence (|rs(i+1)| <= eps ||r0||) and ierr conventions (0, 1, -1;
 * library errors <= -10).  rhs is used as scratch as in the reference
 * (its content on return is unspecified).  The reference writes its
 * residual history to Fortran unit iout (:257-259, :311; src/main3d.f90 opens
 * it as gmres.log); a C library cannot write to a Fortran unit, so with
 * iout >= 0 the history is kept for xt_gmres_log and the caller's shim
 * writes the lines (iout < 0: nothing is kept). */
void kronpgmres_(const double *a, const double *b, const int *q,
                 const int *ki, const int *kj, const double *kv,
                 const int *mi, const int *mj, const double *mv, const int *p,
                 const double *alu, const int *jlu, const int *ju, double *rhs,
                 double *sol, const int *im, const double *eps,
                 const int *maxits, const int *iout, int *ierr);

/* The residual history of this thread's last kronpgmres_ call made with
 * iout >= 0, as the reference writes it: entry 0 is ||r0||/||rhs|| at
 * its = 0 (the line written when iout >= 0), entry k >= 1 the estimate
 * |rs(i+1)|/||rhs|| after iteration k (written when iout > 0).  Copies up
 * to cap entries to rel and returns the number of entries (0 before any
 * such call). */
int xt_gmres_log(double *rel, int cap);

/* src/delelement.f90:109-136  chkelesta on the device: element i fails when
 * one of its ngpe Gauss points has D >= Dc; gpsta/elesta set to 0 for it
 * and nefail gets the 1-based failed elements in ascending order. */
void chkelesta_(const int *nn, const int *ne, const int *nnse, const int *ngpe,
                const double *Dc, const double *D, int *elesta, int *gpsta,
                int *nef, int *nefail);

/* ------------------------------------------------ damage entry point */

/* src/kokkos_host.cpp:37-41  kokkos_host_, same signature and array
 * layouts (scalars by value, arrays flattened as in
 * src/kokkos_damage.f90:51-84).  Runs the two-scale fatigue-damage update
 * of every Gauss point over nip temporal points on the GPU. */
void kokkos_host_(int rank, int ne, int nn, int ndofn, int nnse, int nnte,
                  int ngpe, int ncmp, int nip, int *nodes, double *Nx,
                  double *Ny, double *Nz, double *Nt, double *sol, double *ym,
                  double *nu, double *eps_old, double *eps_pl,
                  double *sig_eff, double *sig_back, double *p, double *D,
                  double *ws, double *del_po, double *sig_d);

/* Status-returning form of kokkos_host_ (no rank argument). */
int xt_damage(int ne, int nn, int ndofn, int nnse, int nnte, int ngpe,
              int ncmp, int nip, const int *nodes, const double *Nx,
              const double *Ny, const double *Nz, const double *Nt,
              const double *sol, const double *ym, const double *nu,
              double *eps_old, double *eps_pl, double *sig_eff,
              double *sig_back, double *p, double *D, double *ws,
              double *del_po, double *sig_d);

/* Allocation-free form of xt_damage.  No counterpart in the reference: it
 * serves callers that keep the damage state resident on the GPU and must
 * not allocate inside their time loop: a driver that hands all device
 * memory to its own pool up front (a cudaMalloc there fails or steals from
 * the pool), and a loop whose streams must keep running while it calls in
 * (cudaMalloc and cudaFree can synchronise the device).
 *   - Every array argument is a DEVICE pointer with the layouts of
 *     xt_damage; nothing is copied to or from the host except counts.
 *   - The kernel's scratch (FP32 copy of Nt, shape-value bounds, step
 *     counters) is a static 1.5 MB array in the library's device image,
 *     held on every GPU that loads the library until the process exits, so
 *     nip must be <= 65536 (XT_ERR_ARG with a message otherwise; use
 *     xt_damage for longer slabs).
 *   - The step counters are cleared at the start of every call (they
 *     accumulate with atomics); counts (host, may be NULL) receives the
 *     plastic, screened-elastic and exact step totals.
 *   - The first call looks up the scratch address (cudaGetSymbolAddress,
 *     once per device, with that device current) and may set up the
 *     library context: make that first call, or xt_init, before any
 *     stream capture.
 *   - One scratch per process and device, keeping the last call's
 *     contents: calls whose work overlaps on the GPU (two host threads)
 *     race on it.
 *   - Ordering: the call starts with cudaDeviceSynchronize, so every kernel
 *     or copy the caller queued before it, on any stream of the device,
 *     has finished writing the inputs and the state before the update
 *     reads them.  It returns after the update has finished.
 *   - The work runs on the library's device (xt_init); the calling
 *     thread's current device is restored before the call returns. */
int xt_damage_device(int ne, int nn, int ndofn, int nnse, int nnte, int ngpe,
                     int ncmp, int nip, const int *nodes, const double *Nx,
                     const double *Ny, const double *Nz, const double *Nt,
                     const double *sol, const double *ym, const double *nu,
                     double *eps_old, double *eps_pl, double *sig_eff,
                     double *sig_back, double *p, double *D, double *ws,
                     double *del_po, double *sig_d, unsigned long long *counts);

/* --------------------------------------------- handle-based interface */

/* A device-resident space-time system: K and M (1-based CSR, order p), the
 * temporal size q, an optional ILUT factor and the current A, B.  This is
 * the form the Fortran entry points use internally; it lets a caller keep
 * the operator on the GPU across slabs. */
typedef struct xt_system_s *xt_system;

int xt_system_create(int p, int q, const int *ki, const int *kj,
                     const double *kv, const int *mi, const int *mj,
                     const double *mv, xt_system *out);
int xt_system_destroy(xt_system s);
/* Factor in SPARSKIT MSR form (src/ilut.f:152-240).  group = rows per node
 * for the level schedule (3 for three DOFs per node; 1 = row levels). */
int xt_system_set_ilu(xt_system s, const double *alu, const int *jlu,
                      const int *ju, int group);
/* The same for a block-Jacobi factor of `blocks` row blocks
 * (xth_ilut_blocks of include/xtfem_gb300_host.h): when the factor has no
 * entry between the blocks, the FP32 register sweep runs each block's
 * triangular solves in a thread block of its own (blocks x q thread
 * blocks per sweep instead of q); other sweeps use the one schedule of the
 * whole factor.  A factor with entries between blocks falls back to that
 * schedule too.  blocks <= 1: xt_system_set_ilu. */
int xt_system_set_ilu_blocks(xt_system s, const double *alu, const int *jlu,
                             const int *ju, int group, int blocks);
/* The row blocks the FP32 register sweep runs as independent solves (1 for
 * the whole factor). */
int xt_system_ilu_blocks(xt_system s);
/* Classical Gram-Schmidt passes per Arnoldi step of the flexible GMRES
 * (precision 2): 2 (the default) or 1, with the switch to two for the rest
 * of a solve after a loss of orthogonality (as xt_slab_config.gs_passes). */
int xt_system_set_gs_passes(xt_system s, int passes);
/* Temporal matrices A (with the slab-start jump) and B, q x q column-major. */
int xt_system_set_temporal(xt_system s, const double *a, const double *b);
/* kronspgemv semantics with explicit temporal matrices (host vectors,
 * block layout). */
int xt_system_apply(xt_system s, const double *a, const double *b,
                    double alpha, double beta, const double *x, double *y);
/* kronlusol semantics with the system's factor and temporal matrix a. */
int xt_system_lusol(xt_system s, const double *a, const double *x, double *y);
/* The same apply with the factor, the vectors and the arithmetic in FP32
 * (the preconditioner of the mixed-precision inner solve); x and y stay
 * FP64 at the boundary.  No counterpart in the reference, whose lusol is
 * FP64 only. */
int xt_system_lusol_f32(xt_system s, const double *a, const double *x, double *y);
/* kronpgmres semantics (host vectors, block layout).  rhs is preserved.
 * its/ierr/est may be NULL; hist (may be NULL) receives up to hist_len
 * residual estimates |rs(i+1)|/||r0||. */
int xt_system_gmres(xt_system s, const double *rhs, double *sol, int im,
                    double eps, int maxits, int *its, int *ierr, double *est,
                    double *hist, int hist_len);
/* Solve to a true relative residual <= tol with FP64 residuals and
 * solution; precision 0 runs FP64 GMRES cycles, 1 runs FP32 operator,
 * factor and Krylov basis (FP64 dot products and Hessenberg) inside FP64
 * iterative refinement, 2 runs flexible GMRES with the FP32 factor and a
 * double-float (FP32 pair) basis and operator on the preconditioned
 * vectors, 3 runs mode 2 with a preconditioner that is itself a short
 * FP32 GMRES (10 steps, ILU-preconditioned) on K and M stored in BF16
 * (rounded to nearest, widened to FP32 and accumulated in FP32; the
 * BF16-stored experiment: with BF16 K and M as the operator of plain
 * refinement the error of a stiff system's K makes it diverge).
 * out_stats (may be NULL) gets 6 values: iterations, cycles,
 * refinement passes, ierr, true relative residual, last estimate. */
int xt_system_solve(xt_system s, const double *rhs, double *sol, int im,
                    double tol, int maxits, int precision, double inner_tol,
                    double *out_stats);

/* Device reassembly of the system's stiffness K from per-Gauss-point
 * moduli: the element loop of mpiglbmtx_m (src/mpisubs.f90:69-139, with
 * setsdstiff and elemtx_m per Gauss point), which a coupled run calls every
 * slab after material_update (src/thermoelastic.f90:1-46), merged into the
 * system's fixed CSR pattern instead of through tricsr
 * (src/spmtx.f90:359-407).  No counterpart as an entry point in the
 * reference, which assembles on the host.  xt_system_set_mesh gives the
 * C3D8 mesh (xyz: nn x 3; conn: ne x 8, 1-based, the reference's node
 * order) and the constrained DOFs (bc: 3 nn entries, 1 = constrained, with
 * csrapplybc semantics: row and column zero, diagonal 1).  K then takes the
 * mesh's full element pattern (every DOF pair of a shared element, explicit
 * zeros kept, so that any moduli fit it) with its current values carried
 * over; it fails when K has an entry outside that pattern.
 * xt_system_assemble_k recomputes K's values from ym and nu (ne x 8; Gauss
 * point l of element e at 8 e + l, the 2x2x2 rule's order with xi
 * outermost) on the device.  The ILU factor is not touched: a caller that
 * wants one for the new K downloads it (xt_system_get_k), refactors on the
 * host and sets it. */
int xt_system_set_mesh(xt_system s, int nn, int ne, const double *xyz, const int *conn,
                       const int *bc);
int xt_system_assemble_k(xt_system s, const double *ym, const double *nu);
/* K's current number of entries, and K itself as 1-based CSR (ia: p + 1,
 * ja and kv: nnz entries; any of the three may be NULL). */
int xt_system_k_nnz(xt_system s);
int xt_system_get_k(xt_system s, int *ia, int *ja, double *kv);

/* ------------------------------------------------ batches of systems */

/* A batch of independent systems (load cases or specimens of uneven
 * sizes) solved together.  No counterpart in the reference, which solves
 * one system per process; these are the batched entries of the many-rod
 * workload (64 rods of n x n x 3n elements).  Each system keeps its own
 * stream; a pool of host worker threads drives them, largest first, so the
 * level-scheduled triangular sweeps of different systems (each a
 * dependent chain on three SMs) and their bandwidth-bound kernels run at
 * the same time on different SMs.  The systems stay owned by the caller
 * and must outlive the batch; a system must not be used elsewhere while a
 * batch solve runs, nor be listed twice (XT_ERR_ARG).  workers <= 0 picks
 * min(count, 16). */
typedef struct xt_batch_s *xt_batch;

int xt_batch_create(int count, const xt_system *systems, int workers, xt_batch *out);
int xt_batch_destroy(xt_batch b);
/* xt_system_solve on every system of the batch: rhs[i] and sol[i] are
 * system i's host vectors (block layout; sol[i] is the initial guess and
 * receives the solution).  im <= 0 uses the batch's tuned restart length
 * and ILU lanes per row; the first such call tunes them (each restart of
 * 30, 60, 120 and 200, capped at the largest system's unknowns, with 2 and
 * with 1 lanes per row of the FP32 register sweep, i.e. 5 or 10 node rows
 * per warp, solves the whole batch once from the given initial guesses;
 * the fastest pair is kept for the batch's later calls).
 * Precision 2 runs the batch in lockstep on the calling thread: every
 * system's refined solve with its Arnoldi bookkeeping on the device, and
 * per round the next 16 Arnoldi steps of every system as one CUDA graph
 * (captured once per call and replayed; each kernel of a step serves every
 * system in one launch, the ILU sweeps one launch per group of equal
 * kernel shape, and a system whose cycle or solve has ended does nothing
 * in it), one host synchronisation per round for all control words.  Other precisions run
 * each system's solve on a pool of `workers` host threads.  Either way
 * each solution equals the system's own xt_system_solve bit for bit.
 * stats (may be NULL) gets 6 values per system as in xt_system_solve;
 * status (may be NULL) gets each system's return code.  Returns XT_OK when
 * every system succeeded, else the first failing system's code (its
 * message is the batch's last error). */
int xt_batch_solve(xt_batch b, const double *const *rhs, double *const *sol, int im,
                   double tol, int maxits, int precision, double inner_tol,
                   double *stats, int *status);
/* The restart length the tuner picked (0 before the first tuned call). */
int xt_batch_restart(xt_batch b);
/* The ILU lanes per row the tuner picked (1 or 2; 0 before the first tuned
 * call).  No counterpart in the reference. */
int xt_batch_ilu_shares(xt_batch b);
/* The Gram-Schmidt passes the tuner picked (precision 2: it tries one pass
 * at the best restart length and lanes per row; 0 before the first tuned
 * call). */
int xt_batch_gs_passes(xt_batch b);

#ifdef __cplusplus
}
#endif
#endif
