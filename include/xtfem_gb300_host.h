/*
 * xtfem_gb300_host.h -- host-side set-up and the slab driver of the GB300
 * library (same shared object as xtfem_gb300.h).
 *
 * The reference's Fortran driver (src/main3d.f90) assembles K and M,
 * applies boundary conditions, factors K with ILUT and marches the
 * space-time slabs.  These entry points provide the same steps to a C, C++
 * or Python caller: the set-up runs on the host in FP64 (as in the
 * reference); the slab loop keeps every per-slab vector on the GPU.
 */
#ifndef XTFEM_GB300_HOST_H
#define XTFEM_GB300_HOST_H

#ifdef __cplusplus
extern "C" {
#endif

/* --------------------------------------------------- problem set-up */
typedef struct xth_problem_s *xth_problem;

/* Mesh from the reference's .inp format (src/main3d.f90:212-231), or a
 * structured rod of nx x ny x nz C3D8 elements over [0,lx]x[0,ly]x[0,lz]
 * numbered like inp/prismaticrod-*.inp; then K, M and the per-Gauss-point
 * strain rows for a uniform isotropic material (src/mpisubs.f90:69-139). */
int xth_problem_from_inp(const char *path, double E, double nu, double rho,
                         xth_problem *out);
/* A problem from a C3D8 mesh in memory: xyz (nn x 3), conn (ne x 8, 1-based,
 * the node order of the reference's shape functions, src/procs.f90:1366-1389). */
int xth_problem_from_mesh(int nn, int ne, const double *xyz, const int *conn, double E,
                          double nu, double rho, xth_problem *out);
int xth_problem_rod(int nx, int ny, int nz, double lx, double ly, double lz,
                    double E, double nu, double rho, xth_problem *out);
int xth_problem_destroy(xth_problem pr);
/* Current sizes (K changes after deletion surgery). */
int xth_problem_sizes(xth_problem pr, int *nn, int *ne, int *nnz_k,
                      int *nnz_m);
int xth_problem_mesh(xth_problem pr, double *xyz, int *conn);
/* Copies of the current 1-based CSR K and M (ia: 3nn+1, ja/a: nnz). */
int xth_problem_k(xth_problem pr, int *ia, int *ja, double *a);
int xth_problem_m(xth_problem pr, int *ia, int *ja, double *a);
/* Strain rows Nx, Ny, Nz, 8 per Gauss point, 8 Gauss points per element. */
int xth_problem_strain_rows(xth_problem pr, double *nx, double *ny,
                            double *nz);
/* Constitutive matrix (6x6 column-major) of the uniform material. */
int xth_problem_stiffness(xth_problem pr, double *d);
/* src/spmtx.f90:268-307 csrapplybc on K and M with a mask over the 3nn
 * spatial DOFs (nonzero = fixed). */
int xth_problem_apply_bc(xth_problem pr, const int *bc);
/* Element deletion surgery of src/main3d.f90:634-687 for the failed
 * elements nefail[0..nef) (1-based): K -= sum of their element stiffness
 * (delelement, src/delelement.f90:1-59), node-element counts decremented
 * (chkcnsta), disconnected nodes found (chkndsta) and given unit diagonals
 * (adddiagonal), their DOFs added to the mask bc (3nn entries, updated in
 * place), then csrapplybc on M and K.  ndf_out gets the number of newly
 * disconnected nodes. */
int xth_problem_delete(xth_problem pr, int nef, const int *nefail, int *bc,
                       int *ndf_out);

/* The first row (0-based) of K that the last xth_problem_delete changed:
 * a DOF row of a failed element, or a row coupled to a newly fixed DOF.
 * Rows above it are unchanged, so it is the first_row for xth_ilut_update.
 * -1 for a null handle. */
int xth_problem_first_changed_row(xth_problem pr);

/* src/ilut.f:152-495 ILUT(lfil, droptol) in FP64; alu/jlu hold iwk entries,
 * ju n entries; returns SPARSKIT's ierr: 0 success, -1 a row's L or U
 * length exceeds n, -2 the L part overflows iwk, -3 the U part overflows
 * iwk (tested as the reference tests it, row by row), -4 lfil < 0, -5 a
 * zero row.  A zero pivot is replaced by (1e-4 + droptol) times the row
 * norm, with 1e-4 rounded to single precision as in the reference. */
int xth_ilut(int n, const int *ia, const int *ja, const double *a, int lfil,
             double droptol, int iwk, double *alu, int *jlu, int *ju);
/* Block-Jacobi ILUT: the ILUT above of A with its entries between `blocks`
 * contiguous row blocks dropped first.  Block b holds whole node groups of
 * `group` rows: rows from floor(ng b / blocks) group on, ng = n / group
 * (group 1 when n is not a multiple of it).  The factor has no entry
 * between blocks, so its triangular solves split into independent ones
 * (xt_system_set_ilu_blocks runs them on separate SMs).  A weaker
 * preconditioner than the ILUT of A (more GMRES iterations) with shorter
 * dependency chains.  blocks <= 1: xth_ilut.  No counterpart in the
 * reference, whose ILUT factors the whole K. */
int xth_ilut_blocks(int n, const int *ia, const int *ja, const double *a, int lfil,
                    double droptol, int iwk, int group, int blocks, double *alu, int *jlu,
                    int *ju);
/* The same factor when rows [0, first_row) of the matrix equal those of the
 * matrix prev_alu/prev_jlu/prev_ju was computed from (same lfil, droptol):
 * those rows are copied and the rest refactored (ILUT row i depends only on
 * rows <= i).  After a deletion, first_row is xth_problem_first_changed_row.
 * No counterpart in the reference, which refactors every row. */
int xth_ilut_update(int n, const int *ia, const int *ja, const double *a, int lfil,
                    double droptol, int iwk, int first_row, const double *prev_alu,
                    const int *prev_jlu, const int *prev_ju, double *alu, int *jlu, int *ju);

/* src/stcoeff.f90:62-356 (mechanical, 6x6) and 1-60 (thermal, 3x3),
 * column-major. */
void xth_stcoeff_m(double t1, double dt, double w, double *k, double *m,
                   double *ktn, double *mtn, double *ktn1, double *mtn1);
void xth_stcoeff_t(double dt, double *k, double *m, double *ktn, double *mtn,
                   double *ktn1, double *mtn1);
/* src/getfextc.f90:22-58 */
void xth_getfextc_m(double t1, double w, double dt, double *fextc,
                    double *fint);
/* src/getfextc.f90:1-20: the thermal load weights fextc[3] of the slab
 * [t1, t1+dt] (load period 24, w = 2 * 3.14159 / 24 as in the reference). */
void xth_getfextc_t(double t1, double dt, double *fextc);
/* src/kokkos_damage.f90:36-47 temporal shape table Nt[jj*6+k]. */
void xth_nt_table(int nip, const double *tcoorde, double w, double *nt);

/* ------------------------------------------------------ slab driver */
/* Mechanical slab loop of src/main3d.f90:609-937 without the thermal part:
 * deletion check, load and jump terms, GMRES solve, damage update, all on
 * the GPU with the slab state resident. */
typedef struct xt_slab_config {
    int clamp_axis;      /* nodes with x[clamp_axis] == clamp_value fixed */
    double clamp_value;
    int load_axis;       /* traction face x[load_axis] == load_value */
    double load_value;
    int load_comp;       /* force component 0,1,2 */
    double amplitude;    /* traction amplitude (MPa) */
    double area;         /* loaded area (mm^2) */
    double freq;         /* load frequency (Hz) */
    double dt0;          /* step time per cycle unit (s) */
    int n1, n2;          /* cycles per slab before / after first deletion */
    int nipc;            /* temporal damage points per cycle */
    int lfil;            /* ILUT fill */
    double droptol;      /* ILUT drop tolerance */
    int im;              /* GMRES restart length */
    double tol;          /* true relative residual target */
    int maxits;          /* Arnoldi steps per slab at most */
    int precision;       /* as in xt_system_solve: 0 FP64 GMRES, 1 FP32 inner
                            + FP64 refinement, 2 flexible (default of the
                            bench), 3 as 2 with a nested FP32 GMRES on
                            BF16-stored K and M as preconditioner */
    double inner_tol;    /* relative tolerance of an FP32 inner solve */
    double Dc;           /* critical damage */
    int damage;          /* 1 = run the damage update */
    int group;           /* rows per node in the ILU level schedule */
    int overlap;         /* 1 = run each slab's damage update on a second,
                            lower-priority stream while the next slab is
                            solved (see xt_slab_step) */
    double load_ratio;   /* R = F_min / F_max of the cyclic traction
                            F(t) = amplitude (m + sin(w t)), m = (1 + R) / (1 - R);
                            -1 (the reference's fully reversed sine) gives
                            m = 0.  The mean part m enters the load blocks
                            with the weights of a load constant in time,
                            N_j(t1 + dt) - N_j(t1) = (-1, 0, 1, 0, 0, 0),
                            beside the sine weights of src/getfextc.f90. */
    int gs_passes;       /* classical Gram-Schmidt passes per Arnoldi step of
                            the flexible GMRES (precision 2 and 3): 2 (also
                            for 0) or 1.  One pass reads the Krylov basis
                            twice per step instead of four times; a solve
                            with one pass switches to two for the rest of the
                            solve when the true residual at a restart
                            exceeds the estimate it followed tenfold (the
                            basis has lost orthogonality). */
    int ilu_blocks;      /* > 1: the block-Jacobi ILUT of that many row
                            blocks (xth_ilut_blocks) in place of the ILUT of
                            K, its blocks' triangular solves on separate SMs
                            (xt_system_set_ilu_blocks); 0 or 1: the ILUT of
                            K, as the reference. */
} xt_slab_config;

typedef struct xt_slab_s *xt_slab;

int xt_slab_create(xth_problem pr, const xt_slab_config *cfg, xt_slab *out);
int xt_slab_destroy(xt_slab s);
/* One slab.  stats (may be NULL) receives 12 values: slab index, GMRES
 * iterations, restart cycles, refinement passes, ierr, true relative
 * residual, max D, failed elements so far, elements deleted this slab,
 * plastic steps, screened elastic steps, exact steps.
 * With cfg.overlap = 1 the slab's damage update is left running on a second
 * stream when the call returns, and the next call solves its slab while it
 * runs: the slab's operator changes only when the damage update deletes
 * elements, so the next solve is started at once and, if the update did
 * delete elements, discarded and repeated on the new operator.  The results
 * are those of the sequential loop; the damage entries of stats (max D and
 * the step counts) then describe the previous slab, and xt_slab_drain
 * returns those of the last one. */
int xt_slab_step(xt_slab s, double *stats);
/* The same slab through host buffers: fext (block layout, p*6) replaces the
 * slab's external load vector, and the slab's displacement (block layout,
 * p*6) and damage (8 per element) are copied back.  With cfg.overlap = 1,
 * D is the damage after the previous slab (the current update is still
 * running). */
int xt_slab_step_host(xt_slab s, const double *fext, double *disp, double *D,
                      double *stats);
/* Waits for a damage update still running (cfg.overlap = 1) and writes its
 * max D and step counts to stats[6], stats[9..11] (stats may be NULL). */
int xt_slab_drain(xt_slab s, double *stats);
/* Replaces the damage D and stored energy ws of every Gauss point (host
 * arrays of 8 per element; either may be NULL), e.g. to resume a run. */
int xt_slab_set_state(xt_slab s, const double *D, const double *ws);
/* The reference's output step (src/postprocess.f90:106-378) for the last
 * slab: nodal displacement and Gauss-point strain, stress, damage, stored
 * energy and element status at the slab's output time, appended to
 * <job>.time, <job>.disp and <job>_0.strain / .stress / .damage / .energy /
 * .status (strain and stress as 6(E16.8,2X) records, list-directed values
 * with 17 significant digits); truncate = 1 empties the files first, as the
 * reference's initfile does (an empty <job>.temp is made too).  Waits for a
 * running damage update. */
int xt_slab_dump(xt_slab s, const char *job, int truncate);
/* Copies of the current state (waits for a running damage update). */
int xt_slab_get(xt_slab s, double *disp, double *D, double *ws, int *elesta);
/* ------------------------------------------------ thermal slab loop */

/* The temperature part of the reference's slab loop (src/main3d.f90:
 * 429-476 set-up, 586-608 initial and boundary terms, 697-734 per slab)
 * (on its own, or advanced by a coupled mechanical loop, xt_slab_couple):
 * q = 3 temporal nodes,
 * conductivity and capacity of the mesh (elemtx_t, src/elesubs.f90:60-116),
 * fixed temperature T0 on the faces x[fixed_axis] == fixed_value[0] or
 * fixed_value[1], heat flux q0 on the faces x[flux_axis] == flux_value[0]
 * or flux_value[1] (the total q0 * area shared by the element-node
 * incidences of the first face, as the reference counts them), initial
 * temperature Tref, GMRES with the ILUT factor of the conductivity (the
 * reference's MPI route uses an exact MUMPS factor instead). */
typedef struct xt_thermal_config {
    int fixed_axis;
    double fixed_value[2];
    double T0;           /* fixed temperature */
    double Tref;         /* initial temperature */
    int flux_axis;
    double flux_value[2];
    double q0;           /* heat flux per unit area */
    double area;         /* area the total flux is referred to */
    double kappa;        /* conductivity */
    double rho;          /* density */
    double cp;           /* specific heat */
    double dt0;          /* slab length dt0 * n1 */
    int n1;
    int lfil;            /* ILUT fill */
    double droptol;      /* ILUT drop tolerance */
    int im;              /* GMRES restart length */
    double tol;          /* true relative residual target */
    int maxits;
    int precision;       /* as in xt_system_solve */
    double inner_tol;
} xt_thermal_config;

typedef struct xt_thermal_s *xt_thermal;

int xt_thermal_create(xth_problem pr, const xt_thermal_config *cfg, xt_thermal *out);
int xt_thermal_destroy(xt_thermal t);
/* One slab; stats (may be NULL) receives 6 values: slab index, GMRES
 * iterations, restart cycles, refinement passes, ierr, true relative
 * residual. */
int xt_thermal_step(xt_thermal t, double *stats);
/* The slab's nodal temperatures, block layout (3 temporal blocks of nn). */
int xt_thermal_get(xt_thermal t, double *temp);

/* ------------------------------------------------ thermo-mechanical coupling */

/* Couples a thermal slab loop to the mechanical one, as the reference's
 * coupled run does every slab (src/main3d.f90:697-813): each xt_slab_step
 * then first advances the thermal loop one slab, then on the device takes
 * the end-of-slab temperatures to every Gauss point, updates the moduli
 * (material_update, src/thermoelastic.f90:1-46; the damage update uses them
 * too), reassembles K with them (mpiglbmtx_m, src/mpisubs.f90:69-139) and
 * forms the thermal stress load vv (calc_thermo_stress and elevec_m,
 * src/thermoelastic.f90:48-78, src/elesubs.f90:119-167), and adds fint(j) vv
 * to load block j (src/main3d.f90:813).  refactor_every = k recomputes the
 * ILUT factor from the reassembled K on the host every k slabs and after
 * every deletion (0: after deletions only; the reference refactors its MUMPS
 * preconditioner every slab).  The thermal loop must have been created on
 * the same problem and outlive the coupling; the slab must not use
 * cfg.overlap. */
typedef struct xt_coupling_config {
    double alpha;        /* thermal expansion coefficient */
    double Tref;         /* reference temperature */
    double ym0, nu0;     /* moduli at Tref */
    int refactor_every;
} xt_coupling_config;

int xt_slab_couple(xt_slab s, xt_thermal t, const xt_coupling_config *cc);

/* Per-kernel CUDA-event timing on the library stream: enable, then read
 * count and total milliseconds per kernel class (0 Kronecker FP64,
 * 1 Kronecker FP32, 2 ILU FP64, 3 ILU FP32, 4 damage, 5 Gram-Schmidt
 * projection of one Arnoldi step with an FP64-class basis, 6 with an FP32
 * basis, 7 Kronecker double-float on an FP32 vector). */
int xt_profile(int enable);
int xt_profile_read(int cls, long long *count, double *ms);
/* Algorithmic bytes summed over the timed launches of a class, for the
 * classes that record them (5, 6: (4i + 6) n values per Arnoldi step i,
 * two dot passes and two update passes over the i basis vectors). */
int xt_profile_bytes(int cls, double *bytes);
/* Kernel launches issued by the library since load. */
long long xt_launch_count(void);
/* CUDA events on the library stream: record slot 0..7, elapsed ms a -> b
 * (waits for b), and a synchronize of the device (every system's stream). */
int xt_mark(int slot);
double xt_elapsed_ms(int a, int b);
int xt_sync(void);

#ifdef __cplusplus
}
#endif
#endif
