// solver.h -- device-resident space-time system and its GMRES solvers.
#pragma once

#include <memory>
#include <vector>

#include "xt_device.h"

namespace xt {

// Process-wide device context: the device, one stream, scratch.
struct Context {
    int device = -1;
    cudaStream_t stream = nullptr;
    bool ready = false;
};
Context& ctx();
int ensure_init(int device = -1);

// The operator (A (x) K + B (x) M) with its ILUT preconditioner, resident
// on the device.  K, M and the factor are uploaded once; the temporal
// matrices A, B may change every slab.
struct System {
    // Every operation on the system runs on its own stream (highest
    // priority), so independent systems driven from different host threads
    // run concurrently on the GPU.
    cudaStream_t stream = nullptr;
    System() = default;
    System(const System&) = delete;
    System& operator=(const System&) = delete;
    ~System()
    {
        if (stream) cudaStreamDestroy(stream);
    }
    int p = 0, q = 0;
    DevCsr K, M;
    std::shared_ptr<DevIlu> ilu;  // may be shared with a factor cache
    DBuf<double> A, B, Ainv, Cj, Mj;  // q x q each, column-major
    std::vector<double> hA, hB, hAinv;
    DBuf<int> bcmask;                 // p entries (0/1), optional
    // GMRES workspace
    int im_cap = 0;
    bool op16 = false;  // FP32 inner operator reads BF16-stored K and M (mode 3)
    // Gram-Schmidt passes per step of the flexible GMRES (1 or 2), and the
    // switch to two for the rest of a solve after a loss of orthogonality
    int gs_passes = 2;
    bool gs_latched = false;
    long long nest_its = 0;  // inner iterations of the last mode-3 solve
    // device-driven flexible GMRES: step control, cycle state, the fixed
    // preconditioned and operator vectors of a step, host copy of the control
    DBuf<int> fctl;
    DBuf<double> fst;
    DBuf<float> zfix;
    DBuf<float2> wfix;
    DBuf<double> V64, z64, w64, u64;
    DBuf<float> V32, z32, w32, u32, d32, r32;
    DBuf<float> Z32;  // flexible GMRES: preconditioned basis, im columns
    DBuf<double> x64, r64, b64, t64;
    DBuf<double> hsave;
    Reduce red;
    DevAssembly asmb;  // device reassembly of K, when a mesh was set
};

// Creates the system's stream if it has none yet.
int system_stream(System& S);

// Status-returning building blocks
int system_create(System& S, int p, int q, const int* ki, const int* kj, const double* kv,
                  const int* mi, const int* mj, const double* mv);
int system_set_ilu(System& S, const double* alu, const int* jlu, const int* ju, int group,
                   int blocks = 1);
int system_set_temporal(System& S, const double* A, const double* B);
// Device reassembly of K from per-Gauss-point moduli (dev_assembly.cu):
// the mesh and constrained DOFs once, then any number of reassemblies.
// gel (may be null): the full-mesh index of each listed element, for
// moduli arrays that cover every element of the mesh.
int system_set_mesh(System& S, int nn, int ne, const double* xyz, const int* conn, const int* bc,
                    const int* gel = nullptr);
int system_assemble_k(System& S, const double* ym, const double* nu);
// The same from moduli already on the device (by_gel: indexed through gel).
int system_assemble_k_device(System& S, const double* ym, const double* nu, bool by_gel);
// Thermal coupling of every element (dev_assembly.cu): Gauss-point moduli
// and element thermal-stress vectors (ne x 24) from the end-of-slab nodal
// temperatures (temp: interleaved, nn x 3).
int thermal_couple_device(int ne, const int* conn0, const double* xyz, const double* temp,
                          double alpha, double Tref, double ym0, double nu0, double* ym, double* nu,
                          double* ve, cudaStream_t s);
// y[k] = sum over t in [ptr[k], ptr[k+1]) of x[idx[t]]
int gather_list(int n, const int* ptr, const int* idx, const double* x, double* y, cudaStream_t s);

// q x q inverse by LU with partial pivoting (host); returns XT_ERR_SINGULAR.
int invert_small(int n, const double* A, double* Ainv);

struct GmresStats {
    int its = 0;         // Arnoldi steps in total
    int cycles = 0;      // restart cycles
    int outer = 0;       // refinement passes
    int ierr = 0;        // 0 converged, 1 maxits, -1 zero residual
    double relres = 0;   // final true relative residual ||b - A x|| / ||b||
    double est = 0;      // last Givens estimate relative to the first residual
};

// kronpgmres semantics (src/kronecker.f90:181-365) on device vectors in the
// interleaved layout, all in FP64: b and x are device arrays of p*q; x is
// the initial guess and receives the solution.  b is not modified.
int gmres_fp64(System& S, const double* b, double* x, int im, double eps, int maxits,
               GmresStats& st, std::vector<double>* hist);

// Solve to a true relative residual <= tol: FP64 residuals and solution,
// inner GMRES in precision `inner`, restarted with the true residual until
// converged or maxits Arnoldi steps in total:
//   0 = FP64 operator, factor and basis;
//   1 = FP32 operator, factor and basis (FP64-class dots, host Hessenberg);
//   2 = flexible GMRES: FP64 operator and basis, FP32 factor, the
//       preconditioned vectors kept (FP32) for the solution update.
int solve_refined(System& S, const double* b, double* x, int im, double tol, int maxits,
                  int inner, double inner_tol, GmresStats& st);

// The refined solve of mode 2 (flexible GMRES, FP64 refinement) with the
// Arnoldi bookkeeping on the device, as a resumable run:
//   start()   sets the solve up (host work and host reads); afterwards the
//             run is either done or in a cycle whose steps can be issued;
//   issue()   enqueues nstep Arnoldi steps on the system's stream and
//             nothing else (no host synchronisation, no allocation): the
//             steps can be captured into a CUDA graph and replayed, since
//             every kernel reads the step index from the control word and
//             does nothing once the cycle has ended;
//   advance() takes the control word read after a chunk of steps and does
//             the host work of a cycle's end, of the next cycle's start and
//             of the refinement steps between inner solves.
// solve_refined drives one run chunk by chunk; the batch drives many in
// lockstep, one graph per round.  Results equal the host-driven loop's bit
// for bit.
struct FlexRun {
    GmresStats st;       // the refined solve's statistics (final once done)
    bool done = false;   // the solve has ended
    int cycle = 0;       // cycles started so far
    int j = 0;           // steps of the current cycle at the last control read
    bool two_pass = true;

    int start(System& S, const double* b, double* x, int im, double tol, int maxits);
    int issue(int nstep, std::vector<int>* prof_tokens);
    int advance(const int* ctl);

  private:
    System* S_ = nullptr;
    const double* b_ = nullptr;
    double* x_ = nullptr;
    int im_ = 0, maxits_ = 0, its_in_ = 0, left_ = 0;
    double tol_ = 0.0, bn_ = 0.0, rn_ = 0.0, predicted_ = -1.0;
    double ro_ = 0.0, ro0_ = 0.0, eps1_ = 0.0, eps_in_ = 0.0;
    GmresStats in_;
    std::vector<double> rs_;
    int hctl_[4] = {0, 0, 0, 0};
    int outer_step();
    int inner_begin();
    int cycle_begin();
    int inner_end(int ierr_in);
};
// y := alpha (A (x) K + B (x) M) x + beta y with the system's current A, B
// (FP64, interleaved).
int system_apply(System& S, double alpha, double beta, const double* x, double* y);
// Same with explicit temporal matrices (device, q x q).
int system_apply_with(System& S, const double* dA, const double* dB, double alpha, double beta,
                      const double* x, double* y);

}  // namespace xt
