// xt_device.h -- device-side data structures and kernel launchers of the
// GB300 space-time solve path (internal to the library).
//
// Layout in HBM.  A space-time vector of p spatial DOFs and q temporal
// blocks is stored node-major ("interleaved"): element (row r, block k) at
// r*q + k, so the q values a CSR column gathers are contiguous (48 B in
// FP64, 24 B in FP32 for q = 6).  The reference's block-major layout (block
// k at k*p + r, src/kronecker.f90:64) is converted at the C-ABI boundary.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "../../include/xtfem_gb300.h"

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace xt {

// ---------------------------------------------------------------- errors
// Status codes are the public ones of include/xtfem_gb300.h (XT_OK, ...).

void set_error(const std::string& msg);
const char* last_error();
// Running count of kernel launches issued by the library.
void note_launches(int n);

// A named NVTX range over this scope on a profiler's timeline (a slab step,
// a refined solve, a GMRES cycle, a round of the lockstep batch); without a
// profiler attached the calls do nothing.
struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};
// Diagnostics: when the environment variable XTFEM_TRACE is set, trace()
// prints the step and synchronizes the device to surface errors early.
void trace(const char* what);

#define XT_CUDA(call)                                                         \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) {                                              \
            ::xt::set_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
            return XT_ERR_CUDA;                                               \
        }                                                                     \
    } while (0)

#define XT_TRY(expr)                        \
    do {                                    \
        int s_ = (expr);                    \
        if (s_ != XT_OK) return s_;         \
    } while (0)

// Owning device buffer (cudaMalloc / cudaFree).
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    int alloc(size_t count) {
        if (count == n && p) return XT_OK;
        release();
        if (count == 0) return XT_OK;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            set_error(std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
            return XT_ERR_ALLOC;
        }
        n = count;
        return XT_OK;
    }
    int upload(const T* h, size_t count, cudaStream_t s) {
        XT_TRY(alloc(count));
        if (count) XT_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
        return XT_OK;
    }
};

// ------------------------------------------------------ sparse operators
// 0-based CSR on the device with FP64 values and an FP32 copy.
// Node-block form of a three-DOF-per-node pair (K, M): for every node row
// the neighbour nodes, K's 3 x 3 block (zeros where the CSR has no entry)
// and M's one scalar per block when M = m_ab I3 blockwise (a consistent
// mass matrix).  One column index and one contiguous gather of the
// neighbour's 3 x q slice of X serve nine K values and one M value.
struct DevNodeBlocks {
    bool ok = false;
    int nodes = 0, nblocks = 0;
    DBuf<int> ptr, col;    // nodes + 1 block pointers, neighbour node per block
    DBuf<float2> kdf;      // 9 per block, row-major, double-float
    DBuf<float2> mdf;      // 1 per block, double-float
    DBuf<int> from_csr;    // K's nnz entries: position of each in kdf
};


// Mesh data and maps of the device reassembly of K (dev_assembly.cu).
struct DevAssembly {
    bool ok = false;
    int nn = 0, ne = 0;
    DBuf<double> xyz;            // nn x 3
    DBuf<int> conn;              // ne x 8, 0-based nodes
    DBuf<int> cptr, cidx;        // per K entry: its element-matrix entries
    DBuf<unsigned char> bcdiag;  // per K entry: diagonal of a constrained DOF
    DBuf<double> ke;             // ne x 576 element matrices
    DBuf<double> ym, nu;         // ne x 8 Gauss-point moduli
    DBuf<int> gel;               // optional: element e's index in full-mesh moduli arrays
};

struct DevCsr {
    int n = 0, nnz = 0;
    DBuf<int> rowptr, col;
    DBuf<double> v64;
    DBuf<float> v32;
    DBuf<float2> vdf;  // double-float (hi, lo) copy, made on first use
    DBuf<__nv_bfloat16> v16;  // BF16 copy (round to nearest), made on first use
    // set on M when its pattern equals K's (same mesh): the Kronecker
    // kernels then read one column index and one X row per nonzero for both
    bool same_pattern = false;
    DevNodeBlocks nb;  // on K: node-block form of (K, M), when it exists
};

// Refreshes K.nb's K values from K's CSR values (after a reassembly on
// the device); no-op when K has no node-block form.
int node_blocks_refresh(DevCsr& K, cudaStream_t s);

// Builds K.nb from the 1-based host CSR pairs after both were uploaded;
// leaves K.nb.ok false when the pair has no exact node-block form (order
// not a multiple of 3, M not m_ab I3 blockwise, or M outside K's blocks).
int csr_build_node_blocks(DevCsr& K, int n, const int* ki, const int* kj, const double* kv,
                          const int* mi, const int* mj, const double* mv, cudaStream_t s);

// Marks M as sharing K's sparsity pattern when the 1-based host arrays are
// identical (both matrices of one mesh), after both were uploaded.
void csr_mark_shared_pattern(const DevCsr& K, DevCsr& M, const int* ki, const int* kj,
                             const int* mi, const int* mj);

// FP64 -> FP32 copy on the device.
int to_f32(const double* a, float* b, size_t n, cudaStream_t s);

// Upload a 1-based host CSR (ia, ja, a) as 0-based device CSR.
int upload_csr(DevCsr& d, int n, const int* ia, const int* ja, const double* a,
               cudaStream_t s);

// Y := alpha * (K X A^T + M X B^T) + beta * Y on interleaved p x q blocks.
// A, B are q x q column-major on the device (FP64).  T is the value/vector
// type (double or float); accumulation is in T.
template <class T>
int kron_spmm(const DevCsr& K, const DevCsr& M, int q, const double* dA,
              const double* dB, double alpha, double beta, const T* x, T* y,
              cudaStream_t s);

// Y := K X A^T + M X B^T with X in FP32 (exact inputs, e.g. preconditioned
// vectors) and Y in double-float (float2 (hi, lo) per entry): FP64-class
// accuracy at FP32 throughput.  Makes the double-float copies of the CSR
// values on first use.
int kron_spmm_df(DevCsr& K, DevCsr& M, int q, const double* dA, const double* dB, const float* x,
                 float2* y, cudaStream_t s, const int* skip = nullptr);

// The same operator with K and M stored in BF16, FP32 vectors and FP32
// accumulation (the BF16-stored experiment of precision mode 3).
int kron_spmm_bf16(DevCsr& K, DevCsr& M, int q, const double* dA, const double* dB,
                   double alpha, double beta, const float* x, float* y, cudaStream_t s);

// -------------------------------------------------- ILU triangular solves
// Level-scheduled form of a SPARSKIT MSR factor.  Rows are handled in groups
// of g consecutive rows (g = 3 for three DOFs per node, else 1); a group's
// level is one more than the deepest group it depends on outside itself.
struct DevTri {
    int ngroups = 0, nlevels = 0, g = 1;
    DBuf<int> level_ptr;   // nlevels+1, into the level-ordered group list
    DBuf<int> group_row0;  // first row of each group, level order
    DBuf<int> ext_ptr;     // per (group, row-in-group): g*ngroups+1
    DBuf<int> ext_col;     // external (outside the group) columns
    DBuf<double> ext_v64;
    DBuf<float> ext_v32;
    DBuf<double> int_v64;  // per group g*g internal coefficients
    DBuf<float> int_v32;
    DBuf<double> dinv64;   // per group g inverted diagonals (upper only)
    DBuf<float> dinv32;
    int max_level_groups = 0;
};

struct IluSched;  // host copy of both level schedules (dev_ilu.cu)
struct IluStage;  // staged-sweep data for one temporal width and precision

struct DevIlu {
    int n = 0;
    DevTri L, U;
    std::shared_ptr<IluSched> sched;
    // built on first use for a (q, precision) pair; key 2*q + (FP32 ? 1 : 0)
    mutable std::map<int, std::shared_ptr<IluStage>> stages;
    // lanes per row of the FP32 register sweep (its rows per warp: 10 node
    // rows at 1, 5 at 2, 2 at 4); 0 = XTFEM_ILU_SHARES or 2.  Set by the
    // batch tuner.
    mutable int shares = 0;
    // block-Jacobi factor: independent row blocks (1 = the whole factor),
    // their row bounds and one schedule per block
    int blocks = 1;
    std::vector<int> bounds;
    std::vector<std::shared_ptr<IluSched>> part_sched;
};

// Build the level schedule from the 1-based MSR arrays and upload it.
// blocks > 1: a block-Jacobi factor of that many row blocks (the bounds of
// ilu_block_bounds); when it has no entry between blocks, each block also
// gets a schedule of its own for the FP32 register sweep.
int build_ilu(DevIlu& d, int n, const double* alu, const int* jlu, const int* ju,
              int group, cudaStream_t s, int blocks = 1);
// Row bounds of the block-Jacobi ILU's blocks (host_ilut.cpp).
std::vector<int> ilu_block_bounds(int n, int g, int blocks);

// z := (Ainv (x) (LU)^-1) v on interleaved blocks: the q x q mixing with the
// inverse temporal matrix is applied to v first (it commutes with the
// spatial solve), then the forward and backward sweeps.  dAinv is q x q
// column-major FP64 on the device.  work has n*q entries.
// skip (optional, device): when skip[0] is non-zero the FP32 register
// sweep does nothing (a step past the end of a device-driven GMRES cycle).
template <class T>
int ilu_apply(const DevIlu& F, int q, const double* dAinv, const T* v, T* z, T* work,
              cudaStream_t s, const int* skip = nullptr);

// Reads and clears the device-side error word of the staged sweeps (a
// bounded wait that gave up); XT_OK when clear.
int ilu_check(cudaStream_t s);

// ----------------------------------------------------- Krylov vector ops
// Reduction scratch sized for the largest restart length in use.
struct Reduce {
    DBuf<double> partial;  // nblocks * kmax
    DBuf<double> out;      // kmax
    int nblocks = 0, kmax = 0;
};
int reduce_init(Reduce& r, int kmax);

// ----------------------------------- device-driven flexible GMRES steps
// Layout of the device state of one cycle (doubles): the (im+1) x im
// Hessenberg matrix (column-major), the rotations, rs, the two projections
// of the new vector, its squared norm, eps1, 1/t, the residual estimate and
// the solution y of the small triangular system.
// the longest restart the device-driven flexible GMRES takes (its rotation
// kernel stages a Hessenberg column in shared memory); longer ones run
// host-driven
constexpr int kFlexdMaxIm = 1024;
struct FlexLayout {
    size_t hh, cs, sn, rs, h1, h2, nrm, eps1, tinv, ro, y, total;
    __host__ __device__ explicit FlexLayout(int im)
    {
        const size_t m = (size_t)im;
        hh = 0;
        cs = (m + 1) * m;
        sn = cs + m;
        rs = sn + m;
        h1 = rs + m + 1;
        h2 = h1 + m;
        nrm = h2 + m;
        eps1 = nrm + 1;
        tinv = eps1 + 1;
        ro = tinv + 1;
        y = ro + 1;
        total = y + m;
    }
};
// ctl = {j, status, its, maxits} on the device (see dev_krylov.cu)
int flexd_hi(const int* ctl, const float2* V, size_t nl, float* d, size_t n, cudaStream_t s);
int flexd_zcopy(const int* ctl, const float* z, float* Z, size_t n, cudaStream_t s);
int flexd_orth(const int* ctl, const float2* V, size_t nl, float2* w, double* st, int im,
               Reduce& r, cudaStream_t s, bool two_pass = true);
int flexd_givens(int* ctl, double* st, int im, cudaStream_t s);
int flexd_scale_copy(const int* ctl, const double* st, int im, const float2* w, float2* V,
                     size_t nl, size_t n, cudaStream_t s);
int flexd_solve(const int* ctl, double* st, int im, cudaStream_t s);

// Arguments of one register sweep (one triangle of one factor or row block;
// dev_ilu.cu): the slots, the right-hand sides in lane-slot order ([q]
// arrays of rstride), the output (forward: the backward sweep's right-hand
// sides, ostride apart; backward: z, interleaved), levels, warps, slot
// bytes, the window's zero slot, the L2 prefetch distance in levels (0 off)
// and an optional skip flag (nothing to do when skip[0] != 0).
struct RegArgs {
    const unsigned char* slots;
    const float* rhs;
    float* out;
    long long rstride, ostride;
    int nl, ncw, slot_bytes, zero_off;
    int pf;
    const int* skip;
};
// A system's default FP32 ILU apply as a batch entry: the pre-pass's lane
// map and right-hand-side arrays and the two sweeps' arguments (output z,
// skip flag skip).  ok is false when the apply is another format (a
// block-Jacobi factor, a fall-back sweep) or has no batched launch.
struct IluRegEntry {
    bool ok = false;
    const int* src = nullptr;  // row of each forward lane slot (-1: none)
    long long lanes = 0;
    float* rrhs = nullptr;     // forward right-hand sides, [q][lanes]
    int H = 0, smax = 0, w16 = 0;
    RegArgs L{}, U{};
    size_t smemL = 0, smemU = 0;  // window bytes
};
int ilu_reg_entry(const DevIlu& F, int q, float* z, const int* skip, cudaStream_t s,
                  IluRegEntry& e);
// One launch of a batch's sweeps: entries with the same shares, steps,
// offset width, warps and direction (args: a device table of count entries).
struct RegGroup {
    int H = 0, smax = 0, w16 = 0, ncw = 0, upper = 0, count = 0;
    size_t smem = 0;
    DBuf<unsigned char> args;
};
int reg_group_prepare(const RegGroup& g);  // outside a capture: kernel attributes
int reg_group_launch(const RegGroup& g, int q, cudaStream_t s);

// ------------------------------------- batched device-driven Arnoldi steps
// One system of a batch in a table that drives kernels serving every system
// of the batch in one launch (blockIdx.y = the system's entry): the buffers
// the system's FlexRun step uses and its node-block operator.  The kernels
// do per system what the per-system step kernels do, with the same row
// partitions, so the results are the same bits.
struct FlexStepItem {
    int* ctl;          // {j, status, its, maxits}
    double* st;        // FlexLayout(im) state of the cycle
    double* partial;   // reduction scratch
    float2* V;         // double-float basis, column stride nl
    float* zfix;       // ILU output
    float* Z;          // preconditioned vectors, column stride n
    float2* wfix;      // operator output, orthogonalised in place
    long long n, nl;
    int im;
    int rowblocks;      // row blocks of the norm pass
    int dotrows;        // row blocks per basis chunk of the dot pass (at most)
    int dotblocks;      // thread blocks of the system's dot pass
    const int* src;     // ILU pre-pass (IluRegEntry): lane map, lanes, right-hand
    long long lanes;    // sides, A^-1 (q x q)
    float* rrhs;
    const double* Ainv;
    int nodes;          // node-block operator: K's 3 x 3 blocks, M's scalars
    const int* bptr;
    const int* bcol;
    const float2* kv;
    const float2* mv;
    const double* A;    // temporal matrices (q x q)
    const double* B;
};
// The largest sizes over a table's entries (launch grids are sized by them).
struct FlexStepDims {
    long long nmax = 0;
    int nodes_max = 0, rb_max = 0, dot_blocks_max = 0, im = 0;
};
// Row blocks of a system's double-float norm and dot passes; the most
// blocks a dot pass over im basis vectors has items for.
int df_row_blocks_for(long long nl, const Reduce& r);
int df_dot_rows_for(long long nl, const Reduce& r);
int df_dot_blocks_max(int im, int dotrows);
// The thread blocks of one wave of a dot pass (a batch deals them to its
// systems by size).
int df_dot_wave();
// The ILU pre-pass of every entry from the hi part of its basis column j;
// the ILU output into Z column j.
int flexb_rhs(const FlexStepItem* t, int count, int q, long long lanes_max, cudaStream_t s);
int flexb_zcopy(const FlexStepItem* t, int count, const FlexStepDims& d, cudaStream_t s);
// Gram-Schmidt of every system's operator output: the first pass of the
// systems in `two` (two passes), h1 = 0 for those in `one`, then the
// projection and norm pass of all.
int flexb_orth(const FlexStepItem* all, int nall, const FlexStepItem* two, int ntwo,
               const FlexStepItem* one, int none, const FlexStepDims& d, cudaStream_t s);
// The rotations and convergence test, then the scaled new basis column.
int flexb_givens_scale(const FlexStepItem* t, int count, const FlexStepDims& d, cudaStream_t s);
// out[4 e .. 4 e + 3] = the control word of entry e.
int flexb_ctl_gather(const FlexStepItem* t, int count, int* out, cudaStream_t s);
// The node-block double-float operator of every system: wfix = op(zfix).
bool kron_nb_batchable(const DevCsr& K, int q);
int kron_nb_batch(const FlexStepItem* t, int count, int q, const FlexStepDims& d, cudaStream_t s);


// h[j] = <V_j, w> for j < k (V column-major, column stride ld), FP64
// accumulation; result in r.out (device).
template <class TV>
int multi_dot(const TV* V, size_t ld, int k, const TV* w, size_t n, Reduce& r,
              cudaStream_t s);
// w := w - V h (h on device, FP64), then h2 = V^T w (fused second pass of
// classical Gram-Schmidt with re-orthogonalisation); result in r.out.
template <class TV>
int update_and_dot(const TV* V, size_t ld, int k, const double* h, TV* w, size_t n,
                   Reduce& r, cudaStream_t s);
// w := w - V h, then ||w||^2 into r.out[0].
template <class TV>
int update_and_norm(const TV* V, size_t ld, int k, const double* h, TV* w, size_t n,
                    Reduce& r, cudaStream_t s);
// y := sum_j c[j] V_j (c on device, FP64 accumulation), y of type TY.
template <class TV, class TY>
int lincomb(const TV* V, size_t ld, int k, const double* c, TY* y, size_t n,
            cudaStream_t s);
// y := a*x (+ y when accumulate); x, y may differ in type.
template <class TX, class TY>
int axpby(size_t n, double a, const TX* x, double b, TY* y, cudaStream_t s);
// Double-float vectors (float2 (hi, lo) per entry, about 48 significant
// bits, FP32 arithmetic only): the CGS2 passes of multi_dot /
// update_and_dot / update_and_norm, conversions, and y *= a.  n, ld even.
int df_multi_dot(const float2* V, size_t ld, int k, const float2* w, size_t n, Reduce& r,
                 cudaStream_t s);
int df_update_and_dot(const float2* V, size_t ld, int k, const double* h, float2* w, size_t n,
                      Reduce& r, cudaStream_t s);
// update_and_norm: the squared norm into out (default r.out[0]); h may be
// r.out itself (the update has read it before the norm is written)
int df_update_and_norm(const float2* V, size_t ld, int k, const double* h, float2* w, size_t n,
                       Reduce& r, cudaStream_t s, double* out = nullptr);
int df_from_f64(const double* x, float2* y, size_t n, cudaStream_t s);
int df_hi(const float2* x, float* y, size_t n, cudaStream_t s);
int df_to_f64(const float2* x, double* y, size_t n, cudaStream_t s);
int df_scale(float2* y, double a, size_t n, cudaStream_t s);
// df_scale, and the hi part of the scaled y into hi
int df_scale_hi(float2* y, double a, float* hi, size_t n, cudaStream_t s);
// ||x||^2 (FP64) into r.out[0].
template <class T>
int norm2(const T* x, size_t n, Reduce& r, cudaStream_t s);
// x[i] = 0 where mask[i / q] is set (BC rows of an interleaved vector, mask
// over the spatial DOFs).
template <class T>
int mask_rows(T* x, const int* mask, int p, int q, cudaStream_t s);

// out[r*q + j] = c[j] * rext[r] (c: q host values) -- the load blocks
// fextc(j) * rext of src/main3d.f90:807-814 in the interleaved layout.
int fill_load(const double* rext, const double* c, double* out, int p, int q, cudaStream_t s);
// max_i x[i] into r.out[0].
int max_value(const double* x, size_t n, Reduce& r, cudaStream_t s);

// Interleaved <-> block-major conversion (reference layout at the boundary).
template <class TI, class TO>
int to_interleaved(const TI* blk, TO* itl, int p, int q, cudaStream_t s);
template <class TI, class TO>
int to_blocks(const TI* itl, TO* blk, int p, int q, cudaStream_t s);

// Per-Gauss-point strain and stress of the reference's output step
// (dev_post.cu): sol_blocks is the slab solution in block layout (6 temporal
// blocks of 3 nn), Nt6 the six temporal shape values at the output time
// (host); strain and stress are ngp x 6, zero at failed points.
int post_strain_stress(int ngp, int nn, const int* nodes, const double* Nx, const double* Ny,
                       const double* Nz, const double* ym, const double* nu, const int* gpsta,
                       const double* sol_blocks, const double* Nt6, double* strain, double* stress,
                       cudaStream_t s);

// ----------------------------------------------------------------- damage
struct DamageArgs {
    int ngp, nn, ndofn, nnse, nnte, ncmp, nip;
    const int* nodes;            // ngp*nnse, 1-based node ids
    const double *Nx, *Ny, *Nz;  // ngp*nnse
    const double* Nt;            // nip*2*nnte (FP64)
    const float* Nt32;           // nip*2*nnte (FP32 copy for the yield screen)
    const double* sol;           // block-major space-time solution, 2*nnte*nn*ndofn
    const double *ym, *nu;       // ngp
    double *eps_old, *eps_pl, *sig_eff, *sig_back;  // ngp*ncmp
    double *p, *D, *ws, *del_po, *sig_d;            // ngp
    const int* gpsta;            // optional: zero D, ws where gpsta == 0
    unsigned long long* counters;  // optional [3]: plastic, screened, exact steps
    float* ntmax;                // device scratch, 6 floats (per-slab |Nt_k| bounds)
};
int damage_update(const DamageArgs& a, cudaStream_t s);

// Static device scratch of the allocation-free damage entry point: FP32
// shape table (6 * kDamageStaticMaxNip floats), 6 shape-value bounds and 3
// step counters.  The address is looked up once per device, under a lock;
// `device` must be the current device.  damage_static_forget() drops the
// looked-up addresses (library teardown).
constexpr int kDamageStaticMaxNip = 65536;
int damage_static_scratch(int device, float** nt32, float** ntmax, unsigned long long** counters);
void damage_static_forget();

// Temporal shape table on the device (FP64 and FP32 copies).
int nt_table_device(int nip, double t0, double t1, double t2, double w, double* Nt64,
                    float* Nt32, cudaStream_t s);

// chkelesta: flags, ascending failed-element list, count.  D, elesta,
// gpsta, nefail, nef on device.
int chkelesta_device(int ne, int ngpe, double Dc, const double* D, int* elesta, int* gpsta,
                     int* nefail, int* nef, cudaStream_t s);

// any(D >= Dc) over ngp points, result (0/1) into *flag (device).
int any_ge_device(const double* D, int ngp, double Dc, int* flag, cudaStream_t s);

}  // namespace xt
