// solver.cpp -- the space-time system on the device and its restarted GMRES.
//
// gmres_core follows the control flow of the reference's kronpgmres
// (src/kronecker.f90:181-365): right preconditioning with
// (A^-1 (x) (LU)^-1), Arnoldi with Givens rotations, the correction of a
// cycle applied before a restart, the restart residual rebuilt from the
// Givens data, convergence when |rs(i+1)| <= eps * ||r0||, maxits tested at
// the end of a cycle, ierr in {0, 1, -1}.  The vectors live on the device in
// the interleaved layout; the (im+1) x im Hessenberg matrix, the rotations
// and the small triangular solve stay on the host in FP64, fed by one
// device-to-host copy per Arnoldi step.  The projection is CGS2 (see
// dev_krylov.cu) instead of the reference's MGS.
#include "solver.h"

#include "prof.h"

#include <cmath>
#include <cstdlib>
#include <algorithm>
#include <string>
#include <cstring>
#include <mutex>

namespace xt {

namespace {
thread_local std::string g_err;
}

void set_error(const std::string& msg) { g_err = msg; }
const char* last_error() { return g_err.c_str(); }

Context& ctx()
{
    static Context c;
    return c;
}

int ensure_init(int device)
{
    Context& c = ctx();
    if (c.ready && (device < 0 || device == c.device)) return XT_OK;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        set_error(std::string("no CUDA device available: ") + cudaGetErrorString(e));
        return XT_ERR_CUDA;
    }
    if (device < 0) device = 0;
    if (device >= count) {
        set_error("device index out of range");
        return XT_ERR_ARG;
    }
    XT_CUDA(cudaSetDevice(device));
    if (c.stream) cudaStreamDestroy(c.stream);
    // the solve stream runs at the highest priority, so work overlapped on
    // lower-priority streams (the slab loop's damage update) yields to it
    int least = 0, greatest = 0;
    XT_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    XT_CUDA(cudaStreamCreateWithPriority(&c.stream, cudaStreamNonBlocking, greatest));
    c.device = device;
    c.ready = true;
    return XT_OK;
}

int invert_small(int n, const double* A, double* Ainv)
{
    std::vector<double> lu(A, A + (size_t)n * n);
    std::vector<int> piv(n);
    auto LU = [&](int i, int j) -> double& { return lu[(size_t)j * n + i]; };
    for (int c = 0; c < n; ++c) {
        int pr = c;
        double best = std::fabs(LU(c, c));
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(LU(r, c)) > best) { best = std::fabs(LU(r, c)); pr = r; }
        piv[c] = pr;
        if (best == 0.0) {
            set_error("temporal matrix is singular");
            return XT_ERR_SINGULAR;
        }
        if (pr != c)
            for (int j = 0; j < n; ++j) std::swap(LU(c, j), LU(pr, j));
        for (int r = c + 1; r < n; ++r) {
            LU(r, c) /= LU(c, c);
            for (int j = c + 1; j < n; ++j) LU(r, j) -= LU(r, c) * LU(c, j);
        }
    }
    for (int col = 0; col < n; ++col) {
        double* e = Ainv + (size_t)col * n;
        for (int r = 0; r < n; ++r) e[r] = (r == col) ? 1.0 : 0.0;
        for (int c = 0; c < n; ++c)
            if (piv[c] != c) std::swap(e[c], e[piv[c]]);
        for (int r = 1; r < n; ++r)
            for (int c = 0; c < r; ++c) e[r] -= LU(r, c) * e[c];
        for (int r = n - 1; r >= 0; --r) {
            for (int c = r + 1; c < n; ++c) e[r] -= LU(r, c) * e[c];
            e[r] /= LU(r, r);
        }
    }
    return XT_OK;
}

int system_stream(System& S)
{
    XT_TRY(ensure_init());
    if (S.stream) return XT_OK;
    int least = 0, greatest = 0;
    XT_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    XT_CUDA(cudaStreamCreateWithPriority(&S.stream, cudaStreamNonBlocking, greatest));
    return XT_OK;
}

// A caller's 1-based CSR, checked on the host before anything touches the
// device: first row pointer 1, row pointers non-decreasing, column indices
// in 1..n.  A corrupt matrix is XT_ERR_ARG with a message, never a fault.
static int check_csr(const char* what, int n, const int* ia, const int* ja)
{
    if (!ia || !ja) {
        set_error(std::string("system_create: null ") + what + " array");
        return XT_ERR_ARG;
    }
    if (ia[0] != 1) {
        set_error(std::string("system_create: ") + what + " row pointers must start at 1");
        return XT_ERR_ARG;
    }
    for (int r = 0; r < n; ++r)
        if (ia[r + 1] < ia[r]) {
            set_error(std::string("system_create: ") + what + " row pointers decrease at row " +
                      std::to_string(r + 1));
            return XT_ERR_ARG;
        }
    const int nnz = ia[n] - 1;
    for (int k = 0; k < nnz; ++k)
        if (ja[k] < 1 || ja[k] > n) {
            set_error(std::string("system_create: ") + what + " column index out of range at entry " +
                      std::to_string(k + 1));
            return XT_ERR_ARG;
        }
    return XT_OK;
}

int system_create(System& S, int p, int q, const int* ki, const int* kj, const double* kv,
                  const int* mi, const int* mj, const double* mv)
{
    if (p <= 0 || q < 1 || q > 8) {
        set_error("system_create: need p > 0 and 1 <= q <= 8");
        return XT_ERR_ARG;
    }
    XT_TRY(check_csr("K", p, ki, kj));
    XT_TRY(check_csr("M", p, mi, mj));
    XT_TRY(ensure_init());
    XT_TRY(system_stream(S));
    cudaStream_t s = S.stream;
    S.p = p;
    S.q = q;
    XT_TRY(upload_csr(S.K, p, ki, kj, kv, s));
    XT_TRY(upload_csr(S.M, p, mi, mj, mv, s));
    csr_mark_shared_pattern(S.K, S.M, ki, kj, mi, mj);
    XT_TRY(csr_build_node_blocks(S.K, p, ki, kj, kv, mi, mj, mv, s));
    XT_TRY(S.A.alloc(64));
    XT_TRY(S.B.alloc(64));
    XT_TRY(S.Ainv.alloc(64));
    XT_TRY(S.Cj.alloc(64));
    XT_TRY(S.Mj.alloc(64));
    XT_CUDA(cudaStreamSynchronize(s));
    return XT_OK;
}

int system_set_ilu(System& S, const double* alu, const int* jlu, const int* ju, int group,
                   int blocks)
{
    // a factorisation that broke down (a pivot at or near zero) leaves
    // infinities or NaNs in the factor; every apply would then return them
    const long long len = (long long)jlu[S.p] - 1;  // MSR, 1-based pointers
    for (long long k = 0; k < len; ++k)
        if (k != S.p && !std::isfinite(alu[k])) {
            set_error("set_ilu: the factor has a non-finite entry (the factorisation broke down)");
            return XT_ERR_NONFINITE;
        }
    auto f = std::make_shared<DevIlu>();
    XT_TRY(system_stream(S));
    XT_TRY(build_ilu(*f, S.p, alu, jlu, ju, group, S.stream, blocks));
    S.ilu = f;
    return XT_OK;
}

int system_set_temporal(System& S, const double* A, const double* B)
{
    const int q = S.q;
    S.hA.assign(A, A + q * q);
    S.hB.assign(B, B + q * q);
    S.hAinv.assign(q * q, 0.0);
    XT_TRY(invert_small(q, A, S.hAinv.data()));
    XT_TRY(system_stream(S));
    cudaStream_t s = S.stream;
    XT_CUDA(cudaMemcpyAsync(S.A.p, A, sizeof(double) * q * q, cudaMemcpyHostToDevice, s));
    XT_CUDA(cudaMemcpyAsync(S.B.p, B, sizeof(double) * q * q, cudaMemcpyHostToDevice, s));
    XT_CUDA(cudaMemcpyAsync(S.Ainv.p, S.hAinv.data(), sizeof(double) * q * q,
                            cudaMemcpyHostToDevice, s));
    XT_CUDA(cudaStreamSynchronize(s));
    return XT_OK;
}

int system_apply_with(System& S, const double* dA, const double* dB, double alpha, double beta,
                      const double* x, double* y)
{
    const int tok = prof_begin(PROF_KRON64, S.stream);
    const int st = kron_spmm<double>(S.K, S.M, S.q, dA, dB, alpha, beta, x, y, S.stream);
    prof_end(tok, S.stream);
    return st;
}

int system_apply(System& S, double alpha, double beta, const double* x, double* y)
{
    return system_apply_with(S, S.A.p, S.B.p, alpha, beta, x, y);
}

namespace {

int ensure_workspace(System& S, int im, bool fp32, bool flex = false)
{
    const size_t n = (size_t)S.p * S.q;
    if (im > S.im_cap || S.red.kmax < im + 1) {
        XT_TRY(reduce_init(S.red, im + 1));
        XT_TRY(S.hsave.alloc((size_t)2 * (im + 1) + 2));
        S.im_cap = im;
        S.V64.release();
        S.V32.release();
    }
    if (!fp32) {
        // columns of an even length: the double-float basis is read two
        // entries at a time (an odd n gets one zero pad entry per column)
        const size_t nl = n + (n & 1);
        if (S.V64.n < nl * (im + 1)) XT_TRY(S.V64.alloc(nl * (size_t)(im + 1)));
        XT_TRY(S.z64.alloc(n));
        XT_TRY(S.w64.alloc(n));
        XT_TRY(S.u64.alloc(n));
    } else {
        if (S.V32.n < n * (im + 1)) XT_TRY(S.V32.alloc(n * (size_t)(im + 1)));
        XT_TRY(S.z32.alloc(n));
        XT_TRY(S.w32.alloc(n));
        XT_TRY(S.u32.alloc(n));
        XT_TRY(S.d32.alloc(n));
        XT_TRY(S.r32.alloc(n));
    }
    if (flex) {
        if (S.Z32.n < n * (size_t)im) XT_TRY(S.Z32.alloc(n * (size_t)im));
        XT_TRY(S.d32.alloc(n));
        XT_TRY(S.w32.alloc(n));
    }
    XT_TRY(S.x64.alloc(n));
    XT_TRY(S.r64.alloc(n));
    XT_TRY(S.t64.alloc(n));
    return XT_OK;
}

template <class T>
struct Ws;
template <>
struct Ws<double> {
    static double* V(System& S) { return S.V64.p; }
    static double* z(System& S) { return S.z64.p; }
    static double* w(System& S) { return S.w64.p; }
    static double* u(System& S) { return S.u64.p; }
};
template <>
struct Ws<float> {
    static float* V(System& S) { return S.V32.p; }
    static float* z(System& S) { return S.z32.p; }
    static float* w(System& S) { return S.w32.p; }
    static float* u(System& S) { return S.u32.p; }
};

// The FP32 inner operator reads K and M as FP32, or as BF16 when S.op16
// (precision mode 3); both accumulate in FP32.
template <class T>
int kron_inner(System& S, double alpha, double beta, const T* x, T* y)
{
    if constexpr (sizeof(T) == 4) {
        if (S.op16)
            return kron_spmm_bf16(S.K, S.M, S.q, S.A.p, S.B.p, alpha, beta, x, y, S.stream);
    }
    return kron_spmm<T>(S.K, S.M, S.q, S.A.p, S.B.p, alpha, beta, x, y, S.stream);
}

template <class T>
int apply_op(System& S, const T* x, T* y)
{
    const int tok = prof_begin(sizeof(T) == 8 ? PROF_KRON64 : PROF_KRON32, S.stream);
    const int st = kron_inner<T>(S, 1.0, 0.0, x, y);
    prof_end(tok, S.stream);
    return st;
}

template <class T>
int apply_op_ab(System& S, double alpha, double beta, const T* x, T* y)
{
    const int tok = prof_begin(sizeof(T) == 8 ? PROF_KRON64 : PROF_KRON32, S.stream);
    const int st = kron_inner<T>(S, alpha, beta, x, y);
    prof_end(tok, S.stream);
    return st;
}

template <class T>
int apply_prec(System& S, const T* v, T* z)
{
    const int tok = prof_begin(sizeof(T) == 8 ? PROF_ILU64 : PROF_ILU32, S.stream);
    const int st = ilu_apply<T>(*S.ilu, S.q, S.Ainv.p, v, z, Ws<T>::w(S), S.stream);
    prof_end(tok, S.stream);
    return st;
}

int fetch(cudaStream_t s, double* h, const double* d, size_t count)
{
    XT_CUDA(cudaMemcpyAsync(h, d, count * sizeof(double), cudaMemcpyDeviceToHost, s));
    XT_CUDA(cudaStreamSynchronize(s));
    return XT_OK;
}

// GMRES in the reference's control flow on vectors of type T; rhs and sol
// are device vectors of type T (sol in/out).  rhs is preserved.
template <class T>
int gmres_core(System& S, const T* rhs, T* sol, int im, double eps, int maxits, GmresStats& st,
               std::vector<double>* hist)
{
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    T* V = Ws<T>::V(S);
    T* z = Ws<T>::z(S);
    auto col = [&](int j) { return V + (size_t)j * n; };
    std::vector<double> hh((size_t)(im + 1) * im, 0.0), c(im, 0.0), sn(im, 0.0), rs(im + 1, 0.0);
    std::vector<double> hbuf(2 * (im + 1) + 2);
    auto HH = [&](int r, int k) -> double& { return hh[(size_t)k * (im + 1) + r]; };
    const double epsmac = 1.0e-16;
    int its = 0, i = 0, ierr = 0;
    double ro = 0.0, eps1 = 0.0, t;

    XT_TRY(norm2<T>(rhs, n, S.red, s));
    XT_TRY(fetch(s, hbuf.data(), S.red.out.p, 1));
    const double ro0 = std::sqrt(hbuf[0]);
    // v1 = rhs - A sol
    XT_CUDA(cudaMemcpyAsync(col(0), rhs, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
    XT_TRY((kron_spmm<T>(S.K, S.M, S.q, S.A.p, S.B.p, -1.0, 1.0, sol, col(0), s)));
    for (;;) {  // label 20
        XT_TRY(norm2<T>(col(0), n, S.red, s));
        XT_TRY(fetch(s, hbuf.data(), S.red.out.p, 1));
        ro = std::sqrt(hbuf[0]);
        if (!std::isfinite(ro)) {
            set_error("gmres: non-finite residual");
            return XT_ERR_NONFINITE;
        }
        if (ro == 0.0) { ierr = -1; break; }
        XT_TRY((axpby<T, T>(n, 1.0 / ro, col(0), 0.0, col(0), s)));
        if (its == 0) eps1 = eps * ro;
        rs[0] = ro;
        i = 0;
        ++st.cycles;
        for (;;) {  // label 4
            ++i;
            ++its;
            const int i1 = i + 1;
            XT_TRY(apply_prec<T>(S, col(i - 1), z));
            XT_TRY(apply_op<T>(S, z, col(i1 - 1)));
            // CGS2 projection against the i previous vectors
            const int otok = prof_begin(sizeof(T) == 8 ? PROF_ORTH64 : PROF_ORTH32, s);
            // two dot passes ((i + 1) n reads each) and two updates (i + 1 reads
            // and one write of n each)
            prof_bytes(otok, (4.0 * i + 6.0) * (double)n * sizeof(T));
            XT_TRY(multi_dot<T>(V, n, i, col(i1 - 1), n, S.red, s));
            XT_CUDA(cudaMemcpyAsync(S.hsave.p, S.red.out.p, i * sizeof(double),
                                    cudaMemcpyDeviceToDevice, s));
            XT_TRY(update_and_dot<T>(V, n, i, S.hsave.p, col(i1 - 1), n, S.red, s));
            XT_CUDA(cudaMemcpyAsync(S.hsave.p + i, S.red.out.p, i * sizeof(double),
                                    cudaMemcpyDeviceToDevice, s));
            XT_TRY(update_and_norm<T>(V, n, i, S.hsave.p + i, col(i1 - 1), n, S.red, s));
            XT_CUDA(cudaMemcpyAsync(S.hsave.p + 2 * i, S.red.out.p, sizeof(double),
                                    cudaMemcpyDeviceToDevice, s));
            prof_end(otok, s);
            XT_TRY(fetch(s, hbuf.data(), S.hsave.p, 2 * i + 1));
            for (int j = 0; j < i; ++j) HH(j, i - 1) = hbuf[j] + hbuf[i + j];
            t = std::sqrt(hbuf[2 * i]);
            if (!std::isfinite(t)) {
                set_error("gmres: non-finite Krylov vector");
                return XT_ERR_NONFINITE;
            }
            HH(i1 - 1, i - 1) = t;
            if (t != 0.0) XT_TRY((axpby<T, T>(n, 1.0 / t, col(i1 - 1), 0.0, col(i1 - 1), s)));
            for (int k = 2; k <= i; ++k) {  // previous rotations
                const int k1 = k - 1;
                t = HH(k1 - 1, i - 1);
                HH(k1 - 1, i - 1) = c[k1 - 1] * t + sn[k1 - 1] * HH(k - 1, i - 1);
                HH(k - 1, i - 1) = -sn[k1 - 1] * t + c[k1 - 1] * HH(k - 1, i - 1);
            }
            double gam = std::sqrt(HH(i - 1, i - 1) * HH(i - 1, i - 1) +
                                   HH(i1 - 1, i - 1) * HH(i1 - 1, i - 1));
            if (gam == 0.0) gam = epsmac;
            c[i - 1] = HH(i - 1, i - 1) / gam;
            sn[i - 1] = HH(i1 - 1, i - 1) / gam;
            rs[i1 - 1] = -sn[i - 1] * rs[i - 1];
            rs[i - 1] = c[i - 1] * rs[i - 1];
            HH(i - 1, i - 1) = c[i - 1] * HH(i - 1, i - 1) + sn[i - 1] * HH(i1 - 1, i - 1);
            ro = std::fabs(rs[i1 - 1]);
            if (hist) hist->push_back(ro / ro0);
            if (i < im && ro > eps1) continue;
            break;
        }
        // upper triangular solve, combination, preconditioner, update
        std::vector<double> y(rs.begin(), rs.begin() + i);
        y[i - 1] = y[i - 1] / HH(i - 1, i - 1);
        for (int ii = 2; ii <= i; ++ii) {
            const int k = i - ii + 1;
            t = y[k - 1];
            for (int j = k + 1; j <= i; ++j) t -= HH(k - 1, j - 1) * y[j - 1];
            y[k - 1] = t / HH(k - 1, k - 1);
        }
        XT_CUDA(cudaMemcpyAsync(S.hsave.p, y.data(), i * sizeof(double), cudaMemcpyHostToDevice, s));
        T* u = Ws<T>::u(S);
        XT_TRY((lincomb<T, T>(V, n, i, S.hsave.p, u, n, s)));
        XT_TRY(apply_prec<T>(S, u, z));
        XT_TRY((axpby<T, T>(n, 1.0, z, 1.0, sol, s)));
        XT_CUDA(cudaStreamSynchronize(s));
        if (ro <= eps1) { ierr = 0; break; }
        if (its >= maxits) { ierr = 1; break; }
        // restart residual from the Givens data: v1 = sum_j rs'(j) v_j
        {
            const int i1 = i + 1;
            std::vector<double> r2(rs);
            for (int j = 1; j <= i; ++j) {
                const int jj = i1 - j + 1;
                r2[jj - 2] = -sn[jj - 2] * r2[jj - 1];
                r2[jj - 1] = c[jj - 2] * r2[jj - 1];
            }
            XT_CUDA(cudaMemcpyAsync(S.hsave.p, r2.data(), i1 * sizeof(double),
                                    cudaMemcpyHostToDevice, s));
            T* u = Ws<T>::u(S);
            XT_TRY((lincomb<T, T>(V, n, i1, S.hsave.p, u, n, s)));
            XT_CUDA(cudaMemcpyAsync(col(0), u, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
            XT_CUDA(cudaStreamSynchronize(s));
        }
    }
    st.its += its;
    st.ierr = ierr;
    st.est = ro0 > 0 ? ro / ro0 : 0.0;
    return XT_OK;
}


// Flexible GMRES (right preconditioning with the preconditioned vectors
// kept): the control flow of kronpgmres (src/kronecker.f90:181-365) with
// an FP64 operator, the ILU applied in FP32, and the Krylov basis V held in
// double-float (two FP32 numbers per entry: FP64's bytes, about 48
// significant bits, FP32 arithmetic).  z_j = M^-1 v_j is stored in FP32 and
// the update is x += Z y, so the Arnoldi relation A Z = V H holds to
// double-float accuracy however the FP32 preconditioner rounds; the
// operator is applied to z_j in double-float too (FP64-class result at FP32
// throughput).  A restart rebuilds the residual explicitly (FP64).
// Preconditioner of the BF16 experiment (mode 3): a few steps of FP32
// GMRES on the BF16-stored operator, right-preconditioned with the FP32
// ILU, from z = 0 (a variable preconditioner, which the flexible outer
// GMRES allows; the outer Arnoldi relation keeps the double-float
// operator, so the BF16 rounding of K and M only slows convergence).
constexpr int kNestSteps = 10;
constexpr double kNestTol = 1e-3;

int nested_prec(System& S, const float* v, float* z)
{
    const size_t n = (size_t)S.p * S.q;
    XT_CUDA(cudaMemsetAsync(z, 0, n * sizeof(float), S.stream));
    GmresStats in;
    XT_TRY(gmres_core<float>(S, v, z, kNestSteps, kNestTol, kNestSteps, in, nullptr));
    S.nest_its += in.its;
    return XT_OK;
}

// Classical Gram-Schmidt passes per Arnoldi step of the flexible GMRES: the
// system's setting (XTFEM_CGS_PASSES=1 or 2 overrides it), two once the
// solve has switched after a loss of orthogonality.  One pass reads the
// basis twice per step instead of four times; the Hessenberg column is then
// that pass's projections.
bool cgs_two_pass(const System& S)
{
    if (S.gs_latched) return true;
    const char* e = std::getenv("XTFEM_CGS_PASSES");
    const int passes = e ? std::atoi(e) : S.gs_passes;
    return passes != 1;
}

// A restart whose true residual exceeds the estimate of the cycle before it
// tenfold: the one-pass basis has lost orthogonality, so the rest of the
// solve takes two passes.
constexpr double kOrthLoss = 10.0;

int gmres_flex(System& S, const double* rhs, double* sol, int im, double eps, int maxits,
               GmresStats& st)
{
    bool two_pass = cgs_two_pass(S);
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    const size_t nl = n + (n & 1);  // basis column stride: even, zero pad when n is odd
    float2* V = reinterpret_cast<float2*>(S.V64.p);  // double-float basis
    float* Z = S.Z32.p;
    auto col = [&](int j) { return V + (size_t)j * nl; };
    if (nl != n) XT_CUDA(cudaMemsetAsync(V, 0, (size_t)(im + 1) * nl * sizeof(float2), s));
    auto zc = [&](int j) { return Z + (size_t)j * n; };
    std::vector<double> hh((size_t)(im + 1) * im, 0.0), c(im, 0.0), sn(im, 0.0), rs(im + 1, 0.0);
    std::vector<double> hbuf(2 * (im + 1) + 2);
    auto HH = [&](int r, int k) -> double& { return hh[(size_t)k * (im + 1) + r]; };
    const double epsmac = 1.0e-16;
    int its = 0, i = 0, ierr = 0;
    double ro = 0.0, eps1 = 0.0, t;

    XT_TRY(norm2<double>(rhs, n, S.red, s));
    XT_TRY(fetch(s, hbuf.data(), S.red.out.p, 1));
    const double ro0 = std::sqrt(hbuf[0]);
    for (;;) {
        TraceRange cycle("xtfem gmres cycle");
        // v1 = (rhs - A sol) / ||rhs - A sol||, the residual formed in FP64
        const double ro_est = ro;  // the previous cycle's estimate
        XT_CUDA(cudaMemcpyAsync(S.w64.p, rhs, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        XT_TRY(apply_op_ab<double>(S, -1.0, 1.0, sol, S.w64.p));
        XT_TRY(norm2<double>(S.w64.p, n, S.red, s));
        XT_TRY(fetch(s, hbuf.data(), S.red.out.p, 1));
        ro = std::sqrt(hbuf[0]);
        if (!std::isfinite(ro)) {
            set_error("gmres: non-finite residual");
            return XT_ERR_NONFINITE;
        }
        if (ro == 0.0) { ierr = -1; break; }
        if (its > 0 && !two_pass && ro > kOrthLoss * ro_est) two_pass = S.gs_latched = true;
        // v1 and its hi part, the first step's ILU input; each step leaves
        // the next one's the same way when it scales its new column
        XT_TRY(df_from_f64(S.w64.p, col(0), n, s));
        XT_TRY(df_scale_hi(col(0), 1.0 / ro, S.d32.p, n, s));
        if (its == 0) eps1 = eps * ro;
        rs.assign(im + 1, 0.0);
        rs[0] = ro;
        i = 0;
        ++st.cycles;
        for (;;) {
            ++i;
            ++its;
            const int i1 = i + 1;
            if (S.op16) XT_TRY(nested_prec(S, S.d32.p, zc(i - 1)));
            else XT_TRY(apply_prec<float>(S, S.d32.p, zc(i - 1)));
            {  // w = A z in double-float, straight into the basis column
                const int tok = prof_begin(PROF_KRONDF, s);
                XT_TRY(kron_spmm_df(S.K, S.M, S.q, S.A.p, S.B.p, zc(i - 1), col(i1 - 1), s));
                prof_end(tok, s);
            }
            const int otok = prof_begin(PROF_ORTH64, s);
            // as above, double-float values of 8 bytes
            prof_bytes(otok, (two_pass ? 4.0 * i + 6.0 : 2.0 * i + 3.0) * (double)nl * 8.0);
            XT_TRY(df_multi_dot(V, nl, i, col(i1 - 1), nl, S.red, s));
            // the last pass's projections h stay in red.out with the squared
            // norm after them, red.out = (h, ||w||^2); two passes keep the
            // first pass's in hsave.  The host's column: h1 + h (h1 = 0 for
            // one pass).
            if (two_pass) {
                XT_CUDA(cudaMemcpyAsync(S.hsave.p, S.red.out.p, i * sizeof(double),
                                        cudaMemcpyDeviceToDevice, s));
                XT_TRY(df_update_and_dot(V, nl, i, S.hsave.p, col(i1 - 1), nl, S.red, s));
            }
            XT_TRY(df_update_and_norm(V, nl, i, S.red.out.p, col(i1 - 1), nl, S.red, s,
                                      S.red.out.p + i));
            prof_end(otok, s);
            if (two_pass)
                XT_CUDA(cudaMemcpyAsync(hbuf.data(), S.hsave.p, i * sizeof(double),
                                        cudaMemcpyDeviceToHost, s));
            else
                std::fill(hbuf.begin(), hbuf.begin() + i, 0.0);
            XT_TRY(fetch(s, hbuf.data() + i, S.red.out.p, i + 1));
            for (int j = 0; j < i; ++j) HH(j, i - 1) = hbuf[j] + hbuf[i + j];
            t = std::sqrt(hbuf[2 * i]);
            if (!std::isfinite(t)) {
                set_error("gmres: non-finite Krylov vector");
                return XT_ERR_NONFINITE;
            }
            HH(i1 - 1, i - 1) = t;
            if (t != 0.0) XT_TRY(df_scale_hi(col(i1 - 1), 1.0 / t, S.d32.p, n, s));
            else XT_TRY(df_hi(col(i1 - 1), S.d32.p, n, s));
            for (int k = 2; k <= i; ++k) {
                const int k1 = k - 1;
                t = HH(k1 - 1, i - 1);
                HH(k1 - 1, i - 1) = c[k1 - 1] * t + sn[k1 - 1] * HH(k - 1, i - 1);
                HH(k - 1, i - 1) = -sn[k1 - 1] * t + c[k1 - 1] * HH(k - 1, i - 1);
            }
            double gam = std::sqrt(HH(i - 1, i - 1) * HH(i - 1, i - 1) +
                                   HH(i1 - 1, i - 1) * HH(i1 - 1, i - 1));
            if (gam == 0.0) gam = epsmac;
            c[i - 1] = HH(i - 1, i - 1) / gam;
            sn[i - 1] = HH(i1 - 1, i - 1) / gam;
            rs[i1 - 1] = -sn[i - 1] * rs[i - 1];
            rs[i - 1] = c[i - 1] * rs[i - 1];
            HH(i - 1, i - 1) = c[i - 1] * HH(i - 1, i - 1) + sn[i - 1] * HH(i1 - 1, i - 1);
            ro = std::fabs(rs[i1 - 1]);
            if (i < im && ro > eps1 && its < maxits) continue;
            break;
        }
        std::vector<double> y(rs.begin(), rs.begin() + i);
        y[i - 1] = y[i - 1] / HH(i - 1, i - 1);
        for (int ii = 2; ii <= i; ++ii) {
            const int k = i - ii + 1;
            t = y[k - 1];
            for (int j = k + 1; j <= i; ++j) t -= HH(k - 1, j - 1) * y[j - 1];
            y[k - 1] = t / HH(k - 1, k - 1);
        }
        XT_CUDA(cudaMemcpyAsync(S.hsave.p, y.data(), i * sizeof(double), cudaMemcpyHostToDevice, s));
        XT_TRY((lincomb<float, double>(Z, n, i, S.hsave.p, S.u64.p, n, s)));
        XT_TRY((axpby<double, double>(n, 1.0, S.u64.p, 1.0, sol, s)));
        XT_CUDA(cudaStreamSynchronize(s));
        if (ro <= eps1) { ierr = 0; break; }
        if (its >= maxits) { ierr = 1; break; }
    }
    st.its += its;
    st.ierr = ierr;
    st.est = ro0 > 0 ? ro / ro0 : 0.0;
    return XT_OK;
}

// XTFEM_GMRES_CHUNK: Arnoldi steps the device-driven GMRES issues between
// two reads of its control word (16).
int gmres_chunk()
{
    const char* e = std::getenv("XTFEM_GMRES_CHUNK");
    const int v = e ? std::atoi(e) : 16;
    return v > 0 ? v : 16;
}

// XTFEM_DEVICE_GMRES=1 selects the device-driven flexible GMRES (measured
// on the C2 rod and the rod batch: slower than the host-driven loop, whose
// one host read per Arnoldi step costs less than the device path's extra
// rotation, copy and control kernels)
bool device_gmres_on()
{
    const char* e = std::getenv("XTFEM_DEVICE_GMRES");
    return e && std::atoi(e) != 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// FlexRun: the device-driven flexible GMRES inside the FP64 refinement loop.
// A step is the same kernels on fixed buffers whatever its index: the hi
// part of basis column j into the ILU input, the FP32 ILU apply into a fixed
// vector and its copy into Z column j, the double-float operator into a
// fixed vector, the control-driven Gram-Schmidt passes, the rotations and
// convergence test (k_flexd_givens), and the scaled copy into V column j+1.
// Every kernel reads j (and whether the cycle still runs) from the control
// word {j, status, its, maxits} on the device.  The host work between
// cycles follows gmres_flex and solve_refined step for step.

int FlexRun::start(System& S, const double* b, double* x, int im, double tol, int maxits)
{
    S_ = &S;
    b_ = b;
    x_ = x;
    im_ = im;
    tol_ = tol;
    maxits_ = maxits;
    st = GmresStats();
    done = false;
    cycle = 0;
    j = 0;
    predicted_ = -1.0;
    if (!S.ilu) {
        set_error("solve: no preconditioner set");
        return XT_ERR_STATE;
    }
    if (im < 1 || im > kFlexdMaxIm) {
        set_error("solve: the device-driven GMRES takes a restart length of 1 to " +
                  std::to_string(kFlexdMaxIm));
        return XT_ERR_ARG;
    }
    XT_TRY(system_stream(S));
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    S.op16 = false;
    S.nest_its = 0;
    S.gs_latched = false;
    XT_TRY(ensure_workspace(S, im, false, true));
    double hb[2];
    XT_TRY(norm2<double>(b, n, S.red, s));
    XT_TRY(fetch(s, hb, S.red.out.p, 1));
    bn_ = std::sqrt(hb[0]);
    if (bn_ == 0.0) {
        XT_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
        XT_CUDA(cudaStreamSynchronize(s));
        st.ierr = -1;
        done = true;
        return XT_OK;
    }
    return outer_step();
}

// A refinement step: the FP64 true residual, the tests, the inner solve's start.
int FlexRun::outer_step()
{
    System& S = *S_;
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    double hb[2];
    XT_CUDA(cudaMemcpyAsync(S.r64.p, b_, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    XT_TRY(system_apply(S, -1.0, 1.0, x_, S.r64.p));
    XT_TRY(norm2<double>(S.r64.p, n, S.red, s));
    XT_TRY(fetch(s, hb, S.red.out.p, 1));
    rn_ = std::sqrt(hb[0]);
    st.relres = rn_ / bn_;
    if (!std::isfinite(rn_)) {
        set_error("solve: non-finite residual");
        return XT_ERR_NONFINITE;
    }
    if (st.relres <= tol_) {
        st.ierr = 0;
        done = true;
        return XT_OK;
    }
    if (st.its >= maxits_) {
        st.ierr = 1;
        done = true;
        return XT_OK;
    }
    if (predicted_ > 0.0 && rn_ > kOrthLoss * predicted_) S.gs_latched = true;
    ++st.outer;
    left_ = maxits_ - st.its;
    XT_CUDA(cudaMemsetAsync(S.t64.p, 0, n * sizeof(double), s));
    eps_in_ = tol_ * bn_ / rn_;
    return inner_begin();
}

// The inner solve of r64 into t64 (gmres_flex's set-up).
int FlexRun::inner_begin()
{
    System& S = *S_;
    two_pass = cgs_two_pass(S);
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    const size_t nl = n + (n & 1);
    float2* V = reinterpret_cast<float2*>(S.V64.p);
    if (nl != n) XT_CUDA(cudaMemsetAsync(V, 0, (size_t)(im_ + 1) * nl * sizeof(float2), s));
    const FlexLayout Lo(im_);
    XT_TRY(S.fst.alloc(Lo.total));
    XT_TRY(S.fctl.alloc(4));
    XT_TRY(S.zfix.alloc(n));
    XT_TRY(S.wfix.alloc(nl));
    XT_CUDA(cudaMemsetAsync(S.wfix.p, 0, nl * sizeof(float2), s));  // the pad entry stays 0
    rs_.assign(im_ + 1, 0.0);
    in_ = GmresStats();
    its_in_ = 0;
    ro_ = 0.0;
    eps1_ = 0.0;
    double hb[2];
    XT_TRY(norm2<double>(S.r64.p, n, S.red, s));
    XT_TRY(fetch(s, hb, S.red.out.p, 1));
    ro0_ = std::sqrt(hb[0]);
    return cycle_begin();
}

// A cycle's start: v1 from the residual formed in FP64, then the cycle state
// {rs = (ro, 0, ...), eps1, control {0, running, its, maxits}} on the device.
int FlexRun::cycle_begin()
{
    System& S = *S_;
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    float2* V = reinterpret_cast<float2*>(S.V64.p);
    const FlexLayout Lo(im_);
    double hb[2];
    const double ro_est = ro_;  // the previous cycle's estimate
    XT_CUDA(cudaMemcpyAsync(S.w64.p, S.r64.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    XT_TRY(apply_op_ab<double>(S, -1.0, 1.0, S.t64.p, S.w64.p));
    XT_TRY(norm2<double>(S.w64.p, n, S.red, s));
    XT_TRY(fetch(s, hb, S.red.out.p, 1));
    ro_ = std::sqrt(hb[0]);
    if (!std::isfinite(ro_)) {
        set_error("gmres: non-finite residual");
        return XT_ERR_NONFINITE;
    }
    if (ro_ == 0.0) return inner_end(-1);
    if (its_in_ > 0 && !two_pass && ro_ > kOrthLoss * ro_est) two_pass = S.gs_latched = true;
    XT_TRY(df_from_f64(S.w64.p, V, n, s));
    XT_TRY(df_scale(V, 1.0 / ro_, n, s));
    if (its_in_ == 0) eps1_ = eps_in_ * ro_;
    std::fill(rs_.begin(), rs_.end(), 0.0);
    rs_[0] = ro_;
    hctl_[0] = 0;
    hctl_[1] = 0;
    hctl_[2] = its_in_;
    hctl_[3] = left_;
    XT_CUDA(cudaMemcpyAsync(S.fst.p + Lo.rs, rs_.data(), (im_ + 1) * sizeof(double),
                            cudaMemcpyHostToDevice, s));
    XT_CUDA(cudaMemcpyAsync(S.fst.p + Lo.eps1, &eps1_, sizeof(double), cudaMemcpyHostToDevice, s));
    XT_CUDA(cudaMemcpyAsync(S.fctl.p, hctl_, sizeof(hctl_), cudaMemcpyHostToDevice, s));
    ++in_.cycles;
    ++cycle;
    j = 0;
    // complete before any step reads it: steps may run from a graph
    // launched on another stream
    XT_CUDA(cudaStreamSynchronize(s));
    return XT_OK;
}

int FlexRun::issue(int nstep, std::vector<int>* tok)
{
    System& S = *S_;
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    const size_t nl = n + (n & 1);
    float2* V = reinterpret_cast<float2*>(S.V64.p);
    int* ctl = S.fctl.p;
    double* dst = S.fst.p;
    if (tok) tok->assign((size_t)3 * nstep, -1);
    for (int k = 0; k < nstep; ++k) {
        XT_TRY(flexd_hi(ctl, V, nl, S.d32.p, n, s));
        if (tok) (*tok)[3 * k] = prof_begin(PROF_ILU32, s);
        XT_TRY(ilu_apply<float>(*S.ilu, S.q, S.Ainv.p, S.d32.p, S.zfix.p, S.w32.p, s, ctl + 1));
        if (tok) prof_end((*tok)[3 * k], s);
        XT_TRY(flexd_zcopy(ctl, S.zfix.p, S.Z32.p, n, s));
        if (tok) (*tok)[3 * k + 1] = prof_begin(PROF_KRONDF, s);
        XT_TRY(kron_spmm_df(S.K, S.M, S.q, S.A.p, S.B.p, S.zfix.p, S.wfix.p, s, ctl + 1));
        if (tok) prof_end((*tok)[3 * k + 1], s);
        if (tok) (*tok)[3 * k + 2] = prof_begin(PROF_ORTH64, s);
        XT_TRY(flexd_orth(ctl, V, nl, S.wfix.p, dst, im_, S.red, s, two_pass));
        XT_TRY(flexd_givens(ctl, dst, im_, s));
        XT_TRY(flexd_scale_copy(ctl, dst, im_, S.wfix.p, V, nl, n, s));
        if (tok) prof_end((*tok)[3 * k + 2], s);
    }
    return XT_OK;
}

// After a chunk: a cycle that has ended (status set) is finished on the
// host side, then the next cycle, refinement step or the end follows.
int FlexRun::advance(const int* c)
{
    j = c[0];
    if (c[1] == 0) return XT_OK;  // the cycle goes on
    if (c[1] == 4) {
        set_error("gmres: non-finite Krylov vector");
        return XT_ERR_NONFINITE;
    }
    System& S = *S_;
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    const FlexLayout Lo(im_);
    const int i = c[0];
    its_in_ = c[2];
    XT_CUDA(cudaMemcpyAsync(&ro_, S.fst.p + Lo.ro, sizeof(double), cudaMemcpyDeviceToHost, s));
    XT_TRY(flexd_solve(S.fctl.p, S.fst.p, im_, s));
    XT_TRY((lincomb<float, double>(S.Z32.p, n, i, S.fst.p + Lo.y, S.u64.p, n, s)));
    XT_TRY((axpby<double, double>(n, 1.0, S.u64.p, 1.0, S.t64.p, s)));
    XT_CUDA(cudaStreamSynchronize(s));
    if (ro_ <= eps1_) return inner_end(0);
    if (its_in_ >= left_) return inner_end(1);
    return cycle_begin();
}

// The inner solve's end and the rest of the refinement step.
int FlexRun::inner_end(int ierr_in)
{
    System& S = *S_;
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    in_.its += its_in_;
    in_.ierr = ierr_in;
    in_.est = ro0_ > 0 ? ro_ / ro0_ : 0.0;
    predicted_ = rn_ * in_.est;
    XT_TRY((axpby<double, double>(n, 1.0, S.t64.p, 1.0, x_, s)));
    XT_CUDA(cudaStreamSynchronize(s));
    XT_TRY(ilu_check(s));
    st.its += in_.its;
    st.cycles += in_.cycles;
    st.est = in_.est;
    if (in_.its == 0) {
        st.ierr = 1;
        done = true;
        return XT_OK;
    }
    return outer_step();
}

int gmres_fp64(System& S, const double* b, double* x, int im, double eps, int maxits,
               GmresStats& st, std::vector<double>* hist)
{
    if (!S.ilu) {
        set_error("gmres: no preconditioner set");
        return XT_ERR_STATE;
    }
    if (im < 1) {
        set_error("gmres: restart length must be >= 1");
        return XT_ERR_ARG;
    }
    XT_TRY(system_stream(S));
    XT_TRY(ensure_workspace(S, im, false));
    XT_TRY(gmres_core<double>(S, b, x, im, eps, maxits, st, hist));
    return ilu_check(S.stream);
}

namespace {
// Mode 2 with the device-driven flexible GMRES on one system: the run's
// steps issued in chunks, the control read once per chunk.  The profile
// tokens of steps past a cycle's end (they do nothing) are cancelled.
int solve_flex_run(System& S, const double* b, double* x, int im, double tol, int maxits,
                   GmresStats& st)
{
    FlexRun R;
    XT_TRY(R.start(S, b, x, im, tol, maxits));
    const int chunk = gmres_chunk();
    const size_t n = (size_t)S.p * S.q;
    const size_t nl = n + (n & 1);
    int issued = 0, cyc = R.cycle;
    std::vector<int> tok;
    int rctl[4] = {0, 0, 0, 0};
    while (!R.done) {
        if (R.cycle != cyc) {
            cyc = R.cycle;
            issued = 0;
        }
        const int nstep = std::min(chunk, im - issued);
        if (nstep <= 0) {
            set_error("gmres: a cycle ran past its restart length");
            return XT_ERR_STATE;
        }
        const int j0 = R.j;
        XT_TRY(R.issue(nstep, &tok));
        issued += nstep;
        XT_CUDA(cudaMemcpyAsync(rctl, S.fctl.p, sizeof(rctl), cudaMemcpyDeviceToHost, S.stream));
        XT_CUDA(cudaStreamSynchronize(S.stream));
        // steps of this chunk that ran: each advanced j by one
        const int ran = rctl[0] - j0;
        for (int k = 0; k < nstep; ++k) {
            if (k < ran) {
                const double jk = j0 + k + 1;
                prof_bytes(tok[3 * k + 2],
                           (R.two_pass ? 4.0 * jk + 6.0 : 2.0 * jk + 3.0) * (double)nl * 8.0);
            } else {
                for (int c = 0; c < 3; ++c) prof_cancel(tok[3 * k + c]);
            }
        }
        XT_TRY(R.advance(rctl));
    }
    st = R.st;
    return XT_OK;
}
}  // namespace

int solve_refined(System& S, const double* b, double* x, int im, double tol, int maxits,
                  int inner, double inner_tol, GmresStats& st)
{
    TraceRange tr("xtfem solve");
    if (!S.ilu) {
        set_error("solve: no preconditioner set");
        return XT_ERR_STATE;
    }
    if (inner == 2 && im <= kFlexdMaxIm && device_gmres_on())
        return solve_flex_run(S, b, x, im, tol, maxits, st);
    XT_TRY(system_stream(S));
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    // mode 3: the flexible GMRES of mode 2 whose preconditioner is a short
    // FP32 GMRES on K and M stored in BF16 (nested_prec)
    const bool bf16 = inner == 3;
    if (bf16) inner = 2;
    struct Op16 {
        System& S;
        ~Op16() { S.op16 = false; }
    } op16_reset{S};
    S.op16 = bf16;
    S.nest_its = 0;
    S.gs_latched = false;
    double predicted = -1.0;  // the last inner solve's estimate of the residual it left
    XT_TRY(ensure_workspace(S, im, inner == 1, inner == 2));
    if (bf16) XT_TRY(ensure_workspace(S, kNestSteps, true));
    double hb[2];
    XT_TRY(norm2<double>(b, n, S.red, s));
    XT_TRY(fetch(s, hb, S.red.out.p, 1));
    const double bn = std::sqrt(hb[0]);
    st = GmresStats();
    if (bn == 0.0) {
        XT_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
        XT_CUDA(cudaStreamSynchronize(s));
        st.ierr = -1;
        return XT_OK;
    }
    for (;;) {
        // true residual in FP64
        XT_CUDA(cudaMemcpyAsync(S.r64.p, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        XT_TRY(system_apply(S, -1.0, 1.0, x, S.r64.p));
        XT_TRY(norm2<double>(S.r64.p, n, S.red, s));
        XT_TRY(fetch(s, hb, S.red.out.p, 1));
        const double rn = std::sqrt(hb[0]);
        st.relres = rn / bn;
        if (!std::isfinite(rn)) {
            set_error("solve: non-finite residual");
            return XT_ERR_NONFINITE;
        }
        if (st.relres <= tol) { st.ierr = 0; break; }
        if (st.its >= maxits) { st.ierr = 1; break; }
        if (inner == 2 && predicted > 0.0 && rn > kOrthLoss * predicted) S.gs_latched = true;
        ++st.outer;
        const int left = maxits - st.its;
        const double want = std::max(tol * bn / rn, inner == 1 ? inner_tol : 0.0);
        GmresStats in;
        if (inner == 1) {
            // FP32 inner solve of A d = r / ||r||, then x += ||r|| d in FP64
            XT_TRY((axpby<double, float>(n, 1.0 / rn, S.r64.p, 0.0, S.r32.p, s)));
            XT_CUDA(cudaMemsetAsync(S.d32.p, 0, n * sizeof(float), s));
            XT_TRY(gmres_core<float>(S, S.r32.p, S.d32.p, im, want, left, in, nullptr));
            XT_TRY((axpby<float, double>(n, rn, S.d32.p, 1.0, x, s)));
        } else if (inner == 2) {
            XT_CUDA(cudaMemsetAsync(S.t64.p, 0, n * sizeof(double), s));
            XT_TRY(gmres_flex(S, S.r64.p, S.t64.p, im, tol * bn / rn, left, in));
            predicted = rn * in.est;
            XT_TRY((axpby<double, double>(n, 1.0, S.t64.p, 1.0, x, s)));
        } else {
            XT_CUDA(cudaMemsetAsync(S.t64.p, 0, n * sizeof(double), s));
            XT_TRY(gmres_core<double>(S, S.r64.p, S.t64.p, im, want, left, in, nullptr));
            XT_TRY((axpby<double, double>(n, 1.0, S.t64.p, 1.0, x, s)));
        }
        XT_CUDA(cudaStreamSynchronize(s));
        XT_TRY(ilu_check(s));
        st.its += in.its;
        st.cycles += in.cycles;
        st.est = in.est;
        if (in.its == 0) { st.ierr = 1; break; }
    }
    return XT_OK;
}

}  // namespace xt
