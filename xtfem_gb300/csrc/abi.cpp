// abi.cpp -- the C ABI of the library (include/xtfem_gb300.h).
//
// The Fortran entry points mirror the reference's subroutines
// (src/kronecker.f90, src/delelement.f90, src/kokkos_host.cpp) argument for
// argument; host arrays in the reference's block layout are converted to the
// device's interleaved layout on the way in and back on the way out.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/xtfem_gb300.h"
#include "solver.h"

extern "C" long long xt_launch_count(void);  // prof.cpp

using namespace xt;

struct xt_system_s {
    System sys;
    DBuf<double> blk;   // block-layout staging, p*q
    DBuf<double> a_in, b_in;  // q x q staging
};

namespace {

// ------------------------------------------------------------ caching
bool g_cache = false;
using OpKey = std::tuple<const void*, const void*, const void*, const void*, const void*,
                         const void*, int, int, int, int>;
using IluKey = std::tuple<const void*, const void*, const void*, int, int>;
std::map<OpKey, std::unique_ptr<xt_system_s>> g_ops;
std::map<IluKey, std::shared_ptr<DevIlu>> g_ilus;

int to_status(int s) { return s; }

// Makes the library's device current for the lifetime of the guard and
// gives the calling thread its own current device back afterwards.
struct DeviceGuard {
    int saved = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int device)
    {
        err = cudaGetDevice(&saved);
        if (err == cudaSuccess && saved != device) err = cudaSetDevice(device);
    }
    ~DeviceGuard()
    {
        if (saved >= 0) cudaSetDevice(saved);
    }
};

int upload_blocks(xt_system_s& h, const double* host, double* dev_itl)
{
    System& S = h.sys;
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    XT_TRY(h.blk.alloc(n));
    XT_CUDA(cudaMemcpyAsync(h.blk.p, host, n * sizeof(double), cudaMemcpyHostToDevice, s));
    XT_TRY((to_interleaved<double, double>(h.blk.p, dev_itl, S.p, S.q, s)));
    return XT_OK;
}

int download_blocks(xt_system_s& h, const double* dev_itl, double* host)
{
    System& S = h.sys;
    cudaStream_t s = S.stream;
    const size_t n = (size_t)S.p * S.q;
    XT_TRY(h.blk.alloc(n));
    XT_TRY((to_blocks<double, double>(dev_itl, h.blk.p, S.p, S.q, s)));
    XT_CUDA(cudaMemcpyAsync(host, h.blk.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    XT_CUDA(cudaStreamSynchronize(s));
    return XT_OK;
}

int ensure_vec(DBuf<double>& d, size_t n) { return d.alloc(n); }

// Fetch (or build) the system for a Fortran call.  With caching off the
// returned object is owned by `tmp` and dies with the call.
int get_system(const int* ki, const int* kj, const double* kv, const int* mi, const int* mj,
               const double* mv, int p, int q, std::unique_ptr<xt_system_s>& tmp,
               xt_system_s*& out)
{
    XT_TRY(ensure_init());
    if (p <= 0 || q < 1 || q > 8 || !ki || !kj || !kv || !mi || !mj || !mv) {
        set_error("invalid operator arguments (need p > 0, 1 <= q <= 8, non-null arrays)");
        return XT_ERR_ARG;
    }
    const int nk = ki[p] - 1, nm = mi[p] - 1;
    if (g_cache) {
        OpKey key{ki, kj, kv, mi, mj, mv, p, q, nk, nm};
        auto it = g_ops.find(key);
        if (it != g_ops.end()) { out = it->second.get(); return XT_OK; }
        auto h = std::make_unique<xt_system_s>();
        XT_TRY(system_create(h->sys, p, q, ki, kj, kv, mi, mj, mv));
        out = h.get();
        g_ops[key] = std::move(h);
        return XT_OK;
    }
    tmp = std::make_unique<xt_system_s>();
    XT_TRY(system_create(tmp->sys, p, q, ki, kj, kv, mi, mj, mv));
    out = tmp.get();
    return XT_OK;
}

int get_ilu(const double* alu, const int* jlu, const int* ju, int p, std::shared_ptr<DevIlu>& out)
{
    if (!alu || !jlu || !ju || p <= 0) {
        set_error("invalid factor arguments");
        return XT_ERR_ARG;
    }
    const int nz = jlu[p] - 1;
    const int group = (p % 3 == 0) ? 3 : 1;
    if (g_cache) {
        IluKey key{alu, jlu, ju, p, nz};
        auto it = g_ilus.find(key);
        if (it != g_ilus.end()) { out = it->second; return XT_OK; }
    }
    auto f = std::make_shared<DevIlu>();
    XT_TRY(build_ilu(*f, p, alu, jlu, ju, group, ctx().stream));
    if (g_cache) g_ilus[IluKey{alu, jlu, ju, p, nz}] = f;
    out = f;
    return XT_OK;
}

int do_spmv(const double* a, const double* b, double alpha, double beta, int q, const int* ki,
            const int* kj, const double* kv, const int* mi, const int* mj, const double* mv,
            int p, const double* x, double* y)
{
    std::unique_ptr<xt_system_s> tmp;
    xt_system_s* h = nullptr;
    XT_TRY(get_system(ki, kj, kv, mi, mj, mv, p, q, tmp, h));
    return xt_system_apply(h, a, b, alpha, beta, x, y);
}

// A system without K and M for kronlusol_: only the factor and the
// temporal inverse are needed.
struct LuOnly {
    System sys;
    DBuf<double> blk;
};

}  // namespace

extern "C" {

const char* xt_last_error(void) { return last_error(); }
void xt_clear_error(void) { set_error(""); }
const char* xt_version(void) { return "xtfem_gb300 0.1"; }

int xt_init(int device) { return ensure_init(device); }

int xt_finalize(void)
{
    g_ops.clear();
    g_ilus.clear();
    damage_static_forget();
    Context& c = ctx();
    if (c.ready) {
        cudaStreamSynchronize(c.stream);
        cudaStreamDestroy(c.stream);
        c.stream = nullptr;
        c.ready = false;
    }
    return XT_OK;
}

void kokkos_init_(void) { (void)ensure_init(0); }
void kokkos_finish_(void) { (void)xt_finalize(); }

void xt_set_cache_(const int* on)
{
    g_cache = on && *on;
    if (!g_cache) {
        g_ops.clear();
        g_ilus.clear();
    }
}

void xt_invalidate_(void)
{
    g_ops.clear();
    g_ilus.clear();
}

// ------------------------------------------------------- handle API
int xt_system_create(int p, int q, const int* ki, const int* kj, const double* kv,
                     const int* mi, const int* mj, const double* mv, xt_system* out)
{
    if (!out) { set_error("xt_system_create: null output"); return XT_ERR_ARG; }
    *out = nullptr;
    if (!ki || !kj || !kv || !mi || !mj || !mv) {
        set_error("xt_system_create: null array");
        return XT_ERR_ARG;
    }
    auto h = std::make_unique<xt_system_s>();
    XT_TRY(system_create(h->sys, p, q, ki, kj, kv, mi, mj, mv));
    *out = h.release();
    return XT_OK;
}

int xt_system_destroy(xt_system s)
{
    delete s;
    return XT_OK;
}

int xt_system_set_ilu_blocks(xt_system s, const double* alu, const int* jlu, const int* ju,
                             int group, int blocks)
{
    if (!s || !alu || !jlu || !ju) { set_error("xt_system_set_ilu: null argument"); return XT_ERR_ARG; }
    return system_set_ilu(s->sys, alu, jlu, ju, group, blocks);
}

int xt_system_set_gs_passes(xt_system s, int passes)
{
    if (!s || (passes != 1 && passes != 2)) {
        set_error("xt_system_set_gs_passes: passes is 1 or 2");
        return XT_ERR_ARG;
    }
    s->sys.gs_passes = passes;
    return XT_OK;
}

int xt_system_ilu_blocks(xt_system s)
{
    return (s && s->sys.ilu) ? std::max(1, s->sys.ilu->blocks) : 0;
}

int xt_system_set_ilu(xt_system s, const double* alu, const int* jlu, const int* ju, int group)
{
    if (!s || !alu || !jlu || !ju) { set_error("xt_system_set_ilu: null argument"); return XT_ERR_ARG; }
    return system_set_ilu(s->sys, alu, jlu, ju, group);
}

int xt_system_set_temporal(xt_system s, const double* a, const double* b)
{
    if (!s || !a || !b) { set_error("xt_system_set_temporal: null argument"); return XT_ERR_ARG; }
    return system_set_temporal(s->sys, a, b);
}

int xt_system_apply(xt_system h, const double* a, const double* b, double alpha, double beta,
                    const double* x, double* y)
{
    if (!h || !a || !b || !x || !y) { set_error("xt_system_apply: null argument"); return XT_ERR_ARG; }
    System& S = h->sys;
    XT_TRY(system_stream(S));
    cudaStream_t s = S.stream;
    const int q = S.q;
    const size_t n = (size_t)S.p * q;
    XT_TRY(h->a_in.alloc(64));
    XT_TRY(h->b_in.alloc(64));
    XT_CUDA(cudaMemcpyAsync(h->a_in.p, a, sizeof(double) * q * q, cudaMemcpyHostToDevice, s));
    XT_CUDA(cudaMemcpyAsync(h->b_in.p, b, sizeof(double) * q * q, cudaMemcpyHostToDevice, s));
    trace("apply: temporal matrices staged");
    XT_TRY(ensure_vec(S.x64, n));
    XT_TRY(ensure_vec(S.r64, n));
    XT_TRY(upload_blocks(*h, x, S.x64.p));
    trace("apply: x uploaded");
    if (beta != 0.0) XT_TRY(upload_blocks(*h, y, S.r64.p));
    XT_TRY(system_apply_with(S, h->a_in.p, h->b_in.p, alpha, beta, S.x64.p, S.r64.p));
    trace("apply: operator applied");
    const int st = download_blocks(*h, S.r64.p, y);
    trace("apply: y downloaded");
    return st;
}

int xt_system_lusol(xt_system h, const double* a, const double* x, double* y)
{
    if (!h || !a || !x || !y) { set_error("xt_system_lusol: null argument"); return XT_ERR_ARG; }
    System& S = h->sys;
    XT_TRY(system_stream(S));
    if (!S.ilu) { set_error("xt_system_lusol: no factor set"); return XT_ERR_STATE; }
    const int q = S.q;
    const size_t n = (size_t)S.p * q;
    std::vector<double> ainv(q * q);
    XT_TRY(invert_small(q, a, ainv.data()));
    cudaStream_t s = S.stream;
    XT_CUDA(cudaMemcpyAsync(S.Ainv.p, ainv.data(), sizeof(double) * q * q, cudaMemcpyHostToDevice, s));
    XT_TRY(ensure_vec(S.x64, n));
    XT_TRY(ensure_vec(S.r64, n));
    XT_TRY(ensure_vec(S.w64, n));
    XT_TRY(upload_blocks(*h, x, S.x64.p));
    XT_TRY(ilu_apply<double>(*S.ilu, q, S.Ainv.p, S.x64.p, S.r64.p, S.w64.p, s));
    XT_TRY(download_blocks(*h, S.r64.p, y));
    if (!S.hAinv.empty())  // restore the solver's temporal inverse
        XT_CUDA(cudaMemcpyAsync(S.Ainv.p, S.hAinv.data(), sizeof(double) * q * q,
                                cudaMemcpyHostToDevice, s));
    XT_CUDA(cudaStreamSynchronize(s));
    return ilu_check(s);
}

int xt_system_lusol_f32(xt_system h, const double* a, const double* x, double* y)
{
    if (!h || !a || !x || !y) { set_error("xt_system_lusol_f32: null argument"); return XT_ERR_ARG; }
    System& S = h->sys;
    XT_TRY(system_stream(S));
    if (!S.ilu) { set_error("xt_system_lusol_f32: no factor set"); return XT_ERR_STATE; }
    const int q = S.q;
    const size_t n = (size_t)S.p * q;
    std::vector<double> ainv(q * q);
    XT_TRY(invert_small(q, a, ainv.data()));
    cudaStream_t s = S.stream;
    XT_CUDA(cudaMemcpyAsync(S.Ainv.p, ainv.data(), sizeof(double) * q * q, cudaMemcpyHostToDevice, s));
    XT_TRY(ensure_vec(S.x64, n));
    XT_TRY(ensure_vec(S.r64, n));
    DBuf<float> x32, y32, w32;
    XT_TRY(x32.alloc(n));
    XT_TRY(y32.alloc(n));
    XT_TRY(w32.alloc(n));
    XT_TRY(upload_blocks(*h, x, S.x64.p));
    XT_TRY((axpby<double, float>(n, 1.0, S.x64.p, 0.0, x32.p, s)));
    XT_TRY(ilu_apply<float>(*S.ilu, q, S.Ainv.p, x32.p, y32.p, w32.p, s));
    XT_TRY((axpby<float, double>(n, 1.0, y32.p, 0.0, S.r64.p, s)));
    XT_TRY(download_blocks(*h, S.r64.p, y));
    if (!S.hAinv.empty())  // restore the solver's temporal inverse
        XT_CUDA(cudaMemcpyAsync(S.Ainv.p, S.hAinv.data(), sizeof(double) * q * q,
                                cudaMemcpyHostToDevice, s));
    XT_CUDA(cudaStreamSynchronize(s));
    return ilu_check(s);
}

int xt_system_gmres(xt_system h, const double* rhs, double* sol, int im, double eps, int maxits,
                    int* its, int* ierr, double* est, double* hist, int hist_len)
{
    if (!h || !rhs || !sol) { set_error("xt_system_gmres: null argument"); return XT_ERR_ARG; }
    System& S = h->sys;
    XT_TRY(system_stream(S));
    const size_t n = (size_t)S.p * S.q;
    XT_TRY(ensure_vec(S.b64, n));
    XT_TRY(ensure_vec(S.x64, n));
    XT_TRY(upload_blocks(*h, rhs, S.b64.p));
    XT_TRY(upload_blocks(*h, sol, S.x64.p));
    GmresStats st;
    std::vector<double> hv;
    XT_TRY(gmres_fp64(S, S.b64.p, S.x64.p, im, eps, maxits, st, hist ? &hv : nullptr));
    XT_TRY(download_blocks(*h, S.x64.p, sol));
    if (its) *its = st.its;
    if (ierr) *ierr = st.ierr;
    if (est) *est = st.est;
    if (hist)
        for (int k = 0; k < hist_len && k < (int)hv.size(); ++k) hist[k] = hv[k];
    return XT_OK;
}

// xt_system_solve's body, shared with the batch workers.
static int system_solve_host(xt_system h, const double* rhs, double* sol, int im, double tol,
                             int maxits, int precision, double inner_tol, double* out_stats)
{
    if (!h || !rhs || !sol) { set_error("xt_system_solve: null argument"); return XT_ERR_ARG; }
    if (precision < 0 || precision > 3) { set_error("xt_system_solve: precision is 0, 1, 2 or 3"); return XT_ERR_ARG; }
    System& S = h->sys;
    XT_TRY(system_stream(S));
    const size_t n = (size_t)S.p * S.q;
    XT_TRY(ensure_vec(S.b64, n));
    XT_TRY(ensure_vec(S.x64, n));
    XT_TRY(upload_blocks(*h, rhs, S.b64.p));
    XT_TRY(upload_blocks(*h, sol, S.x64.p));
    GmresStats st;
    XT_TRY(solve_refined(S, S.b64.p, S.x64.p, im, tol, maxits, precision, inner_tol, st));
    XT_TRY(download_blocks(*h, S.x64.p, sol));
    if (out_stats) {
        out_stats[0] = st.its;
        out_stats[1] = st.cycles;
        out_stats[2] = st.outer;
        out_stats[3] = st.ierr;
        out_stats[4] = st.relres;
        out_stats[5] = st.est;
    }
    return XT_OK;
}

int xt_system_solve(xt_system h, const double* rhs, double* sol, int im, double tol, int maxits,
                    int precision, double inner_tol, double* out_stats)
{
    return system_solve_host(h, rhs, sol, im, tol, maxits, precision, inner_tol, out_stats);
}

int xt_system_set_mesh(xt_system h, int nn, int ne, const double* xyz, const int* conn,
                       const int* bc)
{
    if (!h || !xyz || !conn || !bc) { set_error("xt_system_set_mesh: null argument"); return XT_ERR_ARG; }
    XT_TRY(system_stream(h->sys));
    try {
        return system_set_mesh(h->sys, nn, ne, xyz, conn, bc);
    } catch (const std::bad_alloc&) {
        set_error("xt_system_set_mesh: out of host memory");
        return XT_ERR_ALLOC;
    }
}

int xt_system_assemble_k(xt_system h, const double* ym, const double* nu)
{
    if (!h || !ym || !nu) { set_error("xt_system_assemble_k: null argument"); return XT_ERR_ARG; }
    return system_assemble_k(h->sys, ym, nu);
}

int xt_system_k_nnz(xt_system h) { return h ? h->sys.K.nnz : 0; }

int xt_system_get_k(xt_system h, int* ia, int* ja, double* kv)
{
    if (!h) { set_error("xt_system_get_k: null argument"); return XT_ERR_ARG; }
    System& S = h->sys;
    XT_TRY(system_stream(S));
    cudaStream_t s = S.stream;
    const size_t nnz = (size_t)S.K.nnz;
    if (ia) XT_CUDA(cudaMemcpyAsync(ia, S.K.rowptr.p, sizeof(int) * ((size_t)S.p + 1), cudaMemcpyDeviceToHost, s));
    if (ja) XT_CUDA(cudaMemcpyAsync(ja, S.K.col.p, sizeof(int) * nnz, cudaMemcpyDeviceToHost, s));
    if (kv) XT_CUDA(cudaMemcpyAsync(kv, S.K.v64.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost, s));
    XT_CUDA(cudaStreamSynchronize(s));
    if (ia) for (int r = 0; r <= S.p; ++r) ++ia[r];  // the device keeps 0-based indices
    if (ja) for (size_t k = 0; k < nnz; ++k) ++ja[k];
    return XT_OK;
}

// ------------------------------------------------------------- batches
struct xt_batch_s {
    std::vector<xt_system> sys;
    std::vector<int> order;  // largest system first
    int workers = 1;
    int tuned_im = 0;        // restart length picked by the tuner, 0 before
    int tuned_shares = 0;    // ILU lanes per row picked by the tuner
    int tuned_passes = 0;    // Gram-Schmidt passes picked by the tuner
};

int xt_batch_create(int count, const xt_system* systems, int workers, xt_batch* out)
{
    if (!out || count <= 0 || !systems) { set_error("xt_batch_create: bad arguments"); return XT_ERR_ARG; }
    *out = nullptr;
    for (int i = 0; i < count; ++i)
        if (!systems[i]) { set_error("xt_batch_create: null system"); return XT_ERR_ARG; }
    {  // one worker per system at a time: a system listed twice would race
        std::vector<xt_system> sorted(systems, systems + count);
        std::sort(sorted.begin(), sorted.end());
        if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) {
            set_error("xt_batch_create: a system is listed twice");
            return XT_ERR_ARG;
        }
    }
    XT_TRY(ensure_init());
    auto b = std::make_unique<xt_batch_s>();
    b->sys.assign(systems, systems + count);
    b->order.resize(count);
    for (int i = 0; i < count; ++i) b->order[i] = i;
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) {
        return (long long)b->sys[x]->sys.p * b->sys[x]->sys.q > (long long)b->sys[y]->sys.p * b->sys[y]->sys.q;
    });
    b->workers = std::max(1, std::min(count, workers > 0 ? workers : 16));
    *out = b.release();
    return XT_OK;
}

int xt_batch_destroy(xt_batch b)
{
    delete b;
    return XT_OK;
}

namespace {
int batch_run(xt_batch b, const double* const* rhs, double* const* sol, int im, double tol,
              int maxits, int precision, double inner_tol, double* stats, int* status);

// Tuner of the restart length and of the ILU sweep's lanes per row (the
// register sweep's rows per warp): each candidate pair solves the whole
// batch from the caller's initial guesses; the fastest (host wall clock,
// device work included: every solve ends with its download) is kept.
void set_shares(xt_batch b, int shares)
{
    for (xt_system h : b->sys)
        if (h->sys.ilu) h->sys.ilu->shares = shares;
}

void set_passes(xt_batch b, int passes)
{
    for (xt_system h : b->sys) h->sys.gs_passes = passes;
}

int batch_tune(xt_batch b, const double* const* rhs, double* const* sol, double tol, int maxits,
               int precision, double inner_tol)
{
    const int count = (int)b->sys.size();
    long long nmax = 0;
    for (xt_system h : b->sys) nmax = std::max(nmax, (long long)h->sys.p * h->sys.q);
    std::vector<std::vector<double>> x0(count);
    for (int i = 0; i < count; ++i) {
        const size_t n = (size_t)b->sys[i]->sys.p * b->sys[i]->sys.q;
        x0[i].assign(sol[i], sol[i] + n);
    }
    double best = 0.0;
    int best_im = 0, best_sh = 0;
    for (int sh : {2, 1}) {
        set_shares(b, sh);
        int last_im = 0;
        for (int cand : {30, 60, 120, 200}) {
            const int im = (int)std::min<long long>(cand, nmax);
            if (im == last_im) continue;
            last_im = im;
            for (int i = 0; i < count; ++i) std::copy(x0[i].begin(), x0[i].end(), sol[i]);
            const auto t0 = std::chrono::steady_clock::now();
            XT_TRY(batch_run(b, rhs, sol, im, tol, maxits, precision, inner_tol, nullptr, nullptr));
            const double t =
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (best_im == 0 || t < best) {
                best = t;
                best_im = im;
                best_sh = sh;
            }
        }
    }
    // one Gram-Schmidt pass at the best pair (mode 2 only; two are the default)
    int best_passes = 2;
    if (precision == 2) {
        set_shares(b, best_sh);
        set_passes(b, 1);
        for (int i = 0; i < count; ++i) std::copy(x0[i].begin(), x0[i].end(), sol[i]);
        const auto t0 = std::chrono::steady_clock::now();
        XT_TRY(batch_run(b, rhs, sol, best_im, tol, maxits, precision, inner_tol, nullptr, nullptr));
        const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (t < best) best_passes = 1;
        set_passes(b, 2);
    }
    for (int i = 0; i < count; ++i) std::copy(x0[i].begin(), x0[i].end(), sol[i]);
    b->tuned_im = best_im;
    b->tuned_shares = best_sh;
    b->tuned_passes = best_passes;
    set_shares(b, best_sh);
    set_passes(b, best_passes);
    return XT_OK;
}
}  // namespace

int xt_batch_restart(xt_batch b) { return b ? b->tuned_im : 0; }
int xt_batch_ilu_shares(xt_batch b) { return b ? b->tuned_shares : 0; }
int xt_batch_gs_passes(xt_batch b) { return b ? b->tuned_passes : 0; }

int xt_batch_solve(xt_batch b, const double* const* rhs, double* const* sol, int im, double tol,
                   int maxits, int precision, double inner_tol, double* stats, int* status)
{
    if (!b || !rhs || !sol) { set_error("xt_batch_solve: null argument"); return XT_ERR_ARG; }
    const int count = (int)b->sys.size();
    for (int i = 0; i < count; ++i)
        if (!rhs[i] || !sol[i]) { set_error("xt_batch_solve: null vector"); return XT_ERR_ARG; }
    if (im <= 0) {
        if (b->tuned_im == 0) XT_TRY(batch_tune(b, rhs, sol, tol, maxits, precision, inner_tol));
        im = b->tuned_im;
        set_shares(b, b->tuned_shares);
        set_passes(b, b->tuned_passes);
    }
    return batch_run(b, rhs, sol, im, tol, maxits, precision, inner_tol, stats, status);
}

namespace {
// The batch in lockstep (mode 2, the default): every system runs the
// refined solve with the device-driven flexible GMRES (FlexRun), and a round
// issues the next kRound Arnoldi steps of every system (16,
// XTFEM_BATCH_ROUND) as kRound launches of one CUDA graph that holds one
// step of every system, one branch per system, each branch ending with the
// copy of its control word into pinned host memory.  The graph is captured
// in the second round, after every run has issued a
// round directly (so the device data built on first use exists); it is
// replayed every round after that, and runs whose cycle or solve has ended
// do nothing in it (their kernels read the ended status).  One host
// synchronisation per round reads every control word; the host work between
// cycles (residuals, the least-squares update, refinement) is each run's
// own, on its stream.  XTFEM_BATCH_GRAPH=0: the same rounds issued directly.
// The results equal each system's own solve bit for bit.
// Arnoldi steps per round (XTFEM_BATCH_ROUND, 16)
int batch_round()
{
    const char* e = std::getenv("XTFEM_BATCH_ROUND");
    const int v = e ? std::atoi(e) : 16;
    return v > 0 && v <= 256 ? v : 16;
}

struct PinnedInts {
    int* p = nullptr;
    ~PinnedInts() { if (p) cudaFreeHost(p); }
};
struct GraphParts {
    cudaStream_t master = nullptr;
    std::vector<cudaEvent_t> ev;
    cudaGraphExec_t exec = nullptr;
    ~GraphParts()
    {
        if (exec) cudaGraphExecDestroy(exec);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        if (master) cudaStreamDestroy(master);
    }
};

bool batch_graph_on()
{
    const char* e = std::getenv("XTFEM_BATCH_GRAPH");
    return !e || std::atoi(e) != 0;
}

// The round graph's step of the systems whose operator has the node-block
// form (XTFEM_BATCH_FUSED=0: none): batched kernels that serve all of them
// in one launch each (flexb_*, kron_nb_batch), driven by a device table of
// their buffers, with each system's two ILU sweeps as its own branch; the
// step is about 20 graph nodes however many systems there are, instead of
// 15 per system.  One gathered copy brings their control words back.
bool batch_fused_on()
{
    const char* e = std::getenv("XTFEM_BATCH_FUSED");
    return !e || std::atoi(e) != 0;
}

struct FusedStep {
    DBuf<unsigned char> table;  // entries of all, then of two, then of one
    DBuf<int> dctl;             // gathered control words, four per entry of all
    int* hgat = nullptr;        // their pinned host copy
    std::vector<int> sys;       // batch index of each entry of all
    int nall = 0, ntwo = 0, none = 0, q = 0;
    long long lanes_max = 0;
    FlexStepDims dims;
    // the ILU sweeps: one launch per group of equal kernel shape, forward
    // groups, then backward groups, each group on a branch of its own
    std::vector<std::unique_ptr<RegGroup>> gl, gu;
    std::vector<cudaEvent_t> gev;
    ~FusedStep()
    {
        if (hgat) cudaFreeHost(hgat);
        for (cudaEvent_t e : gev)
            if (e) cudaEventDestroy(e);
    }
};

// A live system's entry of the fused step; false when its ILU apply or its
// operator has no batched launch (it then runs its own step kernels).
bool fused_item(System& S, int im, FlexStepItem& e, IluRegEntry& r)
{
    if (!S.ilu || !kron_nb_batchable(S.K, S.q)) return false;
    if (ilu_reg_entry(*S.ilu, S.q, S.zfix.p, S.fctl.p + 1, S.stream, r) != XT_OK) {
        cudaGetLastError();
        return false;
    }
    if (!r.ok) return false;
    const long long n = (long long)S.p * S.q, nl = n + (n & 1);
    e = FlexStepItem{};
    e.ctl = S.fctl.p;
    e.st = S.fst.p;
    e.partial = S.red.partial.p;
    e.V = reinterpret_cast<float2*>(S.V64.p);
    e.zfix = S.zfix.p;
    e.Z = S.Z32.p;
    e.wfix = S.wfix.p;
    e.n = n;
    e.nl = nl;
    e.im = im;
    e.rowblocks = df_row_blocks_for(nl, S.red);
    e.dotrows = df_dot_rows_for(nl, S.red);
    e.dotblocks = 1;  // set from the batch's sizes
    e.src = r.src;
    e.lanes = r.lanes;
    e.rrhs = r.rrhs;
    e.Ainv = S.Ainv.p;
    e.nodes = S.K.nb.nodes;
    e.bptr = S.K.nb.ptr.p;
    e.bcol = S.K.nb.col.p;
    e.kv = S.K.nb.kdf.p;
    e.mv = S.K.nb.mdf.p;
    e.A = S.A.p;
    e.B = S.B.p;
    return e.ctl && e.st && e.partial && e.V && e.zfix && e.Z && e.wfix && e.src && e.rrhs &&
           e.Ainv && e.A && e.B;
}

// Sweep groups of one direction: entries with equal shares, steps, offset
// width and warps, their argument tables uploaded.
int fused_groups(std::vector<std::unique_ptr<RegGroup>>& out, const std::vector<IluRegEntry>& ent,
                 bool upper)
{
    out.clear();
    std::map<std::tuple<int, int, int, int>, std::vector<RegArgs>> by;
    std::map<std::tuple<int, int, int, int>, size_t> smem;
    for (const IluRegEntry& r : ent) {
        const RegArgs& a = upper ? r.U : r.L;
        const auto key = std::make_tuple(r.H, r.smax, r.w16, a.ncw);
        by[key].push_back(a);
        smem[key] = std::max(smem[key], upper ? r.smemU : r.smemL);
    }
    for (auto& kv : by) {
        auto g = std::make_unique<RegGroup>();
        g->H = std::get<0>(kv.first);
        g->smax = std::get<1>(kv.first);
        g->w16 = std::get<2>(kv.first);
        g->ncw = std::get<3>(kv.first);
        g->upper = upper ? 1 : 0;
        g->count = (int)kv.second.size();
        g->smem = smem[kv.first];
        XT_TRY(g->args.alloc(kv.second.size() * sizeof(RegArgs)));
        XT_CUDA(cudaMemcpy(g->args.p, kv.second.data(), kv.second.size() * sizeof(RegArgs),
                           cudaMemcpyHostToDevice));
        XT_TRY(reg_group_prepare(*g));
        out.push_back(std::move(g));
    }
    return XT_OK;
}

// The table of the live systems in `idx` (each with its run's Gram-Schmidt
// passes) and their sweep groups, uploaded before the capture: nothing is
// allocated inside it.
int fused_build(FusedStep& f, const std::vector<int>& idx,
                const std::vector<FlexStepItem>& items, const std::vector<IluRegEntry>& ilu,
                const std::vector<FlexRun>& run, int im, int count)
{
    std::vector<FlexStepItem> all(items), two, one;
    f.sys = idx;
    f.dims = FlexStepDims{};
    f.dims.im = im;
    f.lanes_max = 0;
    double ntot = 0.0;
    for (const FlexStepItem& e : all) ntot += (double)e.n;
    // the dot pass's wave dealt to the systems by size, each at most the
    // items its longest pass has
    for (FlexStepItem& e : all) {
        const int most = df_dot_blocks_max(im, e.dotrows);
        const int share = (int)std::lround(df_dot_wave() * (double)e.n / ntot);
        e.dotblocks = std::max(1, std::min(most, share));
        f.dims.dot_blocks_max = std::max(f.dims.dot_blocks_max, e.dotblocks);
        f.dims.nmax = std::max(f.dims.nmax, e.n);
        f.dims.nodes_max = std::max(f.dims.nodes_max, e.nodes);
        f.dims.rb_max = std::max(f.dims.rb_max, e.rowblocks);
        f.lanes_max = std::max(f.lanes_max, e.lanes);
    }
    for (size_t k = 0; k < idx.size(); ++k) (run[idx[k]].two_pass ? two : one).push_back(all[k]);
    f.nall = (int)all.size();
    f.ntwo = (int)two.size();
    f.none = (int)one.size();
    std::vector<FlexStepItem> tab(all);
    tab.insert(tab.end(), two.begin(), two.end());
    tab.insert(tab.end(), one.begin(), one.end());
    XT_TRY(f.table.alloc(tab.size() * sizeof(FlexStepItem)));
    XT_CUDA(cudaMemcpy(f.table.p, tab.data(), tab.size() * sizeof(FlexStepItem),
                       cudaMemcpyHostToDevice));
    XT_TRY(f.dctl.alloc((size_t)4 * count));
    if (!f.hgat)
        XT_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&f.hgat), sizeof(int) * 4 * (size_t)count,
                              cudaHostAllocDefault));
    XT_TRY(fused_groups(f.gl, ilu, false));
    XT_TRY(fused_groups(f.gu, ilu, true));
    const size_t nev = 2 + f.gl.size() + f.gu.size();
    while (f.gev.size() < nev) {
        cudaEvent_t e = nullptr;
        XT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        f.gev.push_back(e);
    }
    return XT_OK;
}

// The fused step into the capture on `master`: the ILU pre-pass of all, the
// forward sweep groups side by side, then the backward ones, then the
// operator, Gram-Schmidt, rotations and the new basis column of all, and
// the gathered control words.  Group g runs on the stream of the batch's
// g-th entry (distinct streams: there are no more groups than entries).
bool fused_capture(FusedStep& f, xt_batch b, cudaStream_t master)
{
    const FlexStepItem* all = reinterpret_cast<const FlexStepItem*>(f.table.p);
    const FlexStepItem* two = all + f.nall;
    const FlexStepItem* one = two + f.ntwo;
    bool ok = flexb_rhs(all, f.nall, f.q, f.lanes_max, master) == XT_OK;
    size_t ev = 0;
    for (auto* groups : {&f.gl, &f.gu}) {
        const cudaEvent_t fork = f.gev[ev++];
        ok = ok && cudaEventRecord(fork, master) == cudaSuccess;
        for (size_t g = 0; ok && g < groups->size(); ++g) {
            cudaStream_t st = b->sys[f.sys[g]]->sys.stream;
            const cudaEvent_t join = f.gev[ev++];
            ok = cudaStreamWaitEvent(st, fork, 0) == cudaSuccess &&
                 reg_group_launch(*(*groups)[g], f.q, st) == XT_OK &&
                 cudaEventRecord(join, st) == cudaSuccess &&
                 cudaStreamWaitEvent(master, join, 0) == cudaSuccess;
        }
    }
    return ok && flexb_zcopy(all, f.nall, f.dims, master) == XT_OK &&
           kron_nb_batch(all, f.nall, f.q, f.dims, master) == XT_OK &&
           flexb_orth(all, f.nall, two, f.ntwo, one, f.none, f.dims, master) == XT_OK &&
           flexb_givens_scale(all, f.nall, f.dims, master) == XT_OK &&
           flexb_ctl_gather(all, f.nall, f.dctl.p, master) == XT_OK &&
           cudaMemcpyAsync(f.hgat, f.dctl.p, sizeof(int) * 4 * (size_t)f.nall,
                           cudaMemcpyDeviceToHost, master) == cudaSuccess;
}

int batch_run_graph(xt_batch b, const double* const* rhs, double* const* sol, int im, double tol,
                    int maxits, double* stats, int* status)
{
    const int count = (int)b->sys.size();
    const int kRound = batch_round();
    DeviceGuard guard(ctx().device);
    if (guard.err != cudaSuccess) {
        set_error("xt_batch_solve: could not select the library's device");
        return XT_ERR_CUDA;
    }
    std::vector<int> code(count, XT_OK);
    std::vector<std::string> msg(count);
    std::vector<FlexRun> run(count);
    auto fail = [&](int i, int rc) {
        code[i] = rc;
        msg[i] = last_error();
    };
    PinnedInts hctl;
    XT_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&hctl.p), sizeof(int) * 4 * (size_t)count,
                          cudaHostAllocDefault));
    // the host work of the runs (set-up, cycle ends and starts, refinement
    // steps: each with its own host reads) spread over the batch's workers,
    // largest system first; each run is touched by one thread at a time
    const int device = ctx().device;
    bool lost_device = false;
    auto parallel = [&](auto fn) {
        std::atomic<int> next{0};
        std::atomic<bool> lost{false};
        auto work = [&] {
            if (cudaSetDevice(device) != cudaSuccess) {
                lost = true;
                return;
            }
            for (int k; (k = next.fetch_add(1)) < count;) fn(b->order[k]);
        };
        std::vector<std::thread> pool;
        for (int w = 1; w < b->workers; ++w) pool.emplace_back(work);
        work();
        for (auto& t : pool) t.join();
        lost_device = lost_device || lost.load();
    };
    // XTFEM_TRACE: the time of each phase, printed at the end
    const bool tracing = std::getenv("XTFEM_TRACE") != nullptr;
    using clk = std::chrono::steady_clock;
    double t_start = 0, t_capture = 0, t_steps = 0, t_host = 0, t_down = 0;
    int rounds = 0;
    auto since = [](clk::time_point t0) {
        return std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    };
    auto tp = clk::now();
    parallel([&](int i) {
        xt_system_s& h = *b->sys[i];
        System& S = h.sys;
        const size_t n = (size_t)S.p * S.q;
        int rc = system_stream(S);
        if (rc == XT_OK) rc = ensure_vec(S.b64, n);
        if (rc == XT_OK) rc = ensure_vec(S.x64, n);
        if (rc == XT_OK) rc = upload_blocks(h, rhs[i], S.b64.p);
        if (rc == XT_OK) rc = upload_blocks(h, sol[i], S.x64.p);
        if (rc == XT_OK) rc = run[i].start(S, S.b64.p, S.x64.p, im, tol, maxits);
        if (rc != XT_OK) fail(i, rc);
    });
    t_start = since(tp);
    auto live = [&](int i) { return code[i] == XT_OK && !run[i].done; };
    GraphParts gp;
    FusedStep fs;
    std::vector<char> in_graph(count, 0), cap_two(count, 0);
    long long graph_kernels = 0;
    bool tried = false;
    for (int round = 0;; ++round) {
        TraceRange tr("xtfem batch round");
        bool any = false;
        for (int i = 0; i < count; ++i) any = any || live(i);
        if (!any) break;
        // a run that switched to two Gram-Schmidt passes after the capture
        // needs its steps captured again
        if (gp.exec) {
            bool stale = false;
            for (int i = 0; i < count; ++i)
                stale = stale || (live(i) && run[i].two_pass != (bool)cap_two[i]);
            if (stale) {
                cudaGraphExecDestroy(gp.exec);
                gp.exec = nullptr;
                tried = false;
                std::fill(in_graph.begin(), in_graph.end(), 0);
            }
        }
        ++rounds;
        tp = clk::now();
        if (round >= 1 && !tried && batch_graph_on()) {
            tried = true;
            if (!gp.master) {
                XT_CUDA(cudaStreamCreateWithFlags(&gp.master, cudaStreamNonBlocking));
                gp.ev.assign(count + 2, nullptr);
                for (auto& e : gp.ev) XT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            }
            // the live systems of the fused step: node-block operator, the
            // first such system's q
            // largest first (their sweeps, the longest chains, lead the tables)
            std::vector<int> fused;
            std::vector<FlexStepItem> items;
            std::vector<IluRegEntry> ilu;
            fs.q = 0;
            for (int o = 0; batch_fused_on() && o < count; ++o) {
                const int i = b->order[o];
                if (!live(i)) continue;
                System& S = b->sys[i]->sys;
                if ((fs.q && S.q != fs.q) || fused.size() >= 65535)  // entry = blockIdx.y
                    continue;
                FlexStepItem e;
                IluRegEntry r;
                if (!fused_item(S, im, e, r)) continue;
                fs.q = S.q;
                fused.push_back(i);
                items.push_back(e);
                ilu.push_back(r);
            }
            if (!fused.empty() && fused_build(fs, fused, items, ilu, run, im, count) != XT_OK) {
                fused.clear();  // their own branches instead
                fs.sys.clear();
                fs.nall = 0;
                cudaGetLastError();
            }
            std::vector<char> is_fused(count, 0);
            for (int i : fused) is_fused[i] = 1;
            const long long before = xt_launch_count();
            cudaGraph_t g = nullptr;
            bool ok = cudaStreamBeginCapture(gp.master, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            if (ok) {
                ok = cudaEventRecord(gp.ev[count], gp.master) == cudaSuccess;
                if (ok && !fused.empty()) {
                    ok = fused_capture(fs, b, gp.master);
                    for (int i : fused) {
                        in_graph[i] = 1;
                        cap_two[i] = run[i].two_pass;
                    }
                }
                // every other live system: its own step kernels, one branch
                for (int i = 0; ok && i < count; ++i) {
                    if (!live(i) || is_fused[i]) continue;
                    System& S = b->sys[i]->sys;
                    ok = cudaStreamWaitEvent(S.stream, gp.ev[count], 0) == cudaSuccess &&
                         run[i].issue(1, nullptr) == XT_OK &&
                         cudaMemcpyAsync(hctl.p + 4 * i, S.fctl.p, 4 * sizeof(int),
                                         cudaMemcpyDeviceToHost, S.stream) == cudaSuccess &&
                         cudaEventRecord(gp.ev[i], S.stream) == cudaSuccess &&
                         cudaStreamWaitEvent(gp.master, gp.ev[i], 0) == cudaSuccess;
                    in_graph[i] = 1;
                    cap_two[i] = run[i].two_pass;
                }
                const cudaError_t e = cudaStreamEndCapture(gp.master, &g);
                ok = ok && e == cudaSuccess && g != nullptr &&
                     cudaGraphInstantiate(&gp.exec, g, 0) == cudaSuccess;
            }
            if (g) cudaGraphDestroy(g);
            graph_kernels = xt_launch_count() - before;
            if (!ok) {  // issue the rounds directly instead
                if (gp.exec) cudaGraphExecDestroy(gp.exec);
                gp.exec = nullptr;
                cudaGetLastError();
                std::fill(in_graph.begin(), in_graph.end(), 0);
                fs.sys.clear();
                fs.nall = 0;
            }
            note_launches((int)-graph_kernels);  // captured, not run: counted per replay
            t_capture += since(tp);
            tp = clk::now();
        }
        if (gp.exec) {
            for (int k = 0; k < kRound; ++k) XT_CUDA(cudaGraphLaunch(gp.exec, gp.master));
            XT_CUDA(cudaStreamSynchronize(gp.master));
            note_launches((int)(graph_kernels * kRound));
            for (int k = 0; k < fs.nall; ++k)
                std::memcpy(hctl.p + 4 * fs.sys[k], fs.hgat + 4 * k, 4 * sizeof(int));
            for (int i = 0; i < count; ++i)
                if (live(i) && !in_graph[i]) {
                    set_error("xt_batch_solve: a running system is missing from the round graph");
                    fail(i, XT_ERR_STATE);
                }
        } else {
            for (int i = 0; i < count; ++i) {
                if (!live(i)) continue;
                System& S = b->sys[i]->sys;
                int rc = run[i].issue(kRound, nullptr);
                if (rc == XT_OK &&
                    cudaMemcpyAsync(hctl.p + 4 * i, S.fctl.p, 4 * sizeof(int),
                                    cudaMemcpyDeviceToHost, S.stream) != cudaSuccess) {
                    set_error("xt_batch_solve: control read failed");
                    rc = XT_ERR_CUDA;
                }
                if (rc != XT_OK) fail(i, rc);
            }
            for (int i = 0; i < count; ++i)
                if (live(i) && cudaStreamSynchronize(b->sys[i]->sys.stream) != cudaSuccess) {
                    set_error("xt_batch_solve: stream synchronisation failed");
                    fail(i, XT_ERR_CUDA);
                }
        }
        t_steps += since(tp);
        tp = clk::now();
        parallel([&](int i) {
            if (!live(i)) return;
            const int rc = run[i].advance(hctl.p + 4 * i);
            if (rc != XT_OK) fail(i, rc);
        });
        t_host += since(tp);
        if (lost_device) break;
    }
    tp = clk::now();
    parallel([&](int i) {
        if (code[i] != XT_OK) return;
        xt_system_s& h = *b->sys[i];
        const int d = download_blocks(h, h.sys.x64.p, sol[i]);
        if (d != XT_OK) fail(i, d);
    });
    t_down = since(tp);
    if (tracing)
        std::fprintf(stderr,
                     "[xtfem] batch lockstep: %d systems, %d rounds of %d steps, graph %s "
                     "(%lld kernels, %d systems in batched kernels); ms: start %.1f, capture "
                     "%.1f, steps %.1f, host between rounds %.1f, download %.1f\n",
                     count, rounds, kRound, gp.exec ? "yes" : "no", graph_kernels, fs.nall,
                     t_start, t_capture, t_steps, t_host, t_down);
    if (lost_device) {
        set_error("xt_batch_solve: worker thread could not select the device");
        return XT_ERR_CUDA;
    }
    int rc = XT_OK;
    for (int i = 0; i < count; ++i) {
        if (stats && code[i] == XT_OK) {
            const GmresStats& st = run[i].st;
            double* o = stats + (size_t)6 * i;
            o[0] = st.its;
            o[1] = st.cycles;
            o[2] = st.outer;
            o[3] = st.ierr;
            o[4] = st.relres;
            o[5] = st.est;
        }
        if (status) status[i] = code[i];
        if (code[i] != XT_OK && rc == XT_OK) {
            rc = code[i];
            set_error("xt_batch_solve: system " + std::to_string(i) + ": " + msg[i]);
        }
    }
    return rc;
}

int batch_run(xt_batch b, const double* const* rhs, double* const* sol, int im, double tol,
              int maxits, int precision, double inner_tol, double* stats, int* status)
{
    const int count = (int)b->sys.size();
    // XTFEM_BATCH_LOCKSTEP=0: mode 2 on the thread pool below as well
    const char* ls = std::getenv("XTFEM_BATCH_LOCKSTEP");
    if (precision == 2 && im >= 1 && im <= kFlexdMaxIm && (!ls || std::atoi(ls) != 0))
        return batch_run_graph(b, rhs, sol, im, tol, maxits, stats, status);
    std::vector<int> code(count, XT_OK);
    std::vector<std::string> msg(count);
    std::atomic<int> next{0};
    const int device = ctx().device;
    // the caller's thread runs work() too: it gets its current device back
    DeviceGuard guard(device);
    if (guard.err != cudaSuccess) {
        set_error("xt_batch_solve: could not select the library's device");
        return XT_ERR_CUDA;
    }
    auto work = [&] {
        if (cudaSetDevice(device) != cudaSuccess) return;
        for (int k; (k = next.fetch_add(1)) < count;) {
            const int i = b->order[k];
            code[i] = system_solve_host(b->sys[i], rhs[i], sol[i], im, tol, maxits, precision,
                                        inner_tol, stats ? stats + (size_t)6 * i : nullptr);
            if (code[i] != XT_OK) msg[i] = last_error();
        }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < b->workers; ++w) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    if (next.load() < count) {  // a worker could not select the device
        set_error("xt_batch_solve: worker thread could not select the device");
        return XT_ERR_CUDA;
    }
    int rc = XT_OK;
    for (int i = 0; i < count; ++i) {
        if (status) status[i] = code[i];
        if (code[i] != XT_OK && rc == XT_OK) {
            rc = code[i];
            set_error("xt_batch_solve: system " + std::to_string(i) + ": " + msg[i]);
        }
    }
    return rc;
}
}  // namespace


// ------------------------------------------------- Fortran entry points
void kronspmv_(const double* a, const double* b, const int* q, const int* ki, const int* kj,
               const double* kv, const int* mi, const int* mj, const double* mv, const int* p,
               const double* x, double* y)
{
    (void)do_spmv(a, b, 1.0, 0.0, *q, ki, kj, kv, mi, mj, mv, *p, x, y);
}

void kronspgemv_(const double* a, const double* b, const double* alpha, const double* beta,
                 const int* q, const int* ki, const int* kj, const double* kv, const int* mi,
                 const int* mj, const double* mv, const int* p, const double* x, double* y)
{
    (void)do_spmv(a, b, *alpha, *beta, *q, ki, kj, kv, mi, mj, mv, *p, x, y);
}

void kronlusol_(const double* a, const int* q, const double* alu, const int* jlu, const int* ju,
                const int* p, const double* x, double* y)
{
    if (ensure_init() != XT_OK) return;
    if (!q || !p || *q < 1 || *q > 8 || *p <= 0) { set_error("kronlusol_: bad sizes"); return; }
    xt_system_s h;
    h.sys.p = *p;
    h.sys.q = *q;
    if (h.sys.A.alloc(64) != XT_OK || h.sys.Ainv.alloc(64) != XT_OK) return;
    if (get_ilu(alu, jlu, ju, *p, h.sys.ilu) != XT_OK) return;
    (void)xt_system_lusol(&h, a, x, y);
}

// kronpgmres_'s residual history for the caller's Fortran shim (one per
// host thread: each thread drives its own solves)
static thread_local std::vector<double> t_gmres_log;

int xt_gmres_log(double* rel, int cap)
{
    const int n = (int)t_gmres_log.size();
    for (int k = 0; rel && k < cap && k < n; ++k) rel[k] = t_gmres_log[k];
    return n;
}

void kronpgmres_(const double* a, const double* b, const int* q, const int* ki, const int* kj,
                 const double* kv, const int* mi, const int* mj, const double* mv, const int* p,
                 const double* alu, const int* jlu, const int* ju, double* rhs, double* sol,
                 const int* im, const double* eps, const int* maxits, const int* iout, int* ierr)
{
    const bool keep_log = iout && *iout >= 0;
    if (keep_log) t_gmres_log.clear();
    if (!ierr) return;
    *ierr = XT_ERR_ARG;
    if (!q || !p || !im || !eps || !maxits) { set_error("kronpgmres_: null argument"); return; }
    std::unique_ptr<xt_system_s> tmp;
    xt_system_s* h = nullptr;
    int st = get_system(ki, kj, kv, mi, mj, mv, *p, *q, tmp, h);
    if (st != XT_OK) { *ierr = st; return; }
    st = get_ilu(alu, jlu, ju, *p, h->sys.ilu);
    if (st != XT_OK) { *ierr = st; return; }
    st = system_set_temporal(h->sys, a, b);
    if (st != XT_OK) { *ierr = st; return; }
    int its = 0, e = 0;
    if (!keep_log) {
        st = xt_system_gmres(h, rhs, sol, *im, *eps, *maxits, &its, &e, nullptr, nullptr, 0);
        *ierr = (st != XT_OK) ? st : e;
        return;
    }
    // the its = 0 line: ||rhs - A sol|| / ||rhs|| before the first cycle
    const size_t n = (size_t)(*p) * (*q);
    double ro0 = 0.0, ro = 0.0;
    for (size_t k = 0; k < n; ++k) ro0 += rhs[k] * rhs[k];
    bool zero_start = true;
    for (size_t k = 0; k < n && zero_start; ++k) zero_start = sol[k] == 0.0;
    if (zero_start) {
        ro = ro0;
    } else {
        std::vector<double> r(rhs, rhs + n);
        st = xt_system_apply(h, a, b, -1.0, 1.0, sol, r.data());
        if (st != XT_OK) { *ierr = st; return; }
        for (size_t k = 0; k < n; ++k) ro += r[k] * r[k];
    }
    std::vector<double> hist((size_t)std::max(*maxits, 0) + (size_t)std::max(*im, 0) + 1, 0.0);
    st = xt_system_gmres(h, rhs, sol, *im, *eps, *maxits, &its, &e, nullptr, hist.data(),
                         (int)hist.size());
    *ierr = (st != XT_OK) ? st : e;
    if (st != XT_OK) return;
    t_gmres_log.assign(1, std::sqrt(ro) / std::sqrt(ro0));
    t_gmres_log.insert(t_gmres_log.end(), hist.begin(),
                       hist.begin() + std::min((size_t)std::max(its, 0), hist.size()));
}

void chkelesta_(const int* nn, const int* ne, const int* nnse, const int* ngpe, const double* Dc,
                const double* D, int* elesta, int* gpsta, int* nef, int* nefail)
{
    (void)nn;
    (void)nnse;
    if (!ne || !ngpe || !Dc || !D || !elesta || !gpsta || !nef || !nefail) return;
    if (ensure_init() != XT_OK) return;
    const int E = *ne, G = *ngpe;
    if (E <= 0 || G <= 0) { *nef = 0; return; }
    cudaStream_t s = ctx().stream;
    DBuf<double> dD;
    DBuf<int> de, dg, df, dn;
    if (dD.upload(D, (size_t)E * G, s) || de.upload(elesta, E, s) || dg.upload(gpsta, (size_t)E * G, s) ||
        df.alloc(E) || dn.alloc(1))
        return;
    if (chkelesta_device(E, G, *Dc, dD.p, de.p, dg.p, df.p, dn.p, s) != XT_OK) return;
    cudaMemcpyAsync(elesta, de.p, sizeof(int) * E, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(gpsta, dg.p, sizeof(int) * (size_t)E * G, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(nefail, df.p, sizeof(int) * E, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(nef, dn.p, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
}

int xt_damage(int ne, int nn, int ndofn, int nnse, int nnte, int ngpe, int ncmp, int nip,
              const int* nodes, const double* Nx, const double* Ny, const double* Nz,
              const double* Nt, const double* sol, const double* ym, const double* nu,
              double* eps_old, double* eps_pl, double* sig_eff, double* sig_back, double* p,
              double* D, double* ws, double* del_po, double* sig_d)
{
    XT_TRY(ensure_init());
    if (ne <= 0 || nn <= 0 || ngpe <= 0 || nip < 0 || !nodes || !Nx || !Ny || !Nz || !Nt || !sol ||
        !ym || !nu || !eps_old || !eps_pl || !sig_eff || !sig_back || !p || !D || !ws ||
        !del_po || !sig_d) {
        set_error("xt_damage: bad arguments");
        return XT_ERR_ARG;
    }
    if (ndofn != 3 || nnte != 3 || ncmp != 6 || nnse < 1 || nnse > 8) {
        set_error("xt_damage: the C3D8 update needs ndofn=3, nnte=3, ncmp=6, nnse<=8");
        return XT_ERR_ARG;
    }
    const size_t ngp = (size_t)ngpe * ne;
    for (size_t i = 0; i < ngp * nnse; ++i)
        if (nodes[i] < 1 || nodes[i] > nn) {
            set_error("xt_damage: node id out of range");
            return XT_ERR_ARG;
        }
    cudaStream_t s = ctx().stream;
    DBuf<int> dnodes;
    DBuf<double> dNx, dNy, dNz, dNt, dsol, dym, dnu, deo, dep, dse, dsb, dp, dD, dws, ddp, dsd;
    DBuf<float> dNt32, ntmax;
    const size_t nsol = (size_t)2 * nnte * nn * ndofn, nnt = (size_t)2 * nnte * nip;
    XT_TRY(dnodes.upload(nodes, ngp * nnse, s));
    XT_TRY(dNx.upload(Nx, ngp * nnse, s));
    XT_TRY(dNy.upload(Ny, ngp * nnse, s));
    XT_TRY(dNz.upload(Nz, ngp * nnse, s));
    XT_TRY(dNt.upload(Nt, nnt ? nnt : 1, s));
    XT_TRY(dNt32.alloc(nnt ? nnt : 1));
    XT_TRY(ntmax.alloc(8));
    XT_TRY(to_f32(dNt.p, dNt32.p, nnt, s));
    XT_TRY(dsol.upload(sol, nsol, s));
    XT_TRY(dym.upload(ym, ngp, s));
    XT_TRY(dnu.upload(nu, ngp, s));
    XT_TRY(deo.upload(eps_old, ngp * ncmp, s));
    XT_TRY(dep.upload(eps_pl, ngp * ncmp, s));
    XT_TRY(dse.upload(sig_eff, ngp * ncmp, s));
    XT_TRY(dsb.upload(sig_back, ngp * ncmp, s));
    XT_TRY(dp.upload(p, ngp, s));
    XT_TRY(dD.upload(D, ngp, s));
    XT_TRY(dws.upload(ws, ngp, s));
    XT_TRY(ddp.upload(del_po, ngp, s));
    XT_TRY(dsd.upload(sig_d, ngp, s));
    DamageArgs a{};
    a.ngp = (int)ngp; a.nn = nn; a.ndofn = ndofn; a.nnse = nnse; a.nnte = nnte; a.ncmp = ncmp;
    a.nip = nip;
    a.nodes = dnodes.p; a.Nx = dNx.p; a.Ny = dNy.p; a.Nz = dNz.p; a.Nt = dNt.p; a.Nt32 = dNt32.p;
    a.sol = dsol.p; a.ym = dym.p; a.nu = dnu.p;
    a.eps_old = deo.p; a.eps_pl = dep.p; a.sig_eff = dse.p; a.sig_back = dsb.p;
    a.p = dp.p; a.D = dD.p; a.ws = dws.p; a.del_po = ddp.p; a.sig_d = dsd.p;
    a.gpsta = nullptr; a.counters = nullptr; a.ntmax = ntmax.p;
    XT_TRY(damage_update(a, s));
    auto back = [&](double* h, const DBuf<double>& d, size_t n) -> int {
        XT_CUDA(cudaMemcpyAsync(h, d.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
        return XT_OK;
    };
    XT_TRY(back(eps_old, deo, ngp * ncmp));
    XT_TRY(back(eps_pl, dep, ngp * ncmp));
    XT_TRY(back(sig_eff, dse, ngp * ncmp));
    XT_TRY(back(sig_back, dsb, ngp * ncmp));
    XT_TRY(back(p, dp, ngp));
    XT_TRY(back(D, dD, ngp));
    XT_TRY(back(ws, dws, ngp));
    XT_TRY(back(del_po, ddp, ngp));
    XT_TRY(back(sig_d, dsd, ngp));
    XT_CUDA(cudaStreamSynchronize(s));
    return XT_OK;
}

int xt_damage_device(int ne, int nn, int ndofn, int nnse, int nnte, int ngpe, int ncmp, int nip,
                     const int* nodes, const double* Nx, const double* Ny, const double* Nz,
                     const double* Nt, const double* sol, const double* ym, const double* nu,
                     double* eps_old, double* eps_pl, double* sig_eff, double* sig_back,
                     double* p, double* D, double* ws, double* del_po, double* sig_d,
                     unsigned long long* counts)
{
    // Host-side checks first: they need no device and allocate nothing.
    if (ne <= 0 || nn <= 0 || ngpe <= 0 || nip < 0 || !nodes || !Nx || !Ny || !Nz || !Nt || !sol ||
        !ym || !nu || !eps_old || !eps_pl || !sig_eff || !sig_back || !p || !D || !ws ||
        !del_po || !sig_d) {
        set_error("xt_damage_device: bad arguments");
        return XT_ERR_ARG;
    }
    if (ndofn != 3 || nnte != 3 || ncmp != 6 || nnse < 1 || nnse > 8) {
        set_error("xt_damage_device: the C3D8 update needs ndofn=3, nnte=3, ncmp=6, nnse<=8");
        return XT_ERR_ARG;
    }
    if (nip > kDamageStaticMaxNip) {
        set_error("xt_damage_device: nip = " + std::to_string(nip) +
                  " exceeds the static scratch of this entry point (at most " +
                  std::to_string(kDamageStaticMaxNip) + " steps per call); use xt_damage");
        return XT_ERR_ARG;
    }
    if ((long long)ngpe * ne > 2147483647LL) {
        set_error("xt_damage_device: more than 2^31-1 Gauss points");
        return XT_ERR_ARG;
    }
    XT_TRY(ensure_init());
    // The launches go to the library's stream, which belongs to the
    // library's device: make that device current for this call (the
    // caller's thread may have another one current) and give the caller's
    // back on return.
    DeviceGuard guard(ctx().device);
    XT_CUDA(guard.err);
    // The inputs and the state were written by the caller's own kernels, on
    // streams that nothing here orders after (the library's stream is
    // non-blocking).  Wait for all work on the device first; this allocates
    // nothing.
    XT_CUDA(cudaDeviceSynchronize());
    cudaStream_t s = ctx().stream;
    float *nt32 = nullptr, *ntmax = nullptr;
    unsigned long long* counters = nullptr;
    XT_TRY(damage_static_scratch(ctx().device, &nt32, &ntmax, &counters));
    // the step counters accumulate with atomics: they must start at zero
    XT_CUDA(cudaMemsetAsync(counters, 0, 3 * sizeof(unsigned long long), s));
    if (nip > 0) XT_TRY(to_f32(Nt, nt32, (size_t)2 * nnte * nip, s));
    DamageArgs a{};
    a.ngp = ngpe * ne; a.nn = nn; a.ndofn = ndofn; a.nnse = nnse; a.nnte = nnte; a.ncmp = ncmp;
    a.nip = nip;
    a.nodes = nodes; a.Nx = Nx; a.Ny = Ny; a.Nz = Nz; a.Nt = Nt; a.Nt32 = nt32;
    a.sol = sol; a.ym = ym; a.nu = nu;
    a.eps_old = eps_old; a.eps_pl = eps_pl; a.sig_eff = sig_eff; a.sig_back = sig_back;
    a.p = p; a.D = D; a.ws = ws; a.del_po = del_po; a.sig_d = sig_d;
    a.gpsta = nullptr; a.counters = counters; a.ntmax = ntmax;
    XT_TRY(damage_update(a, s));
    if (counts)
        XT_CUDA(cudaMemcpyAsync(counts, counters, 3 * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, s));
    XT_CUDA(cudaStreamSynchronize(s));
    return XT_OK;
}

void kokkos_host_(int rank, int ne, int nn, int ndofn, int nnse, int nnte, int ngpe, int ncmp,
                  int nip, int* nodes, double* Nx, double* Ny, double* Nz, double* Nt,
                  double* sol, double* ym, double* nu, double* eps_old, double* eps_pl,
                  double* sig_eff, double* sig_back, double* p, double* D, double* ws,
                  double* del_po, double* sig_d)
{
    (void)rank;
    (void)xt_damage(ne, nn, ndofn, nnse, nnte, ngpe, ncmp, nip, nodes, Nx, Ny, Nz, Nt, sol, ym,
                    nu, eps_old, eps_pl, sig_eff, sig_back, p, D, ws, del_po, sig_d);
}

}  // extern "C"
