// host_ilut.cpp -- ILUT(lfil, droptol) factorisation on the host in FP64.
//
// The GPU path applies the factor; computing it stays on the host, as in the
// reference, whose solver entry points take the SPARSKIT MSR arrays
// alu/jlu/ju (src/kronecker.f90:130-178).  The algorithm is Saad's ILUT
// (src/ilut.f:152-495): a row-by-row IKJ elimination in ascending column
// order with a dual dropping rule, then a quick-split selection of the
// largest entries of each L and U row (src/ilut.f:2487-2545).  The factor
// must come out identical to the reference's (same entries, same order in
// each row), so the steps below are the published algorithm's steps:
//   * the multiplier test is |w_j * u_jj^-1| <= droptol (absolute);
//   * U entries are kept when |u| > droptol * tnorm (tnorm = mean |a| of
//     the row);
//   * L keeps at most lfil entries, U at most lfil-1 off-diagonal entries;
//   * a zero pivot is replaced by (1e-4 + droptol) * tnorm where 1e-4 is the
//     reference's single-precision literal.
//
// Rows are pipelined over host threads.  Row i eliminates with earlier rows
// in ascending column order, so it needs its nearest predecessors last: a
// thread works on row i while rows i-1, i-2, ... are still being finished
// by other threads, and waits on a row's done flag only when it reaches
// that row.  Every row does the same arithmetic in the same order whatever
// the thread count, so the factor is bit-for-bit the serial one; a failing
// row stops the rows after it, and the lowest failing row's code is the
// result, as in the reference, which stops at its first failing row.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <exception>
#include <functional>
#include <memory>
#include <mutex>
#include <system_error>
#include <thread>
#include <vector>

#include "host_sparse.h"

namespace xt {

namespace {

// Partial quick-sort of v[0..n) by magnitude, descending, until position
// cut-1 (0-based) separates the cut largest entries; idx follows v.
void split_largest(double* v, int* idx, int n, int cut)
{
    int lo = 0, hi = n - 1;
    const int target = cut - 1;
    if (target < lo || target > hi) return;
    for (;;) {
        int mid = lo;
        const double key = std::fabs(v[mid]);
        for (int j = lo + 1; j <= hi; ++j)
            if (std::fabs(v[j]) > key) {
                ++mid;
                std::swap(v[mid], v[j]);
                std::swap(idx[mid], idx[j]);
            }
        std::swap(v[mid], v[lo]);
        std::swap(idx[mid], idx[lo]);
        if (mid == target) return;
        if (mid > target) hi = mid - 1;
        else lo = mid + 1;
    }
}

}  // namespace

namespace {

// Append-only storage of finished rows for one thread: blocks never move,
// so other threads can read a finished row while more rows are appended.
struct RowStore {
    std::vector<std::unique_ptr<double[]>> vals;
    std::vector<std::unique_ptr<int[]>> cols;
    size_t used = 0, cap = 0, block;
    explicit RowStore(size_t b) : block(b) {}
    void take(size_t len, double*& v, int*& c)
    {
        // a block exists before the first row is stored, even an empty row
        if (vals.empty() || used + len > cap) {
            vals.emplace_back(new double[block]);
            cols.emplace_back(new int[block]);
            used = 0;
            cap = block;
        }
        v = vals.back().get() + used;
        c = cols.back().get() + used;
        used += len;
    }
};

// One finished row: L multipliers and U off-diagonals (0-based columns) in
// the order they are stored, and the inverted pivot.
struct RowOut {
    const double* lv = nullptr;
    const int* lc = nullptr;
    const double* uv = nullptr;
    const int* uc = nullptr;
    int nl = 0, nu = 0;
    double dinv = 0.0;
};

struct Shared {
    const Csr& A;
    int n, lfil;
    double droptol;
    std::vector<RowOut> rows;
    std::unique_ptr<std::atomic<int>[]> done;
    std::atomic<int> first_fail;
    std::vector<int> code;  // error code of a failing row
    std::mutex error_m;     // an exception of a thread (allocation), for the caller
    std::exception_ptr error;
    int first_row = 0;           // rows below it are taken from a previous factor
    std::vector<int> prev_cols;  // that factor's columns, 0-based
    Shared(const Csr& a, int lf, double dt)
        : A(a), n(a.n), lfil(lf), droptol(dt), rows(a.n), done(new std::atomic<int>[a.n]),
          first_fail(a.n), code(a.n, 0)
    {
        for (int i = 0; i < n; ++i) done[i].store(0, std::memory_order_relaxed);
    }
    // Rows [0, r0) of the factor from prev (SPARSKIT MSR of the same order),
    // marked done before any thread starts.
    void reuse(const Msr& prev, int r0)
    {
        const size_t nz = prev.jlu.size();
        prev_cols.assign(nz, 0);
        for (size_t k = (size_t)n + 1; k < nz; ++k) prev_cols[k] = prev.jlu[k] - 1;
        for (int i = 0; i < r0; ++i) {
            RowOut& O = rows[i];
            const int b = prev.jlu[i] - 1, m = prev.ju[i] - 1, e = prev.jlu[i + 1] - 1;
            O.lv = prev.alu.data() + b; O.lc = prev_cols.data() + b; O.nl = m - b;
            O.uv = prev.alu.data() + m; O.uc = prev_cols.data() + m; O.nu = e - m;
            O.dinv = prev.alu[i];
            done[i].store(1, std::memory_order_relaxed);
        }
        first_row = r0;
    }
    void fail(int i, int c)
    {
        code[i] = c;
        int cur = first_fail.load();
        while (i < cur && !first_fail.compare_exchange_weak(cur, i)) {}
    }
};

// Rows first, first + stride, ... of the factor, stored in `store` (which
// outlives the call: the rows are read again when the factor is assembled).
// Returns when its rows are done or a row at or below one of its rows has
// failed.
void factor_rows(Shared& S, RowStore& store, int first, int stride)
{
    const int n = S.n, lfil = S.lfil;
    const double droptol = S.droptol;
    const Csr& A = S.A;
    // Row workspace.  Slots [0, lenl) hold the L candidates (column, value),
    // slot i the diagonal and slots (i, i+lenu) the U part; where[c] is the
    // slot of column c in the current row, or -1.
    std::vector<double> w(n + 1);
    std::vector<int> col(n + 1), where(n, -1);
    // L candidates waiting for elimination, as a bit set of columns read
    // upward: the reference picks the smallest remaining column by a linear
    // scan (and swaps it forward), which is the same order, and every fill-in
    // lies above the column being eliminated, so one upward pass over the
    // words below i visits them all.  The kept multipliers go to their own
    // arrays in that order, where the reference compacts them to the front
    // of the row.  Same factor, without the quadratic scan.
    std::vector<unsigned long long> pending((size_t)n / 64 + 2, 0ull);
    std::vector<double> wl(n + 1);
    std::vector<int> cl(n + 1);
    for (int i = first; i < n; i += stride) {
        if (i < S.first_row) continue;  // taken from the previous factor
        if (S.first_fail.load(std::memory_order_relaxed) < i) return;
        const int b = A.ia[i] - 1, e = A.ia[i + 1] - 1;
        double tnorm = 0.0;
        for (int k = b; k < e; ++k) tnorm += std::fabs(A.a[k]);
        if (tnorm == 0.0) { S.fail(i, -5); return; }
        tnorm /= (double)(float)(e - b);
        int lenl = 0, lenu = 1;
        col[i] = i;
        w[i] = 0.0;
        where[i] = i;
        int lo = i;  // lowest candidate column
        for (int k = b; k < e; ++k) {
            const int c = A.ja[k] - 1;
            if (c < i) {
                col[lenl] = c; w[lenl] = A.a[k]; where[c] = lenl; ++lenl;
                pending[(size_t)c >> 6] |= 1ull << (c & 63);
                if (c < lo) lo = c;
            } else if (c == i) {
                w[i] = A.a[k];
            } else {
                const int sl = i + lenu;
                col[sl] = c; w[sl] = A.a[k]; where[c] = sl; ++lenu;
            }
        }
        // eliminate with earlier rows in ascending column order
        int kept = 0;
        size_t wd = (size_t)lo >> 6;
        const size_t wend = ((size_t)i >> 6) + 1;
        for (;;) {
            while (wd < wend && pending[wd] == 0) ++wd;
            if (wd >= wend) break;
            const int r = (int)(wd << 6) + __builtin_ctzll(pending[wd]);
            pending[wd] &= pending[wd] - 1;  // clear the lowest set bit
            // row r finished (by this thread or another)?
            for (int spins = 0; S.done[r].load(std::memory_order_acquire) == 0; ++spins) {
                if (S.first_fail.load(std::memory_order_relaxed) < i) return;
                if (spins > 64) std::this_thread::yield();
            }
            const RowOut& R = S.rows[r];
            const double fact = w[where[r]] * R.dinv;
            where[r] = -1;
            if (std::fabs(fact) <= droptol) continue;
            for (int k = 0; k < R.nu; ++k) {
                const double sv = fact * R.uv[k];
                const int c = R.uc[k];
                const int slot = where[c];
                if (c >= i) {
                    if (slot < 0) {
                        if (lenu + 1 > n) { S.fail(i, -1); return; }
                        const int ns = i + lenu;
                        col[ns] = c; where[c] = ns; w[ns] = -sv; ++lenu;
                    } else {
                        w[slot] -= sv;
                    }
                } else {
                    if (slot < 0) {
                        if (lenl + 1 > n) { S.fail(i, -1); return; }
                        col[lenl] = c; where[c] = lenl; w[lenl] = -sv; ++lenl;
                        pending[(size_t)c >> 6] |= 1ull << (c & 63);
                    } else {
                        w[slot] -= sv;
                    }
                }
            }
            wl[kept] = fact;
            cl[kept] = r;
            ++kept;
        }
        for (int k = 0; k < lenu; ++k) where[col[i + k]] = -1;
        RowOut& O = S.rows[i];
        // L row: the lfil largest multipliers
        const int nl = kept < lfil ? kept : lfil;
        split_largest(wl.data(), cl.data(), kept, nl);
        // U row: threshold, then the lfil-1 largest off-diagonals
        int nu = 0;
        for (int k = 1; k < lenu; ++k)
            if (std::fabs(w[i + k]) > droptol * tnorm) {
                ++nu;
                w[i + nu] = w[i + k];
                col[i + nu] = col[i + k];
            }
        const int lenu2 = nu + 1;
        const int keep = lenu2 < lfil ? lenu2 : lfil;
        split_largest(w.data() + i + 1, col.data() + i + 1, lenu2 - 1, keep);
        double* v;
        int* c;
        store.take((size_t)nl + (keep > 1 ? keep - 1 : 0), v, c);
        for (int k = 0; k < nl; ++k) { v[k] = wl[k]; c[k] = cl[k]; }
        O.lv = v; O.lc = c; O.nl = nl;
        for (int k = 1; k <= keep - 1; ++k) { v[nl + k - 1] = w[i + k]; c[nl + k - 1] = col[i + k]; }
        O.uv = v + nl; O.uc = c + nl; O.nu = keep > 1 ? keep - 1 : 0;
        if (w[i] == 0.0) w[i] = ((double)0.0001f + droptol) * tnorm;
        O.dinv = 1.0 / w[i];
        S.done[i].store(1, std::memory_order_release);
    }
}

// factor_rows for a thread: an exception (an allocation that failed) is
// kept for the calling thread, which rethrows it after the join, and stops
// the other threads; it must not leave a thread function.
void factor_rows_kept(Shared& S, RowStore& store, int first, int stride)
{
    try {
        factor_rows(S, store, first, stride);
    } catch (...) {
        {
            std::lock_guard<std::mutex> g(S.error_m);
            if (!S.error) S.error = std::current_exception();
        }
        S.first_fail.store(-1);
    }
}

int ilut_threads(int n)
{
    if (const char* e = std::getenv("XTFEM_ILUT_THREADS")) {
        const int t = std::atoi(e);
        if (t >= 1) return t < 64 ? t : 64;
    }
    if (n < 16384) return 1;
    const unsigned hw = std::thread::hardware_concurrency();
    return hw == 0 ? 1 : (int)(hw < 16 ? hw : 16);
}

}  // namespace

namespace {

// SPARSKIT MSR, 1-based: alu(1..n) inverted pivots, alu(n+1) unused, rows'
// L then U entries from position n+2; jlu(1..n+1) row starts, jlu(k >= n+2)
// columns; ju(i) the start of row i's U entries.  After a failure only the
// rows before the failing one are filled in (ju has that many entries), for
// a caller that checks storage row by row.
void assemble(const Shared& S, Msr& F)
{
    const int n = S.n;
    const int f = S.first_fail.load();
    size_t tot = 0;
    for (int i = 0; i < f; ++i) tot += (size_t)S.rows[i].nl + S.rows[i].nu;
    F.n = n;
    F.alu.assign((size_t)n + 1 + tot, 0.0);
    F.jlu.assign((size_t)n + 1 + tot, 0);
    F.ju.assign(f, 0);
    size_t pos = (size_t)n + 2;
    for (int i = 0; i < f; ++i) {
        const RowOut& R = S.rows[i];
        F.jlu[i] = (int)pos;
        for (int k = 0; k < R.nl; ++k, ++pos) { F.alu[pos - 1] = R.lv[k]; F.jlu[pos - 1] = R.lc[k] + 1; }
        F.ju[i] = (int)pos;
        for (int k = 0; k < R.nu; ++k, ++pos) { F.alu[pos - 1] = R.uv[k]; F.jlu[pos - 1] = R.uc[k] + 1; }
        F.alu[i] = R.dinv;
    }
    F.jlu[f] = (int)pos;
}

// The factor on T threads, assembled into F with its code in ierr; false
// when a thread could not be started (the threads already running are
// stopped and joined first, and F is left alone).
bool ilut_on(const Csr& A, int lfil, double droptol, int T, Msr& F, int& ierr,
             const Msr* prev, int r0)
{
    const int n = A.n;
    Shared S(A, lfil, droptol);
    if (prev && r0 > 0) S.reuse(*prev, r0);
    // one row store per thread; blocks hold at least one row's L and U
    const size_t row_max = (size_t)(lfil < n ? lfil : n) * 2 + 2;
    std::vector<RowStore> stores;
    stores.reserve(T);
    for (int t = 0; t < T; ++t) stores.emplace_back(row_max > 65536 ? row_max : 65536);
    if (T <= 1) {
        factor_rows_kept(S, stores[0], 0, 1);
    } else {
        std::vector<std::thread> pool;
        pool.reserve(T - 1);
        bool all = true;
        try {
            for (int t = 1; t < T; ++t)
                pool.emplace_back(factor_rows_kept, std::ref(S), std::ref(stores[t]), t, T);
        } catch (const std::system_error&) {
            all = false;
            S.first_fail.store(-1);  // every row is "after" it: the started threads stop
        }
        if (all) factor_rows_kept(S, stores[0], 0, T);
        for (auto& th : pool) th.join();
        if (S.error) std::rethrow_exception(S.error);
        if (!all) return false;
    }
    if (S.error) std::rethrow_exception(S.error);
    assemble(S, F);
    const int f = S.first_fail.load();
    ierr = f < n ? S.code[f] : 0;
    return true;
}

}  // namespace

// factorisations running in this process: concurrent callers (specimens
// set up side by side) each take one thread instead of all of them
static std::atomic<int> g_running{0};

std::vector<int> ilu_block_bounds(int n, int g, int blocks)
{
    if (g < 1 || n % g) g = 1;
    const long long ng = n / g;
    blocks = std::max(1, std::min<int>(blocks, (int)std::max<long long>(ng, 1)));
    std::vector<int> b(blocks + 1);
    for (int k = 0; k <= blocks; ++k) b[k] = (int)(ng * k / blocks) * g;
    return b;
}

Csr block_diagonal(const Csr& A, int g, int blocks)
{
    if (blocks <= 1) return A;
    const std::vector<int> bd = ilu_block_bounds(A.n, g, blocks);
    Csr B;
    B.n = A.n;
    B.ia.assign(A.n + 1, 1);
    B.ja.reserve(A.ja.size());
    B.a.reserve(A.a.size());
    int blk = 0;
    for (int r = 0; r < A.n; ++r) {
        while (r >= bd[blk + 1]) ++blk;
        for (int k = A.ia[r] - 1; k < A.ia[r + 1] - 1; ++k) {
            const int c = A.ja[k] - 1;
            if (c >= bd[blk] && c < bd[blk + 1]) {
                B.ja.push_back(A.ja[k]);
                B.a.push_back(A.a[k]);
            }
        }
        B.ia[r + 1] = (int)B.ja.size() + 1;
    }
    return B;
}

int ilut(const Csr& A, int lfil, double droptol, Msr& F, const Msr* prev, int first_row)
{
    if (lfil < 0) return -4;
    const int others = g_running.fetch_add(1);
    struct Leave {
        ~Leave() { g_running.fetch_sub(1); }
    } leave;
    const int n = A.n;
    // a previous factor is used only when it has this matrix's order and
    // its row pointers are consistent; first_row is clamped to [0, n]
    int r0 = 0;
    if (prev && first_row > 0 && prev->n == n && (int)prev->ju.size() == n &&
        (int)prev->jlu.size() > n && prev->jlu[0] == n + 2) {
        r0 = first_row < n ? first_row : n;
        for (int i = 0; i < r0; ++i)
            if (prev->ju[i] < prev->jlu[i] || prev->jlu[i + 1] < prev->ju[i] ||
                prev->jlu[i + 1] - 1 > (int)prev->jlu.size()) {
                r0 = 0;
                break;
            }
    }
    const int T = (n > 0 && others == 0) ? std::min(ilut_threads(n), n) : 1;
    int ierr = 0;
    if (!ilut_on(A, lfil, droptol, T, F, ierr, prev, r0))
        ilut_on(A, lfil, droptol, 1, F, ierr, prev, r0);
    return ierr;
}

}  // namespace xt
