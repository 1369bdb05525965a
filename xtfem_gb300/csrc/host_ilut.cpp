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
#include <cmath>
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

int ilut(const Csr& A, int lfil, double droptol, Msr& F)
{
    const int n = A.n;
    if (lfil < 0) return -4;
    F.n = n;
    // Built in SPARSKIT's 1-based position space (vector index == position,
    // index 0 a pad dropped at the end): alu[1..n] inverted diagonal,
    // jlu[1..n+1] row starts, off-diagonal entries from position n+2.
    F.ju.assign(n, 0);
    F.jlu.assign(n + 2, 0);
    F.alu.assign(n + 2, 0.0);
    // Row workspace.  Slots [0, lenl) hold the L part (column, value), slot
    // i the diagonal and slots (i, i+lenu) the U part; where[c] is the slot
    // of column c in the current row, or -1.
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
    F.jlu[1] = n + 2;
    F.alu.reserve((size_t)n * (2 * lfil + 2));
    F.jlu.reserve((size_t)n * (2 * lfil + 2));
    for (int i = 0; i < n; ++i) {
        const int b = A.ia[i] - 1, e = A.ia[i + 1] - 1;
        double tnorm = 0.0;
        for (int k = b; k < e; ++k) tnorm += std::fabs(A.a[k]);
        if (tnorm == 0.0) return -5;
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
                const int s = i + lenu;
                col[s] = c; w[s] = A.a[k]; where[c] = s; ++lenu;
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
            const double fact = w[where[r]] * F.alu[r + 1];
            where[r] = -1;
            if (std::fabs(fact) <= droptol) continue;
            // row r of U: MSR positions ju[r] .. jlu[r+1]-1 (1-based)
            for (int k = F.ju[r]; k <= F.jlu[r + 2] - 1; ++k) {
                const double s = fact * F.alu[k];
                const int c = F.jlu[k] - 1;
                const int slot = where[c];
                if (c >= i) {
                    if (slot < 0) {
                        if (lenu + 1 > n) return -1;
                        const int ns = i + lenu;
                        col[ns] = c; where[c] = ns; w[ns] = -s; ++lenu;
                    } else {
                        w[slot] -= s;
                    }
                } else {
                    if (slot < 0) {
                        if (lenl + 1 > n) return -1;
                        col[lenl] = c; where[c] = lenl; w[lenl] = -s; ++lenl;
                        pending[(size_t)c >> 6] |= 1ull << (c & 63);
                    } else {
                        w[slot] -= s;
                    }
                }
            }
            wl[kept] = fact;
            cl[kept] = r;
            ++kept;
        }
        for (int k = 0; k < lenu; ++k) where[col[i + k]] = -1;
        // L row: the lfil largest multipliers
        const int nl = kept < lfil ? kept : lfil;
        split_largest(wl.data(), cl.data(), kept, nl);
        for (int k = 0; k < nl; ++k) {
            F.alu.push_back(wl[k]);
            F.jlu.push_back(cl[k] + 1);
        }
        F.ju[i] = (int)F.jlu.size();  // 1-based start of U row i
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
        for (int k = 1; k <= keep - 1; ++k) {
            F.alu.push_back(w[i + k]);
            F.jlu.push_back(col[i + k] + 1);
        }
        if (w[i] == 0.0) w[i] = ((double)0.0001f + droptol) * tnorm;
        F.alu[i + 1] = 1.0 / w[i];
        F.jlu[i + 2] = (int)F.jlu.size();
    }
    F.alu.erase(F.alu.begin());
    F.jlu.erase(F.jlu.begin());
    return 0;
}

}  // namespace xt
