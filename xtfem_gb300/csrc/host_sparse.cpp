// host_sparse.cpp -- CSR construction and surgery on the host (FP64).
//
// The reference builds CSR from element triplets with a CSparse-style
// pipeline (src/spmtx.f90:359-407, 497-698).  The order in which duplicate
// entries are summed decides the last bits of K and M, so the pipeline below
// keeps the reference's stable ordering: rows grouped in input order, then
// columns sorted stably, then duplicates summed left to right.
#include "host_sparse.h"

#include <algorithm>
#include <numeric>
#include <stdexcept>

namespace xt {

namespace {

// Stable counting sort of (row, col, val) by row, then stable by column
// inside each row: the net effect of cs_compress followed by two
// cs_transpose calls (src/spmtx.f90:497-648).
void sort_rows_then_cols(int n, const std::vector<int>& ri,
                         const std::vector<int>& cj,
                         const std::vector<double>& v, std::vector<int>& ia,
                         std::vector<int>& ja, std::vector<double>& a)
{
    const size_t nz = ri.size();
    // bucket by column first (stable), then by row (stable): rows end up
    // grouped with ascending columns, ties keep input order.
    std::vector<int> cnt(n + 1, 0);
    for (size_t k = 0; k < nz; ++k) cnt[cj[k]]++;
    std::vector<int> start(n + 2, 0);
    for (int c = 1; c <= n; ++c) start[c + 1] = start[c] + cnt[c];
    std::vector<size_t> byc(nz);
    {
        std::vector<int> pos(start);
        for (size_t k = 0; k < nz; ++k) byc[pos[cj[k]]++] = k;
    }
    std::fill(cnt.begin(), cnt.end(), 0);
    for (size_t k = 0; k < nz; ++k) cnt[ri[k]]++;
    ia.assign(n + 1, 0);
    ia[0] = 1;
    for (int r = 1; r <= n; ++r) ia[r] = ia[r - 1] + cnt[r];
    std::vector<int> pos(n + 1);
    for (int r = 1; r <= n; ++r) pos[r] = ia[r - 1] - 1;
    ja.resize(nz);
    a.resize(nz);
    for (size_t t = 0; t < nz; ++t) {
        const size_t k = byc[t];
        const int p = pos[ri[k]]++;
        ja[p] = cj[k];
        a[p] = v[k];
    }
}

// cs_dupl (src/spmtx.f90:651-698) on a row-sorted CSR: equal columns are
// adjacent after the sort, summed in order.
void sum_duplicates(Csr& m)
{
    int out = 0;
    std::vector<int> nia(m.n + 1);
    nia[0] = 1;
    for (int r = 0; r < m.n; ++r) {
        const int b = m.ia[r] - 1, e = m.ia[r + 1] - 1;
        int last = -1;
        for (int k = b; k < e; ++k) {
            if (m.ja[k] == last) {
                m.a[out - 1] = m.a[out - 1] + m.a[k];
            } else {
                m.ja[out] = m.ja[k];
                m.a[out] = m.a[k];
                last = m.ja[k];
                ++out;
            }
        }
        nia[r + 1] = out + 1;
    }
    m.ia.swap(nia);
    m.ja.resize(out);
    m.a.resize(out);
}

}  // namespace

void rm0csr(Csr& m)
{
    int out = 0;
    std::vector<int> nia(m.n + 1);
    nia[0] = 1;
    for (int r = 0; r < m.n; ++r) {
        for (int k = m.ia[r] - 1; k < m.ia[r + 1] - 1; ++k)
            if (m.a[k] != 0.0) {
                m.ja[out] = m.ja[k];
                m.a[out] = m.a[k];
                ++out;
            }
        nia[r + 1] = out + 1;
    }
    m.ia.swap(nia);
    m.ja.resize(out);
    m.a.resize(out);
}

Csr tricsr(const Triplets& t, int n)
{
    Csr m;
    m.n = n;
    for (size_t k = 0; k < t.i.size(); ++k)
        if (t.i[k] < 1 || t.i[k] > n || t.j[k] < 1 || t.j[k] > n)
            throw std::runtime_error("tricsr: index out of range");
    sort_rows_then_cols(n, t.i, t.j, t.v, m.ia, m.ja, m.a);
    sum_duplicates(m);
    rm0csr(m);
    return m;
}

void csrapplybc(Csr& m, const int* bc)
{
    for (int r = 0; r < m.n; ++r)
        for (int k = m.ia[r] - 1; k < m.ia[r + 1] - 1; ++k) {
            const int c = m.ja[k] - 1;
            if (bc[r] != 0 || bc[c] != 0) m.a[k] = (r == c) ? 1.0 : 0.0;
        }
    rm0csr(m);
}

void cs_add(Csr& A, const Csr& B, double alpha, double beta)
{
    // cs_add scatters alpha*A(j,:) then beta*B(j,:) into a dense work row;
    // each entry is alpha*a (+ beta*b when both exist), see
    // src/spmtx.f90:725-740 and cs_scatter.
    Csr C;
    C.n = A.n;
    C.ia.assign(A.n + 1, 0);
    C.ia[0] = 1;
    std::vector<int> mark(A.n, -1);
    std::vector<double> x(A.n, 0.0);
    std::vector<int> cols;
    for (int r = 0; r < A.n; ++r) {
        cols.clear();
        for (int k = A.ia[r] - 1; k < A.ia[r + 1] - 1; ++k) {
            const int c = A.ja[k] - 1;
            if (mark[c] != r) { mark[c] = r; cols.push_back(c); x[c] = alpha * A.a[k]; }
            else x[c] += alpha * A.a[k];
        }
        for (int k = B.ia[r] - 1; k < B.ia[r + 1] - 1; ++k) {
            const int c = B.ja[k] - 1;
            if (mark[c] != r) { mark[c] = r; cols.push_back(c); x[c] = beta * B.a[k]; }
            else x[c] += beta * B.a[k];
        }
        std::sort(cols.begin(), cols.end());
        for (int c : cols) {
            C.ja.push_back(c + 1);
            C.a.push_back(x[c]);
        }
        C.ia[r + 1] = (int)C.ja.size() + 1;
    }
    rm0csr(C);
    A = std::move(C);
}

}  // namespace xt
