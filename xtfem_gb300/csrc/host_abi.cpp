// host_abi.cpp -- C ABI of the host-side set-up (include/xtfem_gb300_host.h)
// and the element-deletion surgery of src/main3d.f90:634-687.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>

#include "../../include/xtfem_gb300_host.h"
#include "host_problem.h"
#include "xt_device.h"

using namespace xt;

namespace xt {

namespace {

// The surgery on the rows it can change, each row taken through the same
// steps and arithmetic as the whole-matrix form below:
//   1. K - T (cs_add: 1.0 * k + (-1.0) * t over the union of the row's
//      columns), exact zeros removed;
//   2. + I on the DOFs of disconnected nodes (cs_add: 1.0 * k + 1.0 * 1.0,
//      or a new diagonal 1.0), exact zeros removed;
//   3. the boundary conditions (csrapplybc: entries of a fixed row or
//      column become 1 on the diagonal and 0 elsewhere), zeros removed;
// and M through step 3.  Steps 1 and 2 change only the DOF rows of the
// failed elements' nodes (T and the new diagonal live there).  Step 3
// changes those rows and any row with a column among the newly fixed DOFs:
// a disconnected node's neighbours through elements deleted earlier keep
// their couplings to it (M keeps the mass of deleted elements, K may keep
// rounding residues).  Every other row is copied unchanged (it holds no
// zeros and already satisfies the old conditions), so both forms give the
// same arrays.
void surgery_rows(Csr& K, Csr& M, const Csr& T, const std::vector<int>& diag_rows,
                  const std::vector<char>& touched, const int* bc)
{
    const int n = K.n;
    std::vector<char> add_diag(n, 0);  // the newly fixed DOFs
    for (int r : diag_rows) add_diag[r] = 1;
    std::vector<int> cols;
    std::vector<double> vals;
    auto rebuild = [&](Csr& A, bool stiffness) {
        Csr C;
        C.n = n;
        C.ia.assign(n + 1, 0);
        C.ia[0] = 1;
        C.ja.reserve(A.ja.size() + (stiffness ? T.ja.size() : 0));
        C.a.reserve(C.ja.capacity());
        for (int r = 0; r < n; ++r) {
            const int b = A.ia[r] - 1, e = A.ia[r + 1] - 1;
            bool fixed_col = false;
            if (!touched[r] && !diag_rows.empty())
                for (int k = b; k < e && !fixed_col; ++k) fixed_col = add_diag[A.ja[k] - 1] != 0;
            if (!touched[r] && !fixed_col) {
                C.ja.insert(C.ja.end(), A.ja.begin() + b, A.ja.begin() + e);
                C.a.insert(C.a.end(), A.a.begin() + b, A.a.begin() + e);
                C.ia[r + 1] = (int)C.ja.size() + 1;
                continue;
            }
            cols.clear();
            vals.clear();
            if (stiffness && touched[r]) {
                // step 1: merge the sorted rows of A and T
                int p = b, q = T.ia[r] - 1;
                const int qe = T.ia[r + 1] - 1;
                while (p < e || q < qe) {
                    int c;
                    double v;
                    if (q >= qe || (p < e && A.ja[p] < T.ja[q])) {
                        c = A.ja[p]; v = 1.0 * A.a[p]; ++p;
                    } else if (p >= e || T.ja[q] < A.ja[p]) {
                        c = T.ja[q]; v = -1.0 * T.a[q]; ++q;
                    } else {
                        c = A.ja[p]; v = 1.0 * A.a[p] + -1.0 * T.a[q]; ++p; ++q;
                    }
                    if (v != 0.0) { cols.push_back(c); vals.push_back(v); }
                }
                // step 2
                if (add_diag[r]) {
                    const int dc = r + 1;
                    size_t k = 0;
                    while (k < cols.size() && cols[k] < dc) ++k;
                    if (k < cols.size() && cols[k] == dc) {
                        vals[k] = 1.0 * vals[k] + 1.0 * 1.0;
                        if (vals[k] == 0.0) { cols.erase(cols.begin() + k); vals.erase(vals.begin() + k); }
                    } else {
                        cols.insert(cols.begin() + k, dc);
                        vals.insert(vals.begin() + k, 1.0);
                    }
                }
            } else {
                cols.assign(A.ja.begin() + b, A.ja.begin() + e);
                vals.assign(A.a.begin() + b, A.a.begin() + e);
            }
            // step 3
            for (size_t k = 0; k < cols.size(); ++k) {
                const int c = cols[k] - 1;
                if (bc[r] != 0 || bc[c] != 0) vals[k] = (r == c) ? 1.0 : 0.0;
                if (vals[k] != 0.0) { C.ja.push_back(cols[k]); C.a.push_back(vals[k]); }
            }
            C.ia[r + 1] = (int)C.ja.size() + 1;
        }
        A = std::move(C);
    };
    rebuild(K, true);
    rebuild(M, false);
}

bool whole_matrix_surgery()
{
    const char* e = std::getenv("XTFEM_SURGERY");
    return e && std::strcmp(e, "full") == 0;
}

}  // namespace

int Problem::delete_elements(int nef, const int* nefail, int* bc, int* ndf_out)
{
    if (ndf_out) *ndf_out = 0;
    if (nef <= 0) return XT_OK;
    const int ndof = 3 * mesh.nn;
    for (int k = 0; k < nef; ++k)
        if (nefail[k] < 1 || nefail[k] > mesh.ne) {
            set_error("delete: element number out of range");
            return XT_ERR_ARG;
        }
    // delelement: the reference passes the per-Gauss-point stiffness array
    // where one 6x6 matrix is expected (src/delelement.f90:46-47 into
    // src/elesubs.f90:217), so every failed element's ke uses the first
    // Gauss point's constitutive matrix; with a uniform material this is
    // the material's matrix.
    Triplets t;
    t.i.reserve((size_t)nef * 576);
    t.j.reserve((size_t)nef * 576);
    t.v.reserve((size_t)nef * 576);
    double ke[576];
    std::vector<char> touched(ndof, 0);
    for (int k = 0; k < nef; ++k) {
        const int e = nefail[k] - 1;
        element_stiffness(mesh, e, sys.stiff.data(), ke);
        int dofs[24];
        for (int i = 0; i < 8; ++i)
            for (int c = 0; c < 3; ++c) dofs[3 * i + c] = 3 * (mesh.conn[(size_t)e * 8 + i] - 1) + c + 1;
        for (int r = 0; r < 24; ++r) {
            touched[dofs[r] - 1] = 1;
            for (int c = 0; c < 24; ++c) {
                t.i.push_back(dofs[r]);
                t.j.push_back(dofs[c]);
                t.v.push_back(ke[r * 24 + c]);
            }
        }
    }
    const Csr T = tricsr(t, ndof);
    // chkcnsta, then chkndsta (src/delelement.f90:139-201)
    for (int k = 0; k < nef; ++k) {
        const int e = nefail[k] - 1;
        for (int i = 0; i < 8; ++i) necnt[mesh.conn[(size_t)e * 8 + i] - 1] -= 1;
    }
    std::vector<int> ndfail;
    std::vector<char> seen(mesh.nn, 0);
    for (int k = 0; k < nef; ++k) {
        const int e = nefail[k] - 1;
        for (int i = 0; i < 8; ++i) {
            const int nd = mesh.conn[(size_t)e * 8 + i] - 1;
            if (necnt[nd] == 0 && !seen[nd]) {
                seen[nd] = 1;
                ndfail.push_back(nd + 1);
            }
        }
    }
    // adddiagonal (src/delelement.f90:204-247): a unit diagonal on the
    // disconnected nodes' DOFs, which become fixed
    std::vector<int> diag_rows;
    for (int nd : ndfail)
        for (int c = 0; c < 3; ++c) diag_rows.push_back((nd - 1) * 3 + c);
    // the first row of K this surgery changes: a failed element's DOF row,
    // or a row with a column among the newly fixed DOFs (a neighbour through
    // an element deleted earlier)
    int first = ndof;
    for (int r = 0; r < ndof; ++r)
        if (touched[r]) { first = r; break; }
    if (!diag_rows.empty()) {
        std::vector<char> fixed_now(ndof, 0);
        for (int r : diag_rows) fixed_now[r] = 1;
        for (int r = 0; r < first; ++r) {
            bool hit = false;
            for (int k = sys.K.ia[r] - 1; k < sys.K.ia[r + 1] - 1 && !hit; ++k)
                hit = fixed_now[sys.K.ja[k] - 1] != 0;
            if (hit) { first = r; break; }
        }
    }
    first_changed = first;
    if (whole_matrix_surgery()) {
        // the same steps on the whole matrices (the reference's form)
        cs_add(sys.K, T, 1.0, -1.0);
        if (!diag_rows.empty()) {
            Triplets d;
            for (int r : diag_rows) {
                d.i.push_back(r + 1);
                d.j.push_back(r + 1);
                d.v.push_back(1.0);
            }
            cs_add(sys.K, tricsr(d, ndof), 1.0, 1.0);
        }
        for (int r : diag_rows) bc[r] = 1;
        csrapplybc(sys.M, bc);
        csrapplybc(sys.K, bc);
    } else {
        for (int r : diag_rows) bc[r] = 1;
        surgery_rows(sys.K, sys.M, T, diag_rows, touched, bc);
    }
    if (ndf_out) *ndf_out = (int)ndfail.size();
    return XT_OK;
}

}  // namespace xt

namespace {

template <class F>
int guarded(F&& f)
{
    try {
        return f();
    } catch (const std::exception& e) {
        set_error(e.what());
        return XT_ERR_HOST;
    }
}

int finish_problem(std::unique_ptr<Problem>& pr, double E, double nu, double rho,
                   xth_problem* out)
{
    pr->sys = assemble_mech(pr->mesh, E, nu, rho);
    pr->E = E;
    pr->nu = nu;
    pr->rho = rho;
    pr->necnt.assign(pr->mesh.nn, 0);
    for (size_t k = 0; k < pr->mesh.conn.size(); ++k) pr->necnt[pr->mesh.conn[k] - 1] += 1;
    *out = reinterpret_cast<xth_problem>(pr.release());
    return XT_OK;
}

Problem* P(xth_problem h) { return reinterpret_cast<Problem*>(h); }

}  // namespace

extern "C" {

int xth_problem_from_inp(const char* path, double E, double nu, double rho, xth_problem* out)
{
    if (!path || !out) { set_error("xth_problem_from_inp: null argument"); return XT_ERR_ARG; }
    return guarded([&] {
        auto pr = std::make_unique<Problem>();
        pr->mesh = read_inp(path);
        return finish_problem(pr, E, nu, rho, out);
    });
}

int xth_problem_from_mesh(int nn, int ne, const double* xyz, const int* conn, double E, double nu,
                          double rho, xth_problem* out)
{
    if (!xyz || !conn || !out || nn <= 0 || ne <= 0) {
        set_error("xth_problem_from_mesh: bad arguments");
        return XT_ERR_ARG;
    }
    return guarded([&] {
        auto pr = std::make_unique<Problem>();
        pr->mesh.nn = nn;
        pr->mesh.ne = ne;
        pr->mesh.xyz.assign(xyz, xyz + (size_t)nn * 3);
        pr->mesh.conn.assign(conn, conn + (size_t)ne * 8);
        for (int v : pr->mesh.conn)
            if (v < 1 || v > nn) {
                set_error("xth_problem_from_mesh: connectivity out of range");
                return XT_ERR_ARG;
            }
        return finish_problem(pr, E, nu, rho, out);
    });
}

int xth_problem_rod(int nx, int ny, int nz, double lx, double ly, double lz, double E, double nu,
                    double rho, xth_problem* out)
{
    if (!out) { set_error("xth_problem_rod: null argument"); return XT_ERR_ARG; }
    return guarded([&] {
        auto pr = std::make_unique<Problem>();
        pr->mesh = make_rod(nx, ny, nz, lx, ly, lz);
        return finish_problem(pr, E, nu, rho, out);
    });
}

int xth_problem_destroy(xth_problem pr)
{
    delete P(pr);
    return XT_OK;
}

int xth_problem_sizes(xth_problem h, int* nn, int* ne, int* nnz_k, int* nnz_m)
{
    if (!h) { set_error("null problem"); return XT_ERR_ARG; }
    Problem* pr = P(h);
    if (nn) *nn = pr->mesh.nn;
    if (ne) *ne = pr->mesh.ne;
    if (nnz_k) *nnz_k = pr->sys.K.nnz();
    if (nnz_m) *nnz_m = pr->sys.M.nnz();
    return XT_OK;
}

int xth_problem_mesh(xth_problem h, double* xyz, int* conn)
{
    if (!h) { set_error("null problem"); return XT_ERR_ARG; }
    Problem* pr = P(h);
    if (xyz) std::memcpy(xyz, pr->mesh.xyz.data(), pr->mesh.xyz.size() * sizeof(double));
    if (conn) std::memcpy(conn, pr->mesh.conn.data(), pr->mesh.conn.size() * sizeof(int));
    return XT_OK;
}

static int copy_csr(const Csr& m, int* ia, int* ja, double* a)
{
    if (ia) std::memcpy(ia, m.ia.data(), m.ia.size() * sizeof(int));
    if (ja) std::memcpy(ja, m.ja.data(), m.ja.size() * sizeof(int));
    if (a) std::memcpy(a, m.a.data(), m.a.size() * sizeof(double));
    return XT_OK;
}

int xth_problem_k(xth_problem h, int* ia, int* ja, double* a)
{
    if (!h) { set_error("null problem"); return XT_ERR_ARG; }
    return copy_csr(P(h)->sys.K, ia, ja, a);
}

int xth_problem_m(xth_problem h, int* ia, int* ja, double* a)
{
    if (!h) { set_error("null problem"); return XT_ERR_ARG; }
    return copy_csr(P(h)->sys.M, ia, ja, a);
}

int xth_problem_strain_rows(xth_problem h, double* nx, double* ny, double* nz)
{
    if (!h) { set_error("null problem"); return XT_ERR_ARG; }
    Problem* pr = P(h);
    const size_t n = pr->sys.Nx.size();
    if (nx) std::memcpy(nx, pr->sys.Nx.data(), n * sizeof(double));
    if (ny) std::memcpy(ny, pr->sys.Ny.data(), n * sizeof(double));
    if (nz) std::memcpy(nz, pr->sys.Nz.data(), n * sizeof(double));
    return XT_OK;
}

int xth_problem_stiffness(xth_problem h, double* d)
{
    if (!h || !d) { set_error("null argument"); return XT_ERR_ARG; }
    std::memcpy(d, P(h)->sys.stiff.data(), 36 * sizeof(double));
    return XT_OK;
}

int xth_problem_apply_bc(xth_problem h, const int* bc)
{
    if (!h || !bc) { set_error("null argument"); return XT_ERR_ARG; }
    return guarded([&] {
        csrapplybc(P(h)->sys.K, bc);
        csrapplybc(P(h)->sys.M, bc);
        return XT_OK;
    });
}

int xth_problem_delete(xth_problem h, int nef, const int* nefail, int* bc, int* ndf_out)
{
    if (!h || (nef > 0 && (!nefail || !bc))) { set_error("null argument"); return XT_ERR_ARG; }
    return guarded([&] { return P(h)->delete_elements(nef, nefail, bc, ndf_out); });
}

static int ilut_into(int n, const int* ia, const int* ja, const double* a, int lfil, double droptol,
                     int iwk, double* alu, int* jlu, int* ju, const Msr* prev, int first_row)
{
    if (n <= 0 || !ia || !ja || !a || !alu || !jlu || !ju) {
        set_error("xth_ilut: bad arguments");
        return XT_ERR_ARG;
    }
    return guarded([&] {
        Csr m;
        m.n = n;
        m.ia.assign(ia, ia + n + 1);
        m.ja.assign(ja, ja + (ia[n] - 1));
        m.a.assign(a, a + (ia[n] - 1));
        Msr f;
        const int ierr = ilut(m, lfil, droptol, f, prev, first_row);
        // The storage test of src/ilut.f:152-495, row by row over the rows
        // the factorisation finished: -2 when an L entry would be stored
        // past iwk, -3 when the U part (counted with its diagonal, as the
        // reference counts it) would end past iwk.  The first failing row
        // decides, as in the reference, which stops there: a storage failure
        // before the row that failed otherwise wins.
        long long pos = (long long)n + 2;  // 1-based next free slot
        const int rows = (int)f.ju.size();
        for (int i = 0; i < rows; ++i) {
            const long long nl = f.ju[i] - f.jlu[i];
            if (nl > 0 && pos + nl - 1 > iwk) return -2;
            pos += nl;
            const long long nu = f.jlu[i + 1] - f.ju[i];
            if (nu + 1 + pos > iwk) return -3;
            pos += nu;
        }
        if (ierr != 0) return ierr;
        if ((long long)f.alu.size() > iwk) return -3;
        std::memcpy(alu, f.alu.data(), f.alu.size() * sizeof(double));
        std::memcpy(jlu, f.jlu.data(), f.jlu.size() * sizeof(int));
        std::memcpy(ju, f.ju.data(), f.ju.size() * sizeof(int));
        return 0;
    });
}

int xth_problem_first_changed_row(xth_problem h)
{
    return h ? P(h)->first_changed : -1;
}

int xth_ilut(int n, const int* ia, const int* ja, const double* a, int lfil, double droptol,
             int iwk, double* alu, int* jlu, int* ju)
{
    return ilut_into(n, ia, ja, a, lfil, droptol, iwk, alu, jlu, ju, nullptr, 0);
}

int xth_ilut_blocks(int n, const int* ia, const int* ja, const double* a, int lfil,
                    double droptol, int iwk, int group, int blocks, double* alu, int* jlu, int* ju)
{
    if (n <= 0 || !ia || !ja || !a) {
        set_error("xth_ilut_blocks: bad arguments");
        return XT_ERR_ARG;
    }
    if (blocks <= 1) return ilut_into(n, ia, ja, a, lfil, droptol, iwk, alu, jlu, ju, nullptr, 0);
    Csr m, b;
    const int rc = guarded([&] {
        m.n = n;
        m.ia.assign(ia, ia + n + 1);
        m.ja.assign(ja, ja + (ia[n] - 1));
        m.a.assign(a, a + (ia[n] - 1));
        b = block_diagonal(m, group, blocks);
        return 0;
    });
    if (rc != 0) return rc;
    return ilut_into(n, b.ia.data(), b.ja.data(), b.a.data(), lfil, droptol, iwk, alu, jlu, ju,
                     nullptr, 0);
}

int xth_ilut_update(int n, const int* ia, const int* ja, const double* a, int lfil,
                    double droptol, int iwk, int first_row, const double* prev_alu,
                    const int* prev_jlu, const int* prev_ju, double* alu, int* jlu, int* ju)
{
    if (n <= 0 || !prev_alu || !prev_jlu || !prev_ju || prev_jlu[0] != n + 2) {
        set_error("xth_ilut_update: bad previous factor");
        return XT_ERR_ARG;
    }
    return guarded([&] {
        Msr prev;
        prev.n = n;
        const int end = prev_jlu[n] - 1;  // entries of the previous factor
        prev.alu.assign(prev_alu, prev_alu + end);
        prev.jlu.assign(prev_jlu, prev_jlu + end);
        prev.ju.assign(prev_ju, prev_ju + n);
        return ilut_into(n, ia, ja, a, lfil, droptol, iwk, alu, jlu, ju, &prev, first_row);
    });
}

void xth_stcoeff_m(double t1, double dt, double w, double* k, double* m, double* ktn, double* mtn,
                   double* ktn1, double* mtn1)
{
    stcoeff_m(t1, dt, w, k, m, ktn, mtn, ktn1, mtn1);
}

void xth_stcoeff_t(double dt, double* k, double* m, double* ktn, double* mtn, double* ktn1,
                   double* mtn1)
{
    stcoeff_t(dt, k, m, ktn, mtn, ktn1, mtn1);
}

void xth_getfextc_m(double t1, double w, double dt, double* fextc, double* fint)
{
    getfextc_m(t1, w, dt, fextc, fint);
}

void xth_getfextc_t(double t1, double dt, double* fextc)
{
    getfextc_t(t1, dt, fextc);
}

void xth_nt_table(int nip, const double* tcoorde, double w, double* nt)
{
    nt_table(nip, tcoorde, w, nt);
}

}  // extern "C"
