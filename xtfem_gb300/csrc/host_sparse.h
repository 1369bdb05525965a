// host_sparse.h -- host-side sparse-matrix and finite-element set-up of the
// XTFEM space-time solve (the caller side of the GPU path).
//
// Everything here runs on the host in FP64 and produces the inputs the GPU
// path consumes: the spatial stiffness K and mass M in CSR (1-based, sorted
// columns, duplicates summed, zeros removed), the boundary-condition masks,
// the load vector, the temporal coefficient matrices and the ILUT factor.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace xt {

// CSR matrix with 1-based row pointers and column indices, the layout of the
// reference's ki/kj/kv arrays (src/spmtx.f90:359-407).
struct Csr {
    int n = 0;
    std::vector<int> ia;      // n+1, 1-based
    std::vector<int> ja;      // nnz, 1-based
    std::vector<double> a;    // nnz
    int nnz() const { return n ? ia[n] - 1 : 0; }
};

// Triplet list (1-based rows and columns), element-by-element order.
struct Triplets {
    std::vector<int> i, j;
    std::vector<double> v;
};

// src/spmtx.f90:359-407 tricsr: compress by rows, sort columns with two
// stable transposes, sum duplicates in input order, drop exact zeros.
Csr tricsr(const Triplets& t, int n);

// src/spmtx.f90:410-454 rm0csr.
void rm0csr(Csr& m);

// src/spmtx.f90:268-307 csrapplybc: rows and columns of fixed DOFs cleared,
// their diagonal set to one, zeros removed.  bc has n entries (nonzero =
// fixed).
void csrapplybc(Csr& m, const int* bc);

// src/spmtx.f90:701-770 cs_add: A := alpha*A + beta*B, result sorted,
// duplicates summed, zeros removed.
void cs_add(Csr& A, const Csr& B, double alpha, double beta);

// Hexahedral C3D8 mesh: coordinates (nn x 3) and 1-based connectivity
// (ne x 8), in the order of the reference's .inp files.
struct Mesh {
    int nn = 0, ne = 0;
    std::vector<double> xyz;   // nn*3
    std::vector<int> conn;     // ne*8, 1-based node numbers
};

// Reads the reference's .inp format (src/main3d.f90:212-231).  Throws on a
// malformed file.
Mesh read_inp(const std::string& path);

// Structured rod of nx x ny x nz elements over [0,lx]x[0,ly]x[0,lz] with the
// node and element numbering of inp/prismaticrod-*.inp (x descending
// outermost, then z descending, then y descending; coordinates rounded to
// single precision as in those files).
Mesh make_rod(int nx, int ny, int nz, double lx, double ly, double lz);

// Mechanical set-up of src/mpisubs.f90:69-139 for all elements with a
// uniform material: K and M (3 DOFs per node) and the per-Gauss-point
// strain rows Nx, Ny, Nz (8 per point, ngp = 8*ne points).
struct MechSystem {
    Csr K, M;
    std::vector<double> Nx, Ny, Nz;  // ngp*8
    std::vector<double> stiff;       // 36, column-major, GP-independent
};
MechSystem assemble_mech(const Mesh& mesh, double E, double nu, double rho);

// Thermal set-up (src/mpisubs.f90 mpiglbmtx_t with elemtx_t,
// src/elesubs.f90:60-116): conductivity K (kappa grad N . grad N) and
// capacity M (rho cp N N), one DOF per node, 2x2x2 Gauss rule.
struct ThermSystem {
    Csr K, M;
};
ThermSystem assemble_therm(const Mesh& mesh, double kappa, double rho, double cp);

// Element stiffness (24x24, row-major) of src/elesubs.f90:207-251 for a
// given constitutive matrix (36, column-major).
void element_stiffness(const Mesh& mesh, int elem, const double* stiff,
                       double* ke);

// src/ilut.f:152-495 ILUT(lfil, droptol) on the host in FP64, MSR output
// with inverted diagonal.  Returns SPARSKIT's ierr; the factor is resized to
// what it holds.
struct Msr {
    int n = 0;
    std::vector<double> alu;
    std::vector<int> jlu, ju;  // 1-based
};
// prev / first_row: rows [0, first_row) are taken from prev, the factor of a
// matrix whose rows [0, first_row) equal A's (ILUT row i depends only on
// rows <= i), so the result is the full factor of A bit for bit.
int ilut(const Csr& A, int lfil, double droptol, Msr& out, const Msr* prev = nullptr,
         int first_row = 0);

// Row bounds of the block-Jacobi ILU's `blocks` contiguous row blocks of
// whole node groups of g rows (blocks + 1 entries, 0-based rows):
// floor(ng b / blocks) g with ng = n / g (g = 1 when n is not a multiple of g).
std::vector<int> ilu_block_bounds(int n, int g, int blocks);
// The block-Jacobi part of A: its entries whose row and column lie in the
// same block of ilu_block_bounds(n, g, blocks); blocks <= 1 gives A.  Its
// ILUT has no entry between blocks, so the triangular solves of the blocks
// are independent.
Csr block_diagonal(const Csr& A, int g, int blocks);

// src/stcoeff.f90:62-356 closed forms (6x6 each, column-major).
void stcoeff_m(double t1, double dt, double w, double* k, double* m,
               double* ktn, double* mtn, double* ktn1, double* mtn1);
// src/stcoeff.f90:1-60 (3x3 each, column-major).
void stcoeff_t(double dt, double* k, double* m, double* ktn, double* mtn,
               double* ktn1, double* mtn1);
// src/getfextc.f90:22-58.
void getfextc_m(double t1, double w, double dt, double* fextc, double* fint);
// src/getfextc.f90:1-20 (3 temporal load weights, w = 2 3.14159 / 24).
void getfextc_t(double t1, double dt, double* fextc);
// src/kokkos_damage.f90:36-47 temporal shape table, Nt[jj*6+k].
void nt_table(int nip, const double* tcoorde, double w, double* Nt);

}  // namespace xt
