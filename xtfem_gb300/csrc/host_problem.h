// host_problem.h -- a mechanical problem on the host: mesh, assembled K and
// M (after boundary conditions once applied) and node-element counts.
#pragma once

#include <vector>

#include "host_sparse.h"

namespace xt {

struct Problem {
    Mesh mesh;
    MechSystem sys;
    std::vector<int> necnt;  // elements per node (src/main3d.f90:270-277)
    // the first row of K the last delete_elements changed (rows above it are
    // as before, so a factor's rows above it stay valid); n when none
    int first_changed = 0;
    double E = 0, nu = 0, rho = 0;  // uniform material
    int delete_elements(int nef, const int* nefail, int* bc, int* ndf_out);
};

}  // namespace xt
