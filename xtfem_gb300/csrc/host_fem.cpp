// host_fem.cpp -- C3D8 meshes and the spatial K, M assembly on the host.
//
// The element integrals follow src/elesubs.f90:2-58 (elemtx_m) with the
// 2x2x2 Gauss rule of src/procs.f90:537 (the 15-digit abscissa is kept, not
// 1/sqrt(3), because the reference uses it), the C3D8 shape-function sign
// table of src/procs.f90:1366-1389 and the closed-form 3x3 determinant and
// inverse of src/procs.f90:273-328, 458-516.  The strain rows Nx, Ny, Nz of
// each Gauss point are the first three rows of the strain-displacement
// matrix (src/elesubs.f90:44-48), which the damage update consumes.
#include "host_sparse.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>

namespace xt {

namespace {

// natural coordinates of the 8 nodes, in the order of the reference's
// shape functions N1..N8 (src/procs.f90:1366-1373)
const int kNodeSign[8][3] = {{-1, -1, +1}, {-1, -1, -1}, {-1, +1, -1},
                             {-1, +1, +1}, {+1, -1, +1}, {+1, -1, -1},
                             {+1, +1, -1}, {+1, +1, +1}};
const double kGauss = 0.577350269189626;  // src/procs.f90:537

struct GaussGeom {
    double dNdx[8][3];  // d N_i / d x_m
    double N[8];
    double jacdet;
};

// Geometry of Gauss point l (0..7, xi outermost as in src/elesubs.f90:36-40)
GaussGeom gauss_geom(const double (*xe)[3], int l)
{
    const double g[2] = {-kGauss, kGauss};
    const double xi = g[(l >> 2) & 1], eta = g[(l >> 1) & 1], zeta = g[l & 1];
    GaussGeom G;
    double dN[8][3];
    for (int i = 0; i < 8; ++i) {
        const double sx = kNodeSign[i][0], sy = kNodeSign[i][1], sz = kNodeSign[i][2];
        G.N[i] = 0.125 * (1.0 + sx * xi) * (1.0 + sy * eta) * (1.0 + sz * zeta);
        dN[i][0] = 0.125 * sx * (1.0 + sy * eta) * (1.0 + sz * zeta);
        dN[i][1] = 0.125 * sy * (1.0 + sx * xi) * (1.0 + sz * zeta);
        dN[i][2] = 0.125 * sz * (1.0 + sx * xi) * (1.0 + sy * eta);
    }
    // jac(a, m) = sum_i dN_i/dxi_a * x_i^m  (src/elesubs.f90:41)
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int a = 0; a < 3; ++a)
        for (int m = 0; m < 3; ++m) {
            double s = 0.0;
            for (int i = 0; i < 8; ++i) s += dN[i][a] * xe[i][m];
            J[a][m] = s;
        }
    const double det = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] +
                       J[0][2] * J[1][0] * J[2][1] - J[0][0] * J[1][2] * J[2][1] -
                       J[0][1] * J[1][0] * J[2][2] - J[0][2] * J[1][1] * J[2][0];
    if (!(std::fabs(det) > 10.0 * 2.220446049250313e-16))
        throw std::runtime_error("C3D8 element with singular Jacobian");
    double inv[3][3];
    inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    for (int i = 0; i < 8; ++i)
        for (int m = 0; m < 3; ++m) {
            double s = 0.0;
            for (int a = 0; a < 3; ++a) s += inv[m][a] * dN[i][a];
            G.dNdx[i][m] = s;
        }
    G.jacdet = det;
    return G;
}

void element_coords(const Mesh& mesh, int e, double (*xe)[3])
{
    for (int i = 0; i < 8; ++i) {
        const int nd = mesh.conn[(size_t)e * 8 + i] - 1;
        for (int m = 0; m < 3; ++m) xe[i][m] = mesh.xyz[(size_t)nd * 3 + m];
    }
}

// B^T D B contribution of one Gauss point into ke (24x24 row-major)
void add_btdb(const GaussGeom& G, const double* D, double* ke)
{
    double B[6][24];
    std::memset(B, 0, sizeof(B));
    for (int i = 0; i < 8; ++i) {
        const double nx = G.dNdx[i][0], ny = G.dNdx[i][1], nz = G.dNdx[i][2];
        B[0][3 * i + 0] = nx;
        B[1][3 * i + 1] = ny;
        B[2][3 * i + 2] = nz;
        B[3][3 * i + 0] = ny; B[3][3 * i + 1] = nx;
        B[4][3 * i + 1] = nz; B[4][3 * i + 2] = ny;
        B[5][3 * i + 0] = nz; B[5][3 * i + 2] = nx;
    }
    double DB[6][24];
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 24; ++c) {
            double s = 0.0;
            for (int k = 0; k < 6; ++k) s += D[k * 6 + r] * B[k][c];
            DB[r][c] = s;
        }
    for (int r = 0; r < 24; ++r)
        for (int c = 0; c < 24; ++c) {
            double s = 0.0;
            for (int k = 0; k < 6; ++k) s += B[k][r] * DB[k][c];
            ke[r * 24 + c] += s * G.jacdet;
        }
}

// src/elesubs.f90:374-401 isotropic constitutive matrix, column-major
void iso_stiffness(double E, double nu, double* D)
{
    const double c = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
    for (int k = 0; k < 36; ++k) D[k] = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) D[j * 6 + i] = c * ((i == j) ? 1.0 - nu : nu);
    for (int i = 3; i < 6; ++i) D[i * 6 + i] = c * (0.5 - nu);
}

}  // namespace

Mesh read_inp(const std::string& path)
{
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) throw std::runtime_error("cannot open mesh " + path);
    Mesh m;
    auto fail = [&](const char* what) {
        std::fclose(f);
        throw std::runtime_error(std::string("malformed mesh ") + path + ": " + what);
    };
    if (std::fscanf(f, "%d", &m.nn) != 1 || m.nn <= 0) fail("node count");
    m.xyz.assign((size_t)m.nn * 3, 0.0);
    for (int k = 0; k < m.nn; ++k) {
        int id;
        double x, y, z;
        if (std::fscanf(f, "%d %lf %lf %lf", &id, &x, &y, &z) != 4) fail("node line");
        if (id < 1 || id > m.nn) fail("node id");
        m.xyz[(size_t)(id - 1) * 3 + 0] = x;
        m.xyz[(size_t)(id - 1) * 3 + 1] = y;
        m.xyz[(size_t)(id - 1) * 3 + 2] = z;
    }
    if (std::fscanf(f, "%d", &m.ne) != 1 || m.ne <= 0) fail("element count");
    m.conn.assign((size_t)m.ne * 8, 0);
    for (int k = 0; k < m.ne; ++k) {
        int id, c[8];
        if (std::fscanf(f, "%d %d %d %d %d %d %d %d %d", &id, c, c + 1, c + 2, c + 3,
                        c + 4, c + 5, c + 6, c + 7) != 9)
            fail("element line");
        if (id < 1 || id > m.ne) fail("element id");
        for (int i = 0; i < 8; ++i) {
            if (c[i] < 1 || c[i] > m.nn) fail("connectivity");
            m.conn[(size_t)(id - 1) * 8 + i] = c[i];
        }
    }
    std::fclose(f);
    return m;
}

Mesh make_rod(int nx, int ny, int nz, double lx, double ly, double lz)
{
    if (nx < 1 || ny < 1 || nz < 1) throw std::runtime_error("make_rod: bad size");
    Mesh m;
    const int py = ny + 1, pz = nz + 1, px = nx + 1;
    m.nn = px * py * pz;
    m.ne = nx * ny * nz;
    m.xyz.resize((size_t)m.nn * 3);
    auto node = [&](int ix, int iy, int iz) { return ix * py * pz + iz * py + iy + 1; };
    // The shipped meshes hold single-precision coordinates printed with nine
    // significant digits and read back in double precision: reproduce that.
    auto coord = [](double v) {
        char buf[32];
        std::snprintf(buf, sizeof buf, "%.9g", (double)(float)v);
        return std::strtod(buf, nullptr);
    };
    for (int ix = 0; ix < px; ++ix)
        for (int iz = 0; iz < pz; ++iz)
            for (int iy = 0; iy < py; ++iy) {
                const int id = node(ix, iy, iz) - 1;
                m.xyz[(size_t)id * 3 + 0] = coord(lx - lx * ix / nx);
                m.xyz[(size_t)id * 3 + 1] = coord(ly - ly * iy / ny);
                m.xyz[(size_t)id * 3 + 2] = coord(lz - lz * iz / nz);
            }
    m.conn.resize((size_t)m.ne * 8);
    for (int ix = 0; ix < nx; ++ix)
        for (int iz = 0; iz < nz; ++iz)
            for (int iy = 0; iy < ny; ++iy) {
                const int e = ix * ny * nz + iz * ny + iy;
                int* c = &m.conn[(size_t)e * 8];
                c[0] = node(ix + 1, iy, iz);
                c[1] = node(ix + 1, iy + 1, iz);
                c[2] = node(ix + 1, iy + 1, iz + 1);
                c[3] = node(ix + 1, iy, iz + 1);
                c[4] = node(ix, iy, iz);
                c[5] = node(ix, iy + 1, iz);
                c[6] = node(ix, iy + 1, iz + 1);
                c[7] = node(ix, iy, iz + 1);
            }
    return m;
}

void element_stiffness(const Mesh& mesh, int e, const double* stiff, double* ke)
{
    double xe[8][3];
    element_coords(mesh, e, xe);
    std::memset(ke, 0, sizeof(double) * 576);
    for (int l = 0; l < 8; ++l) add_btdb(gauss_geom(xe, l), stiff, ke);
}

MechSystem assemble_mech(const Mesh& mesh, double E, double nu, double rho)
{
    MechSystem S;
    S.stiff.resize(36);
    iso_stiffness(E, nu, S.stiff.data());
    const size_t ngp = (size_t)mesh.ne * 8;
    S.Nx.resize(ngp * 8);
    S.Ny.resize(ngp * 8);
    S.Nz.resize(ngp * 8);
    Triplets tk, tm;
    const size_t per = 576;
    tk.i.resize(per * mesh.ne); tk.j.resize(per * mesh.ne); tk.v.resize(per * mesh.ne);
    tm.i.resize(per * mesh.ne); tm.j.resize(per * mesh.ne); tm.v.resize(per * mesh.ne);
    double ke[576], me[576];
    for (int e = 0; e < mesh.ne; ++e) {
        double xe[8][3];
        element_coords(mesh, e, xe);
        std::memset(ke, 0, sizeof(ke));
        std::memset(me, 0, sizeof(me));
        for (int l = 0; l < 8; ++l) {
            const GaussGeom G = gauss_geom(xe, l);
            const size_t gp = (size_t)e * 8 + l;
            for (int i = 0; i < 8; ++i) {
                S.Nx[gp * 8 + i] = G.dNdx[i][0];
                S.Ny[gp * 8 + i] = G.dNdx[i][1];
                S.Nz[gp * 8 + i] = G.dNdx[i][2];
            }
            add_btdb(G, S.stiff.data(), ke);
            for (int i = 0; i < 8; ++i)
                for (int j = 0; j < 8; ++j) {
                    const double v = rho * G.N[i] * G.N[j] * G.jacdet;
                    for (int c = 0; c < 3; ++c) me[(3 * i + c) * 24 + 3 * j + c] += v;
                }
        }
        // element DOFs 3*(node-1)+c+1, triplets row-major (src/spmtx.f90:85-97)
        int dofs[24];
        for (int i = 0; i < 8; ++i)
            for (int c = 0; c < 3; ++c) dofs[3 * i + c] = 3 * (mesh.conn[(size_t)e * 8 + i] - 1) + c + 1;
        const size_t base = per * e;
        for (int r = 0; r < 24; ++r)
            for (int c = 0; c < 24; ++c) {
                const size_t k = base + r * 24 + c;
                tk.i[k] = tm.i[k] = dofs[r];
                tk.j[k] = tm.j[k] = dofs[c];
                tk.v[k] = ke[r * 24 + c];
                tm.v[k] = me[r * 24 + c];
            }
    }
    const int ndof = 3 * mesh.nn;
    S.K = tricsr(tk, ndof);
    S.M = tricsr(tm, ndof);
    return S;
}

ThermSystem assemble_therm(const Mesh& mesh, double kappa, double rho, double cp)
{
    ThermSystem S;
    Triplets tk, tm;
    const size_t per = 64;
    tk.i.resize(per * mesh.ne); tk.j.resize(per * mesh.ne); tk.v.resize(per * mesh.ne);
    tm.i.resize(per * mesh.ne); tm.j.resize(per * mesh.ne); tm.v.resize(per * mesh.ne);
    for (int e = 0; e < mesh.ne; ++e) {
        double xe[8][3], ke[64] = {0}, me[64] = {0};
        element_coords(mesh, e, xe);
        for (int l = 0; l < 8; ++l) {
            const GaussGeom G = gauss_geom(xe, l);
            for (int i = 0; i < 8; ++i)
                for (int j = 0; j < 8; ++j) {
                    me[i * 8 + j] += rho * cp * G.N[i] * G.N[j] * G.jacdet;
                    for (int m = 0; m < 3; ++m)
                        ke[i * 8 + j] += kappa * G.dNdx[i][m] * G.dNdx[j][m] * G.jacdet;
                }
        }
        const size_t base = per * e;
        for (int r = 0; r < 8; ++r)
            for (int c = 0; c < 8; ++c) {
                const size_t k = base + r * 8 + c;
                tk.i[k] = tm.i[k] = mesh.conn[(size_t)e * 8 + r];
                tk.j[k] = tm.j[k] = mesh.conn[(size_t)e * 8 + c];
                tk.v[k] = ke[r * 8 + c];
                tm.v[k] = me[r * 8 + c];
            }
    }
    S.K = tricsr(tk, mesh.nn);
    S.M = tricsr(tm, mesh.nn);
    return S;
}

}  // namespace xt
