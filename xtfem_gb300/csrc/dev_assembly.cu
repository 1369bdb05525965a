// dev_assembly.cu -- spatial stiffness reassembly on the device.
//
// The reference reassembles the mechanical stiffness every slab of a coupled
// run, element by element with per-Gauss-point moduli (mpiglbmtx_m,
// src/mpisubs.f90:69-139, calling setsdstiff and elemtx_m after
// material_update, src/thermoelastic.f90:1-46), and then merges the
// element triplets into CSR (tricsr, src/spmtx.f90:359-407).  Here the
// pattern is fixed once per mesh, so reassembly is two kernels:
//
//   k_element_k   one thread block per element: the geometry of the 2x2x2
//                 Gauss points (shape-function derivatives, Jacobian
//                 determinant; the reference's sign table, abscissa and
//                 closed-form 3x3 inverse) in shared memory, then one thread
//                 per entry (i a, j b) of the 24 x 24 element matrix,
//                 summing over the Gauss points the isotropic B^T D B entry
//                   detJ (lambda N_i,a N_j,b + mu N_i,b N_j,a
//                         + mu delta_ab grad N_i . grad N_j)
//                 with lambda = E nu / ((1 + nu)(1 - 2 nu)) and
//                 mu = E / (2 (1 + nu)) of that Gauss point;
//   k_gather_k    one thread per CSR entry: the sum of its element
//                 contributions in ascending element order (a fixed order,
//                 so the result is the same bits run to run), 1 on the
//                 diagonal of a constrained DOF (csrapplybc semantics).
//
// system_set_mesh gives K the full element pattern once (every DOF pair of
// a shared element, explicit zeros kept, so any moduli fit it) and builds
// the map from K's entries to element-matrix entries on the host.  The FP32
// copy and the node-block form of K are refreshed on the device; the ILU
// factor is not touched (it stays a host computation: the caller downloads
// K and refactors when it wants to).
#include <algorithm>
#include <vector>

#include "solver.h"

namespace xt {

namespace {

constexpr double kGaussAbs = 0.577350269189626;  // src/procs.f90:537

// natural coordinates of the 8 nodes (src/procs.f90:1366-1373 sign table)
__constant__ signed char c_sign[8][3] = {{-1, -1, +1}, {-1, -1, -1}, {-1, +1, -1},
                                         {-1, +1, +1}, {+1, -1, +1}, {+1, -1, -1},
                                         {+1, +1, -1}, {+1, +1, +1}};

__global__ void __launch_bounds__(576)
k_element_k(int ne, const int* __restrict__ conn, const double* __restrict__ xyz,
            const int* __restrict__ gel, const double* __restrict__ ym,
            const double* __restrict__ nu, double* __restrict__ ke)
{
    __shared__ double dN[8][8][3];  // [gauss point][node][x, y, z]
    __shared__ double det[8], lam[8], mu[8];
    const int e = blockIdx.x;
    if (e >= ne) return;
    const int t = threadIdx.x;
    if (t < 8) {
        const int l = t;
        const double g[2] = {-kGaussAbs, kGaussAbs};
        const double xi = g[(l >> 2) & 1], eta = g[(l >> 1) & 1], zeta = g[l & 1];
        double xe[8][3], dn[8][3];
        for (int i = 0; i < 8; ++i) {
            const int nd = conn[(size_t)e * 8 + i];
            for (int m = 0; m < 3; ++m) xe[i][m] = xyz[(size_t)nd * 3 + m];
            const double sx = c_sign[i][0], sy = c_sign[i][1], sz = c_sign[i][2];
            dn[i][0] = 0.125 * sx * (1.0 + sy * eta) * (1.0 + sz * zeta);
            dn[i][1] = 0.125 * sy * (1.0 + sx * xi) * (1.0 + sz * zeta);
            dn[i][2] = 0.125 * sz * (1.0 + sx * xi) * (1.0 + sy * eta);
        }
        double J[3][3];
        for (int a = 0; a < 3; ++a)
            for (int m = 0; m < 3; ++m) {
                double s = 0.0;
                for (int i = 0; i < 8; ++i) s += dn[i][a] * xe[i][m];
                J[a][m] = s;
            }
        const double d = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] +
                         J[0][2] * J[1][0] * J[2][1] - J[0][0] * J[1][2] * J[2][1] -
                         J[0][1] * J[1][0] * J[2][2] - J[0][2] * J[1][1] * J[2][0];
        double inv[3][3];
        inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / d;
        inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / d;
        inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / d;
        inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / d;
        inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / d;
        inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / d;
        inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / d;
        inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / d;
        inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / d;
        for (int i = 0; i < 8; ++i)
            for (int m = 0; m < 3; ++m) {
                double s = 0.0;
                for (int a = 0; a < 3; ++a) s += inv[m][a] * dn[i][a];
                dN[l][i][m] = s;
            }
        det[l] = d;
        const size_t gi = (size_t)(gel ? gel[e] : e) * 8 + l;  // the moduli's element
        const double E = ym[gi], v = nu[gi];
        const double c = E / ((1.0 + v) * (1.0 - 2.0 * v));
        lam[l] = c * v;
        mu[l] = c * (0.5 - v);
    }
    __syncthreads();
    // entry (r, c) of the row-major 24 x 24 element matrix, DOF 3 node + comp
    const int r = t / 24, cc = t - r * 24;
    const int i = r / 3, a = r - 3 * i, j = cc / 3, b = cc - 3 * j;
    double s = 0.0;
    for (int l = 0; l < 8; ++l) {
        double v = lam[l] * dN[l][i][a] * dN[l][j][b] + mu[l] * dN[l][i][b] * dN[l][j][a];
        if (a == b)
            v += mu[l] * (dN[l][i][0] * dN[l][j][0] + dN[l][i][1] * dN[l][j][1] +
                          dN[l][i][2] * dN[l][j][2]);
        s += v * det[l];
    }
    ke[(size_t)e * 576 + t] = s;
}

__global__ void k_gather_k(int nnz, const int* __restrict__ cptr, const int* __restrict__ cidx,
                           const double* __restrict__ ke, const unsigned char* __restrict__ bcdiag,
                           double* __restrict__ kv)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int t = cptr[k]; t < cptr[k + 1]; ++t) s += ke[cidx[t]];
        kv[k] = bcdiag[k] ? 1.0 : s;
    }
}

// Thermal coupling of one element (all elements, one block of 32 threads
// each; threads 0..7 own a Gauss point): the point's temperature from the
// end-of-slab nodal temperatures (the third temporal block), the moduli of
// material_update (src/thermoelastic.f90:21-44: E = E0 - 1.6 dT - 0.1 dT^2,
// nu = nu0 + 5e-5 dT for T >= 0, else E0, nu0; dT = T - Tref), the thermal
// stress of calc_thermo_stress (:66-76: the sum of the first three columns
// of D(E, nu) times alpha dT, for the three normal components) and the
// element vector of elevec_m (src/elesubs.f90:119-167):
// ve(3 i + m) = sum_l dN_i/dx_m(l) sigma_m(l) detJ(l).
__global__ void __launch_bounds__(32)
k_thermal_couple(int ne, const int* __restrict__ conn, const double* __restrict__ xyz,
                 const double* __restrict__ temp, double alpha, double Tref, double ym0,
                 double nu0, double* __restrict__ ym, double* __restrict__ nu,
                 double* __restrict__ ve)
{
    __shared__ double contrib[8][24];
    const int e = blockIdx.x;
    if (e >= ne) return;
    const int l = threadIdx.x;
    if (l < 8) {
        const double g[2] = {-kGaussAbs, kGaussAbs};
        const double xi = g[(l >> 2) & 1], eta = g[(l >> 1) & 1], zeta = g[l & 1];
        double xe[8][3], dn[8][3], N[8];
        double T = 0.0;
        for (int i = 0; i < 8; ++i) {
            const int nd = conn[(size_t)e * 8 + i];
            for (int m = 0; m < 3; ++m) xe[i][m] = xyz[(size_t)nd * 3 + m];
            const double sx = c_sign[i][0], sy = c_sign[i][1], sz = c_sign[i][2];
            N[i] = 0.125 * (1.0 + sx * xi) * (1.0 + sy * eta) * (1.0 + sz * zeta);
            dn[i][0] = 0.125 * sx * (1.0 + sy * eta) * (1.0 + sz * zeta);
            dn[i][1] = 0.125 * sy * (1.0 + sx * xi) * (1.0 + sz * zeta);
            dn[i][2] = 0.125 * sz * (1.0 + sx * xi) * (1.0 + sy * eta);
            T += N[i] * temp[(size_t)nd * 3 + 2];
        }
        double J[3][3];
        for (int a = 0; a < 3; ++a)
            for (int m = 0; m < 3; ++m) {
                double s = 0.0;
                for (int i = 0; i < 8; ++i) s += dn[i][a] * xe[i][m];
                J[a][m] = s;
            }
        const double d = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] +
                         J[0][2] * J[1][0] * J[2][1] - J[0][0] * J[1][2] * J[2][1] -
                         J[0][1] * J[1][0] * J[2][2] - J[0][2] * J[1][1] * J[2][0];
        double inv[3][3];
        inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / d;
        inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / d;
        inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / d;
        inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / d;
        inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / d;
        inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / d;
        inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / d;
        inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / d;
        inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / d;
        const double dT = T - Tref;
        double E = ym0, v = nu0;
        if (T >= 0.0) {
            E = ym0 - 1.6 * dT - 0.1 * dT * dT;
            v = nu0 + 5.e-5 * dT;
        }
        ym[(size_t)e * 8 + l] = E;
        nu[(size_t)e * 8 + l] = v;
        const double c = E / ((1.0 + v) * (1.0 - 2.0 * v));
        // D(m, 1) + D(m, 2) + D(m, 3) = c (1 - nu) + 2 c nu for m = 1..3
        const double sig = (c * (1.0 - v) + 2.0 * c * v) * (alpha * dT);
        for (int i = 0; i < 8; ++i)
            for (int m = 0; m < 3; ++m) {
                double dx = 0.0;
                for (int a = 0; a < 3; ++a) dx += inv[m][a] * dn[i][a];
                contrib[l][3 * i + m] = dx * sig * d;
            }
    }
    __syncthreads();
    if (l < 24) {
        double s = 0.0;
        for (int g = 0; g < 8; ++g) s += contrib[g][l];  // Gauss points in order
        ve[(size_t)e * 24 + l] = s;
    }
}

// y[k] = sum of x over the listed entries, in list order
__global__ void k_gather_list(int n, const int* __restrict__ ptr, const int* __restrict__ idx,
                              const double* __restrict__ x, double* __restrict__ y)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int t = ptr[k]; t < ptr[k + 1]; ++t) s += x[idx[t]];
        y[k] = s;
    }
}

}  // namespace

int system_set_mesh(System& S, int nn, int ne, const double* xyz, const int* conn, const int* bc,
                    const int* gel)
{
    DevAssembly& A = S.asmb;
    A.ok = false;
    if (nn <= 0 || ne <= 0 || !xyz || !conn || !bc || 3 * nn != S.p) {
        set_error("system_set_mesh: need 3 nn = p and non-null mesh arrays");
        return XT_ERR_ARG;
    }
    cudaStream_t s = S.stream;
    const int n = S.p;
    std::vector<int> conn0((size_t)ne * 8);
    for (size_t k = 0; k < conn0.size(); ++k) {
        conn0[k] = conn[k] - 1;
        if (conn0[k] < 0 || conn0[k] >= nn) {
            set_error("system_set_mesh: connectivity out of range");
            return XT_ERR_ARG;
        }
    }
    // K's pattern becomes the full element pattern: every DOF pair of a
    // shared element, whatever its value (entries that vanish for one set
    // of moduli need not vanish for another); a constrained DOF's row and
    // column keep only the diagonal.
    std::vector<std::vector<int>> nbr(nn);
    for (int e = 0; e < ne; ++e)
        for (int i = 0; i < 8; ++i)
            for (int j = 0; j < 8; ++j)
                nbr[conn0[(size_t)e * 8 + i]].push_back(conn0[(size_t)e * 8 + j]);
    std::vector<int> rp(n + 1, 0), col;
    for (int a = 0; a < nn; ++a) {
        auto& v = nbr[a];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        for (int c = 0; c < 3; ++c) {
            const int g = 3 * a + c;
            if (bc[g]) {
                col.push_back(g);
            } else {
                for (int b : v)
                    for (int d = 0; d < 3; ++d)
                        if (!bc[3 * b + d]) col.push_back(3 * b + d);
            }
            rp[g + 1] = (int)col.size();
        }
    }
    const int nnz = (int)col.size();
    auto find = [&](int row, int c) {
        const int* b = col.data() + rp[row];
        const int* e = col.data() + rp[row + 1];
        const int* it = std::lower_bound(b, e, c);
        return (it != e && *it == c) ? (int)(it - col.data()) : -1;
    };
    // the current values carried over into the new pattern
    const int onnz = S.K.nnz;
    std::vector<int> orp(n + 1), ocol(onnz);
    std::vector<double> oval(onnz), val(nnz, 0.0);
    XT_CUDA(cudaMemcpyAsync(orp.data(), S.K.rowptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
    XT_CUDA(cudaMemcpyAsync(ocol.data(), S.K.col.p, sizeof(int) * onnz, cudaMemcpyDeviceToHost, s));
    XT_CUDA(cudaMemcpyAsync(oval.data(), S.K.v64.p, sizeof(double) * onnz, cudaMemcpyDeviceToHost, s));
    XT_CUDA(cudaStreamSynchronize(s));
    for (int r = 0; r < n; ++r)
        for (int k = orp[r]; k < orp[r + 1]; ++k) {
            const int at = find(r, ocol[k]);
            if (at < 0) {
                set_error("system_set_mesh: K has an entry outside the mesh's element pattern");
                return XT_ERR_ARG;
            }
            val[at] = oval[k];
        }
    // element-matrix entries per K entry, in ascending element order
    std::vector<int> cnt(nnz + 1, 0), where((size_t)ne * 576, -1);
    for (int e = 0; e < ne; ++e)
        for (int r = 0; r < 24; ++r) {
            const int gr = 3 * conn0[(size_t)e * 8 + r / 3] + r % 3;
            if (bc[gr]) continue;
            for (int c = 0; c < 24; ++c) {
                const int gc = 3 * conn0[(size_t)e * 8 + c / 3] + c % 3;
                if (bc[gc]) continue;
                const int k = find(gr, gc);
                where[(size_t)e * 576 + r * 24 + c] = k;
                ++cnt[k + 1];
            }
        }
    std::vector<unsigned char> bcd(nnz, 0);
    for (int g = 0; g < n; ++g)
        if (bc[g]) bcd[rp[g]] = 1;
    for (int k = 0; k < nnz; ++k) cnt[k + 1] += cnt[k];
    std::vector<int> idx(cnt[nnz]), fill(cnt.begin(), cnt.end() - 1);
    for (size_t t = 0; t < where.size(); ++t)
        if (where[t] >= 0) idx[fill[where[t]]++] = (int)t;
    // the new K (1-based host copy for the upload and the node-block form)
    std::vector<int> ia(n + 1), ja(nnz);
    for (int r = 0; r <= n; ++r) ia[r] = rp[r] + 1;
    for (int k = 0; k < nnz; ++k) ja[k] = col[k] + 1;
    const int mnnz = S.M.nnz;
    std::vector<int> mrp(n + 1), mcol(mnnz);
    std::vector<double> mval(mnnz);
    XT_CUDA(cudaMemcpyAsync(mrp.data(), S.M.rowptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
    XT_CUDA(cudaMemcpyAsync(mcol.data(), S.M.col.p, sizeof(int) * mnnz, cudaMemcpyDeviceToHost, s));
    XT_CUDA(cudaMemcpyAsync(mval.data(), S.M.v64.p, sizeof(double) * mnnz, cudaMemcpyDeviceToHost, s));
    XT_CUDA(cudaStreamSynchronize(s));
    for (int& v : mrp) ++v;
    for (int& v : mcol) ++v;
    XT_TRY(upload_csr(S.K, n, ia.data(), ja.data(), val.data(), s));
    XT_TRY(csr_build_node_blocks(S.K, n, ia.data(), ja.data(), val.data(), mrp.data(), mcol.data(),
                                 mval.data(), s));
    A.nn = nn;
    A.ne = ne;
    XT_TRY(A.xyz.upload(xyz, (size_t)nn * 3, s));
    XT_TRY(A.conn.upload(conn0.data(), conn0.size(), s));
    XT_TRY(A.cptr.upload(cnt.data(), cnt.size(), s));
    XT_TRY(A.cidx.upload(idx.data(), idx.size(), s));
    XT_TRY(A.bcdiag.upload(bcd.data(), bcd.size(), s));
    if (gel) {
        XT_TRY(A.gel.upload(gel, (size_t)ne, s));
    } else {
        A.gel.release();
    }
    XT_TRY(A.ke.alloc((size_t)ne * 576));
    XT_TRY(A.ym.alloc((size_t)ne * 8));
    XT_TRY(A.nu.alloc((size_t)ne * 8));
    XT_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
    A.ok = true;
    return XT_OK;
}

int system_assemble_k(System& S, const double* ym, const double* nu)
{
    DevAssembly& A = S.asmb;
    if (!A.ok) {
        set_error("system_assemble_k: no mesh set");
        return XT_ERR_STATE;
    }
    cudaStream_t s = S.stream;
    XT_CUDA(cudaMemcpyAsync(A.ym.p, ym, sizeof(double) * A.ne * 8, cudaMemcpyHostToDevice, s));
    XT_CUDA(cudaMemcpyAsync(A.nu.p, nu, sizeof(double) * A.ne * 8, cudaMemcpyHostToDevice, s));
    XT_TRY(system_assemble_k_device(S, A.ym.p, A.nu.p, false));
    XT_CUDA(cudaStreamSynchronize(s));  // the host ym, nu may be reused at once
    return XT_OK;
}

int system_assemble_k_device(System& S, const double* ym, const double* nu, bool by_gel)
{
    DevAssembly& A = S.asmb;
    if (!A.ok) {
        set_error("system_assemble_k: no mesh set");
        return XT_ERR_STATE;
    }
    cudaStream_t s = S.stream;
    k_element_k<<<A.ne, 576, 0, s>>>(A.ne, A.conn.p, A.xyz.p, by_gel ? A.gel.p : nullptr, ym, nu,
                                     A.ke.p);
    const int nnz = S.K.nnz;
    const int blocks = std::max(1, std::min(4096, (nnz + 255) / 256));
    k_gather_k<<<blocks, 256, 0, s>>>(nnz, A.cptr.p, A.cidx.p, A.ke.p, A.bcdiag.p, S.K.v64.p);
    note_launches(2);
    XT_CUDA(cudaGetLastError());
    XT_TRY(to_f32(S.K.v64.p, S.K.v32.p, (size_t)nnz, s));
    S.K.vdf.release();  // remade from the new values on first use
    XT_TRY(node_blocks_refresh(S.K, s));
    return XT_OK;
}

int thermal_couple_device(int ne, const int* conn0, const double* xyz, const double* temp,
                          double alpha, double Tref, double ym0, double nu0, double* ym, double* nu,
                          double* ve, cudaStream_t s)
{
    k_thermal_couple<<<ne, 32, 0, s>>>(ne, conn0, xyz, temp, alpha, Tref, ym0, nu0, ym, nu, ve);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int gather_list(int n, const int* ptr, const int* idx, const double* x, double* y, cudaStream_t s)
{
    k_gather_list<<<std::max(1, std::min(4096, (n + 255) / 256)), 256, 0, s>>>(n, ptr, idx, x, y);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

}  // namespace xt
