// dev_post.cu -- the per-Gauss-point strain and stress of the reference's
// output step (mpipostprocess, src/postprocess.f90:106-200) on the device.
//
// For every Gauss point: the element's nodal displacements interpolated at
// the output time with the six temporal shape values (dispinterp,
// src/postprocess.f90:54-76), the six engineering strains from the strain
// rows Nx, Ny, Nz (calstrain, :79-104), the stress D(E, nu) strain with the
// point's own moduli, both zero at a failed point (:184-189).  One thread per
// Gauss point; the solution is read in the reference's block layout.
#include "xt_device.h"

namespace xt {

namespace {

__global__ void k_post_strain(int ngp, int nn, const int* __restrict__ nodes,
                              const double* __restrict__ Nx, const double* __restrict__ Ny,
                              const double* __restrict__ Nz, const double* __restrict__ ym,
                              const double* __restrict__ nu, const int* __restrict__ gpsta,
                              const double* __restrict__ sol, double nt0, double nt1, double nt2,
                              double nt3, double nt4, double nt5, double* __restrict__ strain,
                              double* __restrict__ stress)
{
    const int gp = blockIdx.x * blockDim.x + threadIdx.x;
    if (gp >= ngp) return;
    const double Nt[6] = {nt0, nt1, nt2, nt3, nt4, nt5};
    double e[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 8; ++i) {
        const int nd = nodes[(size_t)gp * 8 + i] - 1;
        double u[3] = {0, 0, 0};
        for (int k = 0; k < 6; ++k)
            for (int c = 0; c < 3; ++c) u[c] += Nt[k] * sol[(size_t)k * nn * 3 + (size_t)nd * 3 + c];
        const double nx = Nx[(size_t)gp * 8 + i], ny = Ny[(size_t)gp * 8 + i], nz = Nz[(size_t)gp * 8 + i];
        e[0] += nx * u[0];
        e[1] += ny * u[1];
        e[2] += nz * u[2];
        e[3] += ny * u[0] + nx * u[1];
        e[4] += nz * u[1] + ny * u[2];
        e[5] += nz * u[0] + nx * u[2];
    }
    double s[6];
    const double E = ym[gp], v = nu[gp];
    const double coef = E / ((1.0 + v) * (1.0 - 2.0 * v));
    for (int i = 0; i < 3; ++i) {
        s[i] = 0.0;
        for (int j = 0; j < 3; ++j) s[i] += (i == j ? coef * (1.0 - v) : coef * v) * e[j];
        s[i + 3] = coef * (1.0 - 2.0 * v) / 2.0 * e[i + 3];
    }
    const bool live = gpsta[gp] != 0;
    for (int i = 0; i < 6; ++i) {
        strain[(size_t)gp * 6 + i] = live ? e[i] : 0.0;
        stress[(size_t)gp * 6 + i] = live ? s[i] : 0.0;
    }
}

}  // namespace

int post_strain_stress(int ngp, int nn, const int* nodes, const double* Nx, const double* Ny,
                       const double* Nz, const double* ym, const double* nu, const int* gpsta,
                       const double* sol_blocks, const double* Nt6, double* strain, double* stress,
                       cudaStream_t s)
{
    if (ngp <= 0) return XT_OK;
    k_post_strain<<<(ngp + 127) / 128, 128, 0, s>>>(ngp, nn, nodes, Nx, Ny, Nz, ym, nu, gpsta,
                                                    sol_blocks, Nt6[0], Nt6[1], Nt6[2], Nt6[3],
                                                    Nt6[4], Nt6[5], strain, stress);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

}  // namespace xt
