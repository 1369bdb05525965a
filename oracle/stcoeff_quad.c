/*
 * stcoeff_quad.c -- oracle statement of the temporal coefficient matrices of
 * src/stcoeff.f90:62-356 and the temporal load weights of
 * src/getfextc.f90:22-58, obtained from their definitions instead of the
 * reference's closed forms:
 *
 *   basis on the slab [t1, t1+dt] with nodes t_a = t1 + (a-1) dt/2:
 *     N_a      quadratic Lagrange, a = 1..3
 *     N_{3+a}  = N_a(t) (sin(w t) - sin(w t_a))      (src/kokkos_damage.f90:44-46)
 *   k(i,j)    = int N_i'(t) N_j(t) dt
 *   m(i,j)    = int N_i'(t) N_j''(t) dt
 *   ktn(i,j)  = N_i(t1) N_j(t1)
 *   mtn(i,j)  = N_i'(t1) N_j'(t1)
 *   ktn1(i,j) = N_i(t1) N_j(t1+dt)
 *   mtn1(i,j) = N_i'(t1) N_j'(t1+dt)
 *   fextc(j)  = int N_j'(t) sin(w t) dt
 *
 * The integrals are evaluated by composite Gauss-Legendre quadrature fine
 * enough for the oscillating enrichment.  ktn1/mtn1 take the column
 * functions at the end of the same slab, which is how the reference's closed
 * forms are written (its column terms carry sin/cos of (t1+dt) w).
 *
 * The thermal slab (src/stcoeff.f90:1-60) uses the three quadratic
 * Lagrange functions alone, first order in time:
 *   k(i,j)    = int N_i(t) N_j(t) dt        (with the conductivity)
 *   m(i,j)    = int N_i(t) N_j'(t) dt       (with the capacity)
 *   mtn(i,j)  = N_i(t1) N_j(t1),  mtn1(i,j) = N_i(t1) N_j(t1+dt)
 *   ktn = ktn1 = 0
 *
 * TEST INFRASTRUCTURE ONLY (the checker); see xt_oracle.h.
 */
#include "xt_oracle.h"

#include <math.h>

typedef struct { double v, d1, d2; } jet;

/* value, first and second derivative of basis function a (0..5) at t */
static jet basis(int a, double t, double t1, double dt, double w)
{
    const double tn[3] = {t1, t1 + 0.5 * dt, t1 + dt};
    const int b = a % 3;
    const int o1 = (b + 1) % 3, o2 = (b + 2) % 3;
    const double den = (tn[b] - tn[o1]) * (tn[b] - tn[o2]);
    jet L;
    L.v = (t - tn[o1]) * (t - tn[o2]) / den;
    L.d1 = ((t - tn[o1]) + (t - tn[o2])) / den;
    L.d2 = 2.0 / den;
    if (a < 3) return L;
    const double g = sin(w * t) - sin(w * tn[b]);
    const double g1 = w * cos(w * t);
    const double g2 = -w * w * sin(w * t);
    jet E;
    E.v = L.v * g;
    E.d1 = L.d1 * g + L.v * g1;
    E.d2 = L.d2 * g + 2.0 * L.d1 * g1 + L.v * g2;
    return E;
}

/* 8-point Gauss-Legendre on [-1, 1] */
static const double GX[8] = {-0.9602898564975363, -0.7966664774136267,
                             -0.5255324099163290, -0.1834346424956498,
                             0.1834346424956498,  0.5255324099163290,
                             0.7966664774136267,  0.9602898564975363};
static const double GW[8] = {0.1012285362903763, 0.2223810344533745,
                             0.3137066458778873, 0.3626837833783620,
                             0.3626837833783620, 0.3137066458778873,
                             0.2223810344533745, 0.1012285362903763};

#define NSUB 512

void orc_stcoeff_m_quad(double t1, double dt, double w, double *k, double *m,
                        double *ktn, double *mtn, double *ktn1, double *mtn1)
{
    for (int e = 0; e < 36; ++e) k[e] = m[e] = 0.0;
    const double h = dt / NSUB;
    for (int s = 0; s < NSUB; ++s) {
        const double c = t1 + (s + 0.5) * h;
        for (int g = 0; g < 8; ++g) {
            const double t = c + 0.5 * h * GX[g];
            const double wt = 0.5 * h * GW[g];
            jet B[6];
            for (int a = 0; a < 6; ++a) B[a] = basis(a, t, t1, dt, w);
            for (int i = 0; i < 6; ++i)
                for (int j = 0; j < 6; ++j) {
                    k[j * 6 + i] += wt * B[i].d1 * B[j].v;
                    m[j * 6 + i] += wt * B[i].d1 * B[j].d2;
                }
        }
    }
    jet S[6], T[6];
    for (int a = 0; a < 6; ++a) {
        S[a] = basis(a, t1, t1, dt, w);
        T[a] = basis(a, t1 + dt, t1, dt, w);
    }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            ktn[j * 6 + i] = S[i].v * S[j].v;
            mtn[j * 6 + i] = S[i].d1 * S[j].d1;
            ktn1[j * 6 + i] = S[i].v * T[j].v;
            mtn1[j * 6 + i] = S[i].d1 * T[j].d1;
        }
}

void orc_getfextc_m_quad(double t1, double w, double dt, double *fextc)
{
    for (int j = 0; j < 6; ++j) fextc[j] = 0.0;
    const double h = dt / NSUB;
    for (int s = 0; s < NSUB; ++s) {
        const double c = t1 + (s + 0.5) * h;
        for (int g = 0; g < 8; ++g) {
            const double t = c + 0.5 * h * GX[g];
            const double wt = 0.5 * h * GW[g];
            for (int j = 0; j < 6; ++j)
                fextc[j] += wt * basis(j, t, t1, dt, w).d1 * sin(w * t);
        }
    }
}

void orc_stcoeff_t_quad(double dt, double *k, double *m, double *ktn,
                        double *mtn, double *ktn1, double *mtn1)
{
    for (int e = 0; e < 9; ++e) k[e] = m[e] = ktn[e] = mtn[e] = ktn1[e] = mtn1[e] = 0.0;
    const double h = dt / NSUB;
    for (int s = 0; s < NSUB; ++s) {
        const double c = (s + 0.5) * h;
        for (int g = 0; g < 8; ++g) {
            const double t = c + 0.5 * h * GX[g];
            const double wt = 0.5 * h * GW[g];
            jet B[3];
            for (int a = 0; a < 3; ++a) B[a] = basis(a, t, 0.0, dt, 0.0);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    k[j * 3 + i] += wt * B[i].v * B[j].v;
                    m[j * 3 + i] += wt * B[i].v * B[j].d1;
                }
        }
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const jet Si = basis(i, 0.0, 0.0, dt, 0.0);
            mtn[j * 3 + i] = Si.v * basis(j, 0.0, 0.0, dt, 0.0).v;
            mtn1[j * 3 + i] = Si.v * basis(j, dt, 0.0, dt, 0.0).v;
        }
}

void orc_fint_m_def(double t1, double w, double dt, double *fint)
{
    /* int N_j'(t) dt over the slab = N_j(t1+dt) - N_j(t1), exactly */
    for (int j = 0; j < 6; ++j)
        fint[j] = basis(j, t1 + dt, t1, dt, w).v - basis(j, t1, t1, dt, w).v;
}
