/*
 * damage.c -- oracle restatement of the two-scale fatigue-damage update
 * (src/kokkos_kernel.h:45-344 with constants src/damage.h:9-17), of the
 * temporal shape table built by src/kokkos_damage.f90:36-47, a second
 * statement of the same law after src/getdfinal.f:10-397, of the
 * failed-point clean-up src/kokkos_damage.f90:102-107 and of the element
 * status test chkelesta (src/delelement.f90:109-136).
 *
 * TEST INFRASTRUCTURE ONLY (the checker); see xt_oracle.h.
 *
 * The floating-point expressions keep the association order of the
 * reference so that the oracle is a faithful FP64 statement of it; the
 * library is built with -ffp-contract=off so that x86 and Arm hosts give
 * identical results.
 */
#include "xt_oracle.h"

#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/damage.h:9-17 */
#define DM_CY 1740.0
#define DM_H 0.2
#define DM_S 0.5
#define DM_SEXP 0.5
#define DM_SIGF 180.0
#define DM_SIGU 577.0
#define DM_EPSD 0.08
#define DM_WD ((DM_SIGU - DM_SIGF) * DM_EPSD)

/* src/kokkos_damage.f90:36-47 */
void orc_nt_table(int nip, const double *tc, double w, double *Nt)
{
    const double dt = tc[2] - tc[0];
    for (int i = 0; i < nip; ++i) {
        const double t = tc[0] + (double)i * dt / (double)nip;
        const double n1 = 2.0 * (tc[1] - t) * (tc[2] - t) / (dt * dt);
        const double n2 = -4.0 * (tc[0] - t) * (tc[2] - t) / (dt * dt);
        const double n3 = 2.0 * (tc[0] - t) * (tc[1] - t) / (dt * dt);
        double *row = Nt + (size_t)i * 6;
        row[0] = n1;
        row[1] = n2;
        row[2] = n3;
        row[3] = n1 * (sin(w * t) - sin(w * tc[0]));
        row[4] = n2 * (sin(w * t) - sin(w * tc[1]));
        row[5] = n3 * (sin(w * t) - sin(w * tc[2]));
    }
}

/* von Mises-type equivalent of a symmetric tensor in Voigt order with
 * engineering shear components: sqrt(1.5 sum s_n^2 + 3 sum s_s^2) of the
 * given (already deviatoric) vector. */
static double vm_equiv(const double s[6])
{
    double e = 0.0;
    for (int i = 0; i < 3; ++i) e += 1.5 * s[i] * s[i];
    for (int i = 3; i < 6; ++i) e += 3.0 * s[i] * s[i];
    return sqrt(e);
}

/* deviator of a Voigt vector: normal parts minus the mean of the three */
static void deviator(const double s[6], double out[6])
{
    double tr = 0.0;
    for (int i = 0; i < 3; ++i) tr += s[i];
    tr = tr / 3.0;
    out[0] = s[0] - tr;
    out[1] = s[1] - tr;
    out[2] = s[2] - tr;
    out[3] = s[3];
    out[4] = s[4];
    out[5] = s[5];
}

/* One Gauss point over all nip temporal points (src/kokkos_kernel.h:45-344). */
static void damage_point(int gp, int nn, int ndofn, int nnse, int nnte,
                         int ncmp, int nip, const int *nodes,
                         const double *Nx, const double *Ny, const double *Nz,
                         const double *Nt, const double *sol,
                         const double *ym, const double *nu,
                         double *eps_old, double *eps_pl, double *sig_eff,
                         double *sig_back, double *pp, double *D, double *ws,
                         double *del_po, double *sig_d)
{
    const double v = nu[gp], E = ym[gp];
    const double ca = (1.0 + v) / (3.0 * (1.0 - v));
    const double cb = 2.0 * (4.0 - 5.0 * v) / (15.0 * (1.0 - v));
    const double G = E / (2.0 * (1.0 + v));
    const double Kb = E / (3.0 * (1.0 - 2.0 * v));
    const double coef = E / ((1.0 + v) * (1.0 - 2.0 * v));
    double dmat[6][6];
    memset(dmat, 0, sizeof(dmat));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) dmat[i][j] = coef * v;
    for (int i = 0; i < 3; ++i) {
        dmat[i][i] = coef * (1.0 - v);
        dmat[i + 3][i + 3] = coef * (1.0 - 2.0 * v) / 2.0;
    }
    double *epo = eps_old + (size_t)gp * ncmp;
    double *epl = eps_pl + (size_t)gp * ncmp;
    double *sef = sig_eff + (size_t)gp * ncmp;
    double *sbk = sig_back + (size_t)gp * ncmp;
    const int nt = 2 * nnte;

    for (int jj = 0; jj < nip; ++jj) {
        /* displacement at the temporal point, then the strain */
        double disp[24] = {0.0};
        for (int i = 0; i < nnse; ++i) {
            const int nd = nodes[(size_t)gp * nnse + i] - 1;
            for (int j = 0; j < ndofn; ++j)
                for (int k = 0; k < nt; ++k) {
                    const size_t dof = (size_t)k * nn * ndofn + (size_t)nd * ndofn + j;
                    disp[i * ndofn + j] += Nt[(size_t)jj * nt + k] * sol[dof];
                }
        }
        double eps[6] = {0.0};
        for (int i = 0; i < nnse; ++i) {
            const double nx = Nx[(size_t)gp * nnse + i];
            const double ny = Ny[(size_t)gp * nnse + i];
            const double nz = Nz[(size_t)gp * nnse + i];
            const double *u = disp + i * ndofn;
            eps[0] += nx * u[0];
            eps[1] += ny * u[1];
            eps[2] += nz * u[2];
            eps[3] += ny * u[0] + nx * u[1];
            eps[4] += nz * u[1] + ny * u[2];
            eps[5] += nz * u[0] + nx * u[2];
        }
        const double d = D[gp];
        /* elastic prediction */
        const double c1 = 1.0 / (1.0 - cb * d);
        const double c2 = (ca - cb) * d / ((1.0 - cb * d) * (1.0 - ca * d));
        const double c3 = cb * (1.0 - d) / (1.0 - cb * d);
        double tel[6], tee[6], tse[6], tdev[6], tsig[6];
        for (int i = 0; i < 6; ++i) tel[i] = c1 * eps[i] + c3 * epl[i];
        double tr = 0.0;
        for (int i = 0; i < 3; ++i) tr += eps[i];
        tr = c2 * tr / 3.0;
        for (int i = 0; i < 3; ++i) tel[i] += tr;
        for (int i = 0; i < 6; ++i) tee[i] = tel[i] - epl[i];
        for (int i = 0; i < 6; ++i) {
            double acc = 0.0;
            for (int j = 0; j < 6; ++j) acc += dmat[i][j] * tee[j];
            tse[i] = acc;
        }
        deviator(tse, tdev);
        for (int i = 0; i < 6; ++i) tsig[i] = tdev[i] - sbk[i];
        const double teq = vm_equiv(tsig);
        if (teq <= DM_SIGF) {
            for (int i = 0; i < 6; ++i) { sef[i] = tse[i]; epo[i] = eps[i]; }
            sig_d[gp] = teq;
            continue;
        }
        /* plastic correction */
        double de[6], ds[6], qs[6], dq[6];
        for (int i = 0; i < 6; ++i) de[i] = eps[i] - epo[i];
        for (int i = 0; i < 6; ++i) {
            double acc = 0.0;
            for (int j = 0; j < 6; ++j) acc += dmat[i][j] * de[j];
            ds[i] = acc / (1.0 - cb * d);
        }
        const double c4 = Kb * (ca - cb) * d / ((1.0 - cb * d) * (1.0 - ca * d));
        double trd = 0.0;
        for (int i = 0; i < 3; ++i) trd += de[i];
        for (int i = 0; i < 3; ++i) ds[i] += c4 * trd;
        for (int i = 0; i < 6; ++i) qs[i] = sbk[i] - sef[i] - ds[i];
        const double gam = DM_CY * (1.0 - d) + 3.0 * G * (1.0 - cb) / (1.0 - cb * d);
        double trq = 0.0;
        for (int i = 0; i < 3; ++i) trq += qs[i];
        trq = trq / 3.0;
        dq[0] = qs[0] - trq;
        dq[1] = qs[1] - trq;
        dq[2] = qs[2] - trq;
        dq[3] = qs[3];
        dq[4] = qs[4];
        dq[5] = qs[5];
        const double qeq = vm_equiv(dq);
        const double trs = -trq;
        const double dp = (qeq - DM_SIGF) / gam;
        pp[gp] += dp;
        const double c5 = 1.0 + gam * dp / DM_SIGF;
        double dsg[6], sg[6], dpl[6];
        for (int i = 0; i < 6; ++i) dsg[i] = -dq[i] / c5;
        sg[0] = dsg[0] + trs;
        sg[1] = dsg[1] + trs;
        sg[2] = dsg[2] + trs;
        sg[3] = dsg[3];
        sg[4] = dsg[4];
        sg[5] = dsg[5];
        for (int i = 0; i < 6; ++i) {
            dpl[i] = 3.0 * dsg[i] * dp / (2.0 * DM_SIGF);
            epl[i] += dpl[i];
        }
        for (int i = 0; i < 6; ++i) sbk[i] += 2.0 * DM_CY * (1.0 - d) * dpl[i] / 3.0;
        for (int i = 0; i < 6; ++i) sef[i] = sg[i] + sbk[i];
        double sdev[6];
        deviator(sef, sdev);
        const double seq = vm_equiv(sdev);
        const double snew = fabs(seq - DM_SIGF);
        const double sold = fabs(sig_d[gp] - DM_SIGF);
        ws[gp] += (snew * dp + sold * del_po[gp]) / 2.0;
        if (ws[gp] >= DM_WD) {
            double sp[3] = {0.0, 0.0, 0.0}, sn[3] = {0.0, 0.0, 0.0};
            for (int i = 0; i < 3; ++i) {
                if (sef[i] < 0.0) sn[i] = sef[i];
                else sp[i] = sef[i];
            }
            const double x = (1.0 - d) / (1.0 - DM_H * d);
            const double yp = (1.0 + v) / (2.0 * E) *
                (sp[0] * sp[0] + sp[1] * sp[1] + sp[2] * sp[2] +
                 DM_H * x * x * (sn[0] * sn[0] + sn[1] * sn[1] + sn[2] * sn[2]));
            double trs2 = 0.0;
            for (int i = 0; i < 3; ++i) trs2 += sef[i];
            double yn;
            if (trs2 >= 0.0) yn = v / (2.0 * E) * trs2 * trs2;
            else yn = v / (2.0 * E) * DM_H * x * x * trs2 * trs2;
            const double Y = yp - yn;
            D[gp] += pow(Y / DM_S, DM_SEXP) * dp;
        } else {
            D[gp] = 0.0;
        }
        for (int i = 0; i < 6; ++i) epo[i] = eps[i];
        sig_d[gp] = seq;
        del_po[gp] = dp;
    }
}

void orc_damage(int ne, int nn, int ndofn, int nnse, int nnte, int ngpe,
                int ncmp, int nip, const int *nodes, const double *Nx,
                const double *Ny, const double *Nz, const double *Nt,
                const double *sol, const double *ym, const double *nu,
                double *eps_old, double *eps_pl, double *sig_eff,
                double *sig_back, double *p, double *D, double *ws,
                double *del_po, double *sig_d, int nthreads)
{
    const int ngp = ngpe * ne;
#ifdef _OPENMP
    if (nthreads > 1) {
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
        for (int gp = 0; gp < ngp; ++gp)
            damage_point(gp, nn, ndofn, nnse, nnte, ncmp, nip, nodes, Nx, Ny,
                         Nz, Nt, sol, ym, nu, eps_old, eps_pl, sig_eff,
                         sig_back, p, D, ws, del_po, sig_d);
        return;
    }
#else
    (void)nthreads;
#endif
    for (int gp = 0; gp < ngp; ++gp)
        damage_point(gp, nn, ndofn, nnse, nnte, ncmp, nip, nodes, Nx, Ny, Nz,
                     Nt, sol, ym, nu, eps_old, eps_pl, sig_eff, sig_back, p,
                     D, ws, del_po, sig_d);
}

/* src/getdfinal.f:10-397, the reference's second (stand-alone, F77)
 * statement of the same two-scale law: one strain increment per call, from
 * the previous global strain strain_tgo to strain_tg.  It is written here
 * independently of damage_point above, following getdfinal's own steps:
 * the elastic stiffness from the Lame constants (lambda + 2G, lambda, G),
 * the localisation constants a, b, the bulk modulus in the plastic
 * corrector, and the equivalent stress 1.5 (sum s_n^2 + 2 sum s_s^2).  The
 * reference hard-codes E = 1.97e5 and nu = 0.3 and takes dmat from its
 * caller; here E and nu are arguments (the per-point override), so both
 * statements can be run on the same point. */
static void getdfinal_step(const double eg[6], double ego[6], double epl[6],
                           double *p, double *D, double *ws, double se[6],
                           double bs[6], double *dpo, double *sd, double E,
                           double nu)
{
    const double G = E / (2.0 * (1.0 + nu));
    const double bulk = E / (3.0 * (1.0 - 2.0 * nu));
    const double lam = bulk - 2.0 / 3.0 * G;
    const double a = (1.0 + nu) / (3.0 * (1.0 - nu));
    const double b = 2.0 * (4.0 - 5.0 * nu) / (15.0 * (1.0 - nu));
    const double d = *D;
    /* isotropic stiffness applied to a Voigt vector (engineering shear) */
#define STIFF(in, out)                                                      \
    do {                                                                    \
        const double tr_ = (in)[0] + (in)[1] + (in)[2];                     \
        for (int j = 0; j < 3; ++j) (out)[j] = lam * tr_ + 2.0 * G * (in)[j]; \
        for (int j = 3; j < 6; ++j) (out)[j] = G * (in)[j];                 \
    } while (0)
    /* elastic predictor: local strain (eq. 40), elastic part (41), stress (42) */
    const double k1 = 1.0 / (1.0 - b * d);
    const double k2 = (a - b) * d / ((1.0 - b * d) * (1.0 - a * d));
    const double k3 = b * (1.0 - d) / (1.0 - b * d);
    double loc[6], el[6], trial[6];
    const double vol = k2 * (eg[0] + eg[1] + eg[2]) / 3.0;
    for (int j = 0; j < 6; ++j) loc[j] = k1 * eg[j] + k3 * epl[j] + (j < 3 ? vol : 0.0);
    for (int j = 0; j < 6; ++j) el[j] = loc[j] - epl[j];
    STIFF(el, trial);
    const double mt = (trial[0] + trial[1] + trial[2]) / 3.0;
    double rel[6];
    for (int j = 0; j < 6; ++j) rel[j] = trial[j] - (j < 3 ? mt : 0.0) - bs[j];
    const double teq = sqrt(1.5 * (rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2] +
                                   2.0 * (rel[3] * rel[3] + rel[4] * rel[4] + rel[5] * rel[5])));
    if (teq <= DM_SIGF) {
        for (int j = 0; j < 6; ++j) { se[j] = trial[j]; ego[j] = eg[j]; }
        *sd = teq;
        return;
    }
    /* plastic corrector (eqs. 162-175) */
    double de[6], dsg[6], q[6];
    for (int j = 0; j < 6; ++j) de[j] = eg[j] - ego[j];
    STIFF(de, dsg);
    for (int j = 0; j < 6; ++j) dsg[j] /= (1.0 - b * d);
    const double k4 = bulk * (a - b) * d / ((1.0 - b * d) * (1.0 - a * d));
    const double trde = de[0] + de[1] + de[2];
    for (int j = 0; j < 3; ++j) dsg[j] += k4 * trde;
    for (int j = 0; j < 6; ++j) q[j] = bs[j] - se[j] - dsg[j];
    const double eta = DM_CY * (1.0 - d) + 3.0 * G * ((1.0 - b) / (1.0 - b * d));
    const double mq = (q[0] + q[1] + q[2]) / 3.0;
    double dq[6];
    for (int j = 0; j < 6; ++j) dq[j] = q[j] - (j < 3 ? mq : 0.0);
    const double qeq = sqrt(1.5 * (dq[0] * dq[0] + dq[1] * dq[1] + dq[2] * dq[2] +
                                   2.0 * (dq[3] * dq[3] + dq[4] * dq[4] + dq[5] * dq[5])));
    const double dp = (qeq - DM_SIGF) / eta;
    *p += dp;
    const double k5 = 1.0 + eta * dp / DM_SIGF;
    double sdev[6], dpl[6];
    for (int j = 0; j < 6; ++j) sdev[j] = -dq[j] / k5;
    for (int j = 0; j < 6; ++j) {
        dpl[j] = 3.0 * sdev[j] * dp / (2.0 * DM_SIGF);
        epl[j] += dpl[j];
    }
    for (int j = 0; j < 6; ++j) bs[j] += 2.0 * DM_CY * (1.0 - d) * dpl[j] / 3.0;
    for (int j = 0; j < 6; ++j) se[j] = sdev[j] + (j < 3 ? -mq : 0.0) + bs[j];
    const double ms = (se[0] + se[1] + se[2]) / 3.0;
    double sv[6];
    for (int j = 0; j < 6; ++j) sv[j] = se[j] - (j < 3 ? ms : 0.0);
    const double seq = sqrt(1.5 * (sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2] +
                                   2.0 * (sv[3] * sv[3] + sv[4] * sv[4] + sv[5] * sv[5])));
    /* stored energy (eq. 147) and damage (eqs. 177-178) */
    *ws += (fabs(seq - DM_SIGF) * dp + fabs(*sd - DM_SIGF) * *dpo) / 2.0;
    if (*ws >= DM_WD) {
        const double x = (1.0 - d) / (1.0 - DM_H * d);
        double pos = 0.0, neg = 0.0;
        for (int j = 0; j < 3; ++j) {
            if (se[j] < 0.0) neg += se[j] * se[j];
            else pos += se[j] * se[j];
        }
        const double tr = se[0] + se[1] + se[2];
        const double yp = (1.0 + nu) / (2.0 * E) * (pos + DM_H * x * x * neg);
        const double yn = tr >= 0.0 ? nu / (2.0 * E) * tr * tr
                                    : nu / (2.0 * E) * (DM_H * x * x * tr * tr);
        *D = d + pow((yp - yn) / DM_S, DM_SEXP) * dp;
    } else {
        *D = 0.0;
    }
    for (int j = 0; j < 6; ++j) ego[j] = eg[j];
    *sd = seq;
    *dpo = dp;
#undef STIFF
}

void orc_getdfinal_history(int nsteps, const double *eps, double *eps_old,
                           double *eps_pl, double *sig_eff, double *sig_back,
                           double *p, double *D, double *ws, double *del_po,
                           double *sig_d, double E, double nu)
{
    for (int s = 0; s < nsteps; ++s)
        getdfinal_step(eps + (size_t)s * 6, eps_old, eps_pl, p, D, ws, sig_eff,
                       sig_back, del_po, sig_d, E, nu);
}

void orc_damage_cleanup(int ngp, const int *gpsta, double *D, double *ws)
{
    for (int i = 0; i < ngp; ++i)
        if (gpsta[i] == 0) { D[i] = 0.0; ws[i] = 0.0; }
}

int orc_chkelesta(int ne, int ngpe, double Dc, const double *D, int *elesta,
                  int *gpsta, int *nefail)
{
    int nef = 0;
    for (int i = 0; i < ne; ++i) nefail[i] = 0;
    for (int e = 0; e < ne; ++e) {
        int hit = 0;
        for (int g = 0; g < ngpe; ++g)
            if (D[(size_t)e * ngpe + g] >= Dc) hit = 1;
        if (hit) {
            for (int g = 0; g < ngpe; ++g) gpsta[(size_t)e * ngpe + g] = 0;
            elesta[e] = 0;
            nefail[nef++] = e + 1;
        }
    }
    return nef;
}
