// dev_damage.cu -- per-Gauss-point two-scale fatigue damage on the GPU.
//
// Implements the update of src/kokkos_kernel.h:45-344 (constants
// src/damage.h:9-17): for every spatial Gauss point and every temporal
// interpolation point of the slab, interpolate the strain, run the elastic
// predictor and, when the trial von Mises stress exceeds sig_f, the plastic
// corrector with stored energy ws and damage D.  One thread per Gauss point,
// all state in FP64.
//
// The reference spends 144 FMAs per step re-interpolating the displacement
// of the 8 nodes (src/kokkos_kernel.h:55-71).  The strain is linear in the
// six temporal shape values Nt_k(t), so each point first forms its six
// strain "basis" vectors E_k = B u_k once per slab; the strain at any step is
// then sum_k Nt_k(t) E_k.  In the elastic predictor the deviatoric trial
// stress is affine in the strain as long as the internal variables (D,
// eps_pl, sig_back) do not change, i.e. between plastic steps:
//     tsig(t) = sum_k Nt_k(t) G_k + C0
// with G_k = c1 * m .* dev(E_k), C0 = (c3-1) * m .* dev(eps_pl) - sig_back
// (m = 2 mu on the normal terms, mu on the engineering shears).  A step is
// elastic iff 1.5 sum_n tsig_n^2 + 3 sum_s tsig_s^2 <= sig_f^2.
//
// GB300's FP64 rate is a small fraction of its FP32 rate, so every step is
// first screened in FP32 with a rigorous rounding bound.  Steps the screen
// proves elastic change nothing but the "last elastic" markers (sig_eff,
// eps_old, sig_d are overwritten by every elastic step, so only the last one
// before a plastic step, or before the slab ends, has to be evaluated).
// Steps the screen cannot decide, and plastic steps, are evaluated exactly
// in FP64 with the reference's operation order.
#include <cstdlib>
#include <mutex>

#include "xt_device.h"

namespace xt {

namespace {

// src/damage.h:9-17
constexpr double CY = 1740.0, HH = 0.2, SD = 0.5, SEXP = 0.5, SIGF = 180.0, SIGU = 577.0,
                 EPSD = 0.08;
constexpr double WD = (SIGU - SIGF) * EPSD;
constexpr int kNtChunk = 1024;  // temporal points per shared-memory chunk
constexpr int kRun = 32;        // steps proven elastic by one bound

struct Mat {
    double nu, E, ca, cb, G, Kb, coef;
};

__device__ __forceinline__ double vm_equiv(const double s[6])
{
    double e = 0.0;
    for (int i = 0; i < 3; ++i) e += 1.5 * s[i] * s[i];
    for (int i = 3; i < 6; ++i) e += 3.0 * s[i] * s[i];
    return sqrt(e);
}

__device__ __forceinline__ void deviator(const double s[6], double o[6])
{
    double tr = 0.0;
    for (int i = 0; i < 3; ++i) tr += s[i];
    tr = tr / 3.0;
    o[0] = s[0] - tr; o[1] = s[1] - tr; o[2] = s[2] - tr;
    o[3] = s[3]; o[4] = s[4]; o[5] = s[5];
}

// D times a Voigt vector with the reference's 6x6 dmat
// (src/kokkos_kernel.h:81-92), summed in the reference's order
__device__ __forceinline__ void dmat_mul(const Mat& m, const double v[6], double o[6])
{
    const double off = m.coef * m.nu, dia = m.coef * (1.0 - m.nu);
    const double sh = m.coef * (1.0 - 2.0 * m.nu) / 2.0;
    for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc += (i == j ? dia : off) * v[j];
        for (int j = 3; j < 6; ++j) acc += 0.0 * v[j];
        o[i] = acc;
    }
    for (int i = 3; i < 6; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 6; ++j) acc += (j == i ? sh : 0.0) * v[j];
        o[i] = acc;
    }
}

// Elastic predictor of src/kokkos_kernel.h:96-160 in FP64 and reference
// order.  Returns the equivalent trial stress; tse receives D * tee.
__device__ double predictor(const Mat& m, double d, const double eps[6], const double epl[6],
                            const double sbk[6], double tse[6])
{
    const double c1 = 1.0 / (1.0 - m.cb * d);
    const double c2 = (m.ca - m.cb) * d / ((1.0 - m.cb * d) * (1.0 - m.ca * d));
    const double c3 = m.cb * (1.0 - d) / (1.0 - m.cb * d);
    double tel[6], tee[6], tdev[6], tsig[6];
    for (int i = 0; i < 6; ++i) tel[i] = c1 * eps[i] + c3 * epl[i];
    double tr = 0.0;
    for (int i = 0; i < 3; ++i) tr += eps[i];
    tr = c2 * tr / 3.0;
    for (int i = 0; i < 3; ++i) tel[i] += tr;
    for (int i = 0; i < 6; ++i) tee[i] = tel[i] - epl[i];
    dmat_mul(m, tee, tse);
    deviator(tse, tdev);
    for (int i = 0; i < 6; ++i) tsig[i] = tdev[i] - sbk[i];
    return vm_equiv(tsig);
}

struct State {
    double epo[6], epl[6], sef[6], sbk[6];
    double p, d, ws, dpo, sigd;
};

// Plastic corrector of src/kokkos_kernel.h:175-341 in FP64, reference order.
__device__ void corrector(const Mat& m, const double eps[6], State& st)
{
    const double d = st.d;
    double de[6], ds[6], qs[6], dq[6];
    for (int i = 0; i < 6; ++i) de[i] = eps[i] - st.epo[i];
    dmat_mul(m, de, ds);
    for (int i = 0; i < 6; ++i) ds[i] = ds[i] / (1.0 - m.cb * d);
    const double c4 = m.Kb * (m.ca - m.cb) * d / ((1.0 - m.cb * d) * (1.0 - m.ca * d));
    double trd = 0.0;
    for (int i = 0; i < 3; ++i) trd += de[i];
    for (int i = 0; i < 3; ++i) ds[i] += c4 * trd;
    for (int i = 0; i < 6; ++i) qs[i] = st.sbk[i] - st.sef[i] - ds[i];
    const double gam = CY * (1.0 - d) + 3.0 * m.G * (1.0 - m.cb) / (1.0 - m.cb * d);
    double trq = 0.0;
    for (int i = 0; i < 3; ++i) trq += qs[i];
    trq = trq / 3.0;
    dq[0] = qs[0] - trq; dq[1] = qs[1] - trq; dq[2] = qs[2] - trq;
    dq[3] = qs[3]; dq[4] = qs[4]; dq[5] = qs[5];
    const double qeq = vm_equiv(dq);
    const double trs = -trq;
    const double dp = (qeq - SIGF) / gam;
    st.p += dp;
    const double c5 = 1.0 + gam * dp / SIGF;
    double dsg[6], sg[6];
    for (int i = 0; i < 6; ++i) dsg[i] = -dq[i] / c5;
    sg[0] = dsg[0] + trs; sg[1] = dsg[1] + trs; sg[2] = dsg[2] + trs;
    sg[3] = dsg[3]; sg[4] = dsg[4]; sg[5] = dsg[5];
    for (int i = 0; i < 6; ++i) {
        const double dpl = 3.0 * dsg[i] * dp / (2.0 * SIGF);
        st.epl[i] += dpl;
        st.sbk[i] += 2.0 * CY * (1.0 - d) * dpl / 3.0;
    }
    for (int i = 0; i < 6; ++i) st.sef[i] = sg[i] + st.sbk[i];
    double sdev[6];
    deviator(st.sef, sdev);
    const double seq = vm_equiv(sdev);
    const double snew = fabs(seq - SIGF);
    const double sold = fabs(st.sigd - SIGF);
    st.ws += (snew * dp + sold * st.dpo) / 2.0;
    if (st.ws >= WD) {
        double sp[3] = {0.0, 0.0, 0.0}, sn[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < 3; ++i) {
            if (st.sef[i] < 0.0) sn[i] = st.sef[i];
            else sp[i] = st.sef[i];
        }
        const double x = (1.0 - d) / (1.0 - HH * d);
        const double yp = (1.0 + m.nu) / (2.0 * m.E) *
                          (sp[0] * sp[0] + sp[1] * sp[1] + sp[2] * sp[2] +
                           HH * x * x * (sn[0] * sn[0] + sn[1] * sn[1] + sn[2] * sn[2]));
        double tr2 = 0.0;
        for (int i = 0; i < 3; ++i) tr2 += st.sef[i];
        const double yn = (tr2 >= 0.0) ? m.nu / (2.0 * m.E) * tr2 * tr2
                                       : m.nu / (2.0 * m.E) * HH * x * x * tr2 * tr2;
        st.d += pow((yp - yn) / SD, SEXP) * dp;
    } else {
        st.d = 0.0;
    }
    for (int i = 0; i < 6; ++i) st.epo[i] = eps[i];
    st.sigd = seq;
    st.dpo = dp;
}

// Affine screen coefficients for the current internal state: G (6x6, FP32,
// G[k][i]), C0 (6, FP32) and the absolute rounding bound of the screened
// teq^2.
__device__ void screen_setup(const Mat& m, const State& st, const double E[6][6],
                             const float* __restrict__ ntmax, float G[6][6], float C0[6],
                             float& err2, float ecomp[6])
{
    const double d = st.d;
    const double c1 = 1.0 / (1.0 - m.cb * d);
    const double c3 = m.cb * (1.0 - d) / (1.0 - m.cb * d);
    const double mn = m.coef * (1.0 - 2.0 * m.nu), ms = mn / 2.0;
    double dv[6];
    double S[6];
    deviator(st.epl, dv);
    for (int i = 0; i < 6; ++i) {
        const double c0 = (c3 - 1.0) * (i < 3 ? mn : ms) * dv[i] - st.sbk[i];
        C0[i] = (float)c0;
        S[i] = fabs(c0);
    }
    for (int k = 0; k < 6; ++k) {
        double ed[6];
        deviator(E[k], ed);
        for (int i = 0; i < 6; ++i) {
            const double gk = c1 * (i < 3 ? mn : ms) * ed[i];
            G[k][i] = (float)gk;
            S[i] += (double)ntmax[k] * fabs(gk);
        }
    }
    // Each screened component sums 7 rounded products of rounded inputs;
    // 32 units of 2^-24 of the absolute sum S_i bounds its error e_i, and
    // teq^2 = sum w_i tsig_i^2 then errs by at most sum w_i (2 S_i e_i +
    // e_i^2) plus the rounding of the final sum (another 16 units).
    const double u = 32.0 * 5.9604644775390625e-8;
    double e2 = 0.0, tot = 0.0;
    for (int i = 0; i < 6; ++i) {
        const double w = i < 3 ? 1.5 : 3.0;
        const double ei = u * S[i];
        ecomp[i] = (float)(ei * 1.0001);
        e2 += w * (2.0 * S[i] * ei + ei * ei);
        tot += w * S[i] * S[i];
    }
    err2 = (float)(e2 + 16.0 * 5.9604644775390625e-8 * tot) * 1.0001f + 1e-30f;
}

// Everything the rare exact FP64 path needs lives in one per-thread record
// that only no-inline functions touch, so the FP32 screening loop keeps just
// its 43 coefficients in registers (occupancy, no spills in the hot loop).
struct Slow {
    Mat m;
    State st;
    double E[6][6];
};
struct Screen {
    float G[6][6];
    float C0[6];
    float e[6];  // bound on each screened component's error
    float err2;
};

__device__ __noinline__ void slow_screen(const Slow* s, const float* __restrict__ ntmax, Screen* sc)
{
    screen_setup(s->m, s->st, s->E, ntmax, sc->G, sc->C0, sc->err2, sc->e);
}

__device__ __forceinline__ void strain_at(const Slow* s, const double* __restrict__ Nt, int jj,
                                          double eps[6])
{
    const double* ntr = Nt + (size_t)jj * 6;
    double w[6];
    for (int k = 0; k < 6; ++k) w[k] = ntr[k];
    for (int c = 0; c < 6; ++c) {
        double acc = 0.0;
        for (int k = 0; k < 6; ++k) acc = fma(w[k], s->E[k][c], acc);
        eps[c] = acc;
    }
}

// outputs of an elastic step (sig_eff, eps_old, sig_d), reference order
__device__ __noinline__ void slow_materialize(Slow* s, const double* __restrict__ Nt, int jj)
{
    double eps[6], tse[6];
    strain_at(s, Nt, jj, eps);
    const double teq = predictor(s->m, s->st.d, eps, s->st.epl, s->st.sbk, tse);
    for (int i = 0; i < 6; ++i) { s->st.sef[i] = tse[i]; s->st.epo[i] = eps[i]; }
    s->st.sigd = teq;
}

// exact FP64 step jj.  Returns 1 when the step was plastic (internal
// variables changed; the screen is marked stale with an infinite error
// bound, so the following steps take this exact path too), else 0; an
// elastic step on a stale screen rebuilds it.  A plastic phase therefore
// rebuilds the screen once, at its end, not after every plastic step.
__device__ __noinline__ int slow_step(Slow* s, const double* __restrict__ Nt, int jj, int last_el,
                                      const float* __restrict__ ntmax, Screen* sc)
{
    double eps[6], tse[6];
    strain_at(s, Nt, jj, eps);
    const double teq = predictor(s->m, s->st.d, eps, s->st.epl, s->st.sbk, tse);
    if (teq <= SIGF) {
        for (int i = 0; i < 6; ++i) { s->st.sef[i] = tse[i]; s->st.epo[i] = eps[i]; }
        s->st.sigd = teq;
        if (isinf(sc->err2)) {
            screen_setup(s->m, s->st, s->E, ntmax, sc->G, sc->C0, sc->err2, sc->e);
            return 2;
        }
        return 0;
    }
    if (last_el >= 0) slow_materialize(s, Nt, last_el);
    corrector(s->m, eps, s->st);
    sc->err2 = __int_as_float(0x7f800000);  // +inf: screen stale
    return 1;
}

// The slab's update of point gidx (a copy of the last point, storing
// nothing, when gidx is past it: every thread of the block must reach the
// barriers of the chunk loop).
__device__ __forceinline__ void damage_point(const DamageArgs& a, const float* __restrict__ ntmax,
                                             int run_bound, long long gidx)
{
    const bool live = gidx < a.ngp;
    const int gp = live ? (int)gidx : a.ngp - 1;
    Slow s;
    Mat& m = s.m;
    m.nu = a.nu[gp];
    m.E = a.ym[gp];
    m.ca = (1.0 + m.nu) / (3.0 * (1.0 - m.nu));
    m.cb = 2.0 * (4.0 - 5.0 * m.nu) / (15.0 * (1.0 - m.nu));
    m.G = m.E / (2.0 * (1.0 + m.nu));
    m.Kb = m.E / (3.0 * (1.0 - 2.0 * m.nu));
    m.coef = m.E / ((1.0 + m.nu) * (1.0 - 2.0 * m.nu));

    // strain basis E_k = B u_k (6 temporal blocks, checked on the host)
    for (int k = 0; k < 6; ++k)
        for (int c = 0; c < 6; ++c) s.E[k][c] = 0.0;
    for (int i = 0; i < a.nnse; ++i) {
        const int nd = a.nodes[(size_t)gp * a.nnse + i] - 1;
        const double nx = a.Nx[(size_t)gp * a.nnse + i];
        const double ny = a.Ny[(size_t)gp * a.nnse + i];
        const double nz = a.Nz[(size_t)gp * a.nnse + i];
        for (int k = 0; k < 6; ++k) {
            const double* u = a.sol + (size_t)k * a.nn * a.ndofn + (size_t)nd * a.ndofn;
            const double u0 = u[0], u1 = u[1], u2 = u[2];
            s.E[k][0] += nx * u0;
            s.E[k][1] += ny * u1;
            s.E[k][2] += nz * u2;
            s.E[k][3] += ny * u0 + nx * u1;
            s.E[k][4] += nz * u1 + ny * u2;
            s.E[k][5] += nz * u0 + nx * u2;
        }
    }
    State& st = s.st;
    const size_t b6 = (size_t)gp * a.ncmp;
    for (int i = 0; i < 6; ++i) {
        st.epo[i] = a.eps_old[b6 + i];
        st.epl[i] = a.eps_pl[b6 + i];
        st.sef[i] = a.sig_eff[b6 + i];
        st.sbk[i] = a.sig_back[b6 + i];
    }
    st.p = a.p[gp];
    st.d = a.D[gp];
    st.ws = a.ws[gp];
    st.dpo = a.del_po[gp];
    st.sigd = a.sig_d[gp];

    Screen sc;
    slow_screen(&s, ntmax, &sc);
    float G[6][6], C0[6], ecomp[6], err2;
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int i = 0; i < 6; ++i) G[k][i] = sc.G[k][i];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        C0[i] = sc.C0[i];
        ecomp[i] = sc.e[i];
    }
    err2 = sc.err2;
    // proven elastic when q + err2 < sig_f^2 (margin covers the float add)
    const float thr = (float)(SIGF * SIGF) * 0.99999976f;
    int last_el = -1;  // last step known elastic whose outputs are pending
    unsigned n_exact = 0, n_plastic = 0;
    // The FP32 shape table is shared by every point: the block streams it
    // through shared memory in chunks, so each step's six values are a
    // broadcast shared-memory read instead of an L2 round trip.
    __shared__ float2 sNt[3 * kNtChunk];
    __shared__ float sDel[kNtChunk / kRun][6];
    const float2* nt2 = reinterpret_cast<const float2*>(a.Nt32);
    for (int j0 = 0; j0 < a.nip; j0 += kNtChunk) {
    const int jn = min(kNtChunk, a.nip - j0);
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * jn; i += blockDim.x) sNt[i] = __ldg(nt2 + 3 * (size_t)j0 + i);
    __syncthreads();
    // Run bounds: delta_k >= |Nt_k(t) - Nt_k(t0)| of the FP64 table over each
    // run of kRun steps from its first step t0.  The FP32 table differs from
    // the FP64 one by at most u |Nt_k| <= u ntmax_k per entry (u = 2^-24),
    // and the FP32 difference by one more rounding: inflated accordingly.
    for (int t = threadIdx.x; t < (kNtChunk / kRun) * 8; t += blockDim.x) {
        const int run = t >> 3, k = t & 7;
        const int r0 = run * kRun;
        if (k < 6 && r0 < jn) {
            const float* f = reinterpret_cast<const float*>(sNt);
            const float base = f[r0 * 6 + k];
            float mx = 0.0f;
            for (int j = r0 + 1; j < min(r0 + kRun, jn); ++j) mx = fmaxf(mx, fabsf(f[j * 6 + k] - base));
            sDel[run][k] = mx * 1.000001f + __ldg(ntmax + k) * 2.4e-7f;
        }
    }
    __syncthreads();
    for (int jr = 0; jr < jn; jr += kRun) {
    const int jre = min(jn, jr + kRun);
    // One bound for the whole run (fresh screens only: a stale one has an
    // infinite err2): with acc_i(t0) the screened component at the run's
    // first step, every step of the run has |tsig_i| <= |acc_i(t0)| + e_i +
    // sum_k delta_k |g_ki| =: B_i (g the FP64 coefficient, |g| <= |G|(1 +
    // 1.01u); the FP32 sum of the six non-negative products is inflated by
    // 16u for that and its own rounding), so teq^2 <= sum w_i B_i^2; that
    // sum of non-negative FP32 terms is inflated by 2^-18 (64u) for its own
    // rounding.  Below the threshold, every step of the run is elastic.
    if (run_bound && err2 < thr) {
        const float2 t0 = sNt[3 * jr], t1 = sNt[3 * jr + 1], t2 = sNt[3 * jr + 2];
        const float w[6] = {t0.x, t0.y, t1.x, t1.y, t2.x, t2.y};
        float dl[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) dl[k] = sDel[jr / kRun][k];
        float qb = 0.0f;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            float acc = C0[i], dev = 0.0f;
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                acc = fmaf(w[k], G[k][i], acc);
                dev = fmaf(dl[k], fabsf(G[k][i]), dev);
            }
            const float b = fabsf(acc) + ecomp[i] + dev * 1.000001f;
            qb = fmaf(i < 3 ? 1.5f : 3.0f, b * b, qb);
        }
        if (qb * 1.0000039f < thr) {
            last_el = j0 + jre - 1;
            continue;
        }
    }
    for (int jq = jr; jq < jre; ++jq) {
        const int jj = j0 + jq;
        const float2 t0 = sNt[3 * jq], t1 = sNt[3 * jq + 1], t2 = sNt[3 * jq + 2];
        const float w[6] = {t0.x, t0.y, t1.x, t1.y, t2.x, t2.y};
        float q = 0.0f;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            float acc = C0[i];
#pragma unroll
            for (int k = 0; k < 6; ++k) acc = fmaf(w[k], G[k][i], acc);
            q = fmaf(i < 3 ? 1.5f : 3.0f, acc * acc, q);
        }
        if (q + err2 < thr) {
            last_el = jj;
            continue;
        }
        ++n_exact;
        sc.err2 = err2;
        const int r = slow_step(&s, a.Nt, jj, last_el, ntmax, &sc);
        if (r == 1) {
            ++n_plastic;
            err2 = sc.err2;  // stale: every step is exact until one is elastic
        } else if (r == 2) {  // screen rebuilt after a plastic phase
#pragma unroll
            for (int k = 0; k < 6; ++k)
#pragma unroll
                for (int i = 0; i < 6; ++i) G[k][i] = sc.G[k][i];
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                C0[i] = sc.C0[i];
                ecomp[i] = sc.e[i];
            }
            err2 = sc.err2;
        }
        last_el = -1;
    }
    }
    }
    if (last_el >= 0) slow_materialize(&s, a.Nt, last_el);
    if (!live) return;

    if (a.gpsta && a.gpsta[gp] == 0) {  // src/kokkos_damage.f90:102-107
        st.d = 0.0;
        st.ws = 0.0;
    }
    for (int i = 0; i < 6; ++i) {
        a.eps_old[b6 + i] = st.epo[i];
        a.eps_pl[b6 + i] = st.epl[i];
        a.sig_eff[b6 + i] = st.sef[i];
        a.sig_back[b6 + i] = st.sbk[i];
    }
    a.p[gp] = st.p;
    a.D[gp] = st.d;
    a.ws[gp] = st.ws;
    a.del_po[gp] = st.dpo;
    a.sig_d[gp] = st.sigd;
    if (a.counters) {
        atomicAdd(&a.counters[0], (unsigned long long)n_plastic);
        atomicAdd(&a.counters[1], (unsigned long long)a.nip - n_exact);
        atomicAdd(&a.counters[2], (unsigned long long)n_exact);
    }
}

// Points are dealt to blocks round-robin (pass it, thread t of block b
// takes point (it blockDim + t) gridDim + b): plastic points cluster in
// space, i.e. in consecutive point numbers, and their FP64 steps would
// otherwise pile up in a few blocks on a few SMs while the rest of the GPU
// idles.  One pass per thread is one thread per point; a small grid with
// several passes keeps the update on a few SMs.
__global__ void __launch_bounds__(256)
k_damage(DamageArgs a, const float* __restrict__ ntmax, int run_bound, int passes)
{
    for (int it = 0; it < passes; ++it)
        damage_point(a, ntmax, run_bound,
                     ((long long)it * blockDim.x + threadIdx.x) * gridDim.x + blockIdx.x);
}

// max_t |Nt_k(t)| per k over the slab (single block)
__global__ void k_ntmax(const float* __restrict__ nt32, int nip, float* __restrict__ out)
{
    __shared__ float sh[6][32];
    float m[6] = {0, 0, 0, 0, 0, 0};
    for (int j = threadIdx.x; j < nip; j += blockDim.x)
        for (int k = 0; k < 6; ++k) m[k] = fmaxf(m[k], fabsf(nt32[(size_t)j * 6 + k]));
    for (int k = 0; k < 6; ++k) {
        float v = m[k];
        for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, off));
        if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        float v = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = fmaxf(v, sh[threadIdx.x][w]);
        out[threadIdx.x] = v * 1.000001f;
    }
}

__global__ void k_nt_table(int nip, double t0, double t1, double t2, double w, double* nt64,
                           float* nt32)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nip) return;
    const double dt = t2 - t0;
    const double t = t0 + (double)i * dt / (double)nip;
    const double n1 = 2.0 * (t1 - t) * (t2 - t) / (dt * dt);
    const double n2 = -4.0 * (t0 - t) * (t2 - t) / (dt * dt);
    const double n3 = 2.0 * (t0 - t) * (t1 - t) / (dt * dt);
    const double swt = sin(w * t);
    const double r[6] = {n1, n2, n3, n1 * (swt - sin(w * t0)), n2 * (swt - sin(w * t1)),
                         n3 * (swt - sin(w * t2))};
    for (int k = 0; k < 6; ++k) {
        nt64[(size_t)i * 6 + k] = r[k];
        nt32[(size_t)i * 6 + k] = (float)r[k];
    }
}

// chkelesta: single block, elements in ascending order in chunks of
// blockDim.x, block-wide exclusive scan of the failure flags
__global__ void __launch_bounds__(1024)
k_chkelesta(int ne, int ngpe, double Dc, const double* __restrict__ D, int* elesta, int* gpsta,
            int* nefail, int* nef)
{
    __shared__ int warp_tot[32];
    __shared__ int base;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int e0 = 0; e0 < ne; e0 += blockDim.x) {
        const int e = e0 + threadIdx.x;
        int f = 0;
        if (e < ne)
            for (int g = 0; g < ngpe; ++g)
                if (D[(size_t)e * ngpe + g] >= Dc) f = 1;
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        const int before = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) warp_tot[warp] = __popc(bal);
        __syncthreads();
        int off = base;
        for (int w = 0; w < warp; ++w) off += warp_tot[w];
        if (f) {
            nefail[off + before] = e + 1;
            elesta[e] = 0;
            for (int g = 0; g < ngpe; ++g) gpsta[(size_t)e * ngpe + g] = 0;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += warp_tot[w];
            base += t;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *nef = base;
}

__global__ void k_zero_int(int* a, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = 0;
}

__global__ void k_any_ge(const double* __restrict__ D, int n, double Dc, int* flag)
{
    int f = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (D[i] >= Dc) f = 1;
    if (__any_sync(0xffffffffu, f) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// Scratch of the allocation-free damage entry point (xt_damage_device):
// the FP32 copy of the temporal shape table (6 values per step, up to
// kDamageStaticMaxNip steps), the six shape-value bounds and the three step
// counters.  1.5 MB in all, part of the library image; one set per process
// and device, so concurrent calls share it.
constexpr size_t kStaticNt = (size_t)kDamageStaticMaxNip * 6;
constexpr size_t kStaticBytes = kStaticNt * sizeof(float) + 64 + 3 * sizeof(unsigned long long);
static __device__ __align__(256) unsigned char g_damage_scratch[kStaticBytes];

}  // namespace

namespace {
// Per-device address of g_damage_scratch, looked up once per device and
// context.  A mutex guards it: two host threads making their first call at
// once must not race on the entry.  damage_static_forget() clears it when
// the library context is torn down (a new context may place the symbol at
// another address).
std::mutex g_scratch_mu;
constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {nullptr};
}  // namespace

int damage_static_scratch(int device, float** nt32, float** ntmax, unsigned long long** counters)
{
    if (device < 0 || device >= kMaxDevices) {
        set_error("damage scratch: device index out of range");
        return XT_ERR_ARG;
    }
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_addr[device]) {
            // the caller has made `device` current; cudaGetSymbolAddress can
            // load the module, so the first call must not sit inside a
            // stream capture
            int cur = -1;
            XT_CUDA(cudaGetDevice(&cur));
            if (cur != device) {
                set_error("damage scratch: the library's device is not current");
                return XT_ERR_CUDA;
            }
            void* p = nullptr;
            XT_CUDA(cudaGetSymbolAddress(&p, g_damage_scratch));
            g_scratch_addr[device] = p;
        }
        base = g_scratch_addr[device];
    }
    unsigned char* b = static_cast<unsigned char*>(base);
    *nt32 = reinterpret_cast<float*>(b);
    *ntmax = reinterpret_cast<float*>(b + kStaticNt * sizeof(float));
    *counters = reinterpret_cast<unsigned long long*>(b + kStaticNt * sizeof(float) + 64);
    return XT_OK;
}

void damage_static_forget()
{
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    for (int d = 0; d < kMaxDevices; ++d) g_scratch_addr[d] = nullptr;
}

int nt_table_device(int nip, double t0, double t1, double t2, double w, double* Nt64,
                    float* Nt32, cudaStream_t s)
{
    if (nip <= 0) return XT_OK;
    k_nt_table<<<(nip + 255) / 256, 256, 0, s>>>(nip, t0, t1, t2, w, Nt64, Nt32);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int damage_update(const DamageArgs& a, cudaStream_t s)
{
    if (a.nnte != 3 || a.ndofn != 3 || a.ncmp != 6 || a.nnse < 1 || a.nnse > 8) {
        set_error("damage_update: the C3D8 kernel needs ndofn=3, nnte=3, ncmp=6, nnse<=8");
        return XT_ERR_ARG;
    }
    if (a.ngp <= 0 || a.nip <= 0) return XT_OK;
    if (!a.ntmax) {
        set_error("damage_update: missing scratch for the shape-value bounds");
        return XT_ERR_ARG;
    }
    k_ntmax<<<1, 1024, 0, s>>>(a.Nt32, a.nip, a.ntmax);
    // XTFEM_DAMAGE_RUN=0: screen every step (no per-run bound)
    const char* e = std::getenv("XTFEM_DAMAGE_RUN");
    const int run_bound = (!e || std::atoi(e) != 0) ? 1 : 0;
    // 128 threads per block (XTFEM_DAMAGE_THREADS=256: 256).  A block that
    // holds a plastic point runs for the whole update; at 170 registers a
    // thread, a 128-thread block leaves its SM room for the solve's blocks
    // beside it, where a 256-thread block (43.5 K registers) left room for
    // two dot-pass blocks of six.
    const char* et = std::getenv("XTFEM_DAMAGE_THREADS");
    const int nt = (et && std::atoi(et) == 256) ? 256 : 128;
    // XTFEM_DAMAGE_BLOCKS=B: a grid of B blocks, each thread taking several
    // points in turn (0: one thread per point)
    const char* eb = std::getenv("XTFEM_DAMAGE_BLOCKS");
    const long long want = eb ? std::atoll(eb) : 0;
    const long long full = ((long long)a.ngp + nt - 1) / nt;
    const int grid = (int)((want > 0 && want < full) ? want : full);
    const int passes = (int)(((long long)a.ngp + (long long)grid * nt - 1) / ((long long)grid * nt));
    k_damage<<<grid, nt, 0, s>>>(a, a.ntmax, run_bound, passes);
    note_launches(2);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int chkelesta_device(int ne, int ngpe, double Dc, const double* D, int* elesta, int* gpsta,
                     int* nefail, int* nef, cudaStream_t s)
{
    if (ne <= 0) return XT_OK;
    k_zero_int<<<(ne + 255) / 256, 256, 0, s>>>(nefail, ne);
    k_chkelesta<<<1, 1024, 0, s>>>(ne, ngpe, Dc, D, elesta, gpsta, nefail, nef);
    note_launches(2);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int any_ge_device(const double* D, int ngp, double Dc, int* flag, cudaStream_t s)
{
    XT_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
    if (ngp <= 0) return XT_OK;
    int blocks = (ngp + 255) / 256;
    if (blocks > 1024) blocks = 1024;
    k_any_ge<<<blocks, 256, 0, s>>>(D, ngp, Dc, flag);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

}  // namespace xt
