// thermal.cpp -- the thermal space-time slab loop (q = 3) with its state on
// the GPU.
//
// Restates the temperature part of src/main3d.f90 (alone, or driven by the
// mechanical slab loop through thermal.h when the two are coupled):
//   set-up   conductivity and capacity (mpiglbmtx_t / elemtx_t,
//            src/elesubs.f90:60-116), the fixed-temperature faces
//            (:429-441), K and M kept before the boundary conditions
//            (:443-451) and after them (csrapplybc, :452-453), the flux
//            load rext_t (:454-476), tempst = Tref, fInit = (A (x) K0 + B (x)
//            M0) Tref and, with tempst = the fixed values, fBound =
//            -(A (x) K0 + B (x) M0) tempst (:586-608);
//   slab     fextst_t = fInit (first slab only) + fextc_t(j) rext_t per
//            temporal block (getfextc_t), + the jump term (ktn1 (x) K + mtn1
//            (x) M) tempst, + fBound, fixed rows zeroed; GMRES from zero with
//            A = ck + cktn, B = cm + cmtn (stcoeff_t); fixed rows of the
//            solution set to their values (:697-734).
// The reference's mpipgmres here is preconditioned by MUMPS (an exact
// factor of K); this loop uses the ILUT factor of K_t like the mechanical
// GMRES route.  The flux share counts the element-node incidences of the
// first flux face only while the load goes on both faces, as the reference
// does (:460-476).
#include <cmath>
#include <cstring>
#include <memory>

#include "../../include/xtfem_gb300_host.h"
#include "host_problem.h"
#include "solver.h"
#include "thermal.h"

using namespace xt;

struct xt_thermal_s {
    xt_thermal_config cfg{};
    System S;
    int nn = 0, slab = 0;
    double dt = 0, t0 = 0;  // slab length, start time of the next slab
    std::vector<int> bc;
    std::vector<double> rext, finit, fbound;  // host, block layout (3 nn)
    DBuf<double> temp, fext, work, hblk, dbc;
    double A[9], B[9], C1[9], M1[9];
};

namespace {

// y += alpha (a (x) K + b (x) M) x on the host, block layout, q = 3
void kron_host(const Csr& K, const Csr& M, const double* a, const double* b, double alpha,
               const double* x, double* y)
{
    const int n = K.n;
    std::vector<double> kx(3 * (size_t)n, 0.0), mx(3 * (size_t)n, 0.0);
    for (int j = 0; j < 3; ++j)
        for (int r = 0; r < n; ++r) {
            double sk = 0.0, sm = 0.0;
            for (int k = K.ia[r] - 1; k < K.ia[r + 1] - 1; ++k) sk += K.a[k] * x[(size_t)j * n + K.ja[k] - 1];
            for (int k = M.ia[r] - 1; k < M.ia[r + 1] - 1; ++k) sm += M.a[k] * x[(size_t)j * n + M.ja[k] - 1];
            kx[(size_t)j * n + r] = sk;
            mx[(size_t)j * n + r] = sm;
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double ca = alpha * a[j * 3 + i], cb = alpha * b[j * 3 + i];  // column-major
            for (int r = 0; r < n; ++r)
                y[(size_t)i * n + r] += ca * kx[(size_t)j * n + r] + cb * mx[(size_t)j * n + r];
        }
}

bool on_face(const Mesh& m, int node, int axis, const double* v, int nv)
{
    const double c = m.xyz[(size_t)node * 3 + axis];
    for (int k = 0; k < nv; ++k)
        if (c == v[k]) return true;
    return false;
}

int thermal_create(Problem& pr, const xt_thermal_config& cfg, std::unique_ptr<xt_thermal_s>& t)
{
    const Mesh& m = pr.mesh;
    const int nn = m.nn;
    t->cfg = cfg;
    t->nn = nn;
    ThermSystem ts = assemble_therm(m, cfg.kappa, cfg.rho, cfg.cp);
    const Csr K0 = ts.K, M0 = ts.M;
    t->bc.assign(nn, 0);
    std::vector<double> fixedv(3 * (size_t)nn, 0.0);
    for (int i = 0; i < nn; ++i)
        if (on_face(m, i, cfg.fixed_axis, cfg.fixed_value, 2)) {
            t->bc[i] = 1;
            for (int j = 0; j < 3; ++j) fixedv[(size_t)j * nn + i] = cfg.T0;
        }
    csrapplybc(ts.K, t->bc.data());
    csrapplybc(ts.M, t->bc.data());
    // flux: q0 * area shared by the element-node incidences of the first
    // flux face, applied at the incidences of both faces
    std::vector<double> share(nn, 0.0);
    for (size_t k = 0; k < m.conn.size(); ++k) share[m.conn[k] - 1] += 1.0;
    double ntele = 0.0;
    for (int i = 0; i < nn; ++i)
        if (on_face(m, i, cfg.flux_axis, cfg.flux_value, 1)) ntele += share[i];
    t->rext.assign(nn, 0.0);
    if (ntele > 0.0) {
        const double fnode = cfg.q0 * cfg.area / ntele;
        for (size_t k = 0; k < m.conn.size(); ++k) {
            const int nd = m.conn[k] - 1;
            if (on_face(m, nd, cfg.flux_axis, cfg.flux_value, 2)) t->rext[nd] += fnode;
        }
    }
    // temporal matrices: A = ck + cktn, B = cm + cmtn, jump ktn1, mtn1
    t->dt = cfg.dt0 * cfg.n1;
    double ck[9], cm[9], ckt[9], cmt[9];
    stcoeff_t(t->dt, ck, cm, ckt, cmt, t->C1, t->M1);
    for (int e = 0; e < 9; ++e) {
        t->A[e] = ck[e] + ckt[e];
        t->B[e] = cm[e] + cmt[e];
    }
    // fInit = (A (x) K0 + B (x) M0) Tref; fBound = -(...) fixed values
    std::vector<double> tref(3 * (size_t)nn, cfg.Tref);
    t->finit.assign(3 * (size_t)nn, 0.0);
    t->fbound.assign(3 * (size_t)nn, 0.0);
    kron_host(K0, M0, t->A, t->B, 1.0, tref.data(), t->finit.data());
    kron_host(K0, M0, t->A, t->B, -1.0, fixedv.data(), t->fbound.data());
    // the device system
    System& S = t->S;
    XT_TRY(system_create(S, nn, 3, ts.K.ia.data(), ts.K.ja.data(), ts.K.a.data(), ts.M.ia.data(),
                         ts.M.ja.data(), ts.M.a.data()));
    Msr f;
    const int ierr = ilut(ts.K, cfg.lfil, cfg.droptol, f);
    if (ierr != 0) {
        set_error("xt_thermal_create: ILUT failed with ierr " + std::to_string(ierr));
        return XT_ERR_SINGULAR;
    }
    XT_TRY(system_set_ilu(S, f.alu.data(), f.jlu.data(), f.ju.data(), 1));
    XT_TRY(system_set_temporal(S, t->A, t->B));
    cudaStream_t st = S.stream;
    XT_CUDA(cudaMemcpyAsync(S.Cj.p, t->C1, sizeof(t->C1), cudaMemcpyHostToDevice, st));
    XT_CUDA(cudaMemcpyAsync(S.Mj.p, t->M1, sizeof(t->M1), cudaMemcpyHostToDevice, st));
    XT_TRY(S.bcmask.upload(t->bc.data(), t->bc.size(), st));
    const size_t n = 3 * (size_t)nn;
    XT_TRY(t->temp.alloc(n));
    XT_TRY(t->fext.alloc(n));
    XT_TRY(t->work.alloc(n));
    XT_TRY(t->hblk.alloc(n));
    std::vector<double> bcd(t->bc.begin(), t->bc.end());
    XT_TRY(t->dbc.upload(bcd.data(), bcd.size(), st));
    // tempst = the fixed values (0 elsewhere) before the first slab
    XT_TRY(t->hblk.upload(fixedv.data(), n, st));
    XT_TRY((to_interleaved<double, double>(t->hblk.p, t->temp.p, nn, 3, st)));
    XT_CUDA(cudaStreamSynchronize(st));
    return XT_OK;
}

int thermal_step(xt_thermal_s& t, double* stats)
{
    System& S = t.S;
    cudaStream_t st = S.stream;
    const int nn = t.nn;
    const size_t n = 3 * (size_t)nn;
    t.slab += 1;
    double fc[3];
    getfextc_t(t.t0, t.dt, fc);
    std::vector<double> f(n);
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < nn; ++i) {
            const size_t k = (size_t)j * nn + i;
            f[k] = (t.slab == 1 ? t.finit[k] : 0.0) + fc[j] * t.rext[i] + t.fbound[k];
        }
    XT_CUDA(cudaMemcpyAsync(t.hblk.p, f.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
    XT_TRY((to_interleaved<double, double>(t.hblk.p, t.fext.p, nn, 3, st)));
    XT_TRY(system_apply_with(S, S.Cj.p, S.Mj.p, 1.0, 1.0, t.temp.p, t.fext.p));
    XT_TRY(mask_rows<double>(t.fext.p, S.bcmask.p, nn, 3, st));
    XT_CUDA(cudaMemsetAsync(t.temp.p, 0, n * sizeof(double), st));
    GmresStats gs;
    XT_TRY(solve_refined(S, t.fext.p, t.temp.p, t.cfg.im, t.cfg.tol, t.cfg.maxits, t.cfg.precision,
                         t.cfg.inner_tol, gs));
    // fixed rows take their values: temp = masked temp + T0 * bc
    XT_TRY(mask_rows<double>(t.temp.p, S.bcmask.p, nn, 3, st));
    const double c3[3] = {t.cfg.T0, t.cfg.T0, t.cfg.T0};
    XT_TRY(fill_load(t.dbc.p, c3, t.work.p, nn, 3, st));
    XT_TRY((axpby<double, double>(n, 1.0, t.work.p, 1.0, t.temp.p, st)));
    XT_CUDA(cudaStreamSynchronize(st));
    t.t0 += t.dt;
    if (stats) {
        stats[0] = t.slab;
        stats[1] = gs.its;
        stats[2] = gs.cycles;
        stats[3] = gs.outer;
        stats[4] = gs.ierr;
        stats[5] = gs.relres;
    }
    if (gs.ierr != 0 && gs.ierr != -1) {
        set_error("thermal slab solve did not converge");
        return gs.ierr;
    }
    return XT_OK;
}

}  // namespace

namespace xt {
int thermal_advance(xt_thermal_s& t, double* stats) { return thermal_step(t, stats); }
const double* thermal_temperature(const xt_thermal_s& t) { return t.temp.p; }
int thermal_nodes(const xt_thermal_s& t) { return t.nn; }
}  // namespace xt

extern "C" {

int xt_thermal_create(xth_problem pr, const xt_thermal_config* cfg, xt_thermal* out)
{
    if (!pr || !cfg || !out) { set_error("xt_thermal_create: null argument"); return XT_ERR_ARG; }
    *out = nullptr;
    if (cfg->fixed_axis < 0 || cfg->fixed_axis > 2 || cfg->flux_axis < 0 || cfg->flux_axis > 2 ||
        cfg->n1 <= 0 || cfg->dt0 <= 0 || cfg->im <= 0 || cfg->precision < 0 || cfg->precision > 3) {
        set_error("xt_thermal_create: bad configuration");
        return XT_ERR_ARG;
    }
    XT_TRY(ensure_init());
    try {
        auto t = std::make_unique<xt_thermal_s>();
        XT_TRY(system_stream(t->S));
        XT_TRY(thermal_create(*reinterpret_cast<Problem*>(pr), *cfg, t));
        *out = t.release();
        return XT_OK;
    } catch (const std::exception& e) {
        set_error(std::string("xt_thermal_create: ") + e.what());
        return XT_ERR_HOST;
    }
}

int xt_thermal_destroy(xt_thermal t)
{
    delete t;
    return XT_OK;
}

int xt_thermal_step(xt_thermal t, double* stats)
{
    if (!t) { set_error("xt_thermal_step: null handle"); return XT_ERR_ARG; }
    try {
        return thermal_step(*t, stats);
    } catch (const std::exception& e) {
        set_error(std::string("xt_thermal_step: ") + e.what());
        return XT_ERR_HOST;
    }
}

int xt_thermal_get(xt_thermal t, double* temp)
{
    if (!t || !temp) { set_error("xt_thermal_get: null argument"); return XT_ERR_ARG; }
    cudaStream_t st = t->S.stream;
    XT_TRY((to_blocks<double, double>(t->temp.p, t->hblk.p, t->nn, 3, st)));
    XT_CUDA(cudaMemcpyAsync(temp, t->hblk.p, 3 * (size_t)t->nn * sizeof(double),
                            cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaStreamSynchronize(st));
    return XT_OK;
}

}  // extern "C"
