// slab.cpp -- the mechanical space-time slab loop with its state on the GPU.
//
// Restates src/main3d.f90:609-937 for the mechanical-only run (no thermal
// solve, no per-slab reassembly; the element-deletion subtraction then
// persists, src/main3d.f90:752-783 is not executed):
//   1. slab node times from the previous slab's end (:611-614);
//   2. deletion check: any D >= Dc -> chkelesta, delelement, chkcnsta,
//      chkndsta, adddiagonal, extra fixed DOFs, csrapplybc, refactor, and
//      the slab length and damage resolution switch from n1 to n2 cycles
//      (:625-691);
//   3. load blocks fextc(j) * rext, stcoeff_m, jump term
//      (ktn1 (x) K + mtn1 (x) M) u_prev, fixed rows zeroed (:804-823);
//   4. GMRES solve from a zero start, fixed DOFs of the solution zeroed
//      (:824-845);
//   5. damage update with the failed-point clean-up (:880-883).
// The reference passes the INTEGER slab index as stcoeff_m's REAL t1
// argument (:816, implicit interface); the intended slab start time
// tcoorde(1) is used here.  Every per-slab vector stays on the device; the
// host sees a handful of scalars per slab.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/xtfem_gb300_host.h"
#include "host_problem.h"
#include "prof.h"
#include "solver.h"
#include "thermal.h"

using namespace xt;

struct xt_slab_s {
    Problem* pr = nullptr;
    xt_slab_config cfg{};
    System S;
    int p = 0, q = 6, nn = 0, ne = 0, ngp = 0;
    std::vector<int> bc;
    std::vector<double> rext;
    DBuf<double> drext, fext, disp, dblk;
    // damage state (device)
    DBuf<int> nodes, gpsta, elesta, nefail, nef, flag;
    DBuf<double> Nx, Ny, Nz, ym, nu, eo, ep, se, sb, pp, D, ws, dpo, sd, Nt64;
    DBuf<float> Nt32, ntmax;
    DBuf<unsigned long long> counters;
    double tc[3] = {0, 0, 0};
    double dt = 0, w = 0;
    int nip = 0, slab = 0, nfailed = 0;
    bool switched = false;
    // overlap mode: the damage update of the last slab runs on `ds`
    cudaStream_t ds = nullptr;
    cudaEvent_t ev_sol = nullptr, ev_dmg = nullptr;
    bool pending = false;
    DBuf<double> disp_prev, hblk;  // speculation restore point; host-output staging
    Reduce red_dmg;
    double* hbuf = nullptr;  // pinned: max D, 3 counters, deletion flag
    // results of the last finished update, kept until the next slab uses them
    int del_flag = 0;
    double dmg_stats[4] = {0, 0, 0, 0};
    // thermal coupling (xt_slab_couple)
    xt_thermal_s* therm = nullptr;
    xt_coupling_config cc{};
    DBuf<int> conn0, vptr, vidx;
    DBuf<double> xyzd, ymc, nuc, ve, vv, work;
    int coupled_slabs = 0;
    bool force_refactor = false;
    Msr fac;  // the host factor of the host K (n = 0: none), reused from the first changed row
    ~xt_slab_s()
    {
        if (ds) {
            cudaStreamSynchronize(ds);
            cudaStreamDestroy(ds);
        }
        if (ev_sol) cudaEventDestroy(ev_sol);
        if (ev_dmg) cudaEventDestroy(ev_dmg);
        if (hbuf) cudaFreeHost(hbuf);
    }
};

namespace {

// ILUT of the host K.  first_row > 0: K's rows [0, first_row) are those the
// kept factor was computed from, so its rows there are kept (the same
// factor).
int refactor(xt_slab_s& s, int first_row = 0)
{
    // cfg.ilu_blocks > 1: the block-Jacobi part of K (its rows are as
    // row-local as K's, so the kept rows stay valid)
    Csr Kb;
    if (s.cfg.ilu_blocks > 1) Kb = block_diagonal(s.pr->sys.K, s.cfg.group, s.cfg.ilu_blocks);
    const Csr& K = s.cfg.ilu_blocks > 1 ? Kb : s.pr->sys.K;
    Msr f;
    const Msr* prev = (first_row > 0 && s.fac.n == K.n) ? &s.fac : nullptr;
    const int ierr = ilut(K, s.cfg.lfil, s.cfg.droptol, f, prev, first_row);
    s.fac = Msr{};  // kept again only once the new factor is in place
    if (ierr != 0) {
        set_error("ILUT failed with ierr = " + std::to_string(ierr));
        return XT_ERR_HOST;
    }
    XT_TRY(system_set_ilu(s.S, f.alu.data(), f.jlu.data(), f.ju.data(), s.cfg.group,
                          s.cfg.ilu_blocks));
    s.fac = std::move(f);
    return XT_OK;
}

// ILUT of the device K (after a reassembly on the device)
int refactor_device(xt_slab_s& s)
{
    cudaStream_t st = s.S.stream;
    const int n = s.p, nnz = s.S.K.nnz;
    Csr K;
    K.n = n;
    K.ia.resize(n + 1);
    K.ja.resize(nnz);
    K.a.resize(nnz);
    XT_CUDA(cudaMemcpyAsync(K.ia.data(), s.S.K.rowptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaMemcpyAsync(K.ja.data(), s.S.K.col.p, sizeof(int) * nnz, cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaMemcpyAsync(K.a.data(), s.S.K.v64.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaStreamSynchronize(st));
    for (int& v : K.ia) ++v;
    for (int& v : K.ja) ++v;
    s.fac = Msr{};  // the kept factor no longer matches the host K
    Msr f;
    const int ierr = s.cfg.ilu_blocks > 1
                         ? ilut(block_diagonal(K, s.cfg.group, s.cfg.ilu_blocks), s.cfg.lfil,
                                s.cfg.droptol, f)
                         : ilut(K, s.cfg.lfil, s.cfg.droptol, f);
    if (ierr != 0) {
        set_error("ILUT of the reassembled K failed with ierr = " + std::to_string(ierr));
        return XT_ERR_HOST;
    }
    return system_set_ilu(s.S, f.alu.data(), f.jlu.data(), f.ju.data(), s.cfg.group,
                          s.cfg.ilu_blocks);
}

// Maps of the coupled loop for the live elements: K's element pattern and
// its reassembly map, and per DOF the entries of the element thermal-stress
// vectors that sum into it (ascending element order).
int couple_maps(xt_slab_s& s)
{
    cudaStream_t st = s.S.stream;
    const Mesh& m = s.pr->mesh;
    std::vector<int> el(s.ne);
    XT_CUDA(cudaMemcpyAsync(el.data(), s.elesta.p, sizeof(int) * s.ne, cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaStreamSynchronize(st));
    std::vector<int> conn, gel;
    for (int e = 0; e < s.ne; ++e)
        if (el[e]) {
            gel.push_back(e);
            conn.insert(conn.end(), m.conn.begin() + (size_t)e * 8, m.conn.begin() + (size_t)e * 8 + 8);
        }
    XT_TRY(system_set_mesh(s.S, s.nn, (int)gel.size(), m.xyz.data(), conn.data(), s.bc.data(),
                           gel.data()));
    std::vector<int> cnt(s.p + 1, 0);
    for (int e : gel)
        for (int i = 0; i < 8; ++i)
            for (int c = 0; c < 3; ++c) ++cnt[3 * (m.conn[(size_t)e * 8 + i] - 1) + c + 1];
    for (int g = 0; g < s.p; ++g) cnt[g + 1] += cnt[g];
    std::vector<int> idx(cnt[s.p]), fill(cnt.begin(), cnt.end() - 1);
    for (int e : gel)
        for (int i = 0; i < 8; ++i)
            for (int c = 0; c < 3; ++c)
                idx[fill[3 * (m.conn[(size_t)e * 8 + i] - 1) + c]++] = e * 24 + 3 * i + c;
    XT_TRY(s.vptr.upload(cnt.data(), cnt.size(), st));
    XT_TRY(s.vidx.upload(idx.data(), idx.size(), st));
    XT_CUDA(cudaStreamSynchronize(st));
    return XT_OK;
}

// One thermal slab, then the moduli, K and the thermal stress load vv
int couple_update(xt_slab_s& s)
{
    XT_TRY(thermal_advance(*s.therm, nullptr));
    cudaStream_t st = s.S.stream;
    const size_t ngp = s.ngp;
    XT_TRY(thermal_couple_device(s.ne, s.conn0.p, s.xyzd.p, thermal_temperature(*s.therm),
                                 s.cc.alpha, s.cc.Tref, s.cc.ym0, s.cc.nu0, s.ymc.p, s.nuc.p,
                                 s.ve.p, st));
    XT_CUDA(cudaMemcpyAsync(s.ym.p, s.ymc.p, ngp * sizeof(double), cudaMemcpyDeviceToDevice, st));
    XT_CUDA(cudaMemcpyAsync(s.nu.p, s.nuc.p, ngp * sizeof(double), cudaMemcpyDeviceToDevice, st));
    XT_TRY(system_assemble_k_device(s.S, s.ymc.p, s.nuc.p, true));
    if (s.force_refactor ||
        (s.cc.refactor_every > 0 && s.coupled_slabs % s.cc.refactor_every == 0)) {
        XT_TRY(refactor_device(s));
        s.force_refactor = false;
    }
    XT_TRY(gather_list(s.p, s.vptr.p, s.vidx.p, s.ve.p, s.vv.p, st));
    ++s.coupled_slabs;
    return XT_OK;
}

int upload_operator(xt_slab_s& s)
{
    const Csr &K = s.pr->sys.K, &M = s.pr->sys.M;
    cudaStream_t st = s.S.stream;
    XT_TRY(upload_csr(s.S.K, K.n, K.ia.data(), K.ja.data(), K.a.data(), st));
    XT_TRY(upload_csr(s.S.M, M.n, M.ia.data(), M.ja.data(), M.a.data(), st));
    csr_mark_shared_pattern(s.S.K, s.S.M, K.ia.data(), K.ja.data(), M.ia.data(), M.ja.data());
    XT_TRY(csr_build_node_blocks(s.S.K, K.n, K.ia.data(), K.ja.data(), K.a.data(), M.ia.data(),
                                 M.ja.data(), M.a.data(), st));
    XT_TRY(s.S.bcmask.upload(s.bc.data(), s.bc.size(), st));
    XT_CUDA(cudaStreamSynchronize(st));
    return XT_OK;
}

int deletion_check(xt_slab_s& s, int& deleted)
{
    deleted = 0;
    cudaStream_t st = s.S.stream;
    XT_TRY(any_ge_device(s.D.p, s.ngp, s.cfg.Dc, s.flag.p, st));
    int f = 0;
    XT_CUDA(cudaMemcpyAsync(&f, s.flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaStreamSynchronize(st));
    if (!f) return XT_OK;
    XT_TRY(chkelesta_device(s.ne, 8, s.cfg.Dc, s.D.p, s.elesta.p, s.gpsta.p, s.nefail.p, s.nef.p, st));
    int nef = 0;
    XT_CUDA(cudaMemcpyAsync(&nef, s.nef.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaStreamSynchronize(st));
    std::vector<int> list(nef > 0 ? nef : 1);
    if (nef > 0) {
        XT_CUDA(cudaMemcpyAsync(list.data(), s.nefail.p, sizeof(int) * nef, cudaMemcpyDeviceToHost, st));
        XT_CUDA(cudaStreamSynchronize(st));
    }
    int ndf = 0;
    XT_TRY(s.pr->delete_elements(nef, list.data(), s.bc.data(), &ndf));
    XT_TRY(upload_operator(s));
    if (s.therm) {  // the coupled K is reassembled on the device from the live elements
        XT_TRY(couple_maps(s));
        s.force_refactor = true;
    } else {
        // K's rows above the first one the surgery changed are as before
        XT_TRY(refactor(s, nef > 0 ? s.pr->first_changed : 0));
    }
    s.dt = s.cfg.dt0 * s.cfg.n2;
    s.nip = s.cfg.nipc * s.cfg.n2;
    s.switched = true;
    s.nfailed += nef;
    deleted = nef;
    return XT_OK;
}

// Steps 1-4 of a slab; the load blocks come from fext_host (block layout)
// when given, else from fextc(j) * rext.  check = false skips the deletion
// check (the overlapped loop makes it after a speculative solve).
int solve_slab(xt_slab_s& s, const double* fext_host, double* stats, bool check = true)
{
    cudaStream_t st = s.S.stream;
    const size_t n = (size_t)s.p * s.q;
    s.slab += 1;
    const double t3 = s.tc[2];
    for (int j = 0; j < 3; ++j) s.tc[j] = t3 + j * s.dt / 2.0;
    int deleted = 0;
    if (check && s.cfg.damage && s.slab > 1) XT_TRY(deletion_check(s, deleted));
    // temporal matrices of this slab
    double ck[36], cm[36], ckt[36], cmt[36], ck1[36], cm1[36], A[36], B[36];
    stcoeff_m(s.tc[0], s.dt, s.w, ck, cm, ckt, cmt, ck1, cm1);
    for (int k = 0; k < 36; ++k) {
        A[k] = ck[k] + ckt[k];
        B[k] = cm[k] + cmt[k];
    }
    if (s.therm) XT_TRY(couple_update(s));  // before the jump term: it uses the new K
    XT_TRY(system_set_temporal(s.S, A, B));
    XT_CUDA(cudaMemcpyAsync(s.S.Cj.p, ck1, sizeof(ck1), cudaMemcpyHostToDevice, st));
    XT_CUDA(cudaMemcpyAsync(s.S.Mj.p, cm1, sizeof(cm1), cudaMemcpyHostToDevice, st));
    // load blocks and jump term
    if (fext_host) {  // staged in hblk: dblk may still feed a running damage update
        XT_TRY(s.hblk.alloc(n));
        XT_CUDA(cudaMemcpyAsync(s.hblk.p, fext_host, n * sizeof(double), cudaMemcpyHostToDevice, st));
        XT_TRY((to_interleaved<double, double>(s.hblk.p, s.fext.p, s.p, s.q, st)));
    } else {
        double fextc[6], fint[6];
        getfextc_m(s.tc[0], s.w, s.dt, fextc, fint);
        // a mean load m * amplitude (load ratio R > -1): weights of a load
        // constant over the slab, the integrals of the temporal shape
        // functions' time derivatives, (-1, 0, 1, 0, 0, 0)
        const double R = s.cfg.load_ratio;
        if (R > -1.0) {
            const double m = (1.0 + R) / (1.0 - R);
            fextc[0] -= m;
            fextc[2] += m;
        }
        XT_TRY(fill_load(s.drext.p, fextc, s.fext.p, s.p, s.q, st));
        if (s.therm) {  // + fint(j) vv, the thermal stress load (src/main3d.f90:813)
            XT_TRY(fill_load(s.vv.p, fint, s.work.p, s.p, s.q, st));
            XT_TRY((axpby<double, double>(n, 1.0, s.work.p, 1.0, s.fext.p, st)));
        }
    }
    XT_TRY(system_apply_with(s.S, s.S.Cj.p, s.S.Mj.p, 1.0, 1.0, s.disp.p, s.fext.p));
    XT_TRY(mask_rows<double>(s.fext.p, s.S.bcmask.p, s.p, s.q, st));
    // solve from zero
    XT_CUDA(cudaMemsetAsync(s.disp.p, 0, n * sizeof(double), st));
    GmresStats gs;
    s.S.gs_passes = s.cfg.gs_passes == 1 ? 1 : 2;
    XT_TRY(solve_refined(s.S, s.fext.p, s.disp.p, s.cfg.im, s.cfg.tol, s.cfg.maxits, s.cfg.precision,
                         s.cfg.inner_tol, gs));
    XT_TRY(mask_rows<double>(s.disp.p, s.S.bcmask.p, s.p, s.q, st));
    if (stats) {
        stats[0] = s.slab;
        stats[1] = gs.its;
        stats[2] = gs.cycles;
        stats[3] = gs.outer;
        stats[4] = gs.ierr;
        stats[5] = gs.relres;
        stats[8] = deleted;
    }
    if (gs.ierr != 0 && gs.ierr != -1) {
        set_error("slab solve did not converge");
        return gs.ierr;
    }
    return XT_OK;
}

int damage_slab(xt_slab_s& s, double* stats)
{
    cudaStream_t st = s.S.stream;
    const size_t n = (size_t)s.p * s.q;
    if (s.cfg.damage) {
        XT_TRY(s.dblk.alloc(n));
        XT_TRY((to_blocks<double, double>(s.disp.p, s.dblk.p, s.p, s.q, st)));
        XT_TRY(s.Nt64.alloc((size_t)s.nip * 6));
        XT_TRY(s.Nt32.alloc((size_t)s.nip * 6));
        XT_TRY(nt_table_device(s.nip, s.tc[0], s.tc[1], s.tc[2], s.w, s.Nt64.p, s.Nt32.p, st));
        XT_CUDA(cudaMemsetAsync(s.counters.p, 0, 3 * sizeof(unsigned long long), st));
        DamageArgs a{};
        a.ngp = s.ngp; a.nn = s.nn; a.ndofn = 3; a.nnse = 8; a.nnte = 3; a.ncmp = 6; a.nip = s.nip;
        a.nodes = s.nodes.p; a.Nx = s.Nx.p; a.Ny = s.Ny.p; a.Nz = s.Nz.p;
        a.Nt = s.Nt64.p; a.Nt32 = s.Nt32.p; a.sol = s.dblk.p; a.ym = s.ym.p; a.nu = s.nu.p;
        a.eps_old = s.eo.p; a.eps_pl = s.ep.p; a.sig_eff = s.se.p; a.sig_back = s.sb.p;
        a.p = s.pp.p; a.D = s.D.p; a.ws = s.ws.p; a.del_po = s.dpo.p; a.sig_d = s.sd.p;
        a.gpsta = s.gpsta.p; a.counters = s.counters.p; a.ntmax = s.ntmax.p;
        const int tok = prof_begin(PROF_DAMAGE, st);
        XT_TRY(damage_update(a, st));
        prof_end(tok, st);
    }
    if (stats) {
        double mx = 0.0;
        unsigned long long cnt[3] = {0, 0, 0};
        if (s.cfg.damage) {
            XT_TRY(max_value(s.D.p, (size_t)s.ngp, s.S.red, st));
            XT_CUDA(cudaMemcpyAsync(&mx, s.S.red.out.p, sizeof(double), cudaMemcpyDeviceToHost, st));
            XT_CUDA(cudaMemcpyAsync(cnt, s.counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, st));
        }
        XT_CUDA(cudaStreamSynchronize(st));
        stats[6] = mx;
        stats[7] = s.nfailed;
        stats[9] = (double)cnt[0];
        stats[10] = (double)cnt[1];
        stats[11] = (double)cnt[2];
    } else {
        XT_CUDA(cudaStreamSynchronize(st));
    }
    return XT_OK;
}

// ------------------------------------------------ overlapped damage update
// The damage update of slab k reads only slab k's displacement and the
// damage state; slab k+1's solve reads neither unless the update deletes
// elements.  So the update runs on a second, lower-priority stream behind
// an event on the displacement, the next slab is solved meanwhile, and the
// deletion flag the update leaves decides afterwards whether that solve
// stands (the usual case) or is repeated on the new operator.

int overlap_init(xt_slab_s& s)
{
    if (s.ds) return XT_OK;
    int least = 0, greatest = 0;
    XT_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    XT_CUDA(cudaStreamCreateWithPriority(&s.ds, cudaStreamNonBlocking, least));
    XT_CUDA(cudaEventCreateWithFlags(&s.ev_sol, cudaEventDisableTiming));
    XT_CUDA(cudaEventCreateWithFlags(&s.ev_dmg, cudaEventDisableTiming));
    XT_CUDA(cudaMallocHost(&s.hbuf, 8 * sizeof(double)));
    XT_TRY(reduce_init(s.red_dmg, 1));
    XT_TRY(s.disp_prev.alloc((size_t)s.p * s.q));
    return XT_OK;
}

// Launch the damage update of the slab just solved on s.ds.
int damage_launch(xt_slab_s& s)
{
    cudaStream_t st = s.S.stream;
    const size_t n = (size_t)s.p * s.q;
    XT_TRY(s.dblk.alloc(n));
    XT_TRY((to_blocks<double, double>(s.disp.p, s.dblk.p, s.p, s.q, st)));
    XT_CUDA(cudaEventRecord(s.ev_sol, st));
    cudaStream_t ds = s.ds;
    XT_CUDA(cudaStreamWaitEvent(ds, s.ev_sol, 0));
    XT_TRY(s.Nt64.alloc((size_t)s.nip * 6));
    XT_TRY(s.Nt32.alloc((size_t)s.nip * 6));
    XT_TRY(nt_table_device(s.nip, s.tc[0], s.tc[1], s.tc[2], s.w, s.Nt64.p, s.Nt32.p, ds));
    XT_CUDA(cudaMemsetAsync(s.counters.p, 0, 3 * sizeof(unsigned long long), ds));
    DamageArgs a{};
    a.ngp = s.ngp; a.nn = s.nn; a.ndofn = 3; a.nnse = 8; a.nnte = 3; a.ncmp = 6; a.nip = s.nip;
    a.nodes = s.nodes.p; a.Nx = s.Nx.p; a.Ny = s.Ny.p; a.Nz = s.Nz.p;
    a.Nt = s.Nt64.p; a.Nt32 = s.Nt32.p; a.sol = s.dblk.p; a.ym = s.ym.p; a.nu = s.nu.p;
    a.eps_old = s.eo.p; a.eps_pl = s.ep.p; a.sig_eff = s.se.p; a.sig_back = s.sb.p;
    a.p = s.pp.p; a.D = s.D.p; a.ws = s.ws.p; a.del_po = s.dpo.p; a.sig_d = s.sd.p;
    a.gpsta = s.gpsta.p; a.counters = s.counters.p; a.ntmax = s.ntmax.p;
    const int tok = prof_begin(PROF_DAMAGE, ds);
    XT_TRY(damage_update(a, ds));
    prof_end(tok, ds);
    XT_TRY(any_ge_device(s.D.p, s.ngp, s.cfg.Dc, s.flag.p, ds));
    XT_TRY(max_value(s.D.p, (size_t)s.ngp, s.red_dmg, ds));
    XT_CUDA(cudaMemcpyAsync(s.hbuf, s.red_dmg.out.p, sizeof(double), cudaMemcpyDeviceToHost, ds));
    XT_CUDA(cudaMemcpyAsync(s.hbuf + 1, s.counters.p, 3 * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, ds));
    XT_CUDA(cudaMemcpyAsync(s.hbuf + 4, s.flag.p, sizeof(int), cudaMemcpyDeviceToHost, ds));
    XT_CUDA(cudaEventRecord(s.ev_dmg, ds));
    s.pending = true;
    return XT_OK;
}

// Wait for the running update (if any) and keep its deletion flag and
// stats in the slab object; the stats of the last finished update go to
// stats[6], [9..11] (stats may be NULL).
int damage_wait(xt_slab_s& s, double* stats)
{
    if (s.pending) {
        XT_CUDA(cudaEventSynchronize(s.ev_dmg));
        s.pending = false;
        unsigned long long cnt[3];
        std::memcpy(cnt, s.hbuf + 1, sizeof(cnt));
        int f = 0;
        std::memcpy(&f, s.hbuf + 4, sizeof(int));
        s.del_flag = f;
        s.dmg_stats[0] = s.hbuf[0];
        for (int k = 0; k < 3; ++k) s.dmg_stats[1 + k] = (double)cnt[k];
    }
    if (stats) {
        stats[6] = s.dmg_stats[0];
        stats[7] = s.nfailed;
        stats[9] = s.dmg_stats[1];
        stats[10] = s.dmg_stats[2];
        stats[11] = s.dmg_stats[3];
    }
    return XT_OK;
}

// One slab in overlap mode.  D_host (may be NULL) receives the damage after
// the previous slab, copied before this slab's update starts.
int step_overlap(xt_slab_s& s, const double* fext_host, double* stats, double* D_host)
{
    XT_TRY(overlap_init(s));
    cudaStream_t st = s.S.stream;
    const size_t n = (size_t)s.p * s.q;
    const int slab0 = s.slab;
    const double tc0[3] = {s.tc[0], s.tc[1], s.tc[2]};
    XT_CUDA(cudaMemcpyAsync(s.disp_prev.p, s.disp.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    // speculative solve, concurrent with the previous slab's damage update
    XT_TRY(solve_slab(s, fext_host, stats, false));
    XT_TRY(damage_wait(s, stats));
    const int flag = s.del_flag;
    s.del_flag = 0;
    if (flag && s.cfg.damage) {
        // the update deleted elements: repeat this slab exactly as the
        // sequential loop does it (deletion check first, then the solve)
        s.slab = slab0;
        for (int j = 0; j < 3; ++j) s.tc[j] = tc0[j];
        XT_CUDA(cudaMemcpyAsync(s.disp.p, s.disp_prev.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
        XT_TRY(solve_slab(s, fext_host, stats, true));
    }
    if (D_host)
        XT_CUDA(cudaMemcpyAsync(D_host, s.D.p, (size_t)s.ngp * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (s.cfg.damage) XT_TRY(damage_launch(s));
    return XT_OK;
}

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

}  // namespace

// ------------------------------------------------------------ state dump
// The output step of the reference (mpipostprocess and its writers,
// src/postprocess.f90:106-378): at t = tc1 + (nout - 1) dt / nip with
// nout = nip - (nipc / 4) 3 + 1, the nodal displacement (.disp), the
// Gauss-point strain and stress (.strain, .stress, 6(E16.8,2X)), damage
// (.damage), stored energy (.energy) and element status (.status); the
// time goes to .time.  Files <job>.time and <job>.disp are the root rank's,
// <job>_0.* the per-rank ones of a one-process run; records are appended,
// after truncating every file when asked (initfile).  List-directed
// records carry 17 significant digits, one value per field.
namespace {

void fortran_e16_8(double v, char* out)
{
    // Fortran E16.8: 0.dddddddd with an exponent of two digits
    if (v == 0.0) {
        std::snprintf(out, 17, "%16s", "0.00000000E+00");
        return;
    }
    char buf[32];
    std::snprintf(buf, sizeof buf, "%.7e", std::fabs(v));  // d.ddddddde+XX
    const int ex = std::atoi(buf + 10) + 1;
    char body[24];
    std::snprintf(body, sizeof body, "%s0.%c%.7sE%c%02d", v < 0 ? "-" : "", buf[0], buf + 2,
                  ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
    std::snprintf(out, 17, "%16s", body);
}

FILE* open_dump(const std::string& path, bool truncate)
{
    FILE* f = std::fopen(path.c_str(), truncate ? "w" : "a");
    if (!f) throw std::runtime_error("cannot open " + path);
    return f;
}

int slab_dump(xt_slab_s& s, const std::string& job, bool truncate)
{
    if (s.slab < 1) {
        set_error("xt_slab_dump: no slab solved yet");
        return XT_ERR_STATE;
    }
    cudaStream_t st = s.S.stream;
    const int nn = s.nn, ngp = s.ngp;
    const size_t n = (size_t)s.p * 6;
    const int nip = s.nip, nipc = s.cfg.nipc;
    const double dt = s.tc[2] - s.tc[0];
    const int nout = nip - nipc / 4 * 3 + 1;
    const double t = s.tc[0] + (nout - 1) * dt / nip;
    double Nt[6];
    Nt[0] = 2.0 * (s.tc[1] - t) * (s.tc[2] - t) / (dt * dt);
    Nt[1] = -4.0 * (s.tc[0] - t) * (s.tc[2] - t) / (dt * dt);
    Nt[2] = 2.0 * (s.tc[0] - t) * (s.tc[1] - t) / (dt * dt);
    Nt[3] = Nt[0] * (std::sin(s.w * t) - std::sin(s.w * s.tc[0]));
    Nt[4] = Nt[1] * (std::sin(s.w * t) - std::sin(s.w * s.tc[1]));
    Nt[5] = Nt[2] * (std::sin(s.w * t) - std::sin(s.w * s.tc[2]));
    XT_TRY(s.hblk.alloc(n));
    XT_TRY((to_blocks<double, double>(s.disp.p, s.hblk.p, s.p, 6, st)));
    DBuf<double> strain, stress;
    XT_TRY(strain.alloc((size_t)ngp * 6));
    XT_TRY(stress.alloc((size_t)ngp * 6));
    XT_TRY(post_strain_stress(ngp, nn, s.nodes.p, s.Nx.p, s.Ny.p, s.Nz.p, s.ym.p, s.nu.p,
                              s.gpsta.p, s.hblk.p, Nt, strain.p, stress.p, st));
    std::vector<double> sol(n), hs((size_t)ngp * 6), hst((size_t)ngp * 6), D(ngp), ws(ngp);
    std::vector<int> el(s.ne);
    XT_CUDA(cudaMemcpyAsync(sol.data(), s.hblk.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaMemcpyAsync(hs.data(), strain.p, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaMemcpyAsync(hst.data(), stress.p, hst.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaMemcpyAsync(D.data(), s.D.p, ngp * sizeof(double), cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaMemcpyAsync(ws.data(), s.ws.p, ngp * sizeof(double), cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaMemcpyAsync(el.data(), s.elesta.p, s.ne * sizeof(int), cudaMemcpyDeviceToHost, st));
    XT_CUDA(cudaStreamSynchronize(st));
    const std::string rank = job + "_0";
    if (truncate) {  // initfile: the root's .temp exists too (no thermal part here)
        std::fclose(open_dump(job + ".temp", true));
    }
    FILE* f = open_dump(job + ".time", truncate);
    std::fprintf(f, " %25.17E\n", t);
    std::fclose(f);
    f = open_dump(job + ".disp", truncate);
    for (int j = 0; j < nn; ++j) {
        for (int c = 0; c < 3; ++c) {
            double v = 0.0;
            for (int k = 0; k < 6; ++k) v += Nt[k] * sol[(size_t)k * nn * 3 + (size_t)j * 3 + c];
            std::fprintf(f, " %25.17E", v);
        }
        std::fputc('\n', f);
    }
    std::fclose(f);
    char field[20];
    for (int pass = 0; pass < 2; ++pass) {
        const std::vector<double>& a = pass == 0 ? hs : hst;
        f = open_dump(rank + (pass == 0 ? ".strain" : ".stress"), truncate);
        for (int g = 0; g < ngp; ++g) {
            for (int c = 0; c < 6; ++c) {
                fortran_e16_8(a[(size_t)g * 6 + c], field);
                std::fprintf(f, "%s  ", field);
            }
            std::fputc('\n', f);
        }
        std::fclose(f);
    }
    f = open_dump(rank + ".damage", truncate);
    for (double v : D) std::fprintf(f, " %25.17E\n", v);
    std::fclose(f);
    f = open_dump(rank + ".energy", truncate);
    for (double v : ws) std::fprintf(f, " %25.17E\n", v);
    std::fclose(f);
    f = open_dump(rank + ".status", truncate);
    for (int v : el) std::fprintf(f, " %11d\n", v);
    std::fclose(f);
    return XT_OK;
}

}  // namespace

extern "C" {

int xt_slab_create(xth_problem h, const xt_slab_config* cfg, xt_slab* out)
{
    if (!h || !cfg || !out) { set_error("xt_slab_create: null argument"); return XT_ERR_ARG; }
    *out = nullptr;
    XT_TRY(ensure_init());
    return guarded([&]() -> int {
        auto s = std::make_unique<xt_slab_s>();
        s->pr = reinterpret_cast<Problem*>(h);
        s->cfg = *cfg;
        Problem& pr = *s->pr;
        const Mesh& m = pr.mesh;
        if (cfg->clamp_axis < 0 || cfg->clamp_axis > 2 || cfg->load_axis < 0 || cfg->load_axis > 2 ||
            cfg->load_comp < 0 || cfg->load_comp > 2 || cfg->im < 1 || cfg->dt0 <= 0 || cfg->n1 < 1 ||
            cfg->n2 < 1 || cfg->nipc < 0 || cfg->lfil < 0 || !(cfg->load_ratio >= -1.0) ||
            !(cfg->load_ratio < 1.0) || cfg->gs_passes < 0 || cfg->gs_passes > 2 ||
            cfg->ilu_blocks < 0) {
            set_error("xt_slab_create: invalid configuration");
            return XT_ERR_ARG;
        }
        s->nn = m.nn;
        s->ne = m.ne;
        s->ngp = 8 * m.ne;
        s->p = 3 * m.nn;
        // boundary conditions: all 3 DOFs of nodes on the clamped face
        // (src/main3d.f90:482-497 with an axis-aware face selector)
        s->bc.assign(s->p, 0);
        for (int i = 0; i < m.nn; ++i)
            if (m.xyz[(size_t)i * 3 + cfg->clamp_axis] == cfg->clamp_value)
                for (int c = 0; c < 3; ++c) s->bc[(size_t)i * 3 + c] = 1;
        csrapplybc(pr.sys.K, s->bc.data());
        csrapplybc(pr.sys.M, s->bc.data());
        // traction: the total force amplitude * area shared over the face's
        // element-node incidences (src/main3d.f90:501-530)
        std::vector<double> share(m.nn, 0.0);
        for (size_t k = 0; k < m.conn.size(); ++k) share[m.conn[k] - 1] += 1.0;
        double ntele = 0.0;
        for (int i = 0; i < m.nn; ++i)
            if (m.xyz[(size_t)i * 3 + cfg->load_axis] == cfg->load_value) ntele += share[i];
        if (ntele == 0.0) {
            set_error("xt_slab_create: no node on the loaded face");
            return XT_ERR_ARG;
        }
        const double fnode = cfg->amplitude * cfg->area / ntele;
        s->rext.assign(s->p, 0.0);
        for (size_t k = 0; k < m.conn.size(); ++k) {
            const int nd = m.conn[k] - 1;
            if (m.xyz[(size_t)nd * 3 + cfg->load_axis] == cfg->load_value)
                s->rext[(size_t)nd * 3 + cfg->load_comp] += fnode;
        }
        System& S = s->S;
        S.p = s->p;
        S.q = 6;
        XT_TRY(S.A.alloc(64)); XT_TRY(S.B.alloc(64)); XT_TRY(S.Ainv.alloc(64));
        XT_TRY(S.Cj.alloc(64)); XT_TRY(S.Mj.alloc(64));
        XT_TRY(system_stream(S));
        XT_TRY(upload_operator(*s));
        XT_TRY(refactor(*s));
        cudaStream_t st = s->S.stream;
        const size_t n = (size_t)s->p * 6, ngp = s->ngp;
        XT_TRY(s->drext.upload(s->rext.data(), s->p, st));
        XT_TRY(s->fext.alloc(n));
        XT_TRY(s->disp.alloc(n));
        XT_CUDA(cudaMemsetAsync(s->disp.p, 0, n * sizeof(double), st));
        if (S.red.kmax < cfg->im + 1) XT_TRY(reduce_init(S.red, cfg->im + 1));
        // damage state, zero initial state (src/main3d.f90:583-600)
        std::vector<int> nodes(ngp * 8);
        for (size_t gp = 0; gp < ngp; ++gp)
            for (int i = 0; i < 8; ++i) nodes[gp * 8 + i] = m.conn[(gp / 8) * 8 + i];
        XT_TRY(s->nodes.upload(nodes.data(), nodes.size(), st));
        XT_TRY(s->Nx.upload(pr.sys.Nx.data(), pr.sys.Nx.size(), st));
        XT_TRY(s->Ny.upload(pr.sys.Ny.data(), pr.sys.Ny.size(), st));
        XT_TRY(s->Nz.upload(pr.sys.Nz.data(), pr.sys.Nz.size(), st));
        std::vector<double> ymv(ngp, pr.E), nuv(ngp, pr.nu);
        XT_TRY(s->ym.upload(ymv.data(), ngp, st));
        XT_TRY(s->nu.upload(nuv.data(), ngp, st));
        for (DBuf<double>* b : {&s->eo, &s->ep, &s->se, &s->sb}) {
            XT_TRY(b->alloc(ngp * 6));
            XT_CUDA(cudaMemsetAsync(b->p, 0, ngp * 6 * sizeof(double), st));
        }
        for (DBuf<double>* b : {&s->pp, &s->D, &s->ws, &s->dpo, &s->sd}) {
            XT_TRY(b->alloc(ngp));
            XT_CUDA(cudaMemsetAsync(b->p, 0, ngp * sizeof(double), st));
        }
        std::vector<int> ones(ngp, 1);
        XT_TRY(s->gpsta.upload(ones.data(), ngp, st));
        XT_TRY(s->elesta.upload(ones.data(), s->ne, st));
        XT_TRY(s->nefail.alloc(s->ne));
        XT_TRY(s->nef.alloc(1));
        XT_TRY(s->flag.alloc(1));
        XT_TRY(s->counters.alloc(3));
        XT_TRY(s->ntmax.alloc(8));
        XT_CUDA(cudaStreamSynchronize(st));
        s->w = 2.0 * M_PI * cfg->freq;
        s->dt = cfg->dt0 * cfg->n1;
        s->nip = cfg->nipc * cfg->n1;
        *out = s.release();
        return XT_OK;
    });
}

int xt_slab_destroy(xt_slab s)
{
    delete s;
    return XT_OK;
}

int xt_slab_step(xt_slab s, double* stats)
{
    if (!s) { set_error("null slab"); return XT_ERR_ARG; }
    double local[12] = {0};
    double* st = stats ? stats : local;
    return guarded([&]() -> int {
        TraceRange tr("xtfem slab step");
        if (s->cfg.overlap) {
            XT_TRY(step_overlap(*s, nullptr, st, nullptr));
            XT_CUDA(cudaStreamSynchronize(s->S.stream));
            return XT_OK;
        }
        XT_TRY(solve_slab(*s, nullptr, st));
        return damage_slab(*s, st);
    });
}

int xt_slab_drain(xt_slab s, double* stats)
{
    if (!s) { set_error("null slab"); return XT_ERR_ARG; }
    return guarded([&]() -> int { return damage_wait(*s, stats); });
}

int xt_slab_step_host(xt_slab s, const double* fext, double* disp, double* D, double* stats)
{
    if (!s || !fext) { set_error("xt_slab_step_host: null argument"); return XT_ERR_ARG; }
    double local[12] = {0};
    double* st = stats ? stats : local;
    return guarded([&]() -> int {
        TraceRange tr("xtfem slab step");
        cudaStream_t cs = s->S.stream;
        const size_t n = (size_t)s->p * s->q;
        if (s->cfg.overlap) {
            XT_TRY(step_overlap(*s, fext, st, D));
        } else {
            XT_TRY(solve_slab(*s, fext, st));
            XT_TRY(damage_slab(*s, st));
            if (D) XT_CUDA(cudaMemcpyAsync(D, s->D.p, (size_t)s->ngp * sizeof(double), cudaMemcpyDeviceToHost, cs));
        }
        if (disp) {
            XT_TRY(s->hblk.alloc(n));
            XT_TRY((to_blocks<double, double>(s->disp.p, s->hblk.p, s->p, s->q, cs)));
            XT_CUDA(cudaMemcpyAsync(disp, s->hblk.p, n * sizeof(double), cudaMemcpyDeviceToHost, cs));
        }
        XT_CUDA(cudaStreamSynchronize(cs));
        return XT_OK;
    });
}

int xt_slab_set_state(xt_slab s, const double* D, const double* ws)
{
    if (!s) { set_error("null slab"); return XT_ERR_ARG; }
    XT_TRY(damage_wait(*s, nullptr));
    cudaStream_t cs = s->S.stream;
    const size_t b = (size_t)s->ngp * sizeof(double);
    if (D) XT_CUDA(cudaMemcpyAsync(s->D.p, D, b, cudaMemcpyHostToDevice, cs));
    if (ws) XT_CUDA(cudaMemcpyAsync(s->ws.p, ws, b, cudaMemcpyHostToDevice, cs));
    XT_CUDA(cudaStreamSynchronize(cs));
    return XT_OK;
}

int xt_slab_couple(xt_slab s, xt_thermal t, const xt_coupling_config* cc)
{
    if (!s || !t || !cc) { set_error("xt_slab_couple: null argument"); return XT_ERR_ARG; }
    if (s->cfg.overlap) { set_error("xt_slab_couple: not with cfg.overlap"); return XT_ERR_ARG; }
    if (thermal_nodes(*t) != s->nn) {
        set_error("xt_slab_couple: the thermal loop has another mesh");
        return XT_ERR_ARG;
    }
    if (s->slab > 0) { set_error("xt_slab_couple: couple before the first slab"); return XT_ERR_STATE; }
    try {
        s->therm = t;
        s->cc = *cc;
        const Mesh& m = s->pr->mesh;
        cudaStream_t st = s->S.stream;
        std::vector<int> c0(m.conn.begin(), m.conn.end());
        for (int& v : c0) --v;
        XT_TRY(s->conn0.upload(c0.data(), c0.size(), st));
        XT_TRY(s->xyzd.upload(m.xyz.data(), m.xyz.size(), st));
        for (DBuf<double>* b : {&s->ymc, &s->nuc}) XT_TRY(b->alloc((size_t)s->ngp));
        XT_TRY(s->ve.alloc((size_t)s->ne * 24));
        XT_TRY(s->vv.alloc((size_t)s->p));
        XT_TRY(s->work.alloc((size_t)s->p * s->q));
        XT_TRY(couple_maps(*s));
        return XT_OK;
    } catch (const std::exception& e) {
        s->therm = nullptr;
        set_error(std::string("xt_slab_couple: ") + e.what());
        return XT_ERR_HOST;
    }
}

int xt_slab_dump(xt_slab s, const char* job, int truncate)
{
    if (!s || !job) { set_error("xt_slab_dump: null argument"); return XT_ERR_ARG; }
    XT_TRY(damage_wait(*s, nullptr));
    try {
        return slab_dump(*s, job, truncate != 0);
    } catch (const std::exception& e) {
        set_error(std::string("xt_slab_dump: ") + e.what());
        return XT_ERR_HOST;
    }
}

int xt_slab_get(xt_slab s, double* disp, double* D, double* ws, int* elesta)
{
    if (!s) { set_error("null slab"); return XT_ERR_ARG; }
    XT_TRY(damage_wait(*s, nullptr));
    cudaStream_t cs = s->S.stream;
    const size_t n = (size_t)s->p * s->q;
    if (disp) {
        XT_TRY(s->hblk.alloc(n));
        XT_TRY((to_blocks<double, double>(s->disp.p, s->hblk.p, s->p, s->q, cs)));
        XT_CUDA(cudaMemcpyAsync(disp, s->hblk.p, n * sizeof(double), cudaMemcpyDeviceToHost, cs));
    }
    if (D) XT_CUDA(cudaMemcpyAsync(D, s->D.p, (size_t)s->ngp * sizeof(double), cudaMemcpyDeviceToHost, cs));
    if (ws) XT_CUDA(cudaMemcpyAsync(ws, s->ws.p, (size_t)s->ngp * sizeof(double), cudaMemcpyDeviceToHost, cs));
    if (elesta) XT_CUDA(cudaMemcpyAsync(elesta, s->elesta.p, (size_t)s->ne * sizeof(int), cudaMemcpyDeviceToHost, cs));
    XT_CUDA(cudaStreamSynchronize(cs));
    return XT_OK;
}

}  // extern "C"
