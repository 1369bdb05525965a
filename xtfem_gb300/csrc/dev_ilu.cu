// dev_ilu.cu -- the Kronecker ILUT preconditioner on the GPU.
//
// Applies z = (A^-1 (x) (LU)^-1) v, the operator of src/kronecker.f90:130-178
// (kronlusol), whose spatial part is SPARSKIT lusol (src/ilut.f:2383-2432):
// a forward sweep with the unit lower factor and a backward sweep with the
// upper factor and inverted diagonal, for each of the q temporal blocks.
//
// The factor is computed on the host (ILUT, FP64) and arrives in MSR form.
// Triangular solves are chains of dependent rows, so the work is organised
// by level sets computed once per factor:
//   * rows are grouped by node (g = 3 consecutive DOFs); a group's level is
//     one more than the deepest other group it reads, and one warp solves
//     the g rows of a group in sequence, which roughly halves the number of
//     levels compared with single-row levels on C3D8 meshes;
//   * all q right-hand sides of a row are solved together: lanes are split
//     into q segments of S lanes, each segment walks the row's external
//     nonzeros for one temporal block and reduces with shuffles;
//   * the q x q mixing with A^-1 is applied to v on the fly while the
//     forward sweep reads it (the mixing commutes with the spatial solve);
//   * one thread block runs all levels of a sweep with a block barrier
//     between levels; values solved earlier are read back from global
//     memory (L2-resident) after the barrier.
// The kernel is latency-bound (levels x barrier+gather latency), not
// bandwidth-bound; batching independent systems fills the other SMs.
#include <cooperative_groups.h>
#include <cuda_pipeline.h>

#include <algorithm>
#include <vector>

#include "xt_device.h"

namespace xt {

namespace {

constexpr int kMaxG = 3;

struct TriHost {
    int ngroups = 0, nlevels = 0, g = 1, maxw = 0;
    std::vector<int> level_ptr, level_e, group_row0, ext_ptr, ext_col;
    std::vector<double> ext_v, int_v, dinv;
};

// Level-schedule one triangle.  upper == false: rows' L parts
// (jlu(i) .. ju(i)-1); upper == true: U parts (ju(i) .. jlu(i+1)-1).
TriHost schedule(int n, const double* alu, const int* jlu, const int* ju, int g, bool upper)
{
    TriHost T;
    T.g = g;
    const int ng = n / g;
    T.ngroups = ng;
    std::vector<int> lev(ng, 0);
    auto row_range = [&](int r, int& b, int& e) {  // 0-based positions into alu/jlu
        if (!upper) { b = jlu[r] - 1; e = ju[r] - 1; }
        else { b = ju[r] - 1; e = jlu[r + 1] - 1; }
    };
    int maxl = 0;
    for (int s = 0; s < ng; ++s) {
        const int G = upper ? ng - 1 - s : s;
        int l = 0;
        for (int ri = 0; ri < g; ++ri) {
            int b, e;
            row_range(G * g + ri, b, e);
            for (int k = b; k < e; ++k) {
                const int c = (jlu[k] - 1) / g;
                if (c != G) l = std::max(l, lev[c] + 1);
            }
        }
        lev[G] = l;
        maxl = std::max(maxl, l);
    }
    T.nlevels = maxl + 1;
    std::vector<int> cnt(T.nlevels + 1, 0);
    for (int G = 0; G < ng; ++G) cnt[lev[G] + 1]++;
    for (int l = 0; l < T.nlevels; ++l) {
        cnt[l + 1] += cnt[l];
        T.maxw = std::max(T.maxw, cnt[l + 1] - cnt[l]);
    }
    T.level_ptr = cnt;
    std::vector<int> order(ng), pos(cnt.begin(), cnt.end() - 1);
    for (int G = 0; G < ng; ++G) order[pos[lev[G]]++] = G;
    T.group_row0.resize(ng);
    T.ext_ptr.assign((size_t)ng * g + 1, 0);
    T.int_v.assign((size_t)ng * g * g, 0.0);
    if (upper) T.dinv.assign((size_t)ng * g, 0.0);
    for (int i = 0; i < ng; ++i) {
        const int G = order[i];
        T.group_row0[i] = G * g;
        for (int ri = 0; ri < g; ++ri) {
            const int r = G * g + ri;
            int b, e;
            row_range(r, b, e);
            for (int k = b; k < e; ++k) {
                const int c = jlu[k] - 1;
                if (c / g == G) {
                    T.int_v[((size_t)i * g + ri) * g + (c - G * g)] += alu[k];
                } else {
                    T.ext_col.push_back(c);
                    T.ext_v.push_back(alu[k]);
                }
            }
            T.ext_ptr[(size_t)i * g + ri + 1] = (int)T.ext_col.size();
            if (upper) T.dinv[(size_t)i * g + ri] = alu[r];
        }
    }
    T.level_e.resize(T.nlevels + 1);
    for (int l = 0; l <= T.nlevels; ++l) T.level_e[l] = T.ext_ptr[(size_t)T.level_ptr[l] * g];
    return T;
}

int upload_tri(DevTri& d, const TriHost& h, cudaStream_t s)
{
    d.ngroups = h.ngroups;
    d.nlevels = h.nlevels;
    d.g = h.g;
    d.max_level_groups = h.maxw;
    XT_TRY(d.level_ptr.upload(h.level_ptr.data(), h.level_ptr.size(), s));
    XT_TRY(d.level_e.upload(h.level_e.data(), h.level_e.size(), s));
    XT_TRY(d.group_row0.upload(h.group_row0.data(), h.group_row0.size(), s));
    XT_TRY(d.ext_ptr.upload(h.ext_ptr.data(), h.ext_ptr.size(), s));
    const size_t ne = h.ext_col.size();
    if (ne) {
        XT_TRY(d.ext_col.upload(h.ext_col.data(), ne, s));
        XT_TRY(d.ext_v64.upload(h.ext_v.data(), ne, s));
        std::vector<float> f(h.ext_v.begin(), h.ext_v.end());
        XT_TRY(d.ext_v32.upload(f.data(), ne, s));
        XT_CUDA(cudaStreamSynchronize(s));  // f goes out of scope
    } else {
        XT_TRY(d.ext_col.alloc(1));
        XT_TRY(d.ext_v64.alloc(1));
        XT_TRY(d.ext_v32.alloc(1));
    }
    XT_TRY(d.int_v64.upload(h.int_v.data(), h.int_v.size(), s));
    {
        std::vector<float> f(h.int_v.begin(), h.int_v.end());
        XT_TRY(d.int_v32.upload(f.data(), f.size(), s));
        XT_CUDA(cudaStreamSynchronize(s));
    }
    if (!h.dinv.empty()) {
        XT_TRY(d.dinv64.upload(h.dinv.data(), h.dinv.size(), s));
        std::vector<float> f(h.dinv.begin(), h.dinv.end());
        XT_TRY(d.dinv32.upload(f.data(), f.size(), s));
        XT_CUDA(cudaStreamSynchronize(s));
    }
    return XT_OK;
}

template <class T>
struct TriView {
    int nlevels, g, ngroups;
    const int *level_ptr, *group_row0, *ext_ptr, *ext_col;
    const T *ext_v, *int_v, *dinv;
};

template <class T>
TriView<T> view(const DevTri& d);
template <>
TriView<double> view<double>(const DevTri& d)
{
    return {d.nlevels, d.g, d.ngroups, d.level_ptr.p, d.group_row0.p, d.ext_ptr.p, d.ext_col.p,
            d.ext_v64.p, d.int_v64.p, d.dinv64.p};
}
template <>
TriView<float> view<float>(const DevTri& d)
{
    return {d.nlevels, d.g, d.ngroups, d.level_ptr.p, d.group_row0.p, d.ext_ptr.p, d.ext_col.p,
            d.ext_v32.p, d.int_v32.p, d.dinv32.p};
}

// One sweep (forward when UPPER == false).  x is read and written by the
// kernel itself, so it is accessed through plain (coherent) loads.  For the
// forward sweep the right-hand side is v mixed with Ainv; for the backward
// sweep it is x itself (the forward result) and the output goes to z.
template <class T, int Q, int S, bool UPPER>
__global__ void __launch_bounds__(1024, 1)
k_tri_sweep(TriView<T> t, const double* __restrict__ dAinv, const T* __restrict__ v,
            T* x, T* z)
{
    __shared__ T sAinv[Q * Q];
    for (int i = threadIdx.x; i < Q * Q; i += blockDim.x) sAinv[i] = (T)dAinv[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int rhs = lane / S;
    const int sub = lane % S;
    const bool live = rhs < Q;
    const int g = t.g;
    for (int l = 0; l < t.nlevels; ++l) {
        const int gb = t.level_ptr[l], ge = t.level_ptr[l + 1];
        for (int gi = gb + warp; gi < ge; gi += nwarps) {
            const int row0 = t.group_row0[gi];
            T acc[kMaxG];
#pragma unroll
            for (int ri = 0; ri < kMaxG; ++ri) {
                acc[ri] = T(0);
                if (ri < g && live) {
                    const int kb = t.ext_ptr[gi * g + ri], ke = t.ext_ptr[gi * g + ri + 1];
                    for (int k = kb + sub; k < ke; k += S)
                        acc[ri] = fma(t.ext_v[k], x[(size_t)t.ext_col[k] * Q + rhs], acc[ri]);
                }
            }
#pragma unroll
            for (int off = S / 2; off > 0; off >>= 1)
#pragma unroll
                for (int ri = 0; ri < kMaxG; ++ri)
                    acc[ri] += __shfl_xor_sync(0xffffffffu, acc[ri], off);
            if (live) {
                T sol[kMaxG];
                const T* iv = t.int_v + (size_t)gi * g * g;
                for (int s = 0; s < g; ++s) {
                    const int ri = UPPER ? g - 1 - s : s;
                    const int r = row0 + ri;
                    T b;
                    if (!UPPER) {
                        b = T(0);
#pragma unroll
                        for (int j = 0; j < Q; ++j) b = fma(sAinv[j * Q + rhs], v[(size_t)r * Q + j], b);
                    } else {
                        b = x[(size_t)r * Q + rhs];
                    }
                    T val = b - acc[ri];
                    if (!UPPER) {
                        for (int c = 0; c < ri; ++c) val -= iv[ri * g + c] * sol[c];
                    } else {
                        for (int c = ri + 1; c < g; ++c) val -= iv[ri * g + c] * sol[c];
                        val *= t.dinv[(size_t)gi * g + ri];
                    }
                    sol[ri] = val;
                }
                if (sub == 0)
                    for (int ri = 0; ri < g; ++ri) {
                        T* dst = UPPER ? z : x;
                        dst[(size_t)(row0 + ri) * Q + rhs] = sol[ri];
                        if (UPPER && z != x) x[(size_t)(row0 + ri) * Q + rhs] = sol[ri];
                    }
            }
        }
        __syncthreads();
    }
}

template <class T, int Q>
int launch_tri_simple(const DevIlu& F, const double* dAinv, const T* v, T* z, T* work,
                      cudaStream_t s);

// ---------------------------------------------------------------------------
// Staged sweep.  The factor data of a level does not depend on the solution,
// so it is copied into a three-deep shared-memory ring with asynchronous
// copies issued two levels ahead; a level then costs one block barrier plus
// the gathers of previously solved values, instead of a chain of dependent
// global loads.  Each (group, temporal block) task is handled by kSub
// threads that split the group's external nonzeros and reduce with shuffles.
// Levels larger than the ring (more than kMaxGroups groups or kMaxEnt
// nonzeros, e.g. the clamped face's identity rows) are read from global
// memory directly.
constexpr int kMaxGroups = 64;
constexpr int kMaxEnt = 4096;
constexpr int kRing = 3;
constexpr int kSub = 4;
constexpr int kBatch = 8;  // gathers in flight per lane and batch
constexpr int kLpCap = 2048;

template <class T>
struct Ring {
    // byte offsets inside one ring slot
    static constexpr size_t v_off = 0;                                    // kMaxEnt T
    static constexpr size_t i_off = v_off + sizeof(T) * kMaxEnt;           // 9*kMaxGroups T
    static constexpr size_t d_off = i_off + sizeof(T) * 9 * kMaxGroups;    // 3*kMaxGroups T
    static constexpr size_t c_off = d_off + sizeof(T) * 3 * kMaxGroups;    // kMaxEnt int
    static constexpr size_t e_off = c_off + sizeof(int) * kMaxEnt;         // 3*kMaxGroups+1 int
    static constexpr size_t r_off = e_off + sizeof(int) * (3 * kMaxGroups + 4);
    static constexpr size_t slot = ((r_off + sizeof(int) * kMaxGroups) + 127) / 128 * 128;
    static constexpr size_t lp_off = kRing * slot;                        // 2*(kLpCap+1) int
    static constexpr size_t bytes = lp_off + sizeof(int) * 2 * (kLpCap + 1);
};

template <class T, int Q, bool UPPER>
__global__ void __launch_bounds__(1024, 1)
k_tri_staged(TriView<T> t, const int* __restrict__ level_e, const double* __restrict__ dAinv,
             const T* __restrict__ v, T* x, T* z)
{
    extern __shared__ __align__(128) unsigned char smem[];
    using R = Ring<T>;
    __shared__ T sAinv[Q * Q];
    const int tid = threadIdx.x, nth = blockDim.x;
    const int g = t.g;
    const int nl = t.nlevels;
    const bool lp_in_smem = nl + 1 <= kLpCap + 1;
    int* s_lp = reinterpret_cast<int*>(smem + R::lp_off);
    int* s_le = s_lp + (kLpCap + 1);
    for (int i = tid; i < Q * Q; i += nth) sAinv[i] = (T)dAinv[i];
    if (lp_in_smem)
        for (int i = tid; i <= nl; i += nth) {
            s_lp[i] = t.level_ptr[i];
            s_le[i] = level_e[i];
        }
    __syncthreads();
    const int* lp = lp_in_smem ? s_lp : t.level_ptr;
    const int* le = lp_in_smem ? s_le : level_e;

    auto staged = [&](int L) {
        return lp[L + 1] - lp[L] <= kMaxGroups && le[L + 1] - le[L] <= kMaxEnt;
    };
    auto prefetch = [&](int L) {
        if (L < nl && staged(L)) {
            unsigned char* slot = smem + (size_t)(L % kRing) * R::slot;
            T* sv = reinterpret_cast<T*>(slot + R::v_off);
            T* si = reinterpret_cast<T*>(slot + R::i_off);
            T* sd = reinterpret_cast<T*>(slot + R::d_off);
            int* sc = reinterpret_cast<int*>(slot + R::c_off);
            int* se = reinterpret_cast<int*>(slot + R::e_off);
            int* sr = reinterpret_cast<int*>(slot + R::r_off);
            const int gb = lp[L], ng = lp[L + 1] - gb;
            const int e0 = le[L], ne = le[L + 1] - e0;
            for (int i = tid; i < ne; i += nth) {
                __pipeline_memcpy_async(sc + i, t.ext_col + e0 + i, sizeof(int));
                __pipeline_memcpy_async(sv + i, t.ext_v + e0 + i, sizeof(T));
            }
            for (int i = tid; i <= ng * g; i += nth)
                __pipeline_memcpy_async(se + i, t.ext_ptr + (size_t)gb * g + i, sizeof(int));
            for (int i = tid; i < ng; i += nth)
                __pipeline_memcpy_async(sr + i, t.group_row0 + gb + i, sizeof(int));
            for (int i = tid; i < ng * g * g; i += nth)
                __pipeline_memcpy_async(si + i, t.int_v + (size_t)gb * g * g + i, sizeof(T));
            if (UPPER)
                for (int i = tid; i < ng * g; i += nth)
                    __pipeline_memcpy_async(sd + i, t.dinv + (size_t)gb * g + i, sizeof(T));
        }
        __pipeline_commit();
    };

    prefetch(0);
    prefetch(1);
    __pipeline_wait_prior(1);
    __syncthreads();
    const int sub = tid % kSub;
    const int tasks_per_pass = nth / kSub;
    for (int l = 0; l < nl; ++l) {
        prefetch(l + 2);
        const int gb = lp[l], ng = lp[l + 1] - gb;
        const int e0 = le[l];
        const bool st = staged(l);
        const unsigned char* slot = smem + (size_t)(l % kRing) * R::slot;
        const T* sv = st ? reinterpret_cast<const T*>(slot + R::v_off) : t.ext_v + e0;
        const int* sc = st ? reinterpret_cast<const int*>(slot + R::c_off) : t.ext_col + e0;
        const int* se = st ? reinterpret_cast<const int*>(slot + R::e_off) : t.ext_ptr + (size_t)gb * g;
        const int* sr = st ? reinterpret_cast<const int*>(slot + R::r_off) : t.group_row0 + gb;
        const T* si = st ? reinterpret_cast<const T*>(slot + R::i_off) : t.int_v + (size_t)gb * g * g;
        const T* sd = st ? reinterpret_cast<const T*>(slot + R::d_off) : (UPPER ? t.dinv + (size_t)gb * g : nullptr);
        const int ntask = ng * Q;
        for (int base = 0; base < ntask; base += tasks_per_pass) {
            const int task = base + tid / kSub;
            const bool act = task < ntask;
            const int gi = act ? task / Q : 0, rhs = act ? task % Q : 0;
            const int row0 = act ? sr[gi] : 0;
            // right-hand side of row (row0 + sub), issued before the gathers so
            // its latency overlaps them: forward = Ainv-mixed v, backward = the
            // forward result
            T bmine = T(0);
            if (act && sub < g) {
                const int r = row0 + sub;
                if (!UPPER) {
#pragma unroll
                    for (int j = 0; j < Q; ++j)
                        bmine = fma(sAinv[j * Q + rhs], __ldg(v + (size_t)r * Q + j), bmine);
                } else {
                    bmine = x[(size_t)r * Q + rhs];
                }
            }
            // the group's external nonzeros are contiguous over its g rows;
            // each of the kSub lanes takes every kSub-th one, all gathers of a
            // batch are issued before any is consumed
            T a0 = T(0), a1 = T(0), a2 = T(0);
            if (act) {
                const int kb = se[gi * g] - e0, ke = se[gi * g + g] - e0;
                const int b1 = g > 1 ? se[gi * g + 1] - e0 : ke;
                const int b2 = g > 2 ? se[gi * g + 2] - e0 : ke;
                for (int k0 = kb + sub; k0 < ke; k0 += kBatch * kSub) {
                    int cix[kBatch];
                    T cv[kBatch], xv[kBatch];
#pragma unroll
                    for (int u = 0; u < kBatch; ++u) {
                        const int k = k0 + u * kSub;
                        const bool ok = k < ke;
                        cix[u] = ok ? sc[k] : 0;
                        cv[u] = ok ? sv[k] : T(0);
                    }
#pragma unroll
                    for (int u = 0; u < kBatch; ++u) xv[u] = x[(size_t)cix[u] * Q + rhs];
#pragma unroll
                    for (int u = 0; u < kBatch; ++u) {
                        const int k = k0 + u * kSub;
                        const T pr = cv[u] * xv[u];
                        if (k < b1) a0 += pr;
                        else if (k < b2) a1 += pr;
                        else a2 += pr;
                    }
                }
            }
#pragma unroll
            for (int off = kSub / 2; off > 0; off >>= 1) {
                a0 += __shfl_xor_sync(0xffffffffu, a0, off, kSub);
                a1 += __shfl_xor_sync(0xffffffffu, a1, off, kSub);
                a2 += __shfl_xor_sync(0xffffffffu, a2, off, kSub);
            }
            T bq[kMaxG];
#pragma unroll
            for (int ri = 0; ri < kMaxG; ++ri) bq[ri] = __shfl_sync(0xffffffffu, bmine, ri, kSub);
            if (act) {
                const T acc[kMaxG] = {a0, a1, a2};
                const T* iv = si + (size_t)gi * g * g;
                T sol[kMaxG];
                for (int s2 = 0; s2 < g; ++s2) {
                    const int ri = UPPER ? g - 1 - s2 : s2;
                    T val = bq[ri] - acc[ri];
                    if (!UPPER) {
                        for (int c = 0; c < ri; ++c) val -= iv[ri * g + c] * sol[c];
                    } else {
                        for (int c = ri + 1; c < g; ++c) val -= iv[ri * g + c] * sol[c];
                        val *= sd[gi * g + ri];
                    }
                    sol[ri] = val;
                }
                if (sub == 0)
                    for (int ri = 0; ri < g; ++ri) {
                        x[(size_t)(row0 + ri) * Q + rhs] = sol[ri];
                        if (UPPER && z != x) z[(size_t)(row0 + ri) * Q + rhs] = sol[ri];
                    }
            }
        }
        __pipeline_wait_prior(1);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Cluster sweep.  One thread-block cluster of C CTAs per temporal block c
// (Q clusters run side by side).  The cluster keeps column c of the solution
// in distributed shared memory: group G (g rows) lives in CTA G % C at slot
// (G / C) * g, so every gather of a solved value is a shared-memory or
// DSMEM load instead of an L2 round trip, and levels are separated by the
// cluster barrier.  A warp solves one owned group of the level: its lanes
// split the group's external nonzeros, reduce the g partial sums with
// shuffles and lane 0 finishes the g x g internal solve.  Factor data is
// double-buffered in shared memory with asynchronous copies one level ahead.
constexpr int kCEnt = 3072;
constexpr int kCGrp = 64;

template <class T>
struct CRing {
    static constexpr size_t v_off = 0;
    static constexpr size_t i_off = v_off + sizeof(T) * kCEnt;
    static constexpr size_t d_off = i_off + sizeof(T) * 9 * kCGrp;
    static constexpr size_t c_off = d_off + sizeof(T) * 3 * kCGrp;
    static constexpr size_t e_off = c_off + sizeof(int) * kCEnt;
    static constexpr size_t r_off = e_off + sizeof(int) * (3 * kCGrp + 4);
    static constexpr size_t slot = ((r_off + sizeof(int) * kCGrp) + 127) / 128 * 128;
    static constexpr size_t rings = 2 * slot;
};

template <class T, int Q, bool UPPER>
__global__ void __launch_bounds__(1024, 1)
k_tri_cluster(TriView<T> t, const int* __restrict__ level_e, const double* __restrict__ dAinv,
              const T* __restrict__ v, T* x_io, T* z, int C, int xcap)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(128) unsigned char smem[];
    using R = CRing<T>;
    T* xs = reinterpret_cast<T*>(smem + R::rings);
    __shared__ T sAinv[Q * Q];
    const int rank = (int)cluster.block_rank();
    const int col_c = blockIdx.x / C;  // temporal block handled by this cluster
    const int tid = threadIdx.x, nth = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarps = nth >> 5;
    const int g = t.g, nl = t.nlevels;
    const int* lp = t.level_ptr;
    const int* le = level_e;
    for (int i = tid; i < Q * Q; i += nth) sAinv[i] = (T)dAinv[i];
    // owned slice of the solution: rows of groups G = rank, rank + C, ...
    const int ngroups = t.ngroups;
    if (UPPER)
        for (int i = tid; i < xcap; i += nth) {
            const int G = (i / g) * C + rank, ri = i % g;
            xs[i] = (G < ngroups) ? x_io[(size_t)(G * g + ri) * Q + col_c] : T(0);
        }
    T* xr[8];
    for (int r = 0; r < C; ++r) xr[r] = cluster.map_shared_rank(xs, r);

    auto staged = [&](int L) {
        return lp[L + 1] - lp[L] <= kCGrp && le[L + 1] - le[L] <= kCEnt;
    };
    auto prefetch = [&](int L) {
        if (L < nl && staged(L)) {
            unsigned char* slot = smem + (size_t)(L & 1) * R::slot;
            T* sv = reinterpret_cast<T*>(slot + R::v_off);
            T* si = reinterpret_cast<T*>(slot + R::i_off);
            T* sd = reinterpret_cast<T*>(slot + R::d_off);
            int* sc = reinterpret_cast<int*>(slot + R::c_off);
            int* se = reinterpret_cast<int*>(slot + R::e_off);
            int* sr = reinterpret_cast<int*>(slot + R::r_off);
            const int gb = lp[L], ng = lp[L + 1] - gb;
            const int e0 = le[L], ne = le[L + 1] - e0;
            for (int i = tid; i < ne; i += nth) {
                __pipeline_memcpy_async(sc + i, t.ext_col + e0 + i, sizeof(int));
                __pipeline_memcpy_async(sv + i, t.ext_v + e0 + i, sizeof(T));
            }
            for (int i = tid; i <= ng * g; i += nth)
                __pipeline_memcpy_async(se + i, t.ext_ptr + (size_t)gb * g + i, sizeof(int));
            for (int i = tid; i < ng; i += nth)
                __pipeline_memcpy_async(sr + i, t.group_row0 + gb + i, sizeof(int));
            for (int i = tid; i < ng * g * g; i += nth)
                __pipeline_memcpy_async(si + i, t.int_v + (size_t)gb * g * g + i, sizeof(T));
            if (UPPER)
                for (int i = tid; i < ng * g; i += nth)
                    __pipeline_memcpy_async(sd + i, t.dinv + (size_t)gb * g + i, sizeof(T));
        }
        __pipeline_commit();
    };
    auto xval = [&](int col) -> T {
        const int G = col / g;
        return xr[G % C][(G / C) * g + (col - G * g)];
    };

    prefetch(0);
    __pipeline_wait_prior(0);
    cluster.sync();
    for (int l = 0; l < nl; ++l) {
        prefetch(l + 1);
        const int gb = lp[l], ng = lp[l + 1] - gb;
        const int e0 = le[l];
        const bool st = staged(l);
        const unsigned char* slot = smem + (size_t)(l & 1) * R::slot;
        const T* sv = st ? reinterpret_cast<const T*>(slot + R::v_off) : t.ext_v + e0;
        const int* sc = st ? reinterpret_cast<const int*>(slot + R::c_off) : t.ext_col + e0;
        const int* se = st ? reinterpret_cast<const int*>(slot + R::e_off) : t.ext_ptr + (size_t)gb * g;
        const int* sr = st ? reinterpret_cast<const int*>(slot + R::r_off) : t.group_row0 + gb;
        const T* si = st ? reinterpret_cast<const T*>(slot + R::i_off) : t.int_v + (size_t)gb * g * g;
        const T* sd = st ? reinterpret_cast<const T*>(slot + R::d_off)
                         : (UPPER ? t.dinv + (size_t)gb * g : nullptr);
        for (int gl = warp; gl < ng; gl += nwarps) {  // warp-uniform
            const int row0 = sr[gl];
            const int G = row0 / g;
            if (G % C != rank) continue;
            // right-hand side values of the group's rows, loaded early
            T vv = T(0);
            if (!UPPER && lane < g * Q) vv = __ldg(v + (size_t)(row0 + lane / Q) * Q + lane % Q);
            const int kb = se[gl * g] - e0, ke = se[gl * g + g] - e0;
            const int b1 = g > 1 ? se[gl * g + 1] - e0 : ke, b2 = g > 2 ? se[gl * g + 2] - e0 : ke;
            T a0 = T(0), a1 = T(0), a2 = T(0);
            for (int k = kb + lane; k < ke; k += 32) {
                const T prod = sv[k] * xval(sc[k]);
                if (k < b1) a0 += prod;
                else if (k < b2) a1 += prod;
                else a2 += prod;
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                a0 += __shfl_xor_sync(0xffffffffu, a0, off);
                a1 += __shfl_xor_sync(0xffffffffu, a1, off);
                a2 += __shfl_xor_sync(0xffffffffu, a2, off);
            }
            T bq[kMaxG];
#pragma unroll
            for (int ri = 0; ri < kMaxG; ++ri) {
                T b = T(0);
                if (!UPPER) {
#pragma unroll
                    for (int j = 0; j < Q; ++j)
                        b = fma(sAinv[j * Q + col_c], __shfl_sync(0xffffffffu, vv, ri * Q + j), b);
                }
                bq[ri] = b;
            }
            if (lane == 0) {
                const T acc[kMaxG] = {a0, a1, a2};
                const T* iv = si + (size_t)gl * g * g;
                T* mine = xs + (G / C) * g;
                T sol[kMaxG];
                for (int s2 = 0; s2 < g; ++s2) {
                    const int ri = UPPER ? g - 1 - s2 : s2;
                    T val = (UPPER ? mine[ri] : bq[ri]) - acc[ri];
                    if (!UPPER) {
                        for (int c = 0; c < ri; ++c) val -= iv[ri * g + c] * sol[c];
                    } else {
                        for (int c = ri + 1; c < g; ++c) val -= iv[ri * g + c] * sol[c];
                        val *= sd[gl * g + ri];
                    }
                    sol[ri] = val;
                }
                for (int ri = 0; ri < g; ++ri) mine[ri] = sol[ri];
            }
        }
        __pipeline_wait_prior(0);
        cluster.sync();
    }
    // owned rows out: forward result to x_io, backward result to z
    T* out = UPPER ? z : x_io;
    for (int i = tid; i < xcap; i += nth) {
        const int G = (i / g) * C + rank, ri = i % g;
        if (G < ngroups) out[(size_t)(G * g + ri) * Q + col_c] = xs[i];
    }
}

template <class T, int Q>
int launch_tri_cluster(const DevIlu& F, const double* dAinv, const T* v, T* z, T* work,
                       cudaStream_t s, bool& launched)
{
    launched = false;
    const int g = F.L.g;
    const size_t limit = 227 * 1024 - 1024;
    int C = 0;
    for (int c = 1; c <= 8; c *= 2) {
        const size_t xcap = (size_t)((F.L.ngroups + c - 1) / c) * g;
        if (CRing<T>::rings + xcap * sizeof(T) <= limit) { C = c; break; }
    }
    if (C == 0) return XT_OK;
    const int xcap = ((F.L.ngroups + C - 1) / C) * g;
    const size_t bytes = CRing<T>::rings + (size_t)xcap * sizeof(T);
    static bool attr = false;
    if (!attr) {
        XT_CUDA(cudaFuncSetAttribute(k_tri_cluster<T, Q, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
        XT_CUDA(cudaFuncSetAttribute(k_tri_cluster<T, Q, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
        attr = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(Q * C, 1, 1);
    cfg.blockDim = dim3(1024, 1, 1);
    cfg.dynamicSmemBytes = bytes;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    XT_CUDA(cudaLaunchKernelEx(&cfg, k_tri_cluster<T, Q, false>, view<T>(F.L),
                               (const int*)F.L.level_e.p, dAinv, v, work, (T*)nullptr, C, xcap));
    XT_CUDA(cudaLaunchKernelEx(&cfg, k_tri_cluster<T, Q, true>, view<T>(F.U),
                               (const int*)F.U.level_e.p, dAinv, (const T*)nullptr, work, z, C,
                               xcap));
    note_launches(2);
    launched = true;
    return XT_OK;
}

template <class T, int Q>
int launch_tri(const DevIlu& F, const double* dAinv, const T* v, T* z, T* work,
               cudaStream_t s)
{
    if (F.L.g <= kMaxG && F.U.g <= kMaxG && F.L.level_e.p && F.U.level_e.p) {
        const size_t bytes = Ring<T>::bytes;
        static bool attr_set[2] = {false, false};
        if (!attr_set[0]) {
            XT_CUDA(cudaFuncSetAttribute(k_tri_staged<T, Q, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
            XT_CUDA(cudaFuncSetAttribute(k_tri_staged<T, Q, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
            attr_set[0] = true;
        }
        k_tri_staged<T, Q, false><<<1, 1024, bytes, s>>>(view<T>(F.L), F.L.level_e.p, dAinv, v,
                                                         work, nullptr);
        k_tri_staged<T, Q, true><<<1, 1024, bytes, s>>>(view<T>(F.U), F.U.level_e.p, dAinv,
                                                        nullptr, work, z);
        note_launches(2);
        XT_CUDA(cudaGetLastError());
        return XT_OK;
    }
    return launch_tri_simple<T, Q>(F, dAinv, v, z, work, s);
}

template <class T, int Q>
int launch_tri_simple(const DevIlu& F, const double* dAinv, const T* v, T* z, T* work,
                      cudaStream_t s)
{
    constexpr int S = (32 / Q) >= 32 ? 32 : ((32 / Q) >= 16 ? 16 : ((32 / Q) >= 8 ? 8 : ((32 / Q) >= 4 ? 4 : 2)));
    k_tri_sweep<T, Q, S, false><<<1, 1024, 0, s>>>(view<T>(F.L), dAinv, v, work, nullptr);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    k_tri_sweep<T, Q, S, true><<<1, 1024, 0, s>>>(view<T>(F.U), dAinv, nullptr, work, z);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

}  // namespace

int build_ilu(DevIlu& d, int n, const double* alu, const int* jlu, const int* ju, int group,
              cudaStream_t s)
{
    if (n <= 0 || !alu || !jlu || !ju) {
        set_error("build_ilu: bad arguments");
        return XT_ERR_ARG;
    }
    if (jlu[0] != n + 2) {
        set_error("build_ilu: jlu(1) must be n+2 (SPARSKIT MSR layout)");
        return XT_ERR_ARG;
    }
    const int nnz_end = jlu[n] - 1;
    for (int i = 0; i < n; ++i) {
        if (ju[i] < jlu[i] || ju[i] > jlu[i + 1] || jlu[i + 1] < jlu[i]) {
            set_error("build_ilu: inconsistent MSR row pointers");
            return XT_ERR_ARG;
        }
    }
    for (int k = n + 1; k < nnz_end; ++k)
        if (jlu[k] < 1 || jlu[k] > n) {
            set_error("build_ilu: MSR column index out of range");
            return XT_ERR_ARG;
        }
    int g = (group > 1 && n % group == 0 && group <= kMaxG) ? group : 1;
    d.n = n;
    TriHost L = schedule(n, alu, jlu, ju, g, false);
    TriHost U = schedule(n, alu, jlu, ju, g, true);
    XT_TRY(upload_tri(d.L, L, s));
    XT_TRY(upload_tri(d.U, U, s));
    XT_CUDA(cudaStreamSynchronize(s));
    return XT_OK;
}

template <class T>
int ilu_apply(const DevIlu& F, int q, const double* dAinv, const T* v, T* z, T* work,
              cudaStream_t s)
{
    switch (q) {
    case 1: return launch_tri<T, 1>(F, dAinv, v, z, work, s);
    case 2: return launch_tri<T, 2>(F, dAinv, v, z, work, s);
    case 3: return launch_tri<T, 3>(F, dAinv, v, z, work, s);
    case 4: return launch_tri<T, 4>(F, dAinv, v, z, work, s);
    case 5: return launch_tri<T, 5>(F, dAinv, v, z, work, s);
    case 6: return launch_tri<T, 6>(F, dAinv, v, z, work, s);
    case 7: return launch_tri<T, 7>(F, dAinv, v, z, work, s);
    case 8: return launch_tri<T, 8>(F, dAinv, v, z, work, s);
    default:
        set_error("ilu_apply: 1 <= q <= 8");
        return XT_ERR_ARG;
    }
}

template int ilu_apply<double>(const DevIlu&, int, const double*, const double*, double*,
                               double*, cudaStream_t);
template int ilu_apply<float>(const DevIlu&, int, const double*, const float*, float*, float*,
                              cudaStream_t);

}  // namespace xt
