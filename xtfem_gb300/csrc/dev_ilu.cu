// dev_ilu.cu -- the Kronecker ILUT preconditioner on the GPU.
//
// Applies z = (A^-1 (x) (LU)^-1) v, the operator of src/kronecker.f90:130-178
// (kronlusol), whose spatial part is SPARSKIT lusol (src/ilut.f:2383-2432):
// a forward sweep with the unit lower factor and a backward sweep with the
// upper factor and inverted diagonal, for each of the q temporal blocks.
//
// The factor is computed on the host (ILUT, FP64) and arrives in MSR form.
// A triangular solve is a chain of dependent rows, so it is organised by
// level sets computed once per factor:
//   * rows are grouped by node (g = 3 consecutive DOFs); a group's level is
//     one more than the deepest other group it reads, and the g rows of a
//     group are solved in sequence by the same threads, which halves the
//     level count of C3D8 stiffness factors compared with row levels;
//   * everything a level needs -- the external nonzeros (column, value), the
//     group rows, the row pointers, the g x g in-group coefficients and the
//     inverted diagonal -- is packed into one 16-byte-aligned blob per level,
//     so a level is fetched with a handful of 16-byte asynchronous copies
//     into a three-deep shared-memory ring, two levels ahead of use;
//   * one (group, temporal block) task is handled by two lanes that split
//     each row's nonzeros; all q temporal blocks of a level run at once;
//   * the q x q mixing with A^-1 is applied to v while the forward sweep
//     reads it (the mixing commutes with the spatial solve);
//   * one thread block runs all levels of a sweep with one block barrier per
//     level; values solved in earlier levels are read back through L1/L2.
// A single SM runs the sweep: the kernel is bound by the level count times
// the per-level latency (barrier, gathers) and by instruction issue, not by
// HBM bandwidth.  Independent systems (batches) fill the other SMs.
#include <cuda_pipeline.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "xt_device.h"

namespace xt {

namespace {

constexpr int kMaxG = 3;

struct TriHost {
    int ngroups = 0, nlevels = 0, g = 1, maxw = 0;
    std::vector<int> level_ptr, group_row0, ext_ptr, ext_col;
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
    return T;
}

// Per-level blob layout (all sections 16-byte aligned, offsets in bytes):
//   cols  ne ints | vals ne T | row0 ng ints | eptr ng*g+1 ints (relative
//   to the level's first nonzero) | intv ng*g*g T | dinv ng*g T (upper)
struct BlobDesc {
    int off16;  // blob start in 16-byte units
    int len16;  // blob length in 16-byte units
    int ng;     // groups in the level
    int ne;     // external nonzeros in the level
};

template <class T>
struct BlobLayout {
    size_t cols, vals, row0, eptr, intv, dinv, bytes;
    __host__ __device__ BlobLayout(int ne, int ng, int g)
    {
        cols = 0;
        vals = up16(cols + sizeof(int) * (size_t)ne);
        row0 = up16(vals + sizeof(T) * (size_t)ne);
        eptr = up16(row0 + sizeof(int) * (size_t)ng);
        intv = up16(eptr + sizeof(int) * ((size_t)ng * g + 1));
        dinv = up16(intv + sizeof(T) * (size_t)ng * g * g);
        bytes = up16(dinv + sizeof(T) * (size_t)ng * g);
    }
    __host__ __device__ static size_t up16(size_t b) { return (b + 15) / 16 * 16; }
};

template <class T>
void build_blobs(const TriHost& h, std::vector<unsigned char>& blob, std::vector<BlobDesc>& desc)
{
    const int g = h.g;
    desc.resize(h.nlevels);
    size_t total = 0;
    for (int l = 0; l < h.nlevels; ++l) {
        const int gb = h.level_ptr[l], ng = h.level_ptr[l + 1] - gb;
        const int e0 = h.ext_ptr[(size_t)gb * g], ne = h.ext_ptr[(size_t)(gb + ng) * g] - e0;
        BlobLayout<T> L(ne, ng, g);
        desc[l] = {(int)(total / 16), (int)(L.bytes / 16), ng, ne};
        total += L.bytes;
    }
    blob.assign(total, 0);
    for (int l = 0; l < h.nlevels; ++l) {
        const int gb = h.level_ptr[l], ng = desc[l].ng, ne = desc[l].ne;
        const int e0 = h.ext_ptr[(size_t)gb * g];
        BlobLayout<T> L(ne, ng, g);
        unsigned char* b = blob.data() + (size_t)desc[l].off16 * 16;
        int* cols = reinterpret_cast<int*>(b + L.cols);
        T* vals = reinterpret_cast<T*>(b + L.vals);
        int* row0 = reinterpret_cast<int*>(b + L.row0);
        int* eptr = reinterpret_cast<int*>(b + L.eptr);
        T* intv = reinterpret_cast<T*>(b + L.intv);
        T* dinv = reinterpret_cast<T*>(b + L.dinv);
        for (int k = 0; k < ne; ++k) {
            cols[k] = h.ext_col[(size_t)e0 + k];
            vals[k] = (T)h.ext_v[(size_t)e0 + k];
        }
        for (int i = 0; i < ng; ++i) row0[i] = h.group_row0[(size_t)gb + i];
        for (int i = 0; i <= ng * g; ++i) eptr[i] = h.ext_ptr[(size_t)gb * g + i] - e0;
        for (int i = 0; i < ng * g * g; ++i) intv[i] = (T)h.int_v[(size_t)gb * g * g + i];
        if (!h.dinv.empty())
            for (int i = 0; i < ng * g; ++i) dinv[i] = (T)h.dinv[(size_t)gb * g + i];
    }
}

int upload_tri(DevTri& d, const TriHost& h, cudaStream_t s)
{
    d.ngroups = h.ngroups;
    d.nlevels = h.nlevels;
    d.g = h.g;
    d.max_level_groups = h.maxw;
    XT_TRY(d.level_ptr.upload(h.level_ptr.data(), h.level_ptr.size(), s));
    XT_TRY(d.group_row0.upload(h.group_row0.data(), h.group_row0.size(), s));
    XT_TRY(d.ext_ptr.upload(h.ext_ptr.data(), h.ext_ptr.size(), s));
    const size_t ne = h.ext_col.size();
    std::vector<float> f32(h.ext_v.begin(), h.ext_v.end());
    std::vector<float> i32(h.int_v.begin(), h.int_v.end());
    std::vector<float> d32(h.dinv.begin(), h.dinv.end());
    XT_TRY(d.ext_col.upload(ne ? h.ext_col.data() : nullptr, ne ? ne : 0, s));
    XT_TRY(d.ext_v64.upload(h.ext_v.data(), ne, s));
    XT_TRY(d.ext_v32.upload(f32.data(), ne, s));
    XT_TRY(d.int_v64.upload(h.int_v.data(), h.int_v.size(), s));
    XT_TRY(d.int_v32.upload(i32.data(), i32.size(), s));
    if (!h.dinv.empty()) {
        XT_TRY(d.dinv64.upload(h.dinv.data(), h.dinv.size(), s));
        XT_TRY(d.dinv32.upload(d32.data(), d32.size(), s));
    }
    std::vector<unsigned char> b64, b32;
    std::vector<BlobDesc> e64, e32;
    build_blobs<double>(h, b64, e64);
    build_blobs<float>(h, b32, e32);
    XT_TRY(d.blob64.upload(b64.data(), b64.size(), s));
    XT_TRY(d.blob32.upload(b32.data(), b32.size(), s));
    XT_TRY(d.desc64.upload(reinterpret_cast<const int*>(e64.data()), e64.size() * 4, s));
    XT_TRY(d.desc32.upload(reinterpret_cast<const int*>(e32.data()), e32.size() * 4, s));
    XT_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
    return XT_OK;
}

template <class T>
struct TriView {
    int nlevels, g, ngroups;
    const int *level_ptr, *group_row0, *ext_ptr, *ext_col;
    const T *ext_v, *int_v, *dinv;
    const unsigned char* blob;
    const BlobDesc* desc;
};

template <class T>
TriView<T> view(const DevTri& d);
template <>
TriView<double> view<double>(const DevTri& d)
{
    return {d.nlevels, d.g, d.ngroups, d.level_ptr.p, d.group_row0.p, d.ext_ptr.p, d.ext_col.p,
            d.ext_v64.p, d.int_v64.p, d.dinv64.p, d.blob64.p,
            reinterpret_cast<const BlobDesc*>(d.desc64.p)};
}
template <>
TriView<float> view<float>(const DevTri& d)
{
    return {d.nlevels, d.g, d.ngroups, d.level_ptr.p, d.group_row0.p, d.ext_ptr.p, d.ext_col.p,
            d.ext_v32.p, d.int_v32.p, d.dinv32.p, d.blob32.p,
            reinterpret_cast<const BlobDesc*>(d.desc32.p)};
}

// ---------------------------------------------------------------------------
// Reference-shaped sweep: one warp per group, factor data read from global
// memory.  Used when the staged sweep cannot be configured.
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
                        x[(size_t)(row0 + ri) * Q + rhs] = sol[ri];
                        if (UPPER && z != x) z[(size_t)(row0 + ri) * Q + rhs] = sol[ri];
                    }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Staged sweep over per-level blobs (see the file comment).
constexpr int kRing = 3;
constexpr int kDescCap = 2048;  // levels whose descriptors are kept in shared memory

template <class T>
constexpr size_t slot_bytes() { return sizeof(T) == 8 ? 49152 : 40960; }
template <class T>
constexpr size_t staged_smem() { return kRing * slot_bytes<T>() + sizeof(BlobDesc) * kDescCap; }

// block size, lanes per group and nonzeros in flight per lane: FP32 keeps a
// whole level in one pass of 1024 threads; FP64 halves the threads to give
// each lane the registers for its double accumulators
template <class T>
struct BlobCfg {
    static constexpr int threads = sizeof(T) == 8 ? 512 : 1024;
    static constexpr int lanes = sizeof(T) == 8 ? 8 : 16;
    static constexpr int per = sizeof(T) == 8 ? 2 : 4;
};

template <class T, int Q, bool UPPER>
__global__ void __launch_bounds__(BlobCfg<T>::threads, 1)
k_tri_blob(TriView<T> t, const double* __restrict__ dAinv, const T* __restrict__ v, T* x, T* z)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ T sAinv[Q * Q];
    const int tid = threadIdx.x, nth = blockDim.x;
    const int g = t.g, nl = t.nlevels;
    constexpr size_t SLOT = slot_bytes<T>();
    BlobDesc* sdesc = reinterpret_cast<BlobDesc*>(smem + kRing * SLOT);
    const bool desc_in_smem = nl <= kDescCap;
    for (int i = tid; i < Q * Q; i += nth) sAinv[i] = (T)dAinv[i];
    if (desc_in_smem)
        for (int i = tid; i < nl; i += nth) sdesc[i] = t.desc[i];
    __syncthreads();
    const BlobDesc* desc = desc_in_smem ? sdesc : t.desc;
    const int4* gblob = reinterpret_cast<const int4*>(t.blob);

    auto prefetch = [&](int L) {
        if (L < nl) {
            const BlobDesc d = desc[L];
            if ((size_t)d.len16 * 16 <= SLOT) {
                int4* dst = reinterpret_cast<int4*>(smem + (size_t)(L % kRing) * SLOT);
                const int4* src = gblob + d.off16;
                for (int i = tid; i < d.len16; i += nth) __pipeline_memcpy_async(dst + i, src + i, 16);
            }
        }
        __pipeline_commit();
    };

    prefetch(0);
    prefetch(1);
    __pipeline_wait_prior(1);
    __syncthreads();
    // a group is handled by kLanes lanes: lane `sub` takes every kLanes-th
    // external nonzero of the group (all g rows together), gathers the Q
    // solved values of its column in one go and accumulates all g x Q
    // partial sums; shuffles reduce them, then lane r < Q finishes block r
    constexpr int kLanes = BlobCfg<T>::lanes;
    constexpr int kPer = BlobCfg<T>::per;  // nonzeros per lane in flight (one batch)
    const int sub = tid % kLanes;
    const int groups_per_pass = nth / kLanes;
    for (int l = 0; l < nl; ++l) {
        prefetch(l + 2);
        const BlobDesc d = desc[l];
        const unsigned char* base = ((size_t)d.len16 * 16 <= SLOT)
                                        ? smem + (size_t)(l % kRing) * SLOT
                                        : t.blob + (size_t)d.off16 * 16;
        const BlobLayout<T> Lo(d.ne, d.ng, g);
        const int* cols = reinterpret_cast<const int*>(base + Lo.cols);
        const T* vals = reinterpret_cast<const T*>(base + Lo.vals);
        const int* row0s = reinterpret_cast<const int*>(base + Lo.row0);
        const int* eptr = reinterpret_cast<const int*>(base + Lo.eptr);
        const T* intv = reinterpret_cast<const T*>(base + Lo.intv);
        const T* dinv = reinterpret_cast<const T*>(base + Lo.dinv);
        for (int pass = 0; pass < d.ng; pass += groups_per_pass) {
            const int gi = pass + tid / kLanes;
            const bool act = gi < d.ng;
            const int row0 = act ? row0s[gi] : 0;
            const int rhs = sub;  // temporal block finished by this lane (if < Q)
            // right-hand sides of the group's rows for block `rhs`, issued
            // before the gathers so their latency overlaps them
            T bq[kMaxG] = {T(0), T(0), T(0)};
            if (act && rhs < Q) {
#pragma unroll
                for (int ri = 0; ri < kMaxG; ++ri) {
                    if (ri < g) {
                        if (!UPPER) {
                            const T* vr = v + (size_t)(row0 + ri) * Q;
                            T b = T(0);
#pragma unroll
                            for (int j = 0; j < Q; ++j) b = fma(sAinv[j * Q + rhs], __ldg(vr + j), b);
                            bq[ri] = b;
                        } else {
                            bq[ri] = x[(size_t)(row0 + ri) * Q + rhs];
                        }
                    }
                }
            }
            T acc[kMaxG][Q];
#pragma unroll
            for (int ri = 0; ri < kMaxG; ++ri)
#pragma unroll
                for (int b = 0; b < Q; ++b) acc[ri][b] = T(0);
            if (act) {
                const int kb = eptr[gi * g], ke = eptr[gi * g + g];
                const int b1 = g > 1 ? eptr[gi * g + 1] : ke, b2 = g > 2 ? eptr[gi * g + 2] : ke;
                for (int k0 = kb + sub; k0 < ke; k0 += kPer * kLanes) {
                    int cc[kPer];
                    T cv[kPer];
#pragma unroll
                    for (int u = 0; u < kPer; ++u) {
                        const int k = k0 + u * kLanes;
                        cc[u] = k < ke ? cols[k] : -1;
                        cv[u] = k < ke ? vals[k] : T(0);
                    }
                    T xv[kPer][Q];
#pragma unroll
                    for (int u = 0; u < kPer; ++u) {
                        const T* xr = x + (size_t)(cc[u] < 0 ? 0 : cc[u]) * Q;
#pragma unroll
                        for (int b = 0; b < Q; ++b) xv[u][b] = cc[u] < 0 ? T(0) : xr[b];
                    }
#pragma unroll
                    for (int u = 0; u < kPer; ++u) {
                        const int k = k0 + u * kLanes;
                        const int ri = (k >= b1) + (k >= b2);
#pragma unroll
                        for (int b = 0; b < Q; ++b) {
                            const T pr = cv[u] * xv[u][b];
                            acc[0][b] += ri == 0 ? pr : T(0);
                            acc[1][b] += ri == 1 ? pr : T(0);
                            acc[2][b] += ri == 2 ? pr : T(0);
                        }
                    }
                }
            }
#pragma unroll
            for (int off = kLanes / 2; off > 0; off >>= 1)
#pragma unroll
                for (int ri = 0; ri < kMaxG; ++ri)
#pragma unroll
                    for (int b = 0; b < Q; ++b)
                        acc[ri][b] += __shfl_xor_sync(0xffffffffu, acc[ri][b], off, kLanes);
            if (act && rhs < Q) {
                T accr[kMaxG];
#pragma unroll
                for (int ri = 0; ri < kMaxG; ++ri) {
                    T a = acc[ri][0];
#pragma unroll
                    for (int b = 1; b < Q; ++b) a = (rhs == b) ? acc[ri][b] : a;
                    accr[ri] = a;
                }
                const T* iv = intv + (size_t)gi * g * g;
                T sol[kMaxG];
#pragma unroll
                for (int s2 = 0; s2 < kMaxG; ++s2) {
                    if (s2 < g) {
                        const int ri = UPPER ? g - 1 - s2 : s2;
                        T val = bq[ri] - accr[ri];
                        if (!UPPER) {
                            for (int c = 0; c < ri; ++c) val -= iv[ri * g + c] * sol[c];
                        } else {
                            for (int c = ri + 1; c < g; ++c) val -= iv[ri * g + c] * sol[c];
                            val *= dinv[gi * g + ri];
                        }
                        sol[ri] = val;
                    }
                }
#pragma unroll
                for (int ri = 0; ri < kMaxG; ++ri)
                    if (ri < g) {
                        x[(size_t)(row0 + ri) * Q + rhs] = sol[ri];
                        if (UPPER) z[(size_t)(row0 + ri) * Q + rhs] = sol[ri];
                    }
            }
        }
        __pipeline_wait_prior(1);
        __syncthreads();
    }
}

template <class T, int Q>
int launch_tri_simple(const DevIlu& F, const double* dAinv, const T* v, T* z, T* work,
                      cudaStream_t s)
{
    constexpr int S = (32 / Q) >= 32 ? 32 : ((32 / Q) >= 16 ? 16 : ((32 / Q) >= 8 ? 8 : ((32 / Q) >= 4 ? 4 : 2)));
    k_tri_sweep<T, Q, S, false><<<1, 1024, 0, s>>>(view<T>(F.L), dAinv, v, work, nullptr);
    k_tri_sweep<T, Q, S, true><<<1, 1024, 0, s>>>(view<T>(F.U), dAinv, nullptr, work, z);
    note_launches(2);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

template <class T, int Q>
int launch_tri(const DevIlu& F, const double* dAinv, const T* v, T* z, T* work, cudaStream_t s)
{
    const bool blob = F.L.g <= kMaxG && F.U.g <= kMaxG && (sizeof(T) == 8 ? F.L.blob64.p : F.L.blob32.p);
    if (!blob) return launch_tri_simple<T, Q>(F, dAinv, v, z, work, s);
    const size_t bytes = staged_smem<T>();
    static bool attr = false;
    if (!attr) {
        XT_CUDA(cudaFuncSetAttribute(k_tri_blob<T, Q, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        XT_CUDA(cudaFuncSetAttribute(k_tri_blob<T, Q, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        attr = true;
    }
    constexpr int nt = BlobCfg<T>::threads;
    k_tri_blob<T, Q, false><<<1, nt, bytes, s>>>(view<T>(F.L), dAinv, v, work, nullptr);
    k_tri_blob<T, Q, true><<<1, nt, bytes, s>>>(view<T>(F.U), dAinv, nullptr, work, z);
    note_launches(2);
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
    const int g = (group > 1 && n % group == 0 && group <= kMaxG) ? group : 1;
    d.n = n;
    TriHost L = schedule(n, alu, jlu, ju, g, false);
    TriHost U = schedule(n, alu, jlu, ju, g, true);
    XT_TRY(upload_tri(d.L, L, s));
    XT_TRY(upload_tri(d.U, U, s));
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
