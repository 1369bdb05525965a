// dev_ilu.cu -- the Kronecker ILUT preconditioner on the GPU.
//
// Applies z = (A^-1 (x) (LU)^-1) v, the operator of src/kronecker.f90:130-178
// (kronlusol), whose spatial part is SPARSKIT lusol (src/ilut.f:2383-2432):
// a forward sweep with the unit lower factor and a backward sweep with the
// upper factor and inverted diagonal, for each of the q temporal blocks.
//
// The factor is computed on the host (ILUT, FP64) and arrives in MSR form.
// A triangular solve is a chain of dependent rows, so it is organised by
// level sets computed once per factor.  Rows are grouped by node (g = 3
// consecutive DOFs); a group's level is one more than the deepest other
// group it reads.  The staged sweep runs a whole triangle in one thread
// block and keeps every load on a level's critical path in shared memory:
//
//   * Solution window.  A solved group is read only by groups a few levels
//     later, so its values live in a shared-memory slot from its own level
//     to the last level that reads it.  Slots are assigned on the host by
//     interval colouring of these live ranges; the factor's column indices
//     are rewritten as window offsets.  (C3D8 rod, 80,703 DOFs: at most 697
//     groups are live at once, 50 KB in FP32 for six temporal blocks.)
//   * Level stream.  Each level's factor data (window offsets, values, row
//     pointers, the inverted g x g diagonal block of every group) is one
//     16-byte-aligned blob.  A producer warp copies blob and right-hand
//     sides into a variable-size shared-memory ring with bulk asynchronous
//     copies (TMA, completion counted on an mbarrier per level), several
//     levels ahead of the compute warps; the host places every level in the
//     ring and fixes the level at whose start its copy may be issued.
//   * Compute.  S lanes share a row; each lane gathers its share of the
//     row's nonzeros for all q temporal blocks at once (the q values of a
//     window row are contiguous), the S partial sums are combined with
//     shuffles, and the g rows of a group are finished with the group's
//     inverted diagonal block, also through shuffles.  One named barrier
//     per level separates the levels.
//   * The q x q mixing with A^-1 is applied when the right-hand side is
//     permuted into forward-sweep level order (a parallel pre-pass); the
//     forward sweep writes its result in backward-sweep level order, so both
//     sweeps read their right-hand sides as contiguous per-level chunks.
//
// Waits are bounded: a wait that gives up sets a device error word (read by
// ilu_check) and the block leaves the sweep at the next level boundary.
// A factor whose window does not fit in shared memory uses a plain
// one-warp-per-group sweep that reads everything from global memory.
#include <cuda_pipeline.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>
#include <thread>
#include <vector>

#include "xt_device.h"

namespace xt {

__device__ int g_ilu_error;  // 0 = clear; 1 = ring wait gave up; 2 = producer wait gave up

namespace {

constexpr int kMaxG = 3;
constexpr int kNB = 16;          // mbarriers per direction: levels in flight < kNB
constexpr int kTabLevels = 64;  // level table entries staged in shared memory
constexpr int kHdrBytes = 2 * kNB * 8 + 16 + kTabLevels * 32;
constexpr long long kSpinLimit = 1ll << 20;
constexpr int kStageThreads = 512;  // compute warps + the producer and waiter warps, at most

struct TriHost {
    int ngroups = 0, nlevels = 0, g = 1, maxw = 0;
    std::vector<int> level_ptr, group_row0, ext_ptr, ext_col;
    std::vector<double> ext_v, int_v, dinv;
    std::vector<int> order;  // level order -> group id
    std::vector<int> pos;    // group id -> level-order position
    std::vector<int> slot;   // group id -> window slot
    int nslots = 0;
    std::vector<double> minv;  // level order, g*g: inverse of the group's diagonal block
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
    T.order.resize(ng);
    T.pos.resize(ng);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int G = 0; G < ng; ++G) {
        T.pos[G] = fill[lev[G]]++;
        T.order[T.pos[G]] = G;
    }
    T.group_row0.resize(ng);
    T.ext_ptr.assign((size_t)ng * g + 1, 0);
    T.int_v.assign((size_t)ng * g * g, 0.0);
    if (upper) T.dinv.assign((size_t)ng * g, 0.0);
    for (int i = 0; i < ng; ++i) {
        const int G = T.order[i];
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

    // Inverse of each group's diagonal block, column by column, with the
    // lusol recurrences applied to unit vectors: forward
    // x_r = e_r - sum_{c<r} l_rc x_c, backward x_r = d_r (e_r - sum_{c>r} u_rc x_c).
    T.minv.assign((size_t)ng * g * g, 0.0);
    for (int i = 0; i < ng; ++i) {
        const double* iv = &T.int_v[(size_t)i * g * g];
        double* mi = &T.minv[(size_t)i * g * g];
        for (int col = 0; col < g; ++col) {
            double x[kMaxG] = {0, 0, 0};
            for (int s2 = 0; s2 < g; ++s2) {
                const int r = upper ? g - 1 - s2 : s2;
                double v = (r == col) ? 1.0 : 0.0;
                if (!upper) {
                    for (int c = 0; c < r; ++c) v -= iv[r * g + c] * x[c];
                } else {
                    for (int c = r + 1; c < g; ++c) v -= iv[r * g + c] * x[c];
                    v *= T.dinv[(size_t)i * g + r];
                }
                x[r] = v;
            }
            for (int r = 0; r < g; ++r) mi[r * g + col] = x[r];
        }
    }

    // Window slots: group G is live from its level to the last level that
    // reads it; a slot freed after level e is reused from level e+1 on.
    std::vector<int> last(ng);
    for (int G = 0; G < ng; ++G) last[G] = lev[G];
    for (int i = 0; i < ng; ++i) {
        const int G = T.order[i];
        for (int k = T.ext_ptr[(size_t)i * g]; k < T.ext_ptr[(size_t)(i + 1) * g]; ++k) {
            const int Gc = T.ext_col[k] / g;
            last[Gc] = std::max(last[Gc], lev[G]);
        }
    }
    std::vector<std::vector<int>> release(T.nlevels + 1);
    std::vector<int> free_slots;
    T.slot.assign(ng, -1);
    for (int l = 0; l < T.nlevels; ++l) {
        for (int sl : release[l]) free_slots.push_back(sl);
        for (int i = T.level_ptr[l]; i < T.level_ptr[l + 1]; ++i) {
            const int G = T.order[i];
            int sl;
            if (!free_slots.empty()) { sl = free_slots.back(); free_slots.pop_back(); }
            else sl = T.nslots++;
            T.slot[G] = sl;
            release[last[G] + 1].push_back(sl);
        }
    }
    return T;
}

}  // namespace

// Both schedules, kept on the host to build staged sweeps on first use.
struct IluSched {
    TriHost L, U;
};

namespace {

// Per-level blob layout (sections 16-byte aligned, offsets in bytes):
//   header {ng, ne, 0, 0} | eptr ng*g+1 ints (relative to the level's first
//   nonzero) | gslot ng ints (window element offset of the group's rows) |
//   gdst ng ints (destination record or first row) | minv ng*g*g T |
//   offs ne ints (window element offset of each external column) | vals ne T
template <class T>
struct Layout {
    unsigned eptr, gslot, gdst, minv, offs, vals, bytes;
    __host__ __device__ static unsigned up16(unsigned b) { return (b + 15u) & ~15u; }
    __host__ __device__ Layout(int ng, int ne, int g)
    {
        eptr = 16;
        gslot = up16(eptr + 4u * (unsigned)(ng * g + 1));
        gdst = up16(gslot + 4u * (unsigned)ng);
        minv = up16(gdst + 4u * (unsigned)ng);
        offs = up16(minv + (unsigned)sizeof(T) * (unsigned)(ng * g * g));
        vals = up16(offs + 4u * (unsigned)ne);
        bytes = up16(vals + (unsigned)sizeof(T) * (unsigned)ne);
    }
};

// Staged-sweep data of one triangle for one (q, precision).
struct StageTri {
    bool ok = false;
    int nlevels = 0, g = 1, ring_bytes = 0, window_bytes = 0, p90 = 1;
    int ncw = 0;  // compute warps the blob was laid out for (column format), else 0
    int aux = 0;  // column format: window offset of the all-zero padding slot
    DBuf<unsigned char> blob;
    DBuf<int> table;  // per level {off16, pos16, grp0, iss, len16, rhs16, ng, ne, nb or passes}
};

int max_dyn_smem()
{
    static const int v = [] {
        int dev = 0, r = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&r, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
            r = 48 * 1024;
        return r;
    }();
    return v;
}

bool trace_on() { return std::getenv("XTFEM_TRACE") != nullptr; }

// Runs a() on a second host thread (on the caller's device) while b() runs
// on this one; returns the first failure, its message set on this thread
// (an exception in a() becomes XT_ERR_HOST; one in b() is rethrown after
// the join).
template <class A, class B>
int side_by_side(A&& a, B&& b)
{
    int dev = 0;
    XT_CUDA(cudaGetDevice(&dev));
    int ra = XT_OK;
    std::string ea;
    std::thread t([&] {
        try {
            if (cudaSetDevice(dev) != cudaSuccess) {
                ra = XT_ERR_CUDA;
                ea = "could not select the device on a helper thread";
                return;
            }
            ra = a();
            if (ra != XT_OK) ea = last_error();
        } catch (const std::exception& e) {
            ra = XT_ERR_HOST;
            ea = e.what();
        }
    });
    int rb = XT_OK;
    try {
        rb = b();
    } catch (...) {
        t.join();
        throw;
    }
    t.join();
    if (ra != XT_OK) {
        set_error(ea);
        return ra;
    }
    return rb;
}

int env_int(const char* name, int dflt)
{
    const char* e = std::getenv(name);
    return e ? std::atoi(e) : dflt;
}

// Ring size cap; XTFEM_ILU_RING_KB shrinks it (tests use a tight ring to
// make levels wait for the region of the level just before them).
long long ring_cap()
{
    const int kb = env_int("XTFEM_ILU_RING_KB", 0);
    return kb > 0 ? std::max(2, std::min(192, kb)) * 1024ll : 192 * 1024ll;
}
long long ring_min() { return env_int("XTFEM_ILU_RING_KB", 0) > 0 ? 2 * 1024 : 16 * 1024; }

// Node-block format (FP32, g = 3), per level:
//   header {ng, nb, 0, 0} | ng group records of 64 B {bstart, bcount, gslot,
//   gdst, minv[9] row-major, pad} | nb blocks of 48 B {woff, v[9] row-major
//   3 x 3 (rows of the group x DOFs of the neighbour node), pad}
// woff is the window element offset of the neighbour node's first row.  A
// block holds every factor entry between the group and one neighbour node,
// zeros where ILUT dropped the entry.
constexpr unsigned kGrec = 64, kBrec = 48;

// Window and ring sizes of a triangle; false when they do not fit.
bool stage_sizes(const TriHost& h, int Q, size_t tsize, long long& win_elems,
                 long long& window_bytes, long long& ring)
{
    win_elems = (long long)h.nslots * h.g * Q;
    window_bytes = (win_elems * (long long)tsize + 15) / 16 * 16;
    const long long budget = (long long)max_dyn_smem() - kHdrBytes - window_bytes;
    ring = std::min<long long>(budget, ring_cap()) / 16 * 16;
    if (ring < ring_min() || win_elems >= (1ll << 31)) {
        if (trace_on())
            std::fprintf(stderr, "[xtfem] staged sweep off: window %lld B, ring %lld B\n",
                         window_bytes, ring);
        return false;
    }
    return true;
}

// Ring placement.  Each level's region (blob, then right-hand sides) goes
// after the previous one, wrapping to the start when it does not fit; a
// level larger than half the ring is read from global memory (pos16 = -1).
// The issue level is the first level at whose start every earlier occupant
// of the region has been consumed, with fewer than kNB levels in flight.
// Fills tab[l*8+1] (pos16) and tab[l*8+3] (issue level) and checks the
// result.
bool place_ring(const std::vector<unsigned>& region, long long ring, std::vector<int>& tab)
{
    const int nl = (int)region.size();
    std::vector<long long> posb(nl, -1);
    long long cur = 0;
    int prev_iss = 0;
    auto overlap = [&](int a, int b) {
        return posb[a] >= 0 && posb[b] >= 0 && posb[a] < posb[b] + region[b] &&
               posb[b] < posb[a] + region[a];
    };
    for (int l = 0; l < nl; ++l) {
        int* t = &tab[(size_t)l * 8];
        int iss = std::max(prev_iss, l - kNB + 1);
        if ((long long)region[l] * 2 > ring) {
            t[1] = -1;
        } else {
            long long p = cur;
            if (p + region[l] > ring) p = 0;
            cur = p + region[l];
            posb[l] = p;
            t[1] = (int)(p / 16);
            for (int l2 = l - 1; l2 >= iss; --l2)
                if (overlap(l, l2)) { iss = l2 + 1; break; }
        }
        iss = std::min(iss, l);
        t[3] = iss;
        prev_iss = iss;
    }
    for (int l = 0; l < nl; ++l) {
        const int iss = tab[(size_t)l * 8 + 3];
        if (iss > l || l - iss >= kNB) return false;
        if (posb[l] < 0) continue;
        if (posb[l] % 16 || posb[l] + (long long)region[l] > ring) return false;
        for (int l2 = iss; l2 < l; ++l2)
            if (overlap(l, l2)) return false;
    }
    return true;
}

int finish_stage(StageTri& out, const TriHost& h, long long ring, long long window_bytes,
                 const std::vector<unsigned char>& blob, const std::vector<int>& tab,
                 cudaStream_t s)
{
    std::vector<int> wsz;
    for (int l = 0; l < h.nlevels; ++l) wsz.push_back(h.level_ptr[l + 1] - h.level_ptr[l]);
    std::sort(wsz.begin(), wsz.end());
    out.p90 = std::max(1, wsz[(size_t)(0.9 * (wsz.size() - 1))]);
    if (trace_on()) {
        int tight = 0, global = 0;
        for (int l = 0; l < h.nlevels; ++l) {
            tight += tab[(size_t)l * 8 + 3] == l;
            global += tab[(size_t)l * 8 + 1] < 0;
        }
        std::fprintf(stderr, "[xtfem] staged sweep: %d levels, ring %lld B, %d issued at their own level, %d from global\n",
                     h.nlevels, ring, tight, global);
    }
    out.nlevels = h.nlevels;
    out.g = h.g;
    out.ring_bytes = (int)ring;
    out.window_bytes = (int)window_bytes;
    XT_TRY(out.blob.upload(blob.data(), blob.size(), s));
    XT_TRY(out.table.upload(tab.data(), tab.size(), s));
    XT_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
    out.ok = true;
    return XT_OK;
}

// Row format: blob, ring placement and issue levels of one triangle; leaves
// out.ok false when the window or ring does not fit.
template <class T>
int build_row_tri(const TriHost& h, int Q, const std::vector<int>& gdst, StageTri& out,
                  cudaStream_t s)
{
    out.ok = false;
    const int g = h.g, nl = h.nlevels;
    long long win_elems, window_bytes, ring;
    if (!stage_sizes(h, Q, sizeof(T), win_elems, window_bytes, ring)) return XT_OK;
    const unsigned rs = Layout<T>::up16((unsigned)(g * Q * sizeof(T)));
    std::vector<int> tab((size_t)nl * 8, 0);
    std::vector<unsigned> region(nl);
    size_t total = 0;
    for (int l = 0; l < nl; ++l) {
        const int gb = h.level_ptr[l], ng = h.level_ptr[l + 1] - gb;
        const int ne = h.ext_ptr[(size_t)(gb + ng) * g] - h.ext_ptr[(size_t)gb * g];
        Layout<T> Lo(ng, ne, g);
        region[l] = Lo.bytes + (unsigned)ng * rs;
        int* t = &tab[(size_t)l * 8];
        t[0] = (int)(total / 16);
        t[2] = gb;
        t[4] = (int)(Lo.bytes / 16);
        t[5] = (int)((unsigned)ng * rs / 16);
        t[6] = ng;
        t[7] = ne;
        total += Lo.bytes;
    }
    bool valid = place_ring(region, ring, tab);
    std::vector<unsigned char> blob(total, 0);
    for (int l = 0; l < nl && valid; ++l) {
        const int* t = &tab[(size_t)l * 8];
        const int gb = t[2], ng = t[6], ne = t[7];
        const int e0 = h.ext_ptr[(size_t)gb * g];
        Layout<T> Lo(ng, ne, g);
        unsigned char* b = blob.data() + (size_t)t[0] * 16;
        reinterpret_cast<int*>(b)[0] = ng;
        reinterpret_cast<int*>(b)[1] = ne;
        int* eptr = reinterpret_cast<int*>(b + Lo.eptr);
        int* gslot = reinterpret_cast<int*>(b + Lo.gslot);
        int* gd = reinterpret_cast<int*>(b + Lo.gdst);
        T* minv = reinterpret_cast<T*>(b + Lo.minv);
        int* offs = reinterpret_cast<int*>(b + Lo.offs);
        T* vals = reinterpret_cast<T*>(b + Lo.vals);
        for (int i = 0; i <= ng * g; ++i) eptr[i] = h.ext_ptr[(size_t)gb * g + i] - e0;
        for (int j = 0; j < ng; ++j) {
            const int G = h.order[(size_t)gb + j];
            const long long so = (long long)h.slot[G] * g * Q;
            valid = valid && so >= 0 && so + g * Q <= win_elems;
            gslot[j] = (int)so;
            gd[j] = gdst[G];
            for (int e = 0; e < g * g; ++e)
                minv[(size_t)j * g * g + e] = (T)h.minv[((size_t)gb + j) * g * g + e];
        }
        for (int k = 0; k < ne; ++k) {
            const int c = h.ext_col[(size_t)e0 + k], Gc = c / g;
            const long long o = ((long long)h.slot[Gc] * g + (c - Gc * g)) * Q;
            valid = valid && o >= 0 && o + Q <= win_elems;
            offs[k] = (int)o;
            vals[k] = (T)h.ext_v[(size_t)e0 + k];
        }
    }
    if (!valid) {
        if (trace_on()) std::fprintf(stderr, "[xtfem] staged sweep off: schedule check failed\n");
        return XT_OK;
    }
    return finish_stage(out, h, ring, window_bytes, blob, tab, s);
}

// Node-block format (see kGrec); FP32 values, g = 3, even Q.
int build_block_tri(const TriHost& h, int Q, const std::vector<int>& gdst, StageTri& out,
                    cudaStream_t s)
{
    out.ok = false;
    if (h.g != 3 || Q % 2) return XT_OK;
    const int g = 3, nl = h.nlevels;
    long long win_elems, window_bytes, ring;
    if (!stage_sizes(h, Q, sizeof(float), win_elems, window_bytes, ring)) return XT_OK;
    const unsigned rs = Layout<float>::up16((unsigned)(g * Q * sizeof(float)));
    std::vector<int> tab((size_t)nl * 8, 0);
    std::vector<unsigned> region(nl);
    std::vector<std::vector<unsigned char>> lv(nl);
    bool valid = true;
    size_t total = 0;
    std::vector<int> bn;
    std::vector<float> bv;
    for (int l = 0; l < nl; ++l) {
        const int gb = h.level_ptr[l], ng = h.level_ptr[l + 1] - gb;
        std::vector<unsigned char> grp((size_t)ng * kGrec, 0), blk;
        int nb = 0;
        for (int j = 0; j < ng; ++j) {
            const int i = gb + j, G = h.order[i];
            bn.clear();
            bv.clear();
            for (int ri = 0; ri < g; ++ri)
                for (int k = h.ext_ptr[(size_t)i * g + ri]; k < h.ext_ptr[(size_t)i * g + ri + 1]; ++k) {
                    const int c = h.ext_col[k], Gc = c / g;
                    int bi = (int)(std::find(bn.begin(), bn.end(), Gc) - bn.begin());
                    if (bi == (int)bn.size()) {
                        bn.push_back(Gc);
                        bv.resize(bv.size() + 9, 0.0f);
                    }
                    bv[(size_t)bi * 9 + ri * 3 + (c - Gc * g)] = (float)h.ext_v[k];
                }
            int* gr = reinterpret_cast<int*>(grp.data() + (size_t)j * kGrec);
            const long long so = (long long)h.slot[G] * g * Q;
            valid = valid && so >= 0 && so + g * Q <= win_elems;
            gr[0] = nb;
            gr[1] = (int)bn.size();
            gr[2] = (int)so;
            gr[3] = gdst[G];
            float* mv = reinterpret_cast<float*>(gr + 4);
            for (int e = 0; e < 9; ++e) mv[e] = (float)h.minv[(size_t)i * 9 + e];
            for (size_t bi = 0; bi < bn.size(); ++bi) {
                unsigned char rec[kBrec] = {0};
                const long long wo = (long long)h.slot[bn[bi]] * g * Q;
                valid = valid && wo >= 0 && wo + g * Q <= win_elems;
                const int woff = (int)wo;
                std::memcpy(rec, &woff, 4);
                std::memcpy(rec + 4, &bv[bi * 9], 36);
                blk.insert(blk.end(), rec, rec + kBrec);
            }
            nb += (int)bn.size();
        }
        std::vector<unsigned char>& b = lv[l];
        b.assign(16, 0);
        reinterpret_cast<int*>(b.data())[0] = ng;
        reinterpret_cast<int*>(b.data())[1] = nb;
        b.insert(b.end(), grp.begin(), grp.end());
        b.insert(b.end(), blk.begin(), blk.end());
        region[l] = (unsigned)b.size() + (unsigned)ng * rs;
        int* t = &tab[(size_t)l * 8];
        t[0] = (int)(total / 16);
        t[2] = gb;
        t[4] = (int)(b.size() / 16);
        t[5] = (int)((unsigned)ng * rs / 16);
        t[6] = ng;
        t[7] = nb;
        total += b.size();
    }
    valid = valid && place_ring(region, ring, tab);
    if (!valid) {
        if (trace_on()) std::fprintf(stderr, "[xtfem] block sweep off: schedule check failed\n");
        return XT_OK;
    }
    std::vector<unsigned char> blob;
    blob.reserve(total);
    for (auto& b : lv) blob.insert(blob.end(), b.begin(), b.end());
    return finish_stage(out, h, ring, window_bytes, blob, tab, s);
}

// Column-record format (FP32, g = 3, even Q; one temporal-block pair per
// thread block, so the window holds 3 rows x 2 values per slot).  A lane
// owns (group, column c of the 3 x 3 blocks, share h of the group's
// blocks); at every step it reads one 16-byte record {window offset of the
// neighbour's row c, column c of the block} and one window pair, and adds
// one two-wide FMA per row of the group.  The records of a chunk (GPW
// groups, one warp) are stored step by step, 32 lanes side by side, so a
// warp's record load is one contiguous 512-byte read with no bank
// conflicts; lanes past a group's last block read a zero record pointing at
// an all-zero window slot.  Groups of a level are sorted by block count so
// that the groups sharing a chunk need about the same number of steps.
// Per level:
//   header {ng, passes, chunks, 0} | passes x ncw chunk entries {rec16, steps}
//   (padded to 16 B) | ng group records of 48 B {gslot, gdst, rhs index,
//   minv[9] row-major} in chunk order | the chunks' records.
constexpr unsigned kCgrec = 48;

int col_warps(const TriHost& h, int GPW)
{
    std::vector<int> wsz;
    for (int l = 0; l < h.nlevels; ++l) wsz.push_back(h.level_ptr[l + 1] - h.level_ptr[l]);
    std::sort(wsz.begin(), wsz.end());
    const int p90 = std::max(1, wsz[(size_t)(0.9 * (wsz.size() - 1))]);
    const int w = env_int("XTFEM_ILU_WARPS", (p90 + GPW - 1) / GPW);
    return std::max(1, std::min(kStageThreads / 32 - 2, w));
}

int build_col_tri(const TriHost& h, int Q, int H, const std::vector<int>& gdst, StageTri& out,
                  cudaStream_t s, int vps = 2)
{
    out.ok = false;
    if (h.g != 3 || (vps != 1 && vps != 2) || Q % vps || (H != 1 && H != 2)) return XT_OK;
    const int g = 3, nl = h.nlevels, GS = 3 * H, GPW = 32 / GS;
    const int ncw = col_warps(h, GPW);
    const int sw = 3 * vps;  // window values per slot: 3 rows x vps temporal blocks
    const long long win_elems = ((long long)h.nslots + 1) * sw;
    const long long window_bytes = (win_elems * 4 + 15) / 16 * 16;
    const long long ring =
        std::min<long long>((long long)max_dyn_smem() - kHdrBytes - window_bytes, ring_cap()) / 16 * 16;
    if (ring < ring_min() || win_elems >= (1ll << 31)) return XT_OK;
    const int dummy = h.nslots * sw;
    const unsigned rs = Layout<float>::up16((unsigned)(g * Q * sizeof(float)));
    std::vector<int> tab((size_t)nl * 8, 0);
    std::vector<unsigned> region(nl);
    std::vector<std::vector<unsigned char>> lv(nl);
    bool valid = true;
    size_t total = 0;
    std::vector<std::vector<int>> bn;     // per group: neighbour groups of its blocks
    std::vector<std::vector<float>> bv;   // per group: 9 values per block, row-major
    for (int l = 0; l < nl && valid; ++l) {
        const int gb = h.level_ptr[l], ng = h.level_ptr[l + 1] - gb;
        bn.assign(ng, {});
        bv.assign(ng, {});
        for (int j = 0; j < ng; ++j) {
            const int i = gb + j;
            for (int ri = 0; ri < g; ++ri)
                for (int k = h.ext_ptr[(size_t)i * g + ri]; k < h.ext_ptr[(size_t)i * g + ri + 1]; ++k) {
                    const int c = h.ext_col[k], Gc = c / g;
                    int bi = (int)(std::find(bn[j].begin(), bn[j].end(), Gc) - bn[j].begin());
                    if (bi == (int)bn[j].size()) {
                        bn[j].push_back(Gc);
                        bv[j].resize(bv[j].size() + 9, 0.0f);
                    }
                    bv[j][(size_t)bi * 9 + ri * 3 + (c - Gc * g)] = (float)h.ext_v[k];
                }
        }
        std::vector<int> ord(ng);
        for (int j = 0; j < ng; ++j) ord[j] = j;
        std::stable_sort(ord.begin(), ord.end(),
                         [&](int a, int b) { return bn[a].size() > bn[b].size(); });
        const int nchunk = (ng + GPW - 1) / GPW, npass = (nchunk + ncw - 1) / ncw;
        const size_t ctab = ((size_t)npass * ncw * 8 + 15) / 16 * 16;
        std::vector<unsigned char>& b = lv[l];
        b.assign(16 + ctab + (size_t)ng * kCgrec, 0);
        int* hd = reinterpret_cast<int*>(b.data());
        hd[0] = ng;
        hd[1] = npass;
        hd[2] = nchunk;
        for (int jj = 0; jj < ng; ++jj) {
            const int j = ord[jj], i = gb + j, G = h.order[i];
            int* gr = reinterpret_cast<int*>(b.data() + 16 + ctab + (size_t)jj * kCgrec);
            const long long so = (long long)h.slot[G] * sw;
            valid = valid && so >= 0 && so + sw <= dummy;
            gr[0] = (int)so;
            gr[1] = gdst[G];
            gr[2] = j;
            float* mv = reinterpret_cast<float*>(gr + 3);
            for (int e = 0; e < 9; ++e) mv[e] = (float)h.minv[(size_t)i * 9 + e];
        }
        for (int c = 0; c < nchunk; ++c) {
            int steps = 0;
            for (int jj = c * GPW; jj < std::min(ng, (c + 1) * GPW); ++jj)
                steps = std::max(steps, (int)((bn[ord[jj]].size() + H - 1) / H));
            int* ce = reinterpret_cast<int*>(b.data() + 16 + (size_t)c * 8);
            ce[0] = (int)(b.size() / 16);
            ce[1] = steps;
            for (int st = 0; st < steps; ++st)
                for (int lane = 0; lane < 32; ++lane) {
                    const int gw = lane / GS, inl = lane - gw * GS, col = inl / H, hh = inl - col * H;
                    const int jj = c * GPW + gw, bi = hh + H * st;
                    int off = dummy;
                    float v[3] = {0.0f, 0.0f, 0.0f};
                    if (gw < GPW && jj < ng && bi < (int)bn[ord[jj]].size()) {
                        const int j = ord[jj];
                        const long long wo = (long long)h.slot[bn[j][bi]] * sw + vps * col;
                        valid = valid && wo >= 0 && wo + vps <= dummy;
                        off = (int)wo;
                        for (int r = 0; r < 3; ++r) v[r] = bv[j][(size_t)bi * 9 + r * 3 + col];
                    }
                    unsigned char rec[16];
                    std::memcpy(rec, &off, 4);
                    std::memcpy(rec + 4, v, 12);
                    b.insert(b.end(), rec, rec + 16);
                }
        }
        region[l] = (unsigned)b.size() + (unsigned)ng * rs;
        int* t = &tab[(size_t)l * 8];
        t[0] = (int)(total / 16);
        t[2] = gb;
        t[4] = (int)(b.size() / 16);
        t[5] = (int)((unsigned)ng * rs / 16);
        t[6] = ng;
        t[7] = npass;
        total += b.size();
        valid = valid && total / 16 < (size_t)INT32_MAX;
    }
    valid = valid && place_ring(region, ring, tab);
    if (!valid) {
        if (trace_on()) std::fprintf(stderr, "[xtfem] column sweep off: schedule check failed\n");
        return XT_OK;
    }
    std::vector<unsigned char> blob;
    blob.reserve(total);
    for (auto& b : lv) blob.insert(blob.end(), b.begin(), b.end());
    XT_TRY(finish_stage(out, h, ring, window_bytes, blob, tab, s));
    out.ncw = ncw;
    out.aux = dummy;
    return XT_OK;
}

}  // namespace

struct RegTri;
struct IluStage {
    int q = 0;
    unsigned rs = 0;  // right-hand-side record stride in bytes
    StageTri L, U;
    DBuf<unsigned char> rhsL, rhsU;  // ngroups records each, level order
    // register-prefetched row sweep (fmt 4): both triangles, the pre-pass
    // map and the per-temporal-block right-hand-side arrays
    std::shared_ptr<RegTri> regL, regU;
    DBuf<int> srcL;
    DBuf<float> rrhsL, rrhsU;
    bool reg_ok = false;
    // the same per row block of a block-Jacobi factor: one thread block per
    // (block, temporal block), each block's sweep arguments in a device table
    int parts = 0, ncw = 0, win_elems = 0;
    long long lanesL = 0, lanesU = 0;
    std::vector<std::shared_ptr<RegTri>> regLp, regUp;
    DBuf<unsigned char> argsL, argsU;  // RegArgs per block
};

namespace {

// ---------------------------------------------------------------------------
// Reference-shaped sweep: one warp per group, factor data read from global
// memory.  Used when the staged sweep cannot be configured.
template <class T>
struct TriView {
    int nlevels, g, ngroups;
    const int *level_ptr, *group_row0, *ext_ptr, *ext_col;
    const T *ext_v, *int_v, *dinv;
};

TriView<double> view64(const DevTri& d)
{
    return {d.nlevels, d.g, d.ngroups, d.level_ptr.p, d.group_row0.p, d.ext_ptr.p, d.ext_col.p,
            d.ext_v64.p, d.int_v64.p, d.dinv64.p};
}
TriView<float> view32(const DevTri& d)
{
    return {d.nlevels, d.g, d.ngroups, d.level_ptr.p, d.group_row0.p, d.ext_ptr.p, d.ext_col.p,
            d.ext_v32.p, d.int_v32.p, d.dinv32.p};
}
template <class T>
TriView<T> view(const DevTri& d);
template <>
TriView<double> view<double>(const DevTri& d) { return view64(d); }
template <>
TriView<float> view<float>(const DevTri& d) { return view32(d); }

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
// Staged sweep.
__device__ __forceinline__ unsigned smem_addr(const void* p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* b)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(b)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(unsigned long long* b, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase of the given parity to complete.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned parity,
                                          long long limit = kSpinLimit)
{
    for (long long i = 0; i < limit; ++i)
        if (mbar_try_wait(b, parity)) return true;
    return false;
}
// Bulk asynchronous copy global -> shared, completion counted on bar.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void named_barrier(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <class T>
struct Pair;
template <>
struct Pair<float> { using type = float2; };
template <>
struct Pair<double> { using type = double2; };

// Q consecutive values from p (pairs when Q is even: p is then 2*sizeof(T)
// aligned, as every row offset is a multiple of Q in an aligned buffer).
template <class T, int Q>
__device__ __forceinline__ void load_row(const T* p, T (&r)[Q])
{
    if constexpr (Q % 2 == 0) {
        using P = typename Pair<T>::type;
#pragma unroll
        for (int i = 0; i < Q / 2; ++i) {
            const P v = reinterpret_cast<const P*>(p)[i];
            r[2 * i] = v.x;
            r[2 * i + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < Q; ++i) r[i] = p[i];
    }
}
// Store the values of r owned by lane `sub` of S (pairs when Q is even).
template <class T, int Q, int S>
__device__ __forceinline__ void store_row(T* p, const T (&r)[Q], int sub)
{
    if constexpr (Q % 2 == 0) {
        using P = typename Pair<T>::type;
#pragma unroll
        for (int i = 0; i < Q / 2; ++i)
            if (i % S == sub) reinterpret_cast<P*>(p)[i] = P{r[2 * i], r[2 * i + 1]};
    } else {
#pragma unroll
        for (int i = 0; i < Q; ++i)
            if (i % S == sub) p[i] = r[i];
    }
}

// Forward-sweep right-hand sides in level order: record i (stride rsE
// elements) holds the g rows of group i, each the q values
// sum_j Ainv(q, j) v(row, j).
template <class T, int Q>
__global__ void k_rhs_perm(const int* __restrict__ row0, int ng, int g,
                           const double* __restrict__ dAinv, const T* __restrict__ v,
                           T* __restrict__ rec, unsigned rsE)
{
    __shared__ T sA[Q * Q];
    for (int i = threadIdx.x; i < Q * Q; i += blockDim.x) sA[i] = (T)dAinv[i];
    __syncthreads();
    const long long total = (long long)ng * g * Q;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int gq = g * Q;
        const int i = (int)(t / gq), e = (int)(t - (long long)i * gq);
        const int r = e / Q, q = e - r * Q;
        const T* vr = v + (size_t)(row0[i] + r) * Q;
        T b = T(0);
#pragma unroll
        for (int j = 0; j < Q; ++j) b = fma(sA[j * Q + q], vr[j], b);
        rec[(size_t)i * rsE + e] = b;
    }
}

template <class T>
struct StageArgs {
    const unsigned char* blob;
    const int4* table;
    const unsigned char* rhs;  // level-ordered right-hand-side records
    T* out;                    // forward: backward-order records; backward: z
    int nl, g, ncw, window_bytes;
    unsigned rs;               // record stride in bytes
    int aux;                   // column format: offset of the all-zero window slot
    long long spin;            // polls before a wait for a level gives up (the
                               // drain of copies in flight always polls kSpinLimit)
};

// Producer: one thread copies every level's blob and right-hand-side chunk
// into its ring region once the levels that used that region are consumed.
template <class T>
__device__ void stage_producer(const StageArgs<T>& a, unsigned long long* full,
                               unsigned long long* cons, unsigned char* ring)
{
    for (int L = 0; L < a.nl; ++L) {
        const int4 t0 = a.table[2 * L], t1 = a.table[2 * L + 1];
        const int iss = t0.w;
        if (iss > 0) {
            const int c = iss - 1;
            if (!mbar_wait(cons + c % kNB, (unsigned)(c / kNB) & 1u, a.spin)) {
                atomicExch(&g_ilu_error, 2);
                // let the copies already issued land before the block exits
                for (int L2 = max(0, L - kNB); L2 < L; ++L2)
                    (void)mbar_wait(full + L2 % kNB, (unsigned)(L2 / kNB) & 1u);
                return;
            }
        }
        unsigned long long* fb = full + L % kNB;
        if (t0.y >= 0) {
            const unsigned blen = (unsigned)t1.x * 16u, rlen = (unsigned)t1.y * 16u;
            mbar_arrive_tx(fb, blen + rlen);
            unsigned char* dst = ring + (size_t)t0.y * 16;
            bulk_g2s(dst, a.blob + (size_t)t0.x * 16, blen, fb);
            if (rlen) bulk_g2s(dst + blen, a.rhs + (size_t)t0.z * a.rs, rlen, fb);
        } else {
            mbar_arrive(fb);
        }
    }
}

// Block skeleton shared by both formats: barrier set-up, the producer and
// waiter warps (the last two) and the compute warps' level loop.  Body::level<RING>
// computes one level from the ring (RING: shared-memory addresses) or from
// global memory (levels too large for the ring).
template <class T, class Body>
__device__ __forceinline__ void stage_main(const StageArgs<T>& a, Body& body, unsigned char* smem)
{
    unsigned long long* full = reinterpret_cast<unsigned long long*>(smem);
    unsigned long long* cons = full + kNB;
    volatile int* s_abort = reinterpret_cast<volatile int*>(cons + kNB);
    T* win = reinterpret_cast<T*>(smem + kHdrBytes);
    unsigned char* ring = smem + kHdrBytes + a.window_bytes;
    // the level table: a ring of kTabLevels levels in shared memory, so no
    // global load latency sits on a compute warp's level loop
    int4* tabs = reinterpret_cast<int4*>(smem + 2 * kNB * 8 + 16);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int i = 0; i < kNB; ++i) {
            mbar_init(full + i, 1);
            mbar_init(cons + i, a.ncw);  // one arrival per compute warp
        }
        *s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = tid; i < 2 * min(kTabLevels, a.nl); i += blockDim.x) tabs[i] = a.table[i];
    __syncthreads();
    if (warp == a.ncw) {
        if (lane == 0) stage_producer(a, full, cons, ring);
        return;
    }
    // A waiter warp (after the producer) waits for each level's copies and
    // then joins the level barrier that lets the compute warps start that
    // level, so the mbarrier wait overlaps the previous level's work.  The
    // barrier orders the completed copies before the compute warps' reads.
    const int nbar = (a.ncw + 1) * 32;
    if (warp == a.ncw + 1) {
        for (int l = 0; l < a.nl; ++l) {
            int ok = 1;
            if (lane == 0) ok = mbar_wait(full + l % kNB, (unsigned)(l / kNB) & 1u, a.spin) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok && lane == 0) {
                *s_abort = 1;
                atomicExch(&g_ilu_error, 1);
            }
            named_barrier(1, nbar);  // the compute warps start level l after it
            if (*s_abort) return;
            // levels l-32 .. l-1 are done: their table slots take levels
            // l+32 .. l+63, read from level l+31 on
            if (l % (kTabLevels / 2) == 0 && l > 0)
                for (int i = lane; i < kTabLevels; i += 32) {
                    const int e = 2 * (l + kTabLevels / 2) + i;
                    if (e < 2 * a.nl) tabs[e % (2 * kTabLevels)] = a.table[e];
                }
        }
        return;
    }
    named_barrier(1, nbar);
    int4 c0 = tabs[0], c1 = tabs[1];
    for (int l = 0; l < a.nl && !*s_abort; ++l) {
        const int ln = min(l + 1, a.nl - 1) % kTabLevels;
        const int4 n0 = tabs[2 * ln], n1 = tabs[2 * ln + 1];  // used next level
        if (c0.y >= 0) {
            const unsigned char* base = ring + (size_t)c0.y * 16;
            body.template level<true>(win, base, reinterpret_cast<const T*>(base + (size_t)c1.x * 16),
                                      c1.z, c1.w);
        } else {
            body.template level<false>(win, a.blob + (size_t)c0.x * 16,
                                       reinterpret_cast<const T*>(a.rhs + (size_t)c0.z * a.rs), c1.z,
                                       c1.w);
        }
        // this warp is done with the level's ring region; the region is
        // released by the last warp's arrival, before the level barrier
        // (the next level's copy may need exactly this region)
        __syncwarp();
        if (lane == 0) mbar_arrive(cons + l % kNB);
        if (l + 1 < a.nl) named_barrier(1, nbar);
        c0 = n0;
        c1 = n1;
    }
}

// Row format: S lanes per row, each lane all Q temporal blocks of its share
// of the row's nonzeros; g rows of a group in consecutive lane sets.
template <class T, int Q, int S, bool UPPER>
struct RowBody {
    int g, GS, GPW, gw, ri, sub, lane0, warp, ncw;
    bool lane_ok;
    unsigned rsE;
    T* out;
    __device__ RowBody(const StageArgs<T>& a)
    {
        const int lane = threadIdx.x & 31;
        warp = threadIdx.x >> 5;
        ncw = a.ncw;
        g = a.g;
        GS = g * S;
        GPW = 32 / GS;
        gw = lane / GS;
        const int inl = lane - gw * GS;
        ri = inl / S;
        sub = inl - ri * S;
        lane0 = gw * GS;
        lane_ok = gw < GPW;
        rsE = a.rs / (unsigned)sizeof(T);
        out = a.out;
    }
    template <bool RING>
    __device__ __forceinline__ void level(T* win, const unsigned char* base, const T* rh, int ng,
                                          int ne)
    {
        const Layout<T> Lo(ng, ne, g);
        const int* ep = reinterpret_cast<const int*>(base + Lo.eptr);
        const int* gsl = reinterpret_cast<const int*>(base + Lo.gslot);
        const int* gds = reinterpret_cast<const int*>(base + Lo.gdst);
        const T* mv = reinterpret_cast<const T*>(base + Lo.minv);
        const int* of = reinterpret_cast<const int*>(base + Lo.offs);
        const T* va = reinterpret_cast<const T*>(base + Lo.vals);
        for (int j0 = warp * GPW; j0 < ng; j0 += ncw * GPW) {
            const int j = j0 + gw;
            const bool act = lane_ok && j < ng;
            T acc[Q], b[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) acc[q] = b[q] = T(0);
            if (act) {
                const int kb = ep[j * g + ri], ke = ep[j * g + ri + 1];
                load_row<T, Q>(rh + (size_t)j * rsE + ri * Q, b);
#pragma unroll 2
                for (int k = kb + sub; k < ke; k += S) {
                    const T w = va[k];
                    T xr[Q];
                    load_row<T, Q>(win + of[k], xr);
#pragma unroll
                    for (int q = 0; q < Q; ++q) acc[q] = fma(w, xr[q], acc[q]);
                }
            }
#pragma unroll
            for (int m = 1; m < S; m <<= 1)
#pragma unroll
                for (int q = 0; q < Q; ++q) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], m);
            T d[Q], sol[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                d[q] = b[q] - acc[q];
                sol[q] = T(0);
            }
#pragma unroll
            for (int c = 0; c < kMaxG; ++c) {
                if (c < g) {
                    const T m = act ? mv[(size_t)j * g * g + ri * g + c] : T(0);
#pragma unroll
                    for (int q = 0; q < Q; ++q)
                        sol[q] = fma(m, __shfl_sync(0xffffffffu, d[q], lane0 + c * S), sol[q]);
                }
            }
            if (act) {
                store_row<T, Q, S>(win + gsl[j] + ri * Q, sol, sub);
                const int dst = gds[j];
                T* go = UPPER ? out + (size_t)(dst + ri) * Q : out + (size_t)dst * rsE + ri * Q;
                store_row<T, Q, S>(go, sol, sub);
            }
        }
    }
};

// Node-block format (FP32, g = 3, even Q): one lane per (group, pair of
// temporal blocks, share h of the group's blocks); the H shares are summed
// with shuffles and each lane finishes its pair for all three rows.  The
// temporal blocks are independent in a triangular solve, so the Q/2 pairs
// may be dealt to Q/(2 NPC) thread blocks on as many SMs, NPC pairs each:
// every block streams the whole factor but gathers and updates only its
// own pairs' window entries.
template <int Q, int H, bool UPPER, int NPC = Q / 2>
struct BlockBody {
    static_assert((Q / 2) % NPC == 0, "pairs must divide evenly among the blocks");
    static constexpr int NP = NPC, GS = NP * H, GPW = 32 / GS;
    int gw, p, h, lane0, warp, ncw;
    bool lane_ok;
    unsigned rsE;
    float* out;
    __device__ BlockBody(const StageArgs<float>& a)
    {
        const int lane = threadIdx.x & 31;
        warp = threadIdx.x >> 5;
        ncw = a.ncw;
        gw = lane / GS;
        const int inl = lane - gw * GS;
        h = inl / NP;
        p = inl - h * NP + (int)blockIdx.x * NPC;
        lane0 = gw * GS;
        lane_ok = gw < GPW;
        rsE = a.rs / (unsigned)sizeof(float);
        out = a.out;
    }
    template <bool RING>
    __device__ __forceinline__ void level(float* win, const unsigned char* base, const float* rh,
                                          int ng, int nb)
    {
        (void)nb;
        const unsigned char* grec = base + 16;
        const unsigned char* brec = grec + (size_t)kGrec * ng;
        for (int j0 = warp * GPW; j0 < ng; j0 += ncw * GPW) {
            const int j = j0 + gw;
            const bool act = lane_ok && j < ng;
            // each lane's two temporal blocks are one packed FP32 pair: one
            // two-wide FMA (two independently rounded FMAs) per matrix entry
            float2 acc[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) acc[r] = make_float2(0.0f, 0.0f);
            int4 gh = make_int4(0, 0, 0, 0);
            if (act) {
                gh = *reinterpret_cast<const int4*>(grec + (size_t)j * kGrec);
                const unsigned char* bp = brec + (size_t)gh.x * kBrec;
#pragma unroll 2
                for (int bi = h; bi < gh.y; bi += H) {
                    const unsigned char* rec = bp + (size_t)bi * kBrec;
                    const float4 r0 = *reinterpret_cast<const float4*>(rec);
                    const float4 r1 = *reinterpret_cast<const float4*>(rec + 16);
                    const float2 r2 = *reinterpret_cast<const float2*>(rec + 32);
                    const float* xp = win + __float_as_int(r0.x) + 2 * p;
                    const float2 x0 = *reinterpret_cast<const float2*>(xp);
                    const float2 x1 = *reinterpret_cast<const float2*>(xp + Q);
                    const float2 x2 = *reinterpret_cast<const float2*>(xp + 2 * Q);
                    const float v[9] = {r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y};
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        acc[r] = __ffma2_rn(make_float2(v[r * 3 + 0], v[r * 3 + 0]), x0, acc[r]);
                        acc[r] = __ffma2_rn(make_float2(v[r * 3 + 1], v[r * 3 + 1]), x1, acc[r]);
                        acc[r] = __ffma2_rn(make_float2(v[r * 3 + 2], v[r * 3 + 2]), x2, acc[r]);
                    }
                }
            }
#pragma unroll
            for (int m = 1; m < H; m <<= 1) {
                const int src = lane0 + (h ^ m) * NP + (p - (int)blockIdx.x * NPC);
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    acc[r].x += __shfl_sync(0xffffffffu, acc[r].x, src);
                    acc[r].y += __shfl_sync(0xffffffffu, acc[r].y, src);
                }
            }
            if (act) {
                const float* rr = rh + (size_t)j * rsE + 2 * p;
                float2 d[3];
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const float2 bb = *reinterpret_cast<const float2*>(rr + r * Q);
                    d[r] = make_float2(bb.x - acc[r].x, bb.y - acc[r].y);
                }
                const unsigned char* gm = grec + (size_t)j * kGrec + 16;
                const float4 m0 = *reinterpret_cast<const float4*>(gm);
                const float4 m1 = *reinterpret_cast<const float4*>(gm + 16);
                const float m8 = *reinterpret_cast<const float*>(gm + 32);
                const float mv[9] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w, m8};
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    if (r % H != h) continue;  // row r is stored by share r mod H
                    float2 sv = make_float2(0.0f, 0.0f);
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        sv = __ffma2_rn(make_float2(mv[r * 3 + c], mv[r * 3 + c]), d[c], sv);
                    *reinterpret_cast<float2*>(win + gh.z + r * Q + 2 * p) = sv;
                    float* go = UPPER ? out + (size_t)(gh.w + r) * Q + 2 * p
                                      : out + (size_t)gh.w * rsE + r * Q + 2 * p;
                    *reinterpret_cast<float2*>(go) = sv;
                }
            }
        }
    }
};

template <class T, int Q, int S, bool UPPER>
__global__ void __launch_bounds__(kStageThreads, 1) k_tri_stage(StageArgs<T> a)
{
    extern __shared__ __align__(128) unsigned char smem[];
    RowBody<T, Q, S, UPPER> body(a);
    stage_main<T>(a, body, smem);
}

template <int Q, int H, bool UPPER, int NPC>
__global__ void __launch_bounds__(kStageThreads, 1) k_tri_block(StageArgs<float> a)
{
    extern __shared__ __align__(128) unsigned char smem[];
    BlockBody<Q, H, UPPER, NPC> body(a);
    stage_main<float>(a, body, smem);
}

// Column-record format (see build_col_tri): thread block blockIdx.x solves
// temporal-block pair blockIdx.x; lane = (group, column c, share h).  The
// H shares are summed with shuffles, then the three columns; the lane of
// column c (share 0) finishes row c of its group.
template <int Q, int H, bool UPPER>
struct ColBody {
    static constexpr int GS = 3 * H, GPW = 32 / GS;
    int lane, gw, col, hh, lane0, warp, ncw, pr;
    bool lane_ok;
    unsigned rsE;
    float* out;
    __device__ ColBody(const StageArgs<float>& a)
    {
        lane = threadIdx.x & 31;
        warp = threadIdx.x >> 5;
        ncw = a.ncw;
        gw = lane / GS;
        const int inl = lane - gw * GS;
        col = inl / H;
        hh = inl - col * H;
        lane0 = gw * GS;
        lane_ok = gw < GPW;
        pr = blockIdx.x;
        rsE = a.rs / (unsigned)sizeof(float);
        out = a.out;
    }
    template <bool RING>
    __device__ __forceinline__ void level(float* win, const unsigned char* base, const float* rh,
                                          int ng, int npass)
    {
        const int nchunk = reinterpret_cast<const int*>(base)[2];
        const int2* chunks = reinterpret_cast<const int2*>(base + 16);
        const unsigned char* grec = base + 16 + (((size_t)npass * ncw * 8 + 15) & ~(size_t)15);
        for (int k = 0; k < npass; ++k) {
            const int c = k * ncw + warp;
            if (c >= nchunk) break;  // warp-uniform
            const int2 cd = chunks[c];
            const float4* rp = reinterpret_cast<const float4*>(base + (size_t)cd.x * 16) + lane;
            // the finishing lane's group record and right-hand side, loaded
            // before the gathers so their latency overlaps them
            const int jj = c * GPW + gw;
            const bool fin = lane_ok && hh == 0 && jj < ng;
            int gslot = 0, gdst = 0;
            float mv[3] = {0.0f, 0.0f, 0.0f};
            float2 bb[3] = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f)};
            if (fin) {
                const int* gr = reinterpret_cast<const int*>(grec + (size_t)jj * kCgrec);
                gslot = gr[0];
                gdst = gr[1];
                const float* m = reinterpret_cast<const float*>(gr + 3) + col * 3;
                const float* rr = rh + (size_t)gr[2] * rsE + 2 * pr;
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    mv[r] = m[r];
                    bb[r] = *reinterpret_cast<const float2*>(rr + r * Q);
                }
            }
            float2 acc[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) acc[r] = make_float2(0.0f, 0.0f);
#pragma unroll 4
            for (int st = 0; st < cd.y; ++st) {
                const float4 rec = rp[(size_t)st * 32];
                const float2 x = *reinterpret_cast<const float2*>(win + __float_as_int(rec.x));
                acc[0] = __ffma2_rn(make_float2(rec.y, rec.y), x, acc[0]);
                acc[1] = __ffma2_rn(make_float2(rec.z, rec.z), x, acc[1]);
                acc[2] = __ffma2_rn(make_float2(rec.w, rec.w), x, acc[2]);
            }
#pragma unroll
            for (int m = 1; m < H; m <<= 1)
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    acc[r].x += __shfl_xor_sync(0xffffffffu, acc[r].x, m);
                    acc[r].y += __shfl_xor_sync(0xffffffffu, acc[r].y, m);
                }
            float2 tot[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const float2 t0 = make_float2(__shfl_sync(0xffffffffu, acc[r].x, lane0),
                                              __shfl_sync(0xffffffffu, acc[r].y, lane0));
                const float2 t1 = make_float2(__shfl_sync(0xffffffffu, acc[r].x, lane0 + H),
                                              __shfl_sync(0xffffffffu, acc[r].y, lane0 + H));
                const float2 t2 = make_float2(__shfl_sync(0xffffffffu, acc[r].x, lane0 + 2 * H),
                                              __shfl_sync(0xffffffffu, acc[r].y, lane0 + 2 * H));
                tot[r] = make_float2((t0.x + t1.x) + t2.x, (t0.y + t1.y) + t2.y);
            }
            if (fin) {
                float2 sol = make_float2(0.0f, 0.0f);
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const float2 d = make_float2(bb[r].x - tot[r].x, bb[r].y - tot[r].y);
                    sol = __ffma2_rn(make_float2(mv[r], mv[r]), d, sol);
                }
                *reinterpret_cast<float2*>(win + gslot + 2 * col) = sol;
                float* go = UPPER ? out + (size_t)(gdst + col) * Q + 2 * pr
                                  : out + (size_t)gdst * rsE + col * Q + 2 * pr;
                *reinterpret_cast<float2*>(go) = sol;
            }
        }
    }
};

// The same with one temporal block per thread block (Q thread blocks per
// sweep): the window keeps 3 rows x 1 value per slot, a lane gathers one
// FP32 value per step and adds three scalar FMAs.
template <int Q, int H, bool UPPER>
struct ColBody1 {
    static constexpr int GS = 3 * H, GPW = 32 / GS;
    int lane, gw, col, hh, lane0, warp, ncw, tb;
    bool lane_ok;
    unsigned rsE;
    float* out;
    __device__ ColBody1(const StageArgs<float>& a)
    {
        lane = threadIdx.x & 31;
        warp = threadIdx.x >> 5;
        ncw = a.ncw;
        gw = lane / GS;
        const int inl = lane - gw * GS;
        col = inl / H;
        hh = inl - col * H;
        lane0 = gw * GS;
        lane_ok = gw < GPW;
        tb = blockIdx.x;
        rsE = a.rs / (unsigned)sizeof(float);
        out = a.out;
    }
    template <bool RING>
    __device__ __forceinline__ void level(float* win, const unsigned char* base, const float* rh,
                                          int ng, int npass)
    {
        const int nchunk = reinterpret_cast<const int*>(base)[2];
        const int2* chunks = reinterpret_cast<const int2*>(base + 16);
        const unsigned char* grec = base + 16 + (((size_t)npass * ncw * 8 + 15) & ~(size_t)15);
        for (int k = 0; k < npass; ++k) {
            const int c = k * ncw + warp;
            if (c >= nchunk) break;  // warp-uniform
            const int2 cd = chunks[c];
            const float4* rp = reinterpret_cast<const float4*>(base + (size_t)cd.x * 16) + lane;
            const int jj = c * GPW + gw;
            const bool fin = lane_ok && hh == 0 && jj < ng;
            int gslot = 0, gdst = 0;
            float mv[3] = {0.0f, 0.0f, 0.0f}, bb[3] = {0.0f, 0.0f, 0.0f};
            if (fin) {
                const int* gr = reinterpret_cast<const int*>(grec + (size_t)jj * kCgrec);
                gslot = gr[0];
                gdst = gr[1];
                const float* m = reinterpret_cast<const float*>(gr + 3) + col * 3;
                const float* rr = rh + (size_t)gr[2] * rsE + tb;
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    mv[r] = m[r];
                    bb[r] = rr[r * Q];
                }
            }
            float acc[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll 4
            for (int st = 0; st < cd.y; ++st) {
                const float4 rec = rp[(size_t)st * 32];
                const float x = win[__float_as_int(rec.x)];
                acc[0] = fmaf(rec.y, x, acc[0]);
                acc[1] = fmaf(rec.z, x, acc[1]);
                acc[2] = fmaf(rec.w, x, acc[2]);
            }
#pragma unroll
            for (int m = 1; m < H; m <<= 1)
#pragma unroll
                for (int r = 0; r < 3; ++r) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], m);
            float tot[3];
#pragma unroll
            for (int r = 0; r < 3; ++r)
                tot[r] = (__shfl_sync(0xffffffffu, acc[r], lane0) +
                          __shfl_sync(0xffffffffu, acc[r], lane0 + H)) +
                         __shfl_sync(0xffffffffu, acc[r], lane0 + 2 * H);
            if (fin) {
                float sol = 0.0f;
#pragma unroll
                for (int r = 0; r < 3; ++r) sol = fmaf(mv[r], bb[r] - tot[r], sol);
                win[gslot + col] = sol;
                float* go = UPPER ? out + (size_t)(gdst + col) * Q + tb
                                  : out + (size_t)gdst * rsE + col * Q + tb;
                *go = sol;
            }
        }
    }
};

template <int Q, int H, bool UPPER>
__global__ void __launch_bounds__(kStageThreads, 1) k_tri_col1(StageArgs<float> a)
{
    extern __shared__ __align__(128) unsigned char smem[];
    // the padding slot reads as zero (ordered by the set-up barrier)
    if (threadIdx.x < 3) reinterpret_cast<float*>(smem + kHdrBytes)[a.aux + threadIdx.x] = 0.0f;
    ColBody1<Q, H, UPPER> body(a);
    stage_main<float>(a, body, smem);
}

template <int Q, int H, bool UPPER>
__global__ void __launch_bounds__(kStageThreads, 1) k_tri_col(StageArgs<float> a)
{
    extern __shared__ __align__(128) unsigned char smem[];
    // the padding slot reads as zero (ordered by the set-up barrier)
    if (threadIdx.x < 6) reinterpret_cast<float*>(smem + kHdrBytes)[a.aux + threadIdx.x] = 0.0f;
    ColBody<Q, H, UPPER> body(a);
    stage_main<float>(a, body, smem);
}

}  // namespace

// ---------------------------------------------------------------------------
// Register-prefetched row sweep (FP32, g = 3; the default for FP32).
//
// One thread block per temporal block (Q blocks per sweep, each on its own
// SM), each the whole level chain, as the column format; but the factor
// data never passes through shared memory.  Shared memory holds only the
// solution window (3 rows x 1 value per slot); every record of a level is
// loaded from global memory (L2) straight into registers two levels ahead
// of its use, so a level's critical path is: window reads at byte offsets
// already in registers, one multiply-add per factor entry, the share and
// diagonal-block shuffles, the window store and one block barrier.  A level
// has no branch: every warp has a fixed-size slot at every level.
//
// Layout.  Lane = (group of the warp's chunk, row r of the group, share h
// of the row's entries, H shares): lanes g*3H + r*H + h; a lane owns a
// share of the row's off-diagonal entries, one per step, SMAX steps (a
// multiple of 4; entries past the lane's own read an all-zero window slot
// with value 0).  The groups of a level are sorted by their longest row
// and dealt to chunks of 32/(3H) groups; a level with more chunks than the
// ncw warps is split into consecutive sub-levels (its groups are
// independent).  Chunk w of (sub-)level l sits in the fixed slot l*ncw + w;
// warps without a chunk at a level get an empty slot.  A slot holds, per
// lane (loads of 16 bytes, consecutive lanes adjacent):
//   float4 {minv[r][0..2] (row r of the inverted 3 x 3 diagonal block),
//           window offset of the row (-1: lane stores nothing)}   512 B
//   int    destination (forward: the backward sweep's right-hand-side
//          slot of the row; backward: row * Q of z)               128 B
//   uint4  byte offsets in the window of steps 4k..4k+3          SMAX/4 x 512 B
//   float4 factor values of steps 4k..4k+3                       SMAX/4 x 512 B
// The right-hand sides are per-temporal-block arrays in the same lane-slot
// order (the forward sweep's from a pre-pass that also applies the q x q
// mixing with A^-1; the backward sweep's written by the forward sweep), so
// every load of a level has an address known in advance.  The loads are
// inline-PTX non-coherent loads (volatile, so they are issued where they
// stand, two levels before their use), and the level barrier is a
// volatile bar.sync that they do not cross.  A row's entries are summed in
// a step order chosen on the host so that a warp's window reads of one
// step fall into distinct shared-memory banks where possible.
constexpr int kRegMaxWarps = 16;
constexpr unsigned kRegLaneTab = 640;

struct RegTri {
    int nl = 0, ncw = 0, H = 0, smax = 0, slot_bytes = 0;
    int win_elems = 0, zero_off = 0;
    bool w16 = false;  // 16-bit window byte offsets (window <= 64 KB)
    long long lanes = 0;  // nl * ncw * 32
    DBuf<unsigned char> slots;
    std::vector<int> row_slot;             // host: lane slot of each row's h = 0 lane
    std::vector<std::vector<int>> chunks;  // host (build only): level-order groups per chunk
    std::vector<int> chunk_slot, chunk_steps;
};

namespace {

int reg_warps(const TriHost& h, int GPW)
{
    std::vector<int> nch;
    for (int l = 0; l < h.nlevels; ++l)
        nch.push_back((h.level_ptr[l + 1] - h.level_ptr[l] + GPW - 1) / GPW);
    std::sort(nch.begin(), nch.end());
    const int p90 = nch[(size_t)(0.90 * (nch.size() - 1))];
    const int w = env_int("XTFEM_ILU_WARPS", p90);
    return std::max(1, std::min(kRegMaxWarps, w));
}

// Chunks, sub-levels, slots and steps of one triangle (no device data yet).
bool reg_plan(const TriHost& h, int H, RegTri& t, int force_ncw = 0)
{
    const int g = 3, GS = 3 * H, GPW = 32 / GS;
    t.H = H;
    t.ncw = force_ncw > 0 ? force_ncw : reg_warps(h, GPW);
    t.row_slot.assign((size_t)h.ngroups * g, -1);
    t.chunks.clear();
    t.chunk_slot.clear();
    t.chunk_steps.clear();
    int nl = 0, smax = 0;
    std::vector<int> ord;
    auto rowlen = [&](int i, int r) {
        return h.ext_ptr[(size_t)i * g + r + 1] - h.ext_ptr[(size_t)i * g + r];
    };
    auto longest = [&](int i) { return std::max(rowlen(i, 0), std::max(rowlen(i, 1), rowlen(i, 2))); };
    for (int l = 0; l < h.nlevels; ++l) {
        const int gb = h.level_ptr[l], ng = h.level_ptr[l + 1] - gb;
        ord.resize(ng);
        for (int j = 0; j < ng; ++j) ord[j] = gb + j;
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return longest(a) > longest(b); });
        const int nch = (ng + GPW - 1) / GPW;
        for (int c = 0; c < nch; ++c) {
            if (c % t.ncw == 0) ++nl;  // a new (sub-)level every ncw chunks
            std::vector<int> grp(ord.begin() + c * GPW, ord.begin() + std::min(ng, (c + 1) * GPW));
            const long long slot = (long long)(nl - 1) * t.ncw + c % t.ncw;
            int steps = 0;
            for (int gw = 0; gw < (int)grp.size(); ++gw) {
                const int i = grp[gw], G = h.order[i];
                for (int r = 0; r < g; ++r) {
                    steps = std::max(steps, (rowlen(i, r) + H - 1) / H);
                    t.row_slot[(size_t)G * g + r] = (int)(slot * 32 + gw * GS + r * H);
                }
            }
            if (slot * 32 + 31 >= INT32_MAX) return false;
            smax = std::max(smax, steps);
            t.chunks.push_back(std::move(grp));
            t.chunk_slot.push_back((int)slot);
            t.chunk_steps.push_back(steps);
        }
    }
    t.nl = nl;
    t.smax = (smax + 3) / 4 * 4;
    t.lanes = (long long)nl * t.ncw * 32;
    t.zero_off = h.nslots * g;
    t.win_elems = (h.nslots + 1) * g;
    return t.smax <= 32 && (long long)t.win_elems * 4 <= (long long)max_dyn_smem();
}

// Slots of a planned triangle.  dst: forward, the other triangle's
// row_slot; backward (dst empty): row * Q.
int reg_fill(const TriHost& h, RegTri& t, int smax, int Q, const std::vector<int>* dst,
             cudaStream_t s, int row0 = 0)
{
    const int g = 3, H = t.H, GS = 3 * H, GPW = 32 / GS;
    t.smax = smax;
    const unsigned ob = t.w16 ? 256u : 512u;  // bytes of one offset quad per warp
    t.slot_bytes = (int)(kRegLaneTab + (unsigned)(smax / 4) * (ob + 512u));
    const size_t nslot = (size_t)t.nl * t.ncw;
    std::vector<unsigned char> blob(nslot * t.slot_bytes, 0);
    // every lane of every slot starts empty: no store, all steps on the zero slot
    for (size_t sl = 0; sl < nslot; ++sl) {
        unsigned char* b = blob.data() + sl * t.slot_bytes;
        const int none = -1;
        for (int lane = 0; lane < 32; ++lane) std::memcpy(b + lane * 16 + 12, &none, 4);
        for (int e = 0; e < (smax / 4) * 128; ++e) {
            if (t.w16) reinterpret_cast<unsigned short*>(b + kRegLaneTab)[e] = (unsigned short)(t.zero_off * 4);
            else reinterpret_cast<unsigned*>(b + kRegLaneTab)[e] = (unsigned)t.zero_off * 4u;
        }
    }
    std::vector<int> seen(t.win_elems, 0);
    int epoch = 0;
    bool valid = true;
    const bool banks = env_int("XTFEM_ILU_BANKS", 1) != 0;  // 0: entries in row order
    std::vector<std::vector<std::pair<int, float>>> ent(32);
    std::vector<int> lanes(32);
    for (size_t c = 0; c < t.chunks.size(); ++c) {
        const int slot = t.chunk_slot[c];
        unsigned char* b = blob.data() + (size_t)slot * t.slot_bytes;
        float* gm = reinterpret_cast<float*>(b);
        int* go = reinterpret_cast<int*>(b + 512);
        unsigned* off = reinterpret_cast<unsigned*>(b + kRegLaneTab);
        unsigned short* off16 = reinterpret_cast<unsigned short*>(b + kRegLaneTab);
        float* val = reinterpret_cast<float*>(b + kRegLaneTab + (smax / 4) * ob);
        const auto& grp = t.chunks[c];
        for (int lane = 0; lane < 32; ++lane) {
            ent[lane].clear();
            const int gw = lane / GS, r = (lane % GS) / H, hh = lane % H;
            if (gw >= GPW || gw >= (int)grp.size()) continue;
            const int i = grp[gw], G = h.order[i];
            for (int k = 0; k < 3; ++k) gm[lane * 4 + k] = (float)h.minv[(size_t)i * 9 + r * 3 + k];
            if (hh == 0) {
                const int wo = h.slot[G] * g + r;
                std::memcpy(&gm[lane * 4 + 3], &wo, 4);
                const long long d = dst ? (long long)(*dst)[(size_t)G * g + r]
                                        : ((long long)row0 + (long long)G * g + r) * Q;
                valid = valid && wo >= 0 && wo < t.zero_off && d >= 0 && d < INT32_MAX;
                go[lane] = (int)d;
            }
            const int kb = h.ext_ptr[(size_t)i * g + r], ke = h.ext_ptr[(size_t)i * g + r + 1];
            for (int k = kb + hh; k < ke; k += H) {
                const int col = h.ext_col[k], Gc = col / g;
                ent[lane].push_back({h.slot[Gc] * g + (col - Gc * g), (float)h.ext_v[k]});
            }
        }
        // Step order: at every step each lane takes, of its remaining
        // entries, one whose shared-memory bank the warp's reads of that step
        // use least (an address another lane already reads is a broadcast
        // and costs nothing); lanes with more entries left choose first.
        for (int st = 0; st < smax; ++st) {
            int load[32] = {0};
            ++epoch;
            for (int l2 = 0; l2 < 32; ++l2) lanes[l2] = l2;
            std::stable_sort(lanes.begin(), lanes.end(),
                             [&](int a, int b2) { return ent[a].size() > ent[b2].size(); });
            for (int lane : lanes) {
                int o = t.zero_off;
                float v = 0.0f;
                if (!ent[lane].empty()) {
                    size_t best = 0;
                    int bcost = 1 << 30;
                    for (size_t e = 0; banks && e < ent[lane].size(); ++e) {
                        const int a = ent[lane][e].first;
                        const int cost = seen[a] == epoch ? 0 : load[a & 31] + 1;
                        if (cost < bcost) { bcost = cost; best = e; }
                    }
                    o = ent[lane][best].first;
                    v = ent[lane][best].second;
                    ent[lane].erase(ent[lane].begin() + best);
                }
                valid = valid && o >= 0 && o < t.win_elems;
                if (valid && seen[o] != epoch) {
                    seen[o] = epoch;
                    load[o & 31]++;
                }
                const size_t oi = ((size_t)(st >> 2) * 32 + lane) * 4 + (st & 3);
                if (t.w16) off16[oi] = (unsigned short)(o * 4);
                else off[oi] = (unsigned)o * 4u;
                val[((size_t)(st >> 2) * 32 + lane) * 4 + (st & 3)] = v;
            }
        }
        for (int lane = 0; lane < 32; ++lane) valid = valid && ent[lane].empty();
    }
    if (!valid) return XT_OK;
    XT_TRY(t.slots.upload(blob.data(), blob.size(), s));
    XT_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
    t.chunks.clear();
    t.chunks.shrink_to_fit();
    return XT_OK;
}

// Register capacities (steps per lane) compiled for each share count.
int reg_smax(int H, int need)
{
    static const int caps2[] = {8, 12, 16}, caps1[] = {12, 20}, caps4[] = {8};
    const int* c = H == 2 ? caps2 : (H == 1 ? caps1 : caps4);
    const int n = H == 2 ? 3 : (H == 1 ? 2 : 1);
    for (int i = 0; i < n; ++i)
        if (need <= c[i]) return c[i];
    return 0;
}

int build_reg(const IluSched& S, int Q, int H, IluStage& st, cudaStream_t s)
{
    st.reg_ok = false;
    if (S.L.g != 3 || (H != 1 && H != 2 && H != 4)) return XT_OK;
    auto L = std::make_shared<RegTri>(), U = std::make_shared<RegTri>();
    // the triangles are planned side by side, then filled side by side (the
    // forward fill reads the backward triangle's row slots, set by its plan)
    bool okL = false, okU = false;
    XT_TRY(side_by_side([&] { okU = reg_plan(S.U, H, *U); return XT_OK; },
                        [&] { okL = reg_plan(S.L, H, *L); return XT_OK; }));
    if (!okL || !okU) return XT_OK;
    const int smax = reg_smax(H, std::max(L->smax, U->smax));
    if (smax == 0) return XT_OK;
    // 16-bit window offsets when every byte offset of both windows fits
    // (XTFEM_ILU_W16=0: 32-bit)
    const bool w16 = (long long)std::max(L->win_elems, U->win_elems) * 4 <= 65536 &&
                     env_int("XTFEM_ILU_W16", 1) != 0;
    L->w16 = U->w16 = w16;
    XT_TRY(side_by_side([&] { return reg_fill(S.U, *U, smax, Q, nullptr, s); },
                        [&] { return reg_fill(S.L, *L, smax, Q, &U->row_slot, s); }));
    if (!L->slots.p || !U->slots.p) return XT_OK;
    std::vector<int> src((size_t)L->lanes, -1);
    for (size_t r = 0; r < L->row_slot.size(); ++r) src[(size_t)L->row_slot[r]] = (int)r;
    XT_TRY(st.srcL.upload(src.data(), src.size(), s));
    XT_TRY(st.rrhsL.alloc((size_t)Q * L->lanes));
    XT_TRY(st.rrhsU.alloc((size_t)Q * U->lanes));
    // slots the forward sweep never writes are read (not used) by the
    // backward sweep's other lanes: keep them finite
    XT_CUDA(cudaMemsetAsync(st.rrhsU.p, 0, sizeof(float) * Q * U->lanes, s));
    XT_CUDA(cudaStreamSynchronize(s));
    L->row_slot.clear();
    U->row_slot.clear();
    if (trace_on())
        std::fprintf(stderr, "[xtfem] register sweep: H %d, steps %d, warps %d/%d, levels %d/%d\n",
                     H, smax, L->ncw, U->ncw, L->nl, U->nl);
    st.regL = L;
    st.regU = U;
    st.reg_ok = true;
    return XT_OK;
}

__device__ __forceinline__ float4 nc_v4f(const void* p)
{
    float4 r;
    asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
                 : "l"(p));
    return r;
}
__device__ __forceinline__ uint4 nc_v4u(const void* p)
{
    uint4 r;
    asm volatile("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "l"(p));
    return r;
}
__device__ __forceinline__ float nc_f(const void* p)
{
    float r;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(r) : "l"(p));
    return r;
}
__device__ __forceinline__ int nc_i(const void* p)
{
    int r;
    asm volatile("ld.global.nc.s32 %0, [%1];" : "=r"(r) : "l"(p));
    return r;
}
__device__ __forceinline__ float lds_f(unsigned addr)
{
    float r;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(r) : "r"(addr));
    return r;
}
__device__ __forceinline__ void prefetch_l2(const void* p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
__device__ __forceinline__ void level_barrier()
{
    asm volatile("bar.sync 0;" ::: "memory");
}

// Offsets of four steps: four 32-bit window byte offsets, or (W16) four
// 16-bit ones packed in two words.
template <bool W16> struct RegOff;
template <> struct RegOff<false> {
    uint4 o;
    __device__ __forceinline__ unsigned at(int i) const
    {
        return i == 0 ? o.x : (i == 1 ? o.y : (i == 2 ? o.z : o.w));
    }
};
template <> struct RegOff<true> {
    uint2 o;
    __device__ __forceinline__ unsigned at(int i) const
    {
        const unsigned w = i < 2 ? o.x : o.y;
        return (i & 1) ? (w >> 16) : (w & 0xffffu);
    }
};

template <int SMAX, bool W16>
struct RegSet {
    RegOff<W16> off[SMAX / 4];
    float4 val[SMAX / 4];
    float4 gm;
    int go;
    float b;
};

// The slot at p (already offset to this warp's slot of the level) and the
// right-hand side at bsrc.
__device__ __forceinline__ uint2 nc_v2u(const void* p)
{
    uint2 r;
    asm volatile("ld.global.nc.v2.u32 {%0, %1}, [%2];" : "=r"(r.x), "=r"(r.y) : "l"(p));
    return r;
}

template <int SMAX, bool W16>
__device__ __forceinline__ void reg_load(RegSet<SMAX, W16>& S, const unsigned char* p,
                                         const float* bsrc, int lane)
{
    constexpr int ob = W16 ? 256 : 512;
    S.gm = nc_v4f(p + lane * 16);
    S.go = nc_i(p + 512 + lane * 4);
    S.b = nc_f(bsrc);
#pragma unroll
    for (int k = 0; k < SMAX / 4; ++k) {
        if constexpr (W16) S.off[k].o = nc_v2u(p + kRegLaneTab + k * 256 + lane * 8);
        else S.off[k].o = nc_v4u(p + kRegLaneTab + k * 512 + lane * 16);
        S.val[k] = nc_v4f(p + kRegLaneTab + (SMAX / 4) * ob + k * 512 + lane * 16);
    }
}

template <int H, int SMAX, bool W16>
__device__ __forceinline__ void reg_level(const RegSet<SMAX, W16>& S, unsigned wbase, float* win,
                                          float* out, int lane0)
{
    // four accumulators: dependent chains of SMAX / 4 multiply-adds
    float acc0 = 0.0f, acc1 = 0.0f, acc2 = 0.0f, acc3 = 0.0f;
#pragma unroll
    for (int k = 0; k < SMAX / 4; ++k) {
        const float x0 = lds_f(wbase + S.off[k].at(0)), x1 = lds_f(wbase + S.off[k].at(1));
        const float x2 = lds_f(wbase + S.off[k].at(2)), x3 = lds_f(wbase + S.off[k].at(3));
        acc0 = fmaf(S.val[k].x, x0, acc0);
        acc1 = fmaf(S.val[k].y, x1, acc1);
        acc2 = fmaf(S.val[k].z, x2, acc2);
        acc3 = fmaf(S.val[k].w, x3, acc3);
    }
    float acc = (acc0 + acc1) + (acc2 + acc3);
#pragma unroll
    for (int m = 1; m < H; m <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
    const float d = S.b - acc;
    const float d0 = __shfl_sync(0xffffffffu, d, lane0);
    const float d1 = __shfl_sync(0xffffffffu, d, lane0 + H);
    const float d2 = __shfl_sync(0xffffffffu, d, lane0 + 2 * H);
    const float sol = fmaf(S.gm.z, d2, fmaf(S.gm.y, d1, S.gm.x * d0));
    const int wo = __float_as_int(S.gm.w);
    if (wo >= 0) {
        win[wo] = sol;
        out[S.go] = sol;
    }
}

// One temporal block tb of one sweep (one thread block).  DEP register
// sets (2, 3 or 4): a set's loads have DEP - 1 levels of work to land in.
template <int H, int SMAX, bool UPPER, bool W16, int DEP>
__device__ __forceinline__ void tri_reg_body(const RegArgs& a, int tb)
{
    extern __shared__ __align__(16) float rwin[];
    if (a.skip && a.skip[0] != 0) return;  // uniform: before any barrier
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int GS = 3 * H;
    const int lane0 = (lane / GS) * GS;
    const unsigned wbase = (unsigned)__cvta_generic_to_shared(rwin);
    float* out = UPPER ? a.out + tb : a.out + (size_t)tb * a.ostride;
    if (threadIdx.x < 3) rwin[a.zero_off + threadIdx.x] = 0.0f;
    // this warp's slot and right-hand side advance by one level's worth
    const size_t sstep = (size_t)a.ncw * a.slot_bytes;
    const unsigned char* sp = a.slots + (size_t)warp * a.slot_bytes;
    const float* bp = a.rhs + (size_t)tb * a.rstride + (size_t)warp * 32 + lane;
    // L2 prefetch of the slot and right-hand side a.pf levels ahead of the
    // register loads: the slots of a sweep are read once per apply, from
    // DRAM, and the register loads alone do not cover DRAM latency.  Lane i
    // touches the slot's 128-byte line i, lane 31 the right-hand-side line.
    auto prefetch = [&](int L) {
        if (a.pf > 0 && L < a.nl) {
            const size_t o = (size_t)lane * 128;
            if (o < (size_t)a.slot_bytes)
                prefetch_l2(a.slots + ((size_t)L * a.ncw + warp) * a.slot_bytes + o);
            else if (lane == 31)
                prefetch_l2(a.rhs + (size_t)tb * a.rstride + ((size_t)L * a.ncw + warp) * 32);
        }
    };
    for (int L = DEP; L < DEP + a.pf; ++L) prefetch(L);
    // In the level loop the prefetch is a running pointer: the line this
    // thread touches at level DEP + pf, advanced by one level's worth (no
    // address arithmetic per level).  pfl: the loop's last level index l
    // whose level l + DEP + pf exists.
    const bool pf_slot = a.pf > 0 && lane * 128 < a.slot_bytes;
    const bool pf_rhs = a.pf > 0 && !pf_slot && lane == 31;
    const unsigned char* pp =
        pf_slot ? a.slots + ((size_t)(DEP + a.pf) * a.ncw + warp) * a.slot_bytes + (size_t)lane * 128
                : reinterpret_cast<const unsigned char*>(
                      a.rhs + (size_t)tb * a.rstride + ((size_t)(DEP + a.pf) * a.ncw + warp) * 32);
    const size_t pstep = pf_slot ? sstep : (size_t)a.ncw * 32 * sizeof(float);
    const bool pf_on = pf_slot || pf_rhs;
    const int pfl = a.nl - DEP - a.pf;
    // one level: compute it with set S, reload S with the level DEP ahead,
    // prefetch, advance, barrier
    auto level = [&](RegSet<SMAX, W16>& S, int lk) {
        reg_level<H, SMAX, W16>(S, wbase, rwin, out, lane0);
        if (lk + DEP < a.nl) reg_load<SMAX, W16>(S, sp, bp, lane);
        if (pf_on && lk < pfl) prefetch_l2(pp);
        pp += pstep;
        sp += sstep;
        bp += a.ncw * 32;
        level_barrier();
    };
    if constexpr (DEP == 4) {
        // four register sets, four levels per trip
        RegSet<SMAX, W16> s0, s1, s2, s3;
        reg_load<SMAX, W16>(s0, sp, bp, lane);
        if (a.nl > 1) reg_load<SMAX, W16>(s1, sp + sstep, bp + a.ncw * 32, lane);
        if (a.nl > 2) reg_load<SMAX, W16>(s2, sp + 2 * sstep, bp + 2 * a.ncw * 32, lane);
        if (a.nl > 3) reg_load<SMAX, W16>(s3, sp + 3 * sstep, bp + 3 * a.ncw * 32, lane);
        sp += 4 * sstep;
        bp += 4 * a.ncw * 32;
        level_barrier();  // the zero slot is set
        for (int l = 0; l < a.nl; l += 4) {
            level(s0, l);
            if (l + 1 < a.nl) level(s1, l + 1);
            if (l + 2 < a.nl) level(s2, l + 2);
            if (l + 3 < a.nl) level(s3, l + 3);
        }
        return;
    }
    if constexpr (DEP == 3) {
        // three register sets, three levels per trip
        RegSet<SMAX, W16> s0, s1, s2;
        reg_load<SMAX, W16>(s0, sp, bp, lane);
        if (a.nl > 1) reg_load<SMAX, W16>(s1, sp + sstep, bp + a.ncw * 32, lane);
        if (a.nl > 2) reg_load<SMAX, W16>(s2, sp + 2 * sstep, bp + 2 * a.ncw * 32, lane);
        sp += 3 * sstep;
        bp += 3 * a.ncw * 32;
        level_barrier();  // the zero slot is set
        for (int l = 0; l < a.nl; l += 3) {
            reg_level<H, SMAX, W16>(s0, wbase, rwin, out, lane0);
            if (l + 3 < a.nl) reg_load<SMAX, W16>(s0, sp, bp, lane);
            if (pf_on && l < pfl) prefetch_l2(pp);
            pp += pstep;
            sp += sstep;
            bp += a.ncw * 32;
            level_barrier();
            if (l + 1 < a.nl) {
                reg_level<H, SMAX, W16>(s1, wbase, rwin, out, lane0);
                if (l + 4 < a.nl) reg_load<SMAX, W16>(s1, sp, bp, lane);
                if (pf_on && l + 1 < pfl) prefetch_l2(pp);
                pp += pstep;
                sp += sstep;
                bp += a.ncw * 32;
                level_barrier();
            }
            if (l + 2 < a.nl) {
                reg_level<H, SMAX, W16>(s2, wbase, rwin, out, lane0);
                if (l + 5 < a.nl) reg_load<SMAX, W16>(s2, sp, bp, lane);
                if (pf_on && l + 2 < pfl) prefetch_l2(pp);
                pp += pstep;
                sp += sstep;
                bp += a.ncw * 32;
                level_barrier();
            }
        }
        return;
    }
    // two register sets, a pair of levels per trip: the set a level used is
    // reloaded, right after it, with the level two ahead
    RegSet<SMAX, W16> s0, s1;
    reg_load<SMAX, W16>(s0, sp, bp, lane);
    if (a.nl > 1) reg_load<SMAX, W16>(s1, sp + sstep, bp + a.ncw * 32, lane);
    sp += 2 * sstep;
    bp += 2 * a.ncw * 32;
    level_barrier();  // the zero slot is set
    for (int l = 0; l < a.nl; l += 2) {
        reg_level<H, SMAX, W16>(s0, wbase, rwin, out, lane0);
        if (l + 2 < a.nl) reg_load<SMAX, W16>(s0, sp, bp, lane);
        if (pf_on && l < pfl) prefetch_l2(pp);
        pp += pstep;
        sp += sstep;
        bp += a.ncw * 32;
        level_barrier();
        if (l + 1 < a.nl) {
            reg_level<H, SMAX, W16>(s1, wbase, rwin, out, lane0);
            if (l + 3 < a.nl) reg_load<SMAX, W16>(s1, sp, bp, lane);
            if (pf_on && l + 1 < pfl) prefetch_l2(pp);
            pp += pstep;
            sp += sstep;
            bp += a.ncw * 32;
            level_barrier();
        }
    }
}

// Warps of a sweep with DEP register sets: at most 12 for four sets leave
// each thread the registers (131) the sets need.
__host__ __device__ constexpr int reg_max_warps(int dep)
{
    return dep <= 3 ? kRegMaxWarps : 12;
}

template <int H, int SMAX, bool UPPER, bool W16, int DEP>
__global__ void __launch_bounds__(reg_max_warps(DEP) * 32, 1)
    k_tri_reg(RegArgs a)
{
    tri_reg_body<H, SMAX, UPPER, W16, DEP>(a, blockIdx.x);
}

// One thread block per (entry, temporal block): entry blockIdx.x / q of the
// table, temporal block blockIdx.x % q.  The entries are the row blocks of
// a block-Jacobi factor (the output and the skip flag are the launch's) or
// the sweeps of a batch of systems (each entry's own); the prefetch
// distance is the launch's.
template <int H, int SMAX, bool UPPER, bool W16>
__global__ void __launch_bounds__(kRegMaxWarps * 32, 1)
    k_tri_reg_parts(const RegArgs* __restrict__ args, int q, int pf, const int* skip, float* out)
{
    RegArgs a = args[blockIdx.x / q];
    a.pf = pf;
    if (skip) a.skip = skip;
    if (out) a.out = out;
    tri_reg_body<H, SMAX, UPPER, W16, 2>(a, blockIdx.x % q);
}

// Forward-sweep right-hand sides in lane-slot order, one array per temporal
// block: rhs[q][s] = sum_j Ainv(q, j) v(row(s), j) (0 for unused slots).
template <int Q>
__global__ void k_rhs_slots(const int* __restrict__ src, long long lanes,
                            const double* __restrict__ dAinv, const float* __restrict__ v,
                            float* __restrict__ rhs, const int* __restrict__ skip)
{
    __shared__ float sA[Q * Q];
    if (skip && skip[0] != 0) return;
    for (int i = threadIdx.x; i < Q * Q; i += blockDim.x) sA[i] = (float)dAinv[i];
    __syncthreads();
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < lanes;
         t += (long long)gridDim.x * blockDim.x) {
        const int row = src[t];
        float vr[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j) vr[j] = row >= 0 ? v[(size_t)row * Q + j] : 0.0f;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            float b = 0.0f;
#pragma unroll
            for (int j = 0; j < Q; ++j) b = fmaf(sA[j * Q + q], vr[j], b);
            rhs[(size_t)q * lanes + t] = b;
        }
    }
}

// Register layouts of every row block of a block-Jacobi factor, with the
// warps, steps per lane and offset width of the whole set (the largest
// block's warps, the longest row's steps); the blocks' lanes are laid end
// to end, so the pre-pass and the right-hand-side arrays are those of one
// factor.  Leaves st.reg_ok false when a block does not fit.
int build_reg_parts(const DevIlu& F, int Q, int H, IluStage& st, cudaStream_t s)
{
    st.reg_ok = false;
    const int P = F.blocks;
    if (P < 2 || (int)F.part_sched.size() != P || (H != 1 && H != 2 && H != 4)) return XT_OK;
    const int GPW = 32 / (3 * H);
    int ncw = 1;
    for (const auto& ps : F.part_sched) {
        if (ps->L.g != 3) return XT_OK;
        ncw = std::max(ncw, std::max(reg_warps(ps->L, GPW), reg_warps(ps->U, GPW)));
    }
    std::vector<std::shared_ptr<RegTri>> Ls(P), Us(P);
    int need = 0, win = 0;
    for (int b = 0; b < P; ++b) {
        Ls[b] = std::make_shared<RegTri>();
        Us[b] = std::make_shared<RegTri>();
        if (!reg_plan(F.part_sched[b]->L, H, *Ls[b], ncw) ||
            !reg_plan(F.part_sched[b]->U, H, *Us[b], ncw))
            return XT_OK;
        need = std::max(need, std::max(Ls[b]->smax, Us[b]->smax));
        win = std::max(win, std::max(Ls[b]->win_elems, Us[b]->win_elems));
    }
    const int smax = reg_smax(H, need);
    if (smax == 0) return XT_OK;
    const bool w16 = (long long)win * 4 <= 65536 && env_int("XTFEM_ILU_W16", 1) != 0;
    std::vector<long long> offL(P + 1, 0), offU(P + 1, 0);
    for (int b = 0; b < P; ++b) {
        offL[b + 1] = offL[b] + Ls[b]->lanes;
        offU[b + 1] = offU[b] + Us[b]->lanes;
    }
    if (offL[P] >= INT32_MAX || offU[P] >= INT32_MAX) return XT_OK;
    std::vector<int> src((size_t)offL[P], -1);
    for (int b = 0; b < P; ++b) {
        Ls[b]->w16 = Us[b]->w16 = w16;
        XT_TRY(reg_fill(F.part_sched[b]->U, *Us[b], smax, Q, nullptr, s, F.bounds[b]));
        for (int& v : Us[b]->row_slot)
            if (v >= 0) v += (int)offU[b];
        XT_TRY(reg_fill(F.part_sched[b]->L, *Ls[b], smax, Q, &Us[b]->row_slot, s));
        if (!Ls[b]->slots.p || !Us[b]->slots.p) return XT_OK;
        for (size_t r = 0; r < Ls[b]->row_slot.size(); ++r)
            src[(size_t)(offL[b] + Ls[b]->row_slot[r])] = F.bounds[b] + (int)r;
        Ls[b]->row_slot.clear();
        Us[b]->row_slot.clear();
    }
    XT_TRY(st.srcL.upload(src.data(), src.size(), s));
    XT_TRY(st.rrhsL.alloc((size_t)Q * offL[P]));
    XT_TRY(st.rrhsU.alloc((size_t)Q * offU[P]));
    XT_CUDA(cudaMemsetAsync(st.rrhsU.p, 0, sizeof(float) * Q * offU[P], s));
    std::vector<RegArgs> aL(P), aU(P);
    for (int b = 0; b < P; ++b) {
        aL[b] = RegArgs{Ls[b]->slots.p, st.rrhsL.p + offL[b], nullptr, offL[P], offU[P],
                        Ls[b]->nl, ncw, Ls[b]->slot_bytes, Ls[b]->zero_off, 0, nullptr};
        aU[b] = RegArgs{Us[b]->slots.p, st.rrhsU.p + offU[b], nullptr, offU[P], 0,
                        Us[b]->nl, ncw, Us[b]->slot_bytes, Us[b]->zero_off, 0, nullptr};
    }
    XT_TRY(st.argsL.upload(reinterpret_cast<const unsigned char*>(aL.data()), sizeof(RegArgs) * P, s));
    XT_TRY(st.argsU.upload(reinterpret_cast<const unsigned char*>(aU.data()), sizeof(RegArgs) * P, s));
    XT_CUDA(cudaStreamSynchronize(s));
    if (trace_on()) {
        int nlL = 0, nlU = 0;
        for (int b = 0; b < P; ++b) {
            nlL = std::max(nlL, Ls[b]->nl);
            nlU = std::max(nlU, Us[b]->nl);
        }
        std::fprintf(stderr,
                     "[xtfem] register sweep over %d row blocks: H %d, steps %d, warps %d, "
                     "levels at most %d/%d\n", P, H, smax, ncw, nlL, nlU);
    }
    st.parts = P;
    st.ncw = ncw;
    st.win_elems = win;
    st.lanesL = offL[P];
    st.lanesU = offU[P];
    st.regLp = Ls;
    st.regUp = Us;
    st.regL = Ls[0];  // H, steps and offset width of the set
    st.regU = Us[0];
    st.reg_ok = true;
    return XT_OK;
}

template <int Q, int H, int SMAX, bool W16, int DEP = 2>
int launch_reg(const IluStage& st, const double* dAinv, const float* v, float* z, cudaStream_t s,
               const int* skip)
{
    static std::atomic<bool> attr{false};
    if (!attr.load(std::memory_order_acquire)) {
        XT_CUDA(cudaFuncSetAttribute(k_tri_reg<H, SMAX, false, W16, DEP>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem()));
        XT_CUDA(cudaFuncSetAttribute(k_tri_reg<H, SMAX, true, W16, DEP>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem()));
        attr.store(true, std::memory_order_release);
    }
    const int pf = std::max(0, std::min(64, env_int("XTFEM_ILU_PF", 8)));
    if (st.parts > 1) {
        static std::atomic<bool> pattr{false};
        if (!pattr.load(std::memory_order_acquire)) {
            XT_CUDA(cudaFuncSetAttribute(k_tri_reg_parts<H, SMAX, false, W16>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem()));
            XT_CUDA(cudaFuncSetAttribute(k_tri_reg_parts<H, SMAX, true, W16>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem()));
            pattr.store(true, std::memory_order_release);
        }
        const int nb = (int)std::max(1LL, std::min<long long>((st.lanesL + 255) / 256, 152LL * 8));
        k_rhs_slots<Q><<<nb, 256, 0, s>>>(st.srcL.p, st.lanesL, dAinv, v, st.rrhsL.p, skip);
        const RegArgs* aL = reinterpret_cast<const RegArgs*>(st.argsL.p);
        const RegArgs* aU = reinterpret_cast<const RegArgs*>(st.argsU.p);
        const size_t smem = (size_t)st.win_elems * 4;
        k_tri_reg_parts<H, SMAX, false, W16><<<Q * st.parts, st.ncw * 32, smem, s>>>(aL, Q, pf, skip,
                                                                                  st.rrhsU.p);
        k_tri_reg_parts<H, SMAX, true, W16><<<Q * st.parts, st.ncw * 32, smem, s>>>(aU, Q, pf, skip, z);
        note_launches(3);
        XT_CUDA(cudaGetLastError());
        return XT_OK;
    }
    const RegTri& L = *st.regL;
    const RegTri& U = *st.regU;
    const int nblk = (int)std::max(1LL, std::min<long long>((L.lanes + 255) / 256, 152LL * 8));
    k_rhs_slots<Q><<<nblk, 256, 0, s>>>(st.srcL.p, L.lanes, dAinv, v, st.rrhsL.p, skip);
    RegArgs aL{L.slots.p, st.rrhsL.p, st.rrhsU.p, L.lanes, U.lanes, L.nl, L.ncw, L.slot_bytes,
               L.zero_off, pf, skip};
    RegArgs aU{U.slots.p, st.rrhsU.p, z, U.lanes, 0, U.nl, U.ncw, U.slot_bytes, U.zero_off, pf,
               skip};
    k_tri_reg<H, SMAX, false, W16, DEP><<<Q, L.ncw * 32, (size_t)L.win_elems * 4, s>>>(aL);
    k_tri_reg<H, SMAX, true, W16, DEP><<<Q, U.ncw * 32, (size_t)U.win_elems * 4, s>>>(aU);
    note_launches(3);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

// The kernel for the layout's offset width.
template <int Q, int H, int SMAX>
int launch_reg_width(const IluStage& st, const double* dAinv, const float* v, float* z,
                     cudaStream_t s, const int* skip)
{
    if (st.regL->w16 != st.regU->w16) {
        set_error("register sweep: triangles with different offset widths");
        return XT_ERR_STATE;
    }
    // four register sets (16-bit offsets, at most 12 steps per lane and 12
    // warps), else three; XTFEM_ILU_DEPTH=2 or 3 caps them
    if constexpr (SMAX <= 12) {
        const int dep = env_int("XTFEM_ILU_DEPTH", 4);
        const int w = std::max(st.regL->ncw, st.regU->ncw);
        if (st.regL->w16 && st.parts <= 1) {
            if (dep >= 4 && w <= reg_max_warps(4))
                return launch_reg<Q, H, SMAX, true, 4>(st, dAinv, v, z, s, skip);
            if (dep >= 3) return launch_reg<Q, H, SMAX, true, 3>(st, dAinv, v, z, s, skip);
        }
    }
    if (st.regL->w16) return launch_reg<Q, H, SMAX, true>(st, dAinv, v, z, s, skip);
    return launch_reg<Q, H, SMAX, false>(st, dAinv, v, z, s, skip);
}

template <int Q>
int launch_reg_any(const IluStage& st, const double* dAinv, const float* v, float* z,
                   cudaStream_t s, const int* skip)
{
    const int H = st.regL->H, smax = st.regL->smax;
    if (H == 2 && smax == 8) return launch_reg_width<Q, 2, 8>(st, dAinv, v, z, s, skip);
    if (H == 2 && smax == 12) return launch_reg_width<Q, 2, 12>(st, dAinv, v, z, s, skip);
    if (H == 2 && smax == 16) return launch_reg_width<Q, 2, 16>(st, dAinv, v, z, s, skip);
    if (H == 1 && smax == 12) return launch_reg_width<Q, 1, 12>(st, dAinv, v, z, s, skip);
    if (H == 1 && smax == 20) return launch_reg_width<Q, 1, 20>(st, dAinv, v, z, s, skip);
    if (H == 4 && smax == 8) return launch_reg_width<Q, 4, 8>(st, dAinv, v, z, s, skip);
    set_error("register sweep: no kernel for these shares and steps");
    return XT_ERR_ARG;
}

// ---------------------------------------------------------------------------
// Launchers.
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

// Staged-sweep data for (q, T, format), built on first use; nullptr when
// the factor cannot use that staged sweep.  fmt 0: rows, 1: node blocks.
template <class T>
int get_stage(const DevIlu& F, int q, int fmt, cudaStream_t s, IluStage*& out, int H = 0)
{
    out = nullptr;
    if (!F.sched || env_int("XTFEM_ILU_SIMPLE", 0)) return XT_OK;
    // the column format's layout depends on the shares and the warp count
    const bool col = fmt == 2 || fmt == 3;
    const int wenv = col ? std::max(0, std::min(63, env_int("XTFEM_ILU_WARPS", 0))) : 0;
    const int rkb = std::max(0, std::min(255, env_int("XTFEM_ILU_RING_KB", 0)));
    const bool hkey = col || fmt == 4;
    const int wkey = (col || fmt == 4) ? std::max(0, std::min(31, env_int("XTFEM_ILU_WARPS", 0))) +
                                             (fmt == 4 && env_int("XTFEM_ILU_BANKS", 1) == 0 ? 32 : 0)
                                       : 0;
    const int bkey = (fmt == 4 && F.blocks > 1 && env_int("XTFEM_ILU_BLOCKS", 1) != 0) ? 1 : 0;
    const int key =
        (((((q * 8 + fmt) * 2 + (sizeof(T) == 4 ? 1 : 0)) * 8 + (hkey ? H : 0)) * 64 + wkey) * 2 +
         bkey) * 256 + rkb;
    (void)wenv;
    auto it = F.stages.find(key);
    if (it == F.stages.end()) {
        auto st = std::make_shared<IluStage>();
        st->q = q;
        const TriHost& L = F.sched->L;
        const TriHost& U = F.sched->U;
        const int ng = L.ngroups, g = L.g;
        std::vector<int> gdL(ng), gdU(ng);
        for (int G = 0; G < ng; ++G) {
            gdL[G] = U.pos[G];
            gdU[G] = G * g;
        }
        if (fmt == 4) {
            // XTFEM_ILU_BLOCKS=0: the one schedule of a block-Jacobi factor
            if (sizeof(T) == 4 && F.blocks > 1 && env_int("XTFEM_ILU_BLOCKS", 1) != 0)
                XT_TRY(build_reg_parts(F, q, H, *st, s));
            if (sizeof(T) == 4 && !st->reg_ok) XT_TRY(build_reg(*F.sched, q, H, *st, s));
            it = F.stages.emplace(key, st).first;
            out = st->reg_ok ? st.get() : nullptr;
            return XT_OK;
        }
        if (fmt == 2 || fmt == 3) {
            if (sizeof(T) == 4) {
                const int vps = fmt == 2 ? 2 : 1;
                XT_TRY(build_col_tri(L, q, H, gdL, st->L, s, vps));
                XT_TRY(build_col_tri(U, q, H, gdU, st->U, s, vps));
            }
        } else if (fmt == 1) {
            if (sizeof(T) == 4) {
                XT_TRY(build_block_tri(L, q, gdL, st->L, s));
                XT_TRY(build_block_tri(U, q, gdU, st->U, s));
            }
        } else {
            XT_TRY(build_row_tri<T>(L, q, gdL, st->L, s));
            XT_TRY(build_row_tri<T>(U, q, gdU, st->U, s));
        }
        if (st->L.ok && st->U.ok) {
            st->rs = Layout<T>::up16((unsigned)(g * q * sizeof(T)));
            XT_TRY(st->rhsL.alloc((size_t)ng * st->rs));
            XT_TRY(st->rhsU.alloc((size_t)ng * st->rs));
        }
        it = F.stages.emplace(key, st).first;
    }
    if (fmt == 4) {
        out = it->second->reg_ok ? it->second.get() : nullptr;
        return XT_OK;
    }
    if (it->second->L.ok && it->second->U.ok) out = it->second.get();
    return XT_OK;
}

template <class T>
StageArgs<T> stage_args(const StageTri& t, const unsigned char* rhs, T* out, int ncw, unsigned rs)
{
    // XTFEM_ILU_SPIN_LIMIT shortens the waits for a level's data (tests use
    // it to make a wait run out with the GPU still answering)
    const long long spin = env_int("XTFEM_ILU_SPIN_LIMIT", 0) > 0
                               ? (long long)env_int("XTFEM_ILU_SPIN_LIMIT", 0) : kSpinLimit;
    return {t.blob.p, reinterpret_cast<const int4*>(t.table.p), rhs, out, t.nlevels, t.g, ncw,
            t.window_bytes, rs, t.aux, spin};
}

// Pre-pass, forward sweep kl and backward sweep ku of a staged solve; GPW
// groups per compute warp, each sweep on `grid` thread blocks (independent
// shares of the temporal blocks).
template <class T, int Q>
int run_stage(const DevIlu& F, const IluStage& st, int GPW, void (*kl)(StageArgs<T>),
              void (*ku)(StageArgs<T>), std::atomic<bool>& attr, const double* dAinv, const T* v, T* z,
              cudaStream_t s, int grid = 1)
{
    if (!attr.load(std::memory_order_acquire)) {  // idempotent: concurrent first calls are harmless
        XT_CUDA(cudaFuncSetAttribute(kl, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem()));
        XT_CUDA(cudaFuncSetAttribute(ku, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem()));
        attr.store(true, std::memory_order_release);
    }
    const int g = F.L.g, ng = F.L.ngroups;
    auto warps = [&](const StageTri& t) {
        if (t.ncw > 0) return t.ncw;  // laid out for this warp count
        const int w = env_int("XTFEM_ILU_WARPS", (t.p90 + GPW - 1) / GPW);
        return std::max(1, std::min(kStageThreads / 32 - 2, w));  // + producer + waiter
    };
    const int wL = warps(st.L), wU = warps(st.U);
    const long long total = (long long)ng * g * Q;
    const int nblk = (int)std::max(1LL, std::min<long long>((total + 255) / 256, 152LL * 8));
    T* recL = reinterpret_cast<T*>(st.rhsL.p);
    T* recU = reinterpret_cast<T*>(st.rhsU.p);
    k_rhs_perm<T, Q><<<nblk, 256, 0, s>>>(F.L.group_row0.p, ng, g, dAinv, v, recL,
                                          st.rs / (unsigned)sizeof(T));
    const size_t smL = kHdrBytes + (size_t)st.L.window_bytes + st.L.ring_bytes;
    const size_t smU = kHdrBytes + (size_t)st.U.window_bytes + st.U.ring_bytes;
    kl<<<grid, (wL + 2) * 32, smL, s>>>(stage_args<T>(st.L, st.rhsL.p, recU, wL, st.rs));
    ku<<<grid, (wU + 2) * 32, smU, s>>>(stage_args<T>(st.U, st.rhsU.p, z, wU, st.rs));
    note_launches(3);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

template <class T, int Q, int S>
int launch_rows(const DevIlu& F, const IluStage& st, const double* dAinv, const T* v, T* z,
                cudaStream_t s)
{
    static std::atomic<bool> attr{false};
    return run_stage<T, Q>(F, st, 32 / (F.L.g * S), k_tri_stage<T, Q, S, false>,
                           k_tri_stage<T, Q, S, true>, attr, dAinv, v, z, s);
}

template <int Q, int H, int NPC = Q / 2>
int launch_blocks(const DevIlu& F, const IluStage& st, const double* dAinv, const float* v,
                  float* z, cudaStream_t s)
{
    static std::atomic<bool> attr{false};
    return run_stage<float, Q>(F, st, BlockBody<Q, H, false, NPC>::GPW,
                               k_tri_block<Q, H, false, NPC>, k_tri_block<Q, H, true, NPC>, attr,
                               dAinv, v, z, s, Q / 2 / NPC);
}

template <int Q, int H>
int launch_cols(const DevIlu& F, const IluStage& st, const double* dAinv, const float* v, float* z,
                cudaStream_t s)
{
    static std::atomic<bool> attr{false};
    return run_stage<float, Q>(F, st, ColBody<Q, H, false>::GPW, k_tri_col<Q, H, false>,
                               k_tri_col<Q, H, true>, attr, dAinv, v, z, s, Q / 2);
}

template <int Q, int H>
int launch_cols1(const DevIlu& F, const IluStage& st, const double* dAinv, const float* v,
                 float* z, cudaStream_t s)
{
    static std::atomic<bool> attr{false};
    return run_stage<float, Q>(F, st, ColBody1<Q, H, false>::GPW, k_tri_col1<Q, H, false>,
                               k_tri_col1<Q, H, true>, attr, dAinv, v, z, s, Q);
}

template <class T, int Q>
int launch_tri(const DevIlu& F, const double* dAinv, const T* v, T* z, T* work, cudaStream_t s,
               const int* skip)
{
    IluStage* st = nullptr;
    // 4 (default): rows with register-prefetched records, one temporal
    // block per thread block; 3: column records through a TMA ring, one
    // temporal block per thread block; 2: column records, one pair per
    // thread block; 1: node blocks; 0: rows through the ring.  A format
    // that cannot be laid out for the factor falls back to the next.
    int fmt = env_int("XTFEM_ILU_FMT", 4);
    if constexpr (sizeof(T) == 4) {
        if (F.L.g == 3 && fmt == 4) {
            const int H = F.shares > 0 ? F.shares : env_int("XTFEM_ILU_SHARES", 2);
            XT_TRY(get_stage<T>(F, Q, 4, s, st, H));
            if (st) return launch_reg_any<Q>(*st, dAinv, v, z, s, skip);
            fmt = 3;
        }
    }
    if constexpr (sizeof(T) == 4 && Q % 2 == 0) {
        if (F.L.g == 3 && fmt == 3) {
            const int H = env_int("XTFEM_ILU_SHARES", 2) == 1 ? 1 : 2;
            XT_TRY(get_stage<T>(F, Q, 3, s, st, H));
            if (st) {
                if (H == 1) return launch_cols1<Q, 1>(F, *st, dAinv, v, z, s);
                return launch_cols1<Q, 2>(F, *st, dAinv, v, z, s);
            }
        }
        if (F.L.g == 3 && fmt == 2) {
            const int H = env_int("XTFEM_ILU_SHARES", 1) == 2 ? 2 : 1;
            XT_TRY(get_stage<T>(F, Q, 2, s, st, H));
            if (st) {
                if (H == 1) return launch_cols<Q, 1>(F, *st, dAinv, v, z, s);
                return launch_cols<Q, 2>(F, *st, dAinv, v, z, s);
            }
        }
        if (F.L.g == 3 && fmt >= 1) {
            XT_TRY(get_stage<T>(F, Q, 1, s, st));
            if (st) {
                const int H = env_int("XTFEM_ILU_SHARES", 2);
                if constexpr (Q == 6) {
                    // thread blocks per sweep: 3 (default, one temporal-block
                    // pair each) or 1 (all pairs in one block)
                    if (env_int("XTFEM_ILU_SPLIT", 3) == 3) {
                        if (H == 1) return launch_blocks<Q, 1, 1>(F, *st, dAinv, v, z, s);
                        if (H == 4) return launch_blocks<Q, 4, 1>(F, *st, dAinv, v, z, s);
                        if (H == 8) return launch_blocks<Q, 8, 1>(F, *st, dAinv, v, z, s);
                        return launch_blocks<Q, 2, 1>(F, *st, dAinv, v, z, s);
                    }
                    if (H == 1) return launch_blocks<Q, 1>(F, *st, dAinv, v, z, s);
                    if (H == 4) return launch_blocks<Q, 4>(F, *st, dAinv, v, z, s);
                }
                return launch_blocks<Q, 2>(F, *st, dAinv, v, z, s);
            }
        }
    }
    if (F.L.g <= kMaxG) XT_TRY(get_stage<T>(F, Q, 0, s, st));
    if (!st) return launch_tri_simple<T, Q>(F, dAinv, v, z, work, s);
    if constexpr (Q == 6) {
        const int S = env_int("XTFEM_ILU_LANES", 2);
        if (S == 1) return launch_rows<T, Q, 1>(F, *st, dAinv, v, z, s);
        if (S == 4) return launch_rows<T, Q, 4>(F, *st, dAinv, v, z, s);
    }
    return launch_rows<T, Q, 2>(F, *st, dAinv, v, z, s);
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
    XT_TRY(d.ext_col.upload(ne ? h.ext_col.data() : nullptr, ne, s));
    XT_TRY(d.ext_v64.upload(h.ext_v.data(), ne, s));
    XT_TRY(d.ext_v32.upload(f32.data(), ne, s));
    XT_TRY(d.int_v64.upload(h.int_v.data(), h.int_v.size(), s));
    XT_TRY(d.int_v32.upload(i32.data(), i32.size(), s));
    if (!h.dinv.empty()) {
        XT_TRY(d.dinv64.upload(h.dinv.data(), h.dinv.size(), s));
        XT_TRY(d.dinv32.upload(d32.data(), d32.size(), s));
    }
    XT_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
    return XT_OK;
}

// ---------------------------------------------------------------------------
// Batches of systems (the lockstep batch's step graph): the register
// sweeps of many systems in one launch per group of equal kernel shape.

// The pre-pass of k_rhs_slots for table entry blockIdx.y, its input the hi
// part of the entry's basis column j (what the per-system step copies into
// the ILU input first): the same products in the same order.
template <int Q>
__global__ void kb_rhs_slots(const FlexStepItem* __restrict__ t)
{
    __shared__ float sA[Q * Q];
    const FlexStepItem& e = t[blockIdx.y];
    const int* ctl = e.ctl;
    if (ctl[1] != 0) return;
    for (int i = threadIdx.x; i < Q * Q; i += blockDim.x) sA[i] = (float)e.Ainv[i];
    __syncthreads();
    const float2* col = e.V + (size_t)ctl[0] * (size_t)e.nl;
    const long long lanes = e.lanes;
    const int* src = e.src;
    float* rhs = e.rrhs;
    for (long long tt = blockIdx.x * (long long)blockDim.x + threadIdx.x; tt < lanes;
         tt += (long long)gridDim.x * blockDim.x) {
        const int row = src[tt];
        float vr[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j) vr[j] = row >= 0 ? col[(size_t)row * Q + j].x : 0.0f;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            float b = 0.0f;
#pragma unroll
            for (int j = 0; j < Q; ++j) b = fmaf(sA[j * Q + q], vr[j], b);
            rhs[(size_t)q * lanes + tt] = b;
        }
    }
}

}  // namespace

int flexb_rhs(const FlexStepItem* t, int count, int q, long long lanes_max, cudaStream_t s)
{
    if (count <= 0) return XT_OK;
    const long long bx = std::max(1LL, std::min(4096LL, (lanes_max + 1023) / 1024));
    const dim3 grid((unsigned)bx, (unsigned)count);
    switch (q) {
    case 1: kb_rhs_slots<1><<<grid, 256, 0, s>>>(t); break;
    case 2: kb_rhs_slots<2><<<grid, 256, 0, s>>>(t); break;
    case 3: kb_rhs_slots<3><<<grid, 256, 0, s>>>(t); break;
    case 4: kb_rhs_slots<4><<<grid, 256, 0, s>>>(t); break;
    case 5: kb_rhs_slots<5><<<grid, 256, 0, s>>>(t); break;
    case 6: kb_rhs_slots<6><<<grid, 256, 0, s>>>(t); break;
    case 7: kb_rhs_slots<7><<<grid, 256, 0, s>>>(t); break;
    case 8: kb_rhs_slots<8><<<grid, 256, 0, s>>>(t); break;
    default: set_error("flexb_rhs: 1 <= q <= 8"); return XT_ERR_ARG;
    }
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

namespace {
// The (shares, steps) pairs the register sweep has kernels for (as
// launch_reg_any dispatches them).
bool reg_pair_ok(int H, int smax)
{
    return (H == 2 && (smax == 8 || smax == 12 || smax == 16)) || (H == 1 && (smax == 12 || smax == 20)) ||
           (H == 4 && smax == 8);
}

template <int H, int SMAX>
int reg_group_hs(const RegGroup& g, int q, cudaStream_t s, bool prepare)
{
    const RegArgs* a = reinterpret_cast<const RegArgs*>(g.args.p);
    auto kernel = g.upper ? (g.w16 ? k_tri_reg_parts<H, SMAX, true, true> : k_tri_reg_parts<H, SMAX, true, false>)
                          : (g.w16 ? k_tri_reg_parts<H, SMAX, false, true> : k_tri_reg_parts<H, SMAX, false, false>);
    if (prepare) {
        XT_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem()));
        return XT_OK;
    }
    const int pf = std::max(0, std::min(64, env_int("XTFEM_ILU_PF", 8)));
    kernel<<<q * g.count, g.ncw * 32, g.smem, s>>>(a, q, pf, nullptr, nullptr);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int reg_group_any(const RegGroup& g, int q, cudaStream_t s, bool prepare)
{
    if (g.count < 1 || g.ncw < 1 || g.ncw > kRegMaxWarps || (long long)q * g.count > INT32_MAX ||
        g.smem > (size_t)max_dyn_smem() || !g.args.p) {
        set_error("register sweep group: bad shape");
        return XT_ERR_ARG;
    }
    if (g.H == 2 && g.smax == 8) return reg_group_hs<2, 8>(g, q, s, prepare);
    if (g.H == 2 && g.smax == 12) return reg_group_hs<2, 12>(g, q, s, prepare);
    if (g.H == 2 && g.smax == 16) return reg_group_hs<2, 16>(g, q, s, prepare);
    if (g.H == 1 && g.smax == 12) return reg_group_hs<1, 12>(g, q, s, prepare);
    if (g.H == 1 && g.smax == 20) return reg_group_hs<1, 20>(g, q, s, prepare);
    if (g.H == 4 && g.smax == 8) return reg_group_hs<4, 8>(g, q, s, prepare);
    set_error("register sweep group: no kernel for these shares and steps");
    return XT_ERR_ARG;
}
}  // namespace

int ilu_reg_entry(const DevIlu& F, int q, float* z, const int* skip, cudaStream_t s,
                  IluRegEntry& e)
{
    e = IluRegEntry{};
    // the apply launch_tri would run: FP32, register sweep, one row block
    if (F.L.g != 3 || env_int("XTFEM_ILU_FMT", 4) != 4 || q < 1 || q > 8) return XT_OK;
    const int H = F.shares > 0 ? F.shares : env_int("XTFEM_ILU_SHARES", 2);
    IluStage* st = nullptr;
    XT_TRY(get_stage<float>(F, q, 4, s, st, H));
    if (!st || !st->reg_ok || st->parts > 1 || !st->regL || !st->regU) return XT_OK;
    const RegTri& L = *st->regL;
    const RegTri& U = *st->regU;
    if (L.w16 != U.w16 || L.H != U.H || L.smax != U.smax || !reg_pair_ok(L.H, L.smax)) return XT_OK;
    const int pf = std::max(0, std::min(64, env_int("XTFEM_ILU_PF", 8)));
    e.src = st->srcL.p;
    e.lanes = L.lanes;
    e.rrhs = st->rrhsL.p;
    e.H = L.H;
    e.smax = L.smax;
    e.w16 = L.w16 ? 1 : 0;
    e.L = RegArgs{L.slots.p, st->rrhsL.p, st->rrhsU.p, L.lanes, U.lanes, L.nl, L.ncw,
                  L.slot_bytes, L.zero_off, pf, skip};
    e.U = RegArgs{U.slots.p, st->rrhsU.p, z, U.lanes, 0, U.nl, U.ncw, U.slot_bytes, U.zero_off,
                  pf, skip};
    e.smemL = (size_t)L.win_elems * 4;
    e.smemU = (size_t)U.win_elems * 4;
    e.ok = true;
    return XT_OK;
}

int reg_group_prepare(const RegGroup& g) { return reg_group_any(g, 1, nullptr, true); }

int reg_group_launch(const RegGroup& g, int q, cudaStream_t s)
{
    return reg_group_any(g, q, s, false);
}

namespace {
// The rows [r0, r1) of a 1-based MSR factor with no entry outside them, as
// a factor of their own (local 1-based indices).
void sub_factor(const double* alu, const int* jlu, const int* ju, int r0, int r1,
                std::vector<double>& a, std::vector<int>& jl, std::vector<int>& jd)
{
    const int m = r1 - r0;
    a.assign((size_t)m + 1, 0.0);
    jl.assign((size_t)m + 1, 0);
    jd.assign((size_t)m, 0);
    for (int r = 0; r < m; ++r) a[r] = alu[r0 + r];
    jl[0] = m + 2;
    for (int r = 0; r < m; ++r) {
        const int gr = r0 + r;
        for (int k = jlu[gr] - 1; k < jlu[gr + 1] - 1; ++k) {
            if (k == ju[gr] - 1) jd[r] = (int)jl.size() + 1;
            a.push_back(alu[k]);
            jl.push_back(jlu[k] - r0);
        }
        if (ju[gr] == jlu[gr + 1]) jd[r] = (int)jl.size() + 1;  // no U part
        jl[r + 1] = (int)jl.size() + 1;
    }
}
}  // namespace

int build_ilu(DevIlu& d, int n, const double* alu, const int* jlu, const int* ju, int group,
              cudaStream_t s, int blocks)
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
    auto sc = std::make_shared<IluSched>();
    XT_TRY(side_by_side([&] { sc->U = schedule(n, alu, jlu, ju, g, true); return XT_OK; },
                        [&] { sc->L = schedule(n, alu, jlu, ju, g, false); return XT_OK; }));
    XT_TRY(upload_tri(d.L, sc->L, s));
    XT_TRY(upload_tri(d.U, sc->U, s));
    d.sched = sc;
    d.stages.clear();
    d.blocks = 1;
    d.bounds.clear();
    d.part_sched.clear();
    if (blocks > 1) {
        const std::vector<int> bd = ilu_block_bounds(n, g, blocks);
        const int nb = (int)bd.size() - 1;
        bool diag = nb > 1;
        for (int b = 0; diag && b < nb; ++b)
            for (int r = bd[b]; diag && r < bd[b + 1]; ++r)
                for (int k = jlu[r] - 1; k < jlu[r + 1] - 1; ++k) {
                    const int c = jlu[k] - 1;
                    if (c < bd[b] || c >= bd[b + 1]) {
                        diag = false;
                        break;
                    }
                }
        if (diag) {
            std::vector<double> a;
            std::vector<int> jl, jd;
            for (int b = 0; b < nb; ++b) {
                sub_factor(alu, jlu, ju, bd[b], bd[b + 1], a, jl, jd);
                auto ps = std::make_shared<IluSched>();
                const int m = bd[b + 1] - bd[b];
                ps->L = schedule(m, a.data(), jl.data(), jd.data(), g, false);
                ps->U = schedule(m, a.data(), jl.data(), jd.data(), g, true);
                d.part_sched.push_back(ps);
            }
            d.blocks = nb;
            d.bounds = bd;
        }
    }
    return XT_OK;
}

template <class T>
int ilu_apply(const DevIlu& F, int q, const double* dAinv, const T* v, T* z, T* work,
              cudaStream_t s, const int* skip)
{
    switch (q) {
    case 1: return launch_tri<T, 1>(F, dAinv, v, z, work, s, skip);
    case 2: return launch_tri<T, 2>(F, dAinv, v, z, work, s, skip);
    case 3: return launch_tri<T, 3>(F, dAinv, v, z, work, s, skip);
    case 4: return launch_tri<T, 4>(F, dAinv, v, z, work, s, skip);
    case 5: return launch_tri<T, 5>(F, dAinv, v, z, work, s, skip);
    case 6: return launch_tri<T, 6>(F, dAinv, v, z, work, s, skip);
    case 7: return launch_tri<T, 7>(F, dAinv, v, z, work, s, skip);
    case 8: return launch_tri<T, 8>(F, dAinv, v, z, work, s, skip);
    default:
        set_error("ilu_apply: 1 <= q <= 8");
        return XT_ERR_ARG;
    }
}

template int ilu_apply<double>(const DevIlu&, int, const double*, const double*, double*,
                               double*, cudaStream_t, const int*);
template int ilu_apply<float>(const DevIlu&, int, const double*, const float*, float*, float*,
                              cudaStream_t, const int*);

int ilu_check(cudaStream_t s)
{
    int h = 0;
    XT_CUDA(cudaMemcpyFromSymbolAsync(&h, g_ilu_error, sizeof(int), 0, cudaMemcpyDeviceToHost, s));
    XT_CUDA(cudaStreamSynchronize(s));
    if (h != 0) {
        const int zero = 0;
        XT_CUDA(cudaMemcpyToSymbolAsync(g_ilu_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s));
        XT_CUDA(cudaStreamSynchronize(s));
        set_error(h == 1 ? "ILU sweep: wait for a level's data gave up"
                         : "ILU sweep: producer wait for a consumed level gave up");
        return XT_ERR_CUDA;
    }
    return XT_OK;
}

}  // namespace xt
