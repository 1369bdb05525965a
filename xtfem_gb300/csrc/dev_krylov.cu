// dev_krylov.cu -- vector kernels of the restarted GMRES on the GPU.
//
// The reference orthogonalises each new Krylov vector with modified
// Gram-Schmidt, one ddot + daxpy pair per basis vector (src/kronecker.f90:
// 277-285), i.e. 2j dependent passes over n values at step j.  Here the
// projection is classical Gram-Schmidt applied twice (CGS2), which is as
// stable as MGS in exact terms and needs only four passes over the basis
// per step with no dependency between the basis vectors inside a pass:
//   h1 = V^T w ; w -= V h1 ; h2 = V^T w ; w -= V h2 ; ||w||.
// Every dot product accumulates in FP64 whatever the storage type of the
// basis, and reductions are two-stage with a fixed order so results are
// bitwise repeatable run to run.
#include "df.cuh"
#include "xt_device.h"

#include <algorithm>

namespace xt {

namespace {

constexpr int kThreads = 256;
constexpr int kRowBlocks = 296;  // 2 per SM on a 148-152 SM part
constexpr int kChunk = 8;        // basis vectors per block in a dot pass

__device__ __forceinline__ double block_sum(double v, double* sh)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += sh[w];
    return r;  // valid in thread 0
}

// partial[j * nb + b] = sum over block b's rows of V_j[r] * w[r]
template <class TV>
__global__ void k_multi_dot(const TV* __restrict__ V, size_t ld, int k, const TV* __restrict__ w,
                            size_t n, double* __restrict__ partial)
{
    __shared__ double sh[32];
    const int j0 = blockIdx.y * kChunk;
    const int nb = gridDim.x;
    const size_t per = (n + nb - 1) / nb;
    const size_t r0 = per * blockIdx.x, r1 = min(n, r0 + per);
    double acc[kChunk];
#pragma unroll
    for (int c = 0; c < kChunk; ++c) acc[c] = 0.0;
    for (size_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const double wr = (double)w[r];
#pragma unroll
        for (int c = 0; c < kChunk; ++c)
            if (j0 + c < k) acc[c] = fma((double)V[(size_t)(j0 + c) * ld + r], wr, acc[c]);
    }
    for (int c = 0; c < kChunk && j0 + c < k; ++c) {
        const double s = block_sum(acc[c], sh);
        if (threadIdx.x == 0) partial[(size_t)(j0 + c) * nb + blockIdx.x] = s;
    }
}

// FP32 basis (n and ld even, pairs of rows): each pair of products is
// formed in FP32 and accumulated in double-float, reduced across the block
// in double-float; the block's (hi, lo) pair is stored in the FP64 partial
// slot and k_finish_df adds the pairs in FP64.  The part's FP64 rate is
// 1/64 of its FP32 rate, so no FP64 instruction is issued per element.
__global__ void k_multi_dot_f32(const float2* __restrict__ V, size_t ld2, int k,
                                const float2* __restrict__ w, size_t n2,
                                double* __restrict__ partial)
{
    __shared__ float2 sh[kChunk][32];
    const int j0 = blockIdx.y * kChunk;
    const int nb = gridDim.x;
    const size_t per = (n2 + nb - 1) / nb;
    const size_t r0 = per * blockIdx.x, r1 = min(n2, r0 + per);
    float hi[kChunk], lo[kChunk];
#pragma unroll
    for (int c = 0; c < kChunk; ++c) hi[c] = lo[c] = 0.0f;
    for (size_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const float2 wr = w[r];
        float2 v[kChunk];
#pragma unroll
        for (int c = 0; c < kChunk; ++c)
            v[c] = (j0 + c < k) ? V[(size_t)(j0 + c) * ld2 + r] : make_float2(0.0f, 0.0f);
#pragma unroll
        for (int c = 0; c < kChunk; ++c) df_add(hi[c], lo[c], fmaf(v[c].y, wr.y, v[c].x * wr.x));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < kChunk; ++c) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, hi[c], off);
            const float ol = __shfl_xor_sync(0xffffffffu, lo[c], off);
            df_add_df(hi[c], lo[c], oh, ol);
        }
        if (lane == 0) sh[c][warp] = make_float2(hi[c], lo[c]);
    }
    __syncthreads();
    if (threadIdx.x < kChunk && j0 + (int)threadIdx.x < k) {
        const int c = threadIdx.x;
        float h = 0.0f, l = 0.0f;
        for (int wi = 0; wi < nw; ++wi) df_add_df(h, l, sh[c][wi].x, sh[c][wi].y);
        reinterpret_cast<float2*>(partial)[(size_t)(j0 + c) * nb + blockIdx.x] = make_float2(h, l);
    }
}

// ---------------------------------------------------------------------------
// Double-float vectors: one float2 (hi, lo) per entry, value hi + lo with
// |lo| <= ulp(hi)/2 (about 48 significant bits).  The flexible GMRES keeps
// its FP64-accurate Krylov basis in this form: the same bytes as FP64, but
// every operation runs on the FP32 pipe.

// Row blocks per chunk of kChunk basis vectors in a double-float dot pass:
// one wave of the six blocks per SM that the pass's registers allow, over
// all chunks (row blocks shrink as k grows, so each block's rows outweigh
// its block reduction).  Eight per SM made 1.34 waves (ncu).  The wave is
// sized for 148 of the 152 SMs: a few SMs may hold a long-running block of
// the damage update on the side stream, and a pass sized for every SM
// would leave its last blocks a second wave.
__host__ __device__ __forceinline__ int df_dot_blocks(int k, int nblocks)
{
    const int nchunk = (k + kChunk - 1) / kChunk;
    const int b = (6 * 148) / nchunk;
    const int lo = nblocks < 24 ? nblocks : 24;
    return b < lo ? lo : (b < nblocks ? b : nblocks);
}

// Row blocks of the double-float dot and norm passes of a vector of n2
// entry pairs: one 512-row slice per block up to kRowBlocks (a system of
// fewer than kRowBlocks * 512 pairs gets no empty blocks, so a batch of
// small systems is not a batch of mostly idle grids).  The norm pass's
// partial sums are those of the kRowBlocks grid bit for bit: the blocks
// dropped held no rows, and their zero partials added nothing.
__host__ __device__ __forceinline__ int df_row_blocks(long long n2, int nblocks)
{
    const long long b = (n2 + 511) / 512;
    return b < 1 ? 1 : (b < nblocks ? (int)b : nblocks);
}

// Row blocks of the dot pass: those of the norm pass for a system of at
// least kRowBlocks 512-row slices; a smaller system's row blocks hold 2048
// rows or more (the pass per basis chunk would otherwise be a few hundred
// rows per block, all block reduction and partial sums).
__host__ __device__ __forceinline__ int df_dot_rows(long long n2, int nblocks)
{
    const int b = df_row_blocks(n2, nblocks);
    if (b >= nblocks) return nblocks;
    const long long d = (n2 + 2047) / 2048;
    return d < 1 ? 1 : (int)d;
}

// Blocks of a device-driven dot pass: the most any k <= im asks for with
// nb row blocks (blocks past the step's own count return at once).
inline int df_dot_grid(int im, int nb)
{
    int grid = 1;
    for (int k = 1; k <= im; ++k)
        grid = std::max(grid, df_dot_blocks(k, nb) * ((k + kChunk - 1) / kChunk));
    return grid;
}

// partial[(j0+c) nb + b] = (hi, lo) of sum over row block rb's rows of V_j w
__device__ __forceinline__ void multi_dot_df_body(const float4* __restrict__ V, size_t ld2, int k,
                                                  const float4* __restrict__ w, size_t n2,
                                                  double* __restrict__ partial, int rb, int nb,
                                                  int chunk)
{
    __shared__ float2 sh[kChunk][32];
    const int j0 = chunk * kChunk;
    const size_t per = (n2 + nb - 1) / nb;
    const size_t r0 = per * rb, r1 = min(n2, r0 + per);
    float hi[kChunk], lo[kChunk];
#pragma unroll
    for (int c = 0; c < kChunk; ++c) hi[c] = lo[c] = 0.0f;
    for (size_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const float4 wr = w[r];  // two entries: (hi, lo), (hi, lo)
        float4 v[kChunk];
#pragma unroll
        for (int c = 0; c < kChunk; ++c)
            v[c] = (j0 + c < k) ? V[(size_t)(j0 + c) * ld2 + r] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int c = 0; c < kChunk; ++c) {
            df_mul_acc(hi[c], lo[c], v[c].x, v[c].y, wr.x, wr.y);
            df_mul_acc(hi[c], lo[c], v[c].z, v[c].w, wr.z, wr.w);
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < kChunk; ++c) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, hi[c], off);
            const float ol = __shfl_xor_sync(0xffffffffu, lo[c], off);
            df_add_df(hi[c], lo[c], oh, ol);
        }
        if (lane == 0) sh[c][warp] = make_float2(hi[c], lo[c]);
    }
    __syncthreads();
    if (threadIdx.x < kChunk && j0 + (int)threadIdx.x < k) {
        const int c = threadIdx.x;
        float h = 0.0f, l = 0.0f;
        for (int wi = 0; wi < nw; ++wi) df_add_df(h, l, sh[c][wi].x, sh[c][wi].y);
        reinterpret_cast<float2*>(partial)[(size_t)(j0 + c) * nb + rb] = make_float2(h, l);
    }
}

__global__ void __launch_bounds__(256, 6) k_multi_dot_df(const float4* __restrict__ V, size_t ld2, int k,
                               const float4* __restrict__ w, size_t n2,
                               double* __restrict__ partial)
{
    multi_dot_df_body(V, ld2, k, w, n2, partial, blockIdx.x, gridDim.x, blockIdx.y);
}

// The same pass with k = ctl[0] + 1 read on the device (a step of the
// device-driven GMRES; nothing to do once ctl[1] is set): block b takes row
// block b mod nb of chunk b / nb, nb as the host launch would choose it,
// so the partial sums are those of k_multi_dot_df bit for bit.
__global__ void __launch_bounds__(256, 6) k_multi_dot_df_ctl(const float4* __restrict__ V, size_t ld2,
                               const float4* __restrict__ w, size_t n2,
                               double* __restrict__ partial, int nblocks,
                               const int* __restrict__ ctl)
{
    if (ctl[1] != 0) return;
    const int k = ctl[0] + 1;
    const int nb = df_dot_blocks(k, nblocks), nchunk = (k + kChunk - 1) / kChunk;
    const int chunk = blockIdx.x / nb;
    if (chunk >= nchunk) return;
    multi_dot_df_body(V, ld2, k, w, n2, partial, blockIdx.x - chunk * nb, nb, chunk);
}

// (wh, wl) -= (hh + hl)(vh + vl)
__device__ __forceinline__ void df_sub_mul(float& wh, float& wl, float hh, float hl, float vh,
                                           float vl)
{
    const float p = __fmul_rn(hh, vh);
    const float e = fmaf(hh, vh, -p);
    df_add(wh, wl, -p);
    wl = __fsub_rn(wl, __fadd_rn(e, fmaf(hh, vl, __fmul_rn(hl, vh))));
}

// w -= V h on double-float vectors (two entries per float4); optional
// ||w||^2 as a (hi, lo) partial per block.  This thread block is block bx
// of a gx-block pass (a batched launch runs one such pass per system).
template <bool NORM>
__device__ __forceinline__ void update_df_body(const float4* __restrict__ V, size_t ld2, int k,
                                               const double* __restrict__ h,
                                               float4* __restrict__ w, size_t n2,
                                               double* __restrict__ partial, int bx, int gx)
{
    __shared__ float2 hs[512];
    __shared__ float2 sh[32];
    for (int j = threadIdx.x; j < k && j < 512; j += blockDim.x) {
        const float a = (float)h[j];
        hs[j] = make_float2(a, (float)(h[j] - (double)a));
    }
    __syncthreads();
    float nh = 0.0f, nl = 0.0f;
    const size_t stride = (size_t)gx * blockDim.x;
    for (size_t r = (size_t)bx * blockDim.x + threadIdx.x; r < n2; r += stride) {
        const float4 wv = w[r];
        float ah = wv.x, al = wv.y, bh = wv.z, bl = wv.w;
        for (int jb = 0; jb < k; jb += 8) {
            float4 v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u)
                v[u] = (jb + u < k) ? V[(size_t)(jb + u) * ld2 + r] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int j = jb + u;
                if (j >= k) break;
                float2 hj;
                if (j < 512) hj = hs[j];
                else {
                    const float a = (float)h[j];
                    hj = make_float2(a, (float)(h[j] - (double)a));
                }
                df_sub_mul(ah, al, hj.x, hj.y, v[u].x, v[u].y);
                df_sub_mul(bh, bl, hj.x, hj.y, v[u].z, v[u].w);
            }
        }
        const float2 a2 = df_norm(ah, al), b2 = df_norm(bh, bl);
        w[r] = make_float4(a2.x, a2.y, b2.x, b2.y);
        if (NORM) {
            df_mul_acc(nh, nl, a2.x, a2.y, a2.x, a2.y);
            df_mul_acc(nh, nl, b2.x, b2.y, b2.x, b2.y);
        }
    }
    if (NORM) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, nh, off);
            const float ol = __shfl_xor_sync(0xffffffffu, nl, off);
            df_add_df(nh, nl, oh, ol);
        }
        if (lane == 0) sh[warp] = make_float2(nh, nl);
        __syncthreads();
        if (threadIdx.x == 0) {
            float hh = 0.0f, ll = 0.0f;
            for (int wi = 0; wi < nw; ++wi) df_add_df(hh, ll, sh[wi].x, sh[wi].y);
            reinterpret_cast<float2*>(partial)[bx] = make_float2(hh, ll);
        }
    }
}

template <bool NORM>
__global__ void k_update_df(const float4* __restrict__ V, size_t ld2, int k,
                            const double* __restrict__ h, float4* __restrict__ w, size_t n2,
                            double* __restrict__ partial, const int* __restrict__ ctl)
{
    if (ctl) {  // device-driven step: k = ctl[0] + 1, nothing once ctl[1] is set
        if (ctl[1] != 0) return;
        k = ctl[0] + 1;
    }
    update_df_body<NORM>(V, ld2, k, h, w, n2, partial, blockIdx.x, gridDim.x);
}

// y = (hi, lo) split of x; y = hi part only; y = a * y (a FP64, split)
__global__ void k_df_from_f64(const double* __restrict__ x, float2* __restrict__ y, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double v = x[i];
        const float h = __double2float_rn(v);
        y[i] = make_float2(h, __double2float_rn(v - (double)h));
    }
}
__global__ void k_df_hi(const float2* __restrict__ x, float* __restrict__ y, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        y[i] = x[i].x;
}
__global__ void k_df_to_f64(const float2* __restrict__ x, double* __restrict__ y, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        y[i] = (double)x[i].x + (double)x[i].y;
}
__global__ void k_df_scale(float2* __restrict__ y, float ah, float al, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float2 v = y[i];
        float h = 0.0f, l = 0.0f;
        df_mul_acc(h, l, v.x, v.y, ah, al);
        y[i] = df_norm(h, l);
    }
}
// k_df_scale, and the hi part of the result into hi (the next ILU input)
__global__ void k_df_scale_hi(float2* __restrict__ y, float ah, float al, float* __restrict__ hi,
                              size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float2 v = y[i];
        float h = 0.0f, l = 0.0f;
        df_mul_acc(h, l, v.x, v.y, ah, al);
        const float2 r = df_norm(h, l);
        y[i] = r;
        hi[i] = r.x;
    }
}

// out[j] = sum_b (hi_b + lo_b) in FP64, one block per j, fixed order
__global__ void k_finish_df(const double* __restrict__ partial, int nb, double* __restrict__ out)
{
    __shared__ double sh[32];
    const int j = blockIdx.x;
    const float2* p = reinterpret_cast<const float2*>(partial) + (size_t)j * nb;
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) v += (double)p[b].x + (double)p[b].y;
    const double s = block_sum(v, sh);
    if (threadIdx.x == 0) out[j] = s;
}

// k_finish_df for a device-driven step: dot mode (norm == 0) sums the
// k = ctl[0] + 1 dots of the last k_multi_dot_df_ctl pass (block j < k),
// norm mode sums the nblocks partials of k_update_df<true> (block 0).
__device__ __forceinline__ void finish_df_ctl_body(const double* __restrict__ partial, int nblocks,
                                                   double* __restrict__ out,
                                                   const int* __restrict__ ctl, int norm, int j)
{
    __shared__ double sh[32];
    if (ctl[1] != 0) return;
    const int k = ctl[0] + 1;
    if (norm ? j > 0 : j >= k) return;
    const int nb = norm ? nblocks : df_dot_blocks(k, nblocks);
    const float2* p = reinterpret_cast<const float2*>(partial) + (size_t)j * nb;
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) v += (double)p[b].x + (double)p[b].y;
    const double sum = block_sum(v, sh);
    if (threadIdx.x == 0) out[j] = sum;
}

__global__ void k_finish_df_ctl(const double* __restrict__ partial, int nblocks,
                                double* __restrict__ out, const int* __restrict__ ctl, int norm)
{
    finish_df_ctl_body(partial, nblocks, out, ctl, norm, blockIdx.x);
}

// ---------------------------------------------------------------------------
// Device-driven flexible GMRES (solver.cpp, gmres_flex_dev): the Arnoldi
// step's bookkeeping on the device.  ctl = {j, status, its, maxits}: j is
// the step's input basis column, status 0 while the cycle runs (1 once it
// has ended: converged, restart length or maxits reached; 4 on a
// non-finite vector).  Every kernel that indexes by j does nothing once the
// status is set, so steps issued past the end of a cycle cost only their
// launches.  st holds the Hessenberg matrix, the rotations, rs, the two
// projections, the squared norm and the scalars (FlexLayout).

__global__ void k_flexd_hi(const int* __restrict__ ctl, const float2* __restrict__ V, size_t nl,
                           float* __restrict__ d, size_t n)
{
    if (ctl[1] != 0) return;
    const float2* col = V + (size_t)ctl[0] * nl;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) d[i] = col[i].x;
}

__global__ void k_flexd_zcopy(const int* __restrict__ ctl, const float* __restrict__ z,
                              float* __restrict__ Z, size_t n)
{
    if (ctl[1] != 0) return;
    float* col = Z + (size_t)ctl[0] * n;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) col[i] = z[i];
}

// The Hessenberg column of step i = j + 1 from the two projections and the
// norm, the previous rotations, the new rotation, rs, the convergence test
// -- the arithmetic of the host loop of gmres_flex (src/kronecker.f90:286-312
// in the reference), in the same order and without contraction, so that both
// drivers give the same bits.  The rotations are one dependent chain: the
// block stages the column and the rotations in shared memory (kFlexdMaxIm + 1
// entries each), one thread runs the chain from there, and the block writes
// the column back.
constexpr int kGivensMax = kFlexdMaxIm;

__device__ __forceinline__ void flexd_givens_body(int* __restrict__ ctl, double* __restrict__ st,
                                                  int im)
{
    __shared__ double col[kGivensMax + 1], out[kGivensMax + 1], cs[kGivensMax], sn[kGivensMax];
    __shared__ int bad;
    if (ctl[1] != 0) return;  // the same for every thread of the block
    const FlexLayout Lo(im);
    const int i = ctl[0] + 1;
    for (int jj = threadIdx.x; jj < i; jj += blockDim.x) {
        col[jj] = __dadd_rn(st[Lo.h1 + jj], st[Lo.h2 + jj]);
        if (jj < i - 1) {
            cs[jj] = st[Lo.cs + jj];
            sn[jj] = st[Lo.sn + jj];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = sqrt(st[Lo.nrm]);
        bad = !isfinite(t);
        if (!bad) {
            col[i] = t;
            st[Lo.tinv] = (t != 0.0) ? 1.0 / t : 0.0;
            // rotation k1 = k - 1 maps entries (k1 - 1, k - 1); the carry is
            // the rotated entry k - 1, which the next rotation takes as t
            double carry = col[0];
            for (int k = 2; k <= i; ++k) {
                const double c = cs[k - 2], s = sn[k - 2], h = col[k - 1];
                out[k - 2] = __dadd_rn(__dmul_rn(c, carry), __dmul_rn(s, h));
                carry = __dadd_rn(__dmul_rn(-s, carry), __dmul_rn(c, h));
            }
            const double hd = carry, hs = t;
            double gam = sqrt(__dadd_rn(__dmul_rn(hd, hd), __dmul_rn(hs, hs)));
            if (gam == 0.0) gam = 1.0e-16;
            const double cn = hd / gam, snn = hs / gam;
            st[Lo.cs + i - 1] = cn;
            st[Lo.sn + i - 1] = snn;
            double* rs = st + Lo.rs;
            const double r = rs[i - 1];
            rs[i] = __dmul_rn(-snn, r);
            rs[i - 1] = __dmul_rn(cn, r);
            out[i - 1] = __dadd_rn(__dmul_rn(cn, hd), __dmul_rn(snn, hs));
            out[i] = hs;
            const double ro = fabs(rs[i]);
            st[Lo.ro] = ro;
            const int its = ctl[2] + 1;
            ctl[2] = its;
            ctl[0] = i;
            if (!(i < im && ro > st[Lo.eps1] && its < ctl[3])) ctl[1] = 1;
        } else {
            ctl[1] = 4;
        }
    }
    __syncthreads();
    if (bad) return;
    double* hh = st + Lo.hh + (size_t)(i - 1) * (im + 1);
    for (int jj = threadIdx.x; jj <= i; jj += blockDim.x) hh[jj] = out[jj];
}

__global__ void __launch_bounds__(128) k_flexd_givens(int* __restrict__ ctl,
                                                      double* __restrict__ st, int im)
{
    flexd_givens_body(ctl, st, im);
}

// V column j (the new one) = w / t, as df_scale: the FP64 factor split into
// (hi, lo) FP32 values; unscaled when t = 0.
__device__ __forceinline__ void flexd_scale_copy_body(const int* __restrict__ ctl,
                                                      const double* __restrict__ st,
                                                      size_t tinv_at, const float2* __restrict__ w,
                                                      float2* __restrict__ V, size_t nl, size_t n,
                                                      int bx, int gx)
{
    if (ctl[1] != 0) return;
    const double a = st[tinv_at];
    const float ah = (float)a, al = (float)(a - (double)ah);
    float2* col = V + (size_t)ctl[0] * nl;
    const size_t stride = (size_t)gx * blockDim.x;
    for (size_t i = (size_t)bx * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float2 v = w[i];
        if (a == 0.0) {
            col[i] = v;
        } else {
            float h = 0.0f, l = 0.0f;
            df_mul_acc(h, l, v.x, v.y, ah, al);
            col[i] = df_norm(h, l);
        }
    }
}

__global__ void k_flexd_scale_copy(const int* __restrict__ ctl, const double* __restrict__ st,
                                   size_t tinv_at, const float2* __restrict__ w,
                                   float2* __restrict__ V, size_t nl, size_t n)
{
    flexd_scale_copy_body(ctl, st, tinv_at, w, V, nl, n, blockIdx.x, gridDim.x);
}

// One thread: y = H^-1 rs over the cycle's i = ctl[0] steps by back
// substitution, as the host loop does.
__global__ void k_flexd_solve(const int* __restrict__ ctl, double* __restrict__ st, int im)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const FlexLayout Lo(im);
    const int i = ctl[0];
    if (i < 1) return;
    const double* hh = st + Lo.hh;
    const double* rs = st + Lo.rs;
    double* y = st + Lo.y;
    auto HH = [&](int r, int k) { return hh[(size_t)k * (im + 1) + r]; };
    for (int k = 0; k < i; ++k) y[k] = rs[k];
    y[i - 1] = y[i - 1] / HH(i - 1, i - 1);
    for (int ii = 2; ii <= i; ++ii) {
        const int k = i - ii + 1;
        double t = y[k - 1];
        for (int j = k + 1; j <= i; ++j) t = __dsub_rn(t, __dmul_rn(HH(k - 1, j - 1), y[j - 1]));
        y[k - 1] = t / HH(k - 1, k - 1);
    }
}

// acc := acc - (a + b) v for acc = hi + lo held as two FP32 values: the
// product a v is split exactly (fma), the subtraction is Knuth's two-sum,
// and the low-order terms gather in lo (double-float arithmetic, about 48
// significant bits; explicit _rn intrinsics keep the compiler from fusing
// the error-free steps).
__device__ __forceinline__ void df_sub_prod(float& hi, float& lo, float a, float b, float v)
{
    const float p = __fmul_rn(a, v);
    const float e = fmaf(a, v, -p);
    const float s = __fsub_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float t = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(-p, bb));
    lo = fmaf(-b, v, __fsub_rn(__fadd_rn(lo, t), e));
    hi = s;
}

// w -= V h for an FP32 basis with double-float accumulation (the update can
// cancel most of w, so it is not summed in plain FP32); optional ||w||^2.
template <bool NORM>
__global__ void k_update_f32(const float2* __restrict__ V, size_t ld2, int k,
                             const double* __restrict__ h, float2* __restrict__ w, size_t n2,
                             double* __restrict__ partial)
{
    __shared__ double sh[32];
    __shared__ float2 hs[512];
    for (int j = threadIdx.x; j < k && j < 512; j += blockDim.x) {
        const float a = (float)h[j];
        hs[j] = make_float2(a, (float)(h[j] - (double)a));
    }
    __syncthreads();
    double nrm = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n2; r += stride) {
        const float2 wv = w[r];
        float hx = wv.x, lx = 0.0f, hy = wv.y, ly = 0.0f;
        for (int jb = 0; jb < k; jb += 8) {
            float2 v[8];  // eight independent loads in flight per thread
#pragma unroll
            for (int u = 0; u < 8; ++u)
                v[u] = (jb + u < k) ? V[(size_t)(jb + u) * ld2 + r] : make_float2(0.0f, 0.0f);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int j = jb + u;
                if (j >= k) break;
                float2 hj;
                if (j < 512) hj = hs[j];
                else {
                    const float a = (float)h[j];
                    hj = make_float2(a, (float)(h[j] - (double)a));
                }
                df_sub_prod(hx, lx, hj.x, hj.y, v[u].x);
                df_sub_prod(hy, ly, hj.x, hj.y, v[u].y);
            }
        }
        const float2 out = make_float2(__fadd_rn(hx, lx), __fadd_rn(hy, ly));
        w[r] = out;
        if (NORM) nrm = fma((double)out.x, (double)out.x, fma((double)out.y, (double)out.y, nrm));
    }
    if (NORM) {
        const double s = block_sum(nrm, sh);
        if (threadIdx.x == 0) partial[blockIdx.x] = s;
    }
}

// out[j] = sum_b partial[j * nb + b], one block per j, fixed order
__global__ void k_finish(const double* __restrict__ partial, int nb, double* __restrict__ out,
                         int accumulate)
{
    __shared__ double sh[32];
    const int j = blockIdx.x;
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) v += partial[(size_t)j * nb + b];
    const double s = block_sum(v, sh);
    if (threadIdx.x == 0) out[j] = accumulate ? out[j] + s : s;
}

// w[r] -= sum_j h[j] V_j[r]; optionally partial ||w||^2 per block
template <class TV, bool NORM>
__global__ void k_update(const TV* __restrict__ V, size_t ld, int k, const double* __restrict__ h,
                         TV* __restrict__ w, size_t n, double* __restrict__ partial)
{
    __shared__ double sh[32];
    __shared__ double hs[512];
    for (int j = threadIdx.x; j < k && j < 512; j += blockDim.x) hs[j] = h[j];
    __syncthreads();
    double nrm = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        double acc = (double)w[r];
        for (int j = 0; j < k; ++j) {
            const double hj = j < 512 ? hs[j] : h[j];
            acc = fma(-hj, (double)V[(size_t)j * ld + r], acc);
        }
        const TV out = (TV)acc;
        w[r] = out;
        if (NORM) nrm = fma((double)out, (double)out, nrm);
    }
    if (NORM) {
        const double s = block_sum(nrm, sh);
        if (threadIdx.x == 0) partial[blockIdx.x] = s;
    }
}

template <class TV, class TY>
__global__ void k_lincomb(const TV* __restrict__ V, size_t ld, int k, const double* __restrict__ c,
                          TY* __restrict__ y, size_t n)
{
    __shared__ double cs[512];
    for (int j = threadIdx.x; j < k && j < 512; j += blockDim.x) cs[j] = c[j];
    __syncthreads();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        double acc = 0.0;
        for (int j = 0; j < k; ++j) acc = fma(j < 512 ? cs[j] : c[j], (double)V[(size_t)j * ld + r], acc);
        y[r] = (TY)acc;
    }
}

template <class TX, class TY>
__global__ void k_axpby(size_t n, double a, const TX* __restrict__ x, double b, TY* __restrict__ y)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride)
        y[r] = (TY)(b == 0.0 ? a * (double)x[r] : fma(a, (double)x[r], b * (double)y[r]));
}

template <class T>
__global__ void k_norm2(const T* __restrict__ x, size_t n, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double v = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        const double xr = (double)x[r];
        v = fma(xr, xr, v);
    }
    const double s = block_sum(v, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

template <class T>
__global__ void k_mask_rows(T* x, const int* __restrict__ mask, int p, int q)
{
    const size_t n = (size_t)p * q;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        if (mask[i / q]) x[i] = T(0);
}

template <class TI, class TO>
__global__ void k_to_itl(const TI* __restrict__ blk, TO* __restrict__ itl, int p, int q)
{
    const size_t n = (size_t)p * q;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const size_t r = i / q, k = i % q;
        itl[i] = (TO)blk[k * (size_t)p + r];
    }
}

template <class TI, class TO>
__global__ void k_to_blk(const TI* __restrict__ itl, TO* __restrict__ blk, int p, int q)
{
    const size_t n = (size_t)p * q;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const size_t k = i / p, r = i % p;
        blk[i] = (TO)itl[r * q + k];
    }
}

struct Coef8 {
    double c[8];
};

__global__ void k_fill_load(const double* __restrict__ rext, Coef8 c, double* __restrict__ out,
                            int p, int q)
{
    const size_t n = (size_t)p * q;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = c.c[i % q] * rext[i / q];
}

__global__ void k_max(const double* __restrict__ x, size_t n, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double v = -1.0e300;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride)
        v = fmax(v, x[r]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = sh[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, sh[w]);
        partial[blockIdx.x] = r;
    }
}

__global__ void k_max_finish(const double* __restrict__ partial, int nb, double* out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double r = -1.0e300;
        for (int b = 0; b < nb; ++b) r = fmax(r, partial[b]);
        out[0] = r;
    }
}

// FP32 basis stored as row pairs: n and ld even, 8-byte aligned vectors.
template <class TV>
bool pairs_ok(const TV* V, size_t ld, const TV* w, size_t n)
{
    if (sizeof(TV) != 4) return false;
    return n % 2 == 0 && ld % 2 == 0 && reinterpret_cast<uintptr_t>(V) % 8 == 0 &&
           reinterpret_cast<uintptr_t>(w) % 8 == 0;
}

int grid_for(size_t n)
{
    size_t b = (n + kThreads - 1) / kThreads;
    if (b > 4096) b = 4096;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace

int reduce_init(Reduce& r, int kmax)
{
    if (kmax < 1) kmax = 1;
    r.nblocks = kRowBlocks;
    r.kmax = kmax;
    XT_TRY(r.partial.alloc((size_t)kmax * kRowBlocks + kRowBlocks));
    XT_TRY(r.out.alloc((size_t)kmax + 1));
    return XT_OK;
}

template <class TV>
int multi_dot(const TV* V, size_t ld, int k, const TV* w, size_t n, Reduce& r, cudaStream_t s)
{
    if (k > r.kmax) { set_error("multi_dot: k exceeds reduction capacity"); return XT_ERR_ARG; }
    if (k <= 0) return XT_OK;
    dim3 grid(r.nblocks, (k + kChunk - 1) / kChunk);
    if (pairs_ok<TV>(V, ld, w, n)) {
        k_multi_dot_f32<<<grid, kThreads, 0, s>>>(reinterpret_cast<const float2*>(V), ld / 2, k,
                                                  reinterpret_cast<const float2*>(w), n / 2,
                                                  r.partial.p);
        k_finish_df<<<k, kThreads, 0, s>>>(r.partial.p, r.nblocks, r.out.p);
    } else {
        k_multi_dot<TV><<<grid, kThreads, 0, s>>>(V, ld, k, w, n, r.partial.p);
        k_finish<<<k, kThreads, 0, s>>>(r.partial.p, r.nblocks, r.out.p, 0);
    }
    note_launches(2);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

template <class TV>
int update_and_dot(const TV* V, size_t ld, int k, const double* h, TV* w, size_t n, Reduce& r,
                   cudaStream_t s)
{
    if (k <= 0) return XT_OK;
    if (pairs_ok<TV>(V, ld, w, n))
        k_update_f32<false><<<grid_for(n / 2), kThreads, 0, s>>>(
            reinterpret_cast<const float2*>(V), ld / 2, k, h, reinterpret_cast<float2*>(w), n / 2,
            nullptr);
    else
        k_update<TV, false><<<grid_for(n), kThreads, 0, s>>>(V, ld, k, h, w, n, nullptr);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return multi_dot<TV>(V, ld, k, w, n, r, s);
}

template <class TV>
int update_and_norm(const TV* V, size_t ld, int k, const double* h, TV* w, size_t n, Reduce& r,
                    cudaStream_t s)
{
    const int nb = r.nblocks;
    if (k > 0 && pairs_ok<TV>(V, ld, w, n)) {
        k_update_f32<true><<<nb, 2 * kThreads, 0, s>>>(reinterpret_cast<const float2*>(V), ld / 2,
                                                       k, h, reinterpret_cast<float2*>(w), n / 2,
                                                       r.partial.p);
    } else if (k > 0) {
        k_update<TV, true><<<nb, kThreads, 0, s>>>(V, ld, k, h, w, n, r.partial.p);
    } else {
        k_norm2<TV><<<nb, kThreads, 0, s>>>(w, n, r.partial.p);
    }
    k_finish<<<1, kThreads, 0, s>>>(r.partial.p, nb, r.out.p, 0);
    note_launches(3);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

template <class TV, class TY>
int lincomb(const TV* V, size_t ld, int k, const double* c, TY* y, size_t n, cudaStream_t s)
{
    k_lincomb<TV, TY><<<grid_for(n), kThreads, 0, s>>>(V, ld, k, c, y, n);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

template <class TX, class TY>
int axpby(size_t n, double a, const TX* x, double b, TY* y, cudaStream_t s)
{
    k_axpby<TX, TY><<<grid_for(n), kThreads, 0, s>>>(n, a, x, b, y);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

template <class T>
int norm2(const T* x, size_t n, Reduce& r, cudaStream_t s)
{
    k_norm2<T><<<r.nblocks, kThreads, 0, s>>>(x, n, r.partial.p);
    k_finish<<<1, kThreads, 0, s>>>(r.partial.p, r.nblocks, r.out.p, 0);
    note_launches(2);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

template <class T>
int mask_rows(T* x, const int* mask, int p, int q, cudaStream_t s)
{
    k_mask_rows<T><<<grid_for((size_t)p * q), kThreads, 0, s>>>(x, mask, p, q);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

template <class TI, class TO>
int to_interleaved(const TI* blk, TO* itl, int p, int q, cudaStream_t s)
{
    k_to_itl<TI, TO><<<grid_for((size_t)p * q), kThreads, 0, s>>>(blk, itl, p, q);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

template <class TI, class TO>
int to_blocks(const TI* itl, TO* blk, int p, int q, cudaStream_t s)
{
    k_to_blk<TI, TO><<<grid_for((size_t)p * q), kThreads, 0, s>>>(itl, blk, p, q);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int fill_load(const double* rext, const double* c, double* out, int p, int q, cudaStream_t s)
{
    Coef8 cc{};
    for (int j = 0; j < q && j < 8; ++j) cc.c[j] = c[j];
    k_fill_load<<<grid_for((size_t)p * q), kThreads, 0, s>>>(rext, cc, out, p, q);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int max_value(const double* x, size_t n, Reduce& r, cudaStream_t s)
{
    k_max<<<r.nblocks, kThreads, 0, s>>>(x, n, r.partial.p);
    k_max_finish<<<1, 32, 0, s>>>(r.partial.p, r.nblocks, r.out.p);
    note_launches(2);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int df_multi_dot(const float2* V, size_t ld, int k, const float2* w, size_t n, Reduce& r,
                 cudaStream_t s)
{
    if (k > r.kmax) { set_error("df_multi_dot: k exceeds reduction capacity"); return XT_ERR_ARG; }
    if (k <= 0) return XT_OK;
    if (n % 2 || ld % 2) { set_error("df_multi_dot: n and ld must be even"); return XT_ERR_ARG; }
    // about eight resident blocks per SM over all chunks: row blocks shrink
    // as k grows, so each block's rows outweigh its block reduction
    const int nchunk = (k + kChunk - 1) / kChunk;
    const int nb = df_dot_blocks(k, df_dot_rows((long long)n / 2, r.nblocks));
    dim3 grid(nb, nchunk);
    k_multi_dot_df<<<grid, kThreads, 0, s>>>(reinterpret_cast<const float4*>(V), ld / 2, k,
                                             reinterpret_cast<const float4*>(w), n / 2,
                                             r.partial.p);
    k_finish_df<<<k, kThreads, 0, s>>>(r.partial.p, nb, r.out.p);
    note_launches(2);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int df_update_and_dot(const float2* V, size_t ld, int k, const double* h, float2* w, size_t n,
                      Reduce& r, cudaStream_t s)
{
    if (k <= 0) return XT_OK;
    if (n % 2 || ld % 2) { set_error("df_update: n and ld must be even"); return XT_ERR_ARG; }
    k_update_df<false><<<grid_for(n / 2), kThreads, 0, s>>>(
        reinterpret_cast<const float4*>(V), ld / 2, k, h, reinterpret_cast<float4*>(w), n / 2,
        nullptr, nullptr);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return df_multi_dot(V, ld, k, w, n, r, s);
}

int df_update_and_norm(const float2* V, size_t ld, int k, const double* h, float2* w, size_t n,
                       Reduce& r, cudaStream_t s, double* out)
{
    if (n % 2 || ld % 2) { set_error("df_update: n and ld must be even"); return XT_ERR_ARG; }
    const int nb = df_row_blocks((long long)n / 2, r.nblocks);
    k_update_df<true><<<nb, 2 * kThreads, 0, s>>>(reinterpret_cast<const float4*>(V), ld / 2, k,
                                                  h, reinterpret_cast<float4*>(w), n / 2,
                                                  r.partial.p, nullptr);
    k_finish_df<<<1, kThreads, 0, s>>>(r.partial.p, nb, out ? out : r.out.p);
    note_launches(2);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int df_from_f64(const double* x, float2* y, size_t n, cudaStream_t s)
{
    k_df_from_f64<<<grid_for(n), kThreads, 0, s>>>(x, y, n);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int df_hi(const float2* x, float* y, size_t n, cudaStream_t s)
{
    k_df_hi<<<grid_for(n), kThreads, 0, s>>>(x, y, n);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int df_to_f64(const float2* x, double* y, size_t n, cudaStream_t s)
{
    k_df_to_f64<<<grid_for(n), kThreads, 0, s>>>(x, y, n);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int df_scale(float2* y, double a, size_t n, cudaStream_t s)
{
    const float ah = (float)a;
    k_df_scale<<<grid_for(n), kThreads, 0, s>>>(y, ah, (float)(a - (double)ah), n);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int df_scale_hi(float2* y, double a, float* hi, size_t n, cudaStream_t s)
{
    const float ah = (float)a;
    k_df_scale_hi<<<grid_for(n), kThreads, 0, s>>>(y, ah, (float)(a - (double)ah), hi, n);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int flexd_hi(const int* ctl, const float2* V, size_t nl, float* d, size_t n, cudaStream_t s)
{
    k_flexd_hi<<<grid_for(n), kThreads, 0, s>>>(ctl, V, nl, d, n);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int flexd_zcopy(const int* ctl, const float* z, float* Z, size_t n, cudaStream_t s)
{
    k_flexd_zcopy<<<grid_for(n), kThreads, 0, s>>>(ctl, z, Z, n);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int flexd_orth(const int* ctl, const float2* V, size_t nl, float2* w, double* st, int im,
               Reduce& r, cudaStream_t s, bool two_pass)
{
    if (im > r.kmax) { set_error("flexd_orth: restart length exceeds reduction capacity"); return XT_ERR_ARG; }
    if (nl % 2) { set_error("flexd_orth: the basis stride must be even"); return XT_ERR_ARG; }
    const FlexLayout Lo(im);
    const float4* V4 = reinterpret_cast<const float4*>(V);
    float4* w4 = reinterpret_cast<float4*>(w);
    const size_t n2 = nl / 2;
    const int rb = df_row_blocks((long long)n2, r.nblocks);
    const int rd = df_dot_rows((long long)n2, r.nblocks);
    const int grid = df_dot_grid(im, rd);
    if (two_pass) {
        k_multi_dot_df_ctl<<<grid, kThreads, 0, s>>>(V4, n2, w4, n2, r.partial.p, rd, ctl);
        k_finish_df_ctl<<<im, kThreads, 0, s>>>(r.partial.p, rd, st + Lo.h1, ctl, 0);
        k_update_df<false><<<grid_for(n2), kThreads, 0, s>>>(V4, n2, 0, st + Lo.h1, w4, n2, nullptr, ctl);
        note_launches(3);
    } else {
        // one pass: the projections go to h2 and h1 stays zero, as the host
        // loop's Hessenberg column 0 + h
        XT_CUDA(cudaMemsetAsync(st + Lo.h1, 0, (size_t)im * sizeof(double), s));
    }
    k_multi_dot_df_ctl<<<grid, kThreads, 0, s>>>(V4, n2, w4, n2, r.partial.p, rd, ctl);
    k_finish_df_ctl<<<im, kThreads, 0, s>>>(r.partial.p, rd, st + Lo.h2, ctl, 0);
    k_update_df<true><<<rb, 2 * kThreads, 0, s>>>(V4, n2, 0, st + Lo.h2, w4, n2, r.partial.p, ctl);
    k_finish_df_ctl<<<1, kThreads, 0, s>>>(r.partial.p, rb, st + Lo.nrm, ctl, 1);
    note_launches(4);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int flexd_givens(int* ctl, double* st, int im, cudaStream_t s)
{
    if (im > kGivensMax) { set_error("flexd_givens: restart length exceeds the device rotation buffer"); return XT_ERR_ARG; }
    k_flexd_givens<<<1, 128, 0, s>>>(ctl, st, im);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int flexd_scale_copy(const int* ctl, const double* st, int im, const float2* w, float2* V,
                     size_t nl, size_t n, cudaStream_t s)
{
    k_flexd_scale_copy<<<grid_for(n), kThreads, 0, s>>>(ctl, st, FlexLayout(im).tinv, w, V, nl, n);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int flexd_solve(const int* ctl, double* st, int im, cudaStream_t s)
{
    k_flexd_solve<<<1, 32, 0, s>>>(ctl, st, im);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

// ---------------------------------------------------------------------------
// Batched device-driven steps: blockIdx.y selects the system's table entry,
// blockIdx.x is the block of that system's pass.  Each body is the
// per-system kernel's, with the system's own row partition where a
// reduction depends on it, so a batched step gives each system the bits of
// its own step.

namespace {

// Blocks in x of an elementwise batched pass: about eight entries per
// thread of the largest system (smaller systems leave blocks idle).
int ew_grid(long long nmax)
{
    const long long b = (nmax + 8LL * kThreads - 1) / (8LL * kThreads);
    return (int)std::max(1LL, std::min(b, 4096LL));
}

__global__ void kb_flex_zcopy(const FlexStepItem* __restrict__ t)
{
    const FlexStepItem& e = t[blockIdx.y];
    const int* ctl = e.ctl;
    if (ctl[1] != 0) return;
    const size_t n = (size_t)e.n, stride = (size_t)gridDim.x * blockDim.x;
    float* col = e.Z + (size_t)ctl[0] * n;
    const float* z = e.zfix;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) col[i] = z[i];
}

// The partial sums of k_multi_dot_df_ctl for entry blockIdx.y: the entry's
// (row block, chunk) items dealt to its e.dotblocks blocks in turn (a
// system's share of one wave, by its size), so small and large systems
// finish together and no block of the grid is there for the largest alone.
__global__ void __launch_bounds__(256, 6) kb_dot(const FlexStepItem* __restrict__ t)
{
    const FlexStepItem& e = t[blockIdx.y];
    const int* ctl = e.ctl;
    if (ctl[1] != 0 || (int)blockIdx.x >= e.dotblocks) return;
    const int k = ctl[0] + 1;
    const int nb = df_dot_blocks(k, e.dotrows), nchunk = (k + kChunk - 1) / kChunk;
    const size_t n2 = (size_t)e.nl / 2;
    for (int w = blockIdx.x; w < nb * nchunk; w += e.dotblocks) {
        const int chunk = w / nb;
        multi_dot_df_body(reinterpret_cast<const float4*>(e.V), n2, k,
                          reinterpret_cast<const float4*>(e.wfix), n2, e.partial, w - chunk * nb,
                          nb, chunk);
        __syncthreads();  // the body's shared sums are read before the next item writes them
    }
}

// k_finish_df_ctl of entry blockIdx.y into h1 (which 0), h2 (1) or the norm (2)
__global__ void kb_finish(const FlexStepItem* __restrict__ t, int which)
{
    const FlexStepItem& e = t[blockIdx.y];
    const FlexLayout Lo(e.im);
    double* out = e.st + (which == 0 ? Lo.h1 : (which == 1 ? Lo.h2 : Lo.nrm));
    finish_df_ctl_body(e.partial, which == 2 ? e.rowblocks : e.dotrows, out, e.ctl,
                       which == 2 ? 1 : 0, blockIdx.x);
}

// k_update_df of entry blockIdx.y with h = h1 (NORM false) or h2 and the norm
// partials over the system's own row blocks (NORM true)
template <bool NORM>
__global__ void kb_update(const FlexStepItem* __restrict__ t)
{
    const FlexStepItem& e = t[blockIdx.y];
    const int* ctl = e.ctl;
    if (ctl[1] != 0) return;
    const int gx = NORM ? e.rowblocks : (int)gridDim.x;
    if ((int)blockIdx.x >= gx) return;
    const FlexLayout Lo(e.im);
    const size_t n2 = (size_t)e.nl / 2;
    update_df_body<NORM>(reinterpret_cast<const float4*>(e.V), n2, ctl[0] + 1,
                         e.st + (NORM ? Lo.h2 : Lo.h1), reinterpret_cast<float4*>(e.wfix), n2,
                         e.partial, blockIdx.x, gx);
}

// h1 = 0 for a one-pass step (the host-driven loop's Hessenberg column is 0 + h)
__global__ void kb_zero_h1(const FlexStepItem* __restrict__ t)
{
    const FlexStepItem& e = t[blockIdx.y];
    const FlexLayout Lo(e.im);
    for (int j = threadIdx.x; j < e.im; j += blockDim.x) e.st[Lo.h1 + j] = 0.0;
}

__global__ void __launch_bounds__(128) kb_givens(const FlexStepItem* __restrict__ t)
{
    const FlexStepItem& e = t[blockIdx.x];
    flexd_givens_body(e.ctl, e.st, e.im);
}

__global__ void kb_scale_copy(const FlexStepItem* __restrict__ t)
{
    const FlexStepItem& e = t[blockIdx.y];
    flexd_scale_copy_body(e.ctl, e.st, FlexLayout(e.im).tinv, e.wfix, e.V, (size_t)e.nl,
                          (size_t)e.n, blockIdx.x, gridDim.x);
}

__global__ void kb_ctl_gather(const FlexStepItem* __restrict__ t, int count, int* __restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * count; i += gridDim.x * blockDim.x)
        out[i] = t[i / 4].ctl[i % 4];
}

}  // namespace

int df_row_blocks_for(long long nl, const Reduce& r) { return df_row_blocks(nl / 2, r.nblocks); }
int df_dot_rows_for(long long nl, const Reduce& r) { return df_dot_rows(nl / 2, r.nblocks); }
int df_dot_blocks_max(int im, int dotrows) { return df_dot_grid(im, dotrows); }
int df_dot_wave() { return 6 * 148; }

int flexb_zcopy(const FlexStepItem* t, int count, const FlexStepDims& d, cudaStream_t s)
{
    if (count <= 0) return XT_OK;
    kb_flex_zcopy<<<dim3(ew_grid(d.nmax), count), kThreads, 0, s>>>(t);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int flexb_orth(const FlexStepItem* all, int nall, const FlexStepItem* two, int ntwo,
               const FlexStepItem* one, int none, const FlexStepDims& d, cudaStream_t s)
{
    if (nall <= 0) return XT_OK;
    if (d.im < 1 || d.im > kFlexdMaxIm || d.rb_max < 1 || d.rb_max > kRowBlocks ||
        d.dot_blocks_max < 1 || d.dot_blocks_max > 65535) {
        set_error("flexb_orth: bad batch dimensions");
        return XT_ERR_ARG;
    }
    const int grid = std::max(1, d.dot_blocks_max);
    const int ew = ew_grid((d.nmax + 1) / 2);
    int launches = 0;
    if (ntwo > 0) {
        kb_dot<<<dim3(grid, ntwo), kThreads, 0, s>>>(two);
        kb_finish<<<dim3(d.im, ntwo), kThreads, 0, s>>>(two, 0);
        kb_update<false><<<dim3(ew, ntwo), kThreads, 0, s>>>(two);
        launches += 3;
    }
    if (none > 0) {
        kb_zero_h1<<<dim3(1, none), kThreads, 0, s>>>(one);
        ++launches;
    }
    kb_dot<<<dim3(grid, nall), kThreads, 0, s>>>(all);
    kb_finish<<<dim3(d.im, nall), kThreads, 0, s>>>(all, 1);
    kb_update<true><<<dim3(d.rb_max, nall), 2 * kThreads, 0, s>>>(all);
    kb_finish<<<dim3(1, nall), kThreads, 0, s>>>(all, 2);
    note_launches(launches + 4);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int flexb_givens_scale(const FlexStepItem* t, int count, const FlexStepDims& d, cudaStream_t s)
{
    if (count <= 0) return XT_OK;
    if (d.im > kGivensMax) {
        set_error("flexb_givens_scale: restart length exceeds the device rotation buffer");
        return XT_ERR_ARG;
    }
    kb_givens<<<count, 128, 0, s>>>(t);
    kb_scale_copy<<<dim3(ew_grid(d.nmax), count), kThreads, 0, s>>>(t);
    note_launches(2);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int flexb_ctl_gather(const FlexStepItem* t, int count, int* out, cudaStream_t s)
{
    if (count <= 0) return XT_OK;
    const int th = 256, b = std::max(1, std::min(64, (4 * count + th - 1) / th));
    kb_ctl_gather<<<b, th, 0, s>>>(t, count, out);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

#define XT_INST_V(TV)                                                                       \
    template int multi_dot<TV>(const TV*, size_t, int, const TV*, size_t, Reduce&,          \
                               cudaStream_t);                                               \
    template int update_and_dot<TV>(const TV*, size_t, int, const double*, TV*, size_t,     \
                                    Reduce&, cudaStream_t);                                 \
    template int update_and_norm<TV>(const TV*, size_t, int, const double*, TV*, size_t,    \
                                     Reduce&, cudaStream_t);                                \
    template int norm2<TV>(const TV*, size_t, Reduce&, cudaStream_t);                       \
    template int mask_rows<TV>(TV*, const int*, int, int, cudaStream_t);
XT_INST_V(double)
XT_INST_V(float)
#undef XT_INST_V

template int lincomb<double, double>(const double*, size_t, int, const double*, double*, size_t,
                                     cudaStream_t);
template int lincomb<float, double>(const float*, size_t, int, const double*, double*, size_t,
                                    cudaStream_t);
template int lincomb<float, float>(const float*, size_t, int, const double*, float*, size_t,
                                   cudaStream_t);
template int axpby<double, double>(size_t, double, const double*, double, double*, cudaStream_t);
template int axpby<float, double>(size_t, double, const float*, double, double*, cudaStream_t);
template int axpby<double, float>(size_t, double, const double*, double, float*, cudaStream_t);
template int axpby<float, float>(size_t, double, const float*, double, float*, cudaStream_t);
template int to_interleaved<double, double>(const double*, double*, int, int, cudaStream_t);
template int to_blocks<double, double>(const double*, double*, int, int, cudaStream_t);

}  // namespace xt
