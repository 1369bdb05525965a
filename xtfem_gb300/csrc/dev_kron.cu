// dev_kron.cu -- the Kronecker space-time operator on the GPU.
//
// Computes Y = alpha * (K X A^T + M X B^T) + beta * Y, the operator of
// src/kronecker.f90:19-127 (kronspmv / kronspgemv), where X and Y hold the q
// temporal blocks of a space-time vector node-major (row r, block k at
// r*q + k).  The reference runs 2q serial CSR products and then a q^2 p
// mixing loop, so K and M are each streamed q times; here each CSR row is
// streamed once: a team of LANES threads walks the row's nonzeros, every
// nonzero multiplies the q contiguous values of X's column row (one 24 B or
// 48 B gather), the q partial sums of K and of M are reduced across the team
// with shuffles and the q x q temporal mixing with A and B (kept in shared
// memory) is applied in the epilogue before the single store of Y's row.
//
// Roofline: the kernel streams nnz(K)+nnz(M) column indices and values once
// plus the row pointers, and touches X (gathered, L2-resident) and Y once.
// In FP32 it is HBM-bound; in FP64 the GB300's FP64 pipe (about 1.2 TFLOP/s)
// binds first because every nonzero carries q FMAs.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "df.cuh"
#include <cuda_bf16.h>

#include "xt_device.h"

namespace xt {

namespace {

__global__ void k_dec_index(int* a, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) a[i] -= 1;
}

__global__ void k_to_f32(const double* a, float* b, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) b[i] = (float)a[i];
}

template <class T, int Q>
__device__ __forceinline__ void load_row(const T* __restrict__ p, T (&v)[Q])
{
#pragma unroll
    for (int b = 0; b < Q; ++b) v[b] = p[b];
}

// 6 contiguous values: three 2-wide loads (rows start 8 B / 16 B aligned)
template <>
__device__ __forceinline__ void load_row<float, 6>(const float* __restrict__ p, float (&v)[6])
{
    const float2* q = reinterpret_cast<const float2*>(p);
    float2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = c.x; v[5] = c.y;
}
template <>
__device__ __forceinline__ void load_row<double, 6>(const double* __restrict__ p, double (&v)[6])
{
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = c.x; v[5] = c.y;
}

// value array of the requested precision (host-side selection)
template <class T>
const T* vals(const double* v64, const float* v32);
template <>
const double* vals<double>(const double* v64, const float*) { return v64; }
template <>
const float* vals<float>(const double*, const float* v32) { return v32; }

// stored value -> arithmetic type (BF16 values widen exactly to FP32)
template <class T>
__device__ __forceinline__ T widen(T v) { return v; }
__device__ __forceinline__ float widen(__nv_bfloat16 v) { return __bfloat162float(v); }

template <class T, int Q, int LANES, bool MERGED, class V = T>
__global__ void __launch_bounds__(256)
k_kron_spmm(int p, const int* __restrict__ kptr, const int* __restrict__ kcol,
            const V* __restrict__ kval, const int* __restrict__ mptr,
            const int* __restrict__ mcol, const V* __restrict__ mval,
            const double* __restrict__ dA, const double* __restrict__ dB, T alpha, T beta,
            const T* __restrict__ x, T* __restrict__ y)
{
    __shared__ T sA[Q * Q], sB[Q * Q];
    for (int i = threadIdx.x; i < Q * Q; i += blockDim.x) {
        sA[i] = (T)dA[i];
        sB[i] = (T)dB[i];
    }
    __syncthreads();
    // The loop bound is warp-uniform so that every lane of a warp reaches the
    // shuffles; teams past the last row run with empty ranges.
    constexpr int TPW = 32 / LANES;  // teams per warp
    const int lane = threadIdx.x % LANES;
    const int team = (threadIdx.x % 32) / LANES;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int nwarp = (gridDim.x * blockDim.x) / 32;
    for (int rb = gwarp * TPW; rb < p; rb += nwarp * TPW) {
        const int r = rb + team;
        const bool act = r < p;
        T ak[Q], am[Q];
#pragma unroll
        for (int b = 0; b < Q; ++b) { ak[b] = T(0); am[b] = T(0); }
        const int k0 = act ? kptr[r] : 0, k1 = act ? kptr[r + 1] : 0;
        if constexpr (MERGED) {  // one pattern: one index and one X row for both
#pragma unroll 4
            for (int k = k0 + lane; k < k1; k += LANES) {
                const T vk = widen(kval[k]), vm = widen(mval[k]);
                T xr[Q];
                load_row<T, Q>(x + (size_t)kcol[k] * Q, xr);
#pragma unroll
                for (int b = 0; b < Q; ++b) {
                    ak[b] = fma(vk, xr[b], ak[b]);
                    am[b] = fma(vm, xr[b], am[b]);
                }
            }
        } else {
#pragma unroll 4
            for (int k = k0 + lane; k < k1; k += LANES) {
                const T v = widen(kval[k]);
                T xr[Q];
                load_row<T, Q>(x + (size_t)kcol[k] * Q, xr);
#pragma unroll
                for (int b = 0; b < Q; ++b) ak[b] = fma(v, xr[b], ak[b]);
            }
            const int m0 = act ? mptr[r] : 0, m1 = act ? mptr[r + 1] : 0;
#pragma unroll 4
            for (int k = m0 + lane; k < m1; k += LANES) {
                const T v = widen(mval[k]);
                T xr[Q];
                load_row<T, Q>(x + (size_t)mcol[k] * Q, xr);
#pragma unroll
                for (int b = 0; b < Q; ++b) am[b] = fma(v, xr[b], am[b]);
            }
        }
#pragma unroll
        for (int off = LANES / 2; off > 0; off >>= 1)
#pragma unroll
            for (int b = 0; b < Q; ++b) {
                ak[b] += __shfl_xor_sync(0xffffffffu, ak[b], off, LANES);
                am[b] += __shfl_xor_sync(0xffffffffu, am[b], off, LANES);
            }
        // epilogue: lane a < Q forms output block a of this row
        if (act) {
#pragma unroll
            for (int a = 0; a < Q; ++a) {
                if (lane == a) {
                    T acc = T(0);
#pragma unroll
                    for (int b = 0; b < Q; ++b) {
                        acc = fma(sA[b * Q + a], ak[b], acc);
                        acc = fma(sB[b * Q + a], am[b], acc);
                    }
                    T* yp = y + (size_t)r * Q + a;
                    *yp = (beta == T(0)) ? alpha * acc : fma(beta, *yp, alpha * acc);
                }
            }
        }
    }
}

// XTFEM_KRON_NB=0 keeps the CSR kernel (tests compare the two).
bool nb_enabled()
{
    const char* e = std::getenv("XTFEM_KRON_NB");
    return !e || std::atoi(e) != 0;
}

// b[at[i]] = double-float of a[i]
__global__ void k_scatter_df(const double* __restrict__ a, const int* __restrict__ at,
                             float2* __restrict__ b, size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float h = __double2float_rn(a[i]);
        b[at[i]] = make_float2(h, __double2float_rn(a[i] - (double)h));
    }
}

__global__ void k_to_df(const double* __restrict__ a, float2* __restrict__ b, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) {
        const float h = __double2float_rn(a[i]);
        b[i] = make_float2(h, __double2float_rn(a[i] - (double)h));
    }
}

// (hi, lo) += (vh + vl) x for an FP32 x: vh x exactly (fma), vl x in FP32
__device__ __forceinline__ void df_axpy(float& hi, float& lo, float vh, float vl, float x)
{
    const float p = __fmul_rn(vh, x);
    const float e = fmaf(vh, x, -p);
    df_add(hi, lo, p);
    lo = __fadd_rn(lo, fmaf(vl, x, e));
}

// The same row-team structure as k_kron_spmm, with double-float values and
// accumulators, an FP32 X and a double-float Y (alpha = 1, beta = 0).
template <int Q, int LANES, bool MERGED>
__global__ void __launch_bounds__(256)
k_kron_df(int p, const int* __restrict__ kptr, const int* __restrict__ kcol,
          const float2* __restrict__ kval, const int* __restrict__ mptr,
          const int* __restrict__ mcol, const float2* __restrict__ mval,
          const double* __restrict__ dA, const double* __restrict__ dB,
          const float* __restrict__ x, float2* __restrict__ y)
{
    __shared__ float2 sA[Q * Q], sB[Q * Q];
    for (int i = threadIdx.x; i < Q * Q; i += blockDim.x) {
        const float ah = __double2float_rn(dA[i]), bh = __double2float_rn(dB[i]);
        sA[i] = make_float2(ah, __double2float_rn(dA[i] - (double)ah));
        sB[i] = make_float2(bh, __double2float_rn(dB[i] - (double)bh));
    }
    __syncthreads();
    constexpr int TPW = 32 / LANES;
    const int lane = threadIdx.x % LANES;
    const int team = (threadIdx.x % 32) / LANES;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int nwarp = (gridDim.x * blockDim.x) / 32;
    for (int rb = gwarp * TPW; rb < p; rb += nwarp * TPW) {
        const int r = rb + team;
        const bool act = r < p;
        float kh[Q], kl[Q], mh[Q], ml[Q];
#pragma unroll
        for (int b = 0; b < Q; ++b) kh[b] = kl[b] = mh[b] = ml[b] = 0.0f;
        const int k0 = act ? kptr[r] : 0, k1 = act ? kptr[r + 1] : 0;
        if constexpr (MERGED) {
#pragma unroll 4
            for (int k = k0 + lane; k < k1; k += LANES) {
                const float2 vk = kval[k], vm = mval[k];
                float xr[Q];
                load_row<float, Q>(x + (size_t)kcol[k] * Q, xr);
#pragma unroll
                for (int b = 0; b < Q; ++b) {
                    df_axpy(kh[b], kl[b], vk.x, vk.y, xr[b]);
                    df_axpy(mh[b], ml[b], vm.x, vm.y, xr[b]);
                }
            }
        } else {
#pragma unroll 4
            for (int k = k0 + lane; k < k1; k += LANES) {
                const float2 v = kval[k];
                float xr[Q];
                load_row<float, Q>(x + (size_t)kcol[k] * Q, xr);
#pragma unroll
                for (int b = 0; b < Q; ++b) df_axpy(kh[b], kl[b], v.x, v.y, xr[b]);
            }
            const int m0 = act ? mptr[r] : 0, m1 = act ? mptr[r + 1] : 0;
#pragma unroll 4
            for (int k = m0 + lane; k < m1; k += LANES) {
                const float2 v = mval[k];
                float xr[Q];
                load_row<float, Q>(x + (size_t)mcol[k] * Q, xr);
#pragma unroll
                for (int b = 0; b < Q; ++b) df_axpy(mh[b], ml[b], v.x, v.y, xr[b]);
            }
        }
#pragma unroll
        for (int off = LANES / 2; off > 0; off >>= 1)
#pragma unroll
            for (int b = 0; b < Q; ++b) {
                const float a1 = __shfl_xor_sync(0xffffffffu, kh[b], off, LANES);
                const float a2 = __shfl_xor_sync(0xffffffffu, kl[b], off, LANES);
                const float b1 = __shfl_xor_sync(0xffffffffu, mh[b], off, LANES);
                const float b2 = __shfl_xor_sync(0xffffffffu, ml[b], off, LANES);
                df_add_df(kh[b], kl[b], a1, a2);
                df_add_df(mh[b], ml[b], b1, b2);
            }
        if (act) {
#pragma unroll
            for (int a = 0; a < Q; ++a) {
                if (lane == a) {
                    float h = 0.0f, l = 0.0f;
#pragma unroll
                    for (int b = 0; b < Q; ++b) {
                        df_mul_acc(h, l, sA[b * Q + a].x, sA[b * Q + a].y, kh[b], kl[b]);
                        df_mul_acc(h, l, sB[b * Q + a].x, sB[b * Q + a].y, mh[b], ml[b]);
                    }
                    y[(size_t)r * Q + a] = df_norm(h, l);
                }
            }
        }
    }
}

// Node-block double-float apply, Y = K X A^T + M X B^T (even Q): a lane
// owns (node row a, DOF c, temporal pair qp) and accumulates (KX)[3a+c][2qp..]
// and (MX)[3a+c][2qp..] over the node row's blocks: per block one column
// index, row c of K's block, M's scalar and the neighbour's three X pairs.
// The Q/2 lanes of (a, c) then exchange their sums and each finishes its
// two outputs with the q x q temporal mixing.  3 Q/2 lanes per node row,
// 32 / (3 Q/2) node rows per warp.
// This thread block is block bx of a gx-block pass (a batched launch runs
// one such pass per system).
template <int Q>
__device__ __forceinline__ void kron_nb_body(int nodes, const int* __restrict__ bptr,
                                             const int* __restrict__ bcol,
                                             const float2* __restrict__ kv,
                                             const float2* __restrict__ mv,
                                             const double* __restrict__ dA,
                                             const double* __restrict__ dB,
                                             const float* __restrict__ x, float2* __restrict__ y,
                                             int bx, int gx)
{
    static_assert(Q % 2 == 0 && Q <= 8, "pairs of temporal blocks");
    constexpr int NP = Q / 2, LPR = 3 * NP, RPW = 32 / LPR;
    __shared__ float2 sA[Q * Q], sB[Q * Q];
    for (int i = threadIdx.x; i < Q * Q; i += blockDim.x) {
        const float ah = __double2float_rn(dA[i]), bh = __double2float_rn(dB[i]);
        sA[i] = make_float2(ah, __double2float_rn(dA[i] - (double)ah));
        sB[i] = make_float2(bh, __double2float_rn(dB[i] - (double)bh));
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, slot = lane / LPR, inl = lane - slot * LPR;
    const int c = inl / NP, qp = inl - c * NP;
    const bool lane_ok = slot < RPW;
    const int gwarp = (bx * blockDim.x + threadIdx.x) / 32;
    const int nwarp = (gx * blockDim.x) / 32;
    for (int a0 = gwarp * RPW; a0 < nodes; a0 += nwarp * RPW) {
        const int a = a0 + slot;
        const bool act = lane_ok && a < nodes;
        // (hi, lo) of the lane's two temporal entries, packed: .x entry 2qp,
        // .y entry 2qp+1
        float2 kh = make_float2(0.f, 0.f), kl = kh, mh = kh, ml = kh;
        const int b0 = act ? bptr[a] : 0, b1 = act ? bptr[a + 1] : 0;
#pragma unroll 4
        for (int b = b0; b < b1; ++b) {
            const float* xb = x + (size_t)bcol[b] * (3 * Q) + 2 * qp;
            const float2* kr = kv + (size_t)b * 9 + c * 3;
            const float2 k0 = kr[0], k1 = kr[1], k2 = kr[2], m = mv[b];
            const float2 x0 = *reinterpret_cast<const float2*>(xb);
            const float2 x1 = *reinterpret_cast<const float2*>(xb + Q);
            const float2 x2 = *reinterpret_cast<const float2*>(xb + 2 * Q);
            df2_axpy(kh, kl, k0.x, k0.y, x0);
            df2_axpy(kh, kl, k1.x, k1.y, x1);
            df2_axpy(kh, kl, k2.x, k2.y, x2);
            df2_axpy(mh, ml, m.x, m.y, c == 0 ? x0 : (c == 1 ? x1 : x2));
        }
        const float kh0 = kh.x, kl0 = kl.x, kh1 = kh.y, kl1 = kl.y;
        const float mh0 = mh.x, ml0 = ml.x, mh1 = mh.y, ml1 = ml.y;
        // all Q temporal entries of row 3a+c, from the NP lanes of (a, c)
        float KH[Q], KL[Q], MH[Q], ML[Q];
        const int base = slot * LPR + c * NP;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
            const int src = base + j;
            KH[2 * j] = __shfl_sync(0xffffffffu, kh0, src);
            KL[2 * j] = __shfl_sync(0xffffffffu, kl0, src);
            KH[2 * j + 1] = __shfl_sync(0xffffffffu, kh1, src);
            KL[2 * j + 1] = __shfl_sync(0xffffffffu, kl1, src);
            MH[2 * j] = __shfl_sync(0xffffffffu, mh0, src);
            ML[2 * j] = __shfl_sync(0xffffffffu, ml0, src);
            MH[2 * j + 1] = __shfl_sync(0xffffffffu, mh1, src);
            ML[2 * j + 1] = __shfl_sync(0xffffffffu, ml1, src);
        }
        if (act) {
            float2 out[2];
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                const int i = 2 * qp + t;
                float h = 0.0f, l = 0.0f;
#pragma unroll
                for (int j = 0; j < Q; ++j) {
                    df_mul_acc(h, l, sA[j * Q + i].x, sA[j * Q + i].y, KH[j], KL[j]);
                    df_mul_acc(h, l, sB[j * Q + i].x, sB[j * Q + i].y, MH[j], ML[j]);
                }
                out[t] = df_norm(h, l);
            }
            *reinterpret_cast<float4*>(y + (size_t)(3 * a + c) * Q + 2 * qp) =
                make_float4(out[0].x, out[0].y, out[1].x, out[1].y);
        }
    }
}

template <int Q>
__global__ void __launch_bounds__(256)
k_kron_nb(int nodes, const int* __restrict__ bptr, const int* __restrict__ bcol,
          const float2* __restrict__ kv, const float2* __restrict__ mv,
          const double* __restrict__ dA, const double* __restrict__ dB,
          const float* __restrict__ x, float2* __restrict__ y, const int* __restrict__ skip)
{
    if (skip && skip[0] != 0) return;
    kron_nb_body<Q>(nodes, bptr, bcol, kv, mv, dA, dB, x, y, blockIdx.x, gridDim.x);
}

// The node-block operator of table entry blockIdx.y: wfix = op(zfix), nothing
// once the entry's cycle has ended.
template <int Q>
__global__ void __launch_bounds__(256) kb_kron_nb(const FlexStepItem* __restrict__ t)
{
    const FlexStepItem& e = t[blockIdx.y];
    if (e.ctl[1] != 0) return;
    kron_nb_body<Q>(e.nodes, e.bptr, e.bcol, e.kv, e.mv, e.A, e.B, e.zfix, e.wfix, blockIdx.x,
                    gridDim.x);
}

template <int Q>
int launch_nb(const DevNodeBlocks& nb, const double* dA, const double* dB, const float* x,
              float2* y, cudaStream_t s, const int* skip)
{
    constexpr int RPW = 32 / (3 * (Q / 2));
    const int threads = 256, rows_per_block = (threads / 32) * RPW;
    const int blocks = std::max(1, (nb.nodes + rows_per_block - 1) / rows_per_block);
    k_kron_nb<Q><<<blocks, threads, 0, s>>>(nb.nodes, nb.ptr.p, nb.col.p, nb.kdf.p, nb.mdf.p, dA,
                                            dB, x, y, skip);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

template <int Q>
int launch_df(const DevCsr& K, const DevCsr& M, const double* dA, const double* dB,
              const float* x, float2* y, cudaStream_t s)
{
    constexpr int LANES = 8;
    const int threads = 256;
    const int rows_per_block = threads / LANES;
    int blocks = (K.n + rows_per_block - 1) / rows_per_block;
    if (blocks < 1) blocks = 1;
    if (M.same_pattern && M.nnz == K.nnz)
        k_kron_df<Q, LANES, true><<<blocks, threads, 0, s>>>(K.n, K.rowptr.p, K.col.p, K.vdf.p,
                                                             M.rowptr.p, M.col.p, M.vdf.p, dA, dB,
                                                             x, y);
    else
        k_kron_df<Q, LANES, false><<<blocks, threads, 0, s>>>(K.n, K.rowptr.p, K.col.p, K.vdf.p,
                                                              M.rowptr.p, M.col.p, M.vdf.p, dA, dB,
                                                              x, y);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

__global__ void k_to_bf16(const double* __restrict__ a, __nv_bfloat16* __restrict__ b, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) b[i] = __double2bfloat16(a[i]);  // round to nearest even
}

int ensure_bf16(DevCsr& A, cudaStream_t s)
{
    if (A.v16.p && A.v16.n == (size_t)A.nnz) return XT_OK;
    XT_TRY(A.v16.alloc((size_t)A.nnz));
    if (A.nnz) {
        k_to_bf16<<<1024, 256, 0, s>>>(A.v64.p, A.v16.p, (size_t)A.nnz);
        note_launches(1);
        XT_CUDA(cudaGetLastError());
    }
    return XT_OK;
}

template <int Q>
int launch_bf16(const DevCsr& K, const DevCsr& M, const double* dA, const double* dB,
                double alpha, double beta, const float* x, float* y, cudaStream_t s)
{
    constexpr int LANES = 8;
    const int threads = 256;
    const int rows_per_block = threads / LANES;
    int blocks = (K.n + rows_per_block - 1) / rows_per_block;
    if (blocks < 1) blocks = 1;
    if (M.same_pattern && M.nnz == K.nnz)
        k_kron_spmm<float, Q, LANES, true, __nv_bfloat16><<<blocks, threads, 0, s>>>(
            K.n, K.rowptr.p, K.col.p, K.v16.p, M.rowptr.p, M.col.p, M.v16.p, dA, dB,
            (float)alpha, (float)beta, x, y);
    else
        k_kron_spmm<float, Q, LANES, false, __nv_bfloat16><<<blocks, threads, 0, s>>>(
            K.n, K.rowptr.p, K.col.p, K.v16.p, M.rowptr.p, M.col.p, M.v16.p, dA, dB,
            (float)alpha, (float)beta, x, y);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int ensure_df(DevCsr& A, cudaStream_t s)
{
    if (A.vdf.p && A.vdf.n == (size_t)A.nnz) return XT_OK;
    XT_TRY(A.vdf.alloc((size_t)A.nnz));
    if (A.nnz) {
        k_to_df<<<1024, 256, 0, s>>>(A.v64.p, A.vdf.p, (size_t)A.nnz);
        note_launches(1);
        XT_CUDA(cudaGetLastError());
    }
    return XT_OK;
}

template <class T, int Q>
int launch_q(const DevCsr& K, const DevCsr& M, const double* dA, const double* dB,
             double alpha, double beta, const T* x, T* y, cudaStream_t s)
{
    constexpr int LANES = 8;
    const int threads = 256;
    const int rows_per_block = threads / LANES;
    int blocks = (K.n + rows_per_block - 1) / rows_per_block;
    if (blocks < 1) blocks = 1;
    if (M.same_pattern && M.nnz == K.nnz)
        k_kron_spmm<T, Q, LANES, true><<<blocks, threads, 0, s>>>(
            K.n, K.rowptr.p, K.col.p, vals<T>(K.v64.p, K.v32.p), M.rowptr.p, M.col.p,
            vals<T>(M.v64.p, M.v32.p), dA, dB, (T)alpha, (T)beta, x, y);
    else
        k_kron_spmm<T, Q, LANES, false><<<blocks, threads, 0, s>>>(
            K.n, K.rowptr.p, K.col.p, vals<T>(K.v64.p, K.v32.p), M.rowptr.p, M.col.p,
            vals<T>(M.v64.p, M.v32.p), dA, dB, (T)alpha, (T)beta, x, y);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

}  // namespace

int upload_csr(DevCsr& d, int n, const int* ia, const int* ja, const double* a,
               cudaStream_t s)
{
    if (n <= 0 || !ia || !ja || !a) {
        set_error("upload_csr: bad arguments");
        return XT_ERR_ARG;
    }
    const int nnz = ia[n] - ia[0];
    if (nnz < 0 || ia[0] != 1) {
        set_error("upload_csr: row pointers must be 1-based and non-decreasing");
        return XT_ERR_ARG;
    }
    for (int r = 0; r < n; ++r)
        if (ia[r + 1] < ia[r]) {
            set_error("upload_csr: row pointers decrease");
            return XT_ERR_ARG;
        }
    for (int k = 0; k < nnz; ++k)
        if (ja[k] < 1 || ja[k] > n) {
            set_error("upload_csr: column index out of range");
            return XT_ERR_ARG;
        }
    d.n = n;
    d.nnz = nnz;
    d.same_pattern = false;
    d.vdf.release();  // remade from the new values on first use
    d.nb.ok = false;  // rebuilt by csr_build_node_blocks
    XT_TRY(d.rowptr.upload(ia, (size_t)n + 1, s));
    XT_TRY(d.col.upload(ja, (size_t)(nnz > 0 ? nnz : 0), s));
    XT_TRY(d.v64.upload(a, (size_t)nnz, s));
    XT_TRY(d.v32.alloc((size_t)nnz));
    k_dec_index<<<256, 256, 0, s>>>(d.rowptr.p, (size_t)n + 1);
    if (nnz) {
        k_dec_index<<<1024, 256, 0, s>>>(d.col.p, (size_t)nnz);
        k_to_f32<<<1024, 256, 0, s>>>(d.v64.p, d.v32.p, (size_t)nnz);
    }
    note_launches(3);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

void csr_mark_shared_pattern(const DevCsr& K, DevCsr& M, const int* ki, const int* kj,
                             const int* mi, const int* mj)
{
    M.same_pattern = false;
    if (K.n != M.n || K.nnz != M.nnz) return;
    if (std::memcmp(ki, mi, sizeof(int) * ((size_t)K.n + 1)) != 0) return;
    if (std::memcmp(kj, mj, sizeof(int) * (size_t)K.nnz) != 0) return;
    M.same_pattern = true;
}

int csr_build_node_blocks(DevCsr& K, int n, const int* ki, const int* kj, const double* kv,
                          const int* mi, const int* mj, const double* mv, cudaStream_t s)
{
    DevNodeBlocks& nb = K.nb;
    nb.ok = false;
    if (n <= 0 || n % 3 != 0 || K.n != n) return XT_OK;
    const int nodes = n / 3;
    std::vector<int> ptr(nodes + 1, 0), col;
    std::vector<float2> kdf, mdf;
    std::vector<int> pos(nodes, -1);  // block index of neighbour node b in the current row
    std::vector<int> from_csr((size_t)K.nnz, -1);
    auto split = [](double v) {
        const float h = (float)v;
        return make_float2(h, (float)(v - (double)h));
    };
    for (int a = 0; a < nodes; ++a) {
        const int first = (int)col.size();
        for (int c = 0; c < 3; ++c)
            for (int k = ki[3 * a + c] - 1; k < ki[3 * a + c + 1] - 1; ++k) {
                const int b = (kj[k] - 1) / 3;
                if (pos[b] < 0) {
                    pos[b] = (int)col.size();
                    col.push_back(b);
                    kdf.resize(kdf.size() + 9, make_float2(0.f, 0.f));
                    mdf.push_back(make_float2(0.f, 0.f));
                }
            }
        // neighbour nodes in ascending order (the CSR columns are sorted)
        std::vector<int> order(col.begin() + first, col.end());
        std::sort(order.begin(), order.end());
        for (size_t t = 0; t < order.size(); ++t) pos[order[t]] = first + (int)t;
        std::copy(order.begin(), order.end(), col.begin() + first);
        for (int c = 0; c < 3; ++c)
            for (int k = ki[3 * a + c] - 1; k < ki[3 * a + c + 1] - 1; ++k) {
                const int j = kj[k] - 1, b = j / 3;
                const size_t at = (size_t)pos[b] * 9 + c * 3 + (j - 3 * b);
                kdf[at] = split(kv[k]);
                from_csr[k] = (int)at;
            }
        // M: m_ab on the three diagonal entries of each block, nothing else
        std::vector<double> mval(order.size(), 0.0);
        std::vector<int> mcount(order.size(), 0);
        bool fits = true;
        for (int c = 0; c < 3 && fits; ++c)
            for (int k = mi[3 * a + c] - 1; k < mi[3 * a + c + 1] - 1; ++k) {
                const int j = mj[k] - 1, b = j / 3;
                if (j - 3 * b != c || pos[b] < 0) { fits = false; break; }
                const int t = pos[b] - first;
                if (mcount[t] > 0 && mval[t] != mv[k]) { fits = false; break; }
                mval[t] = mv[k];
                ++mcount[t];
            }
        for (size_t t = 0; t < order.size() && fits; ++t) {
            if (mcount[t] != 0 && mcount[t] != 3) fits = false;
            mdf[first + t] = split(mval[t]);
        }
        for (int b : order) pos[b] = -1;
        if (!fits) return XT_OK;  // no exact node-block form: the CSR kernel stays
        ptr[a + 1] = (int)col.size();
    }
    nb.nodes = nodes;
    nb.nblocks = (int)col.size();
    XT_TRY(nb.ptr.upload(ptr.data(), ptr.size(), s));
    XT_TRY(nb.col.upload(col.data(), col.size(), s));
    XT_TRY(nb.kdf.upload(kdf.data(), kdf.size(), s));
    XT_TRY(nb.mdf.upload(mdf.data(), mdf.size(), s));
    XT_TRY(nb.from_csr.upload(from_csr.data(), from_csr.size(), s));
    XT_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
    nb.ok = true;
    return XT_OK;
}

int node_blocks_refresh(DevCsr& K, cudaStream_t s)
{
    if (!K.nb.ok || K.nnz == 0) return XT_OK;
    k_scatter_df<<<std::max(1, std::min(4096, (K.nnz + 255) / 256)), 256, 0, s>>>(
        K.v64.p, K.nb.from_csr.p, K.nb.kdf.p, (size_t)K.nnz);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int to_f32(const double* a, float* b, size_t n, cudaStream_t s)
{
    if (n == 0) return XT_OK;
    size_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_to_f32<<<(int)blocks, 256, 0, s>>>(a, b, n);
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

template <class T>
int kron_spmm(const DevCsr& K, const DevCsr& M, int q, const double* dA,
              const double* dB, double alpha, double beta, const T* x, T* y,
              cudaStream_t s)
{
    if (K.n != M.n || q < 1 || q > 8) {
        set_error("kron_spmm: K and M must have the same order and 1 <= q <= 8");
        return XT_ERR_ARG;
    }
    if (K.n == 0) return XT_OK;
    switch (q) {
    case 1: return launch_q<T, 1>(K, M, dA, dB, alpha, beta, x, y, s);
    case 2: return launch_q<T, 2>(K, M, dA, dB, alpha, beta, x, y, s);
    case 3: return launch_q<T, 3>(K, M, dA, dB, alpha, beta, x, y, s);
    case 4: return launch_q<T, 4>(K, M, dA, dB, alpha, beta, x, y, s);
    case 5: return launch_q<T, 5>(K, M, dA, dB, alpha, beta, x, y, s);
    case 6: return launch_q<T, 6>(K, M, dA, dB, alpha, beta, x, y, s);
    case 7: return launch_q<T, 7>(K, M, dA, dB, alpha, beta, x, y, s);
    default: return launch_q<T, 8>(K, M, dA, dB, alpha, beta, x, y, s);
    }
}

bool kron_nb_batchable(const DevCsr& K, int q)
{
    return K.nb.ok && q % 2 == 0 && q >= 2 && q <= 8 && nb_enabled();
}

int kron_nb_batch(const FlexStepItem* t, int count, int q, const FlexStepDims& d, cudaStream_t s)
{
    if (count <= 0) return XT_OK;
    // a quarter of the largest system's node rows per block pass: each warp
    // loops over about four row groups (any split gives the same rows)
    const int RPW = q == 2 ? 10 : (q == 4 ? 5 : (q == 6 ? 3 : 2));
    const int rows_per_block = 8 * RPW;
    const int gx = std::max(1, (d.nodes_max + 4 * rows_per_block - 1) / (4 * rows_per_block));
    const dim3 grid(gx, count);
    switch (q) {
    case 2: kb_kron_nb<2><<<grid, 256, 0, s>>>(t); break;
    case 4: kb_kron_nb<4><<<grid, 256, 0, s>>>(t); break;
    case 6: kb_kron_nb<6><<<grid, 256, 0, s>>>(t); break;
    case 8: kb_kron_nb<8><<<grid, 256, 0, s>>>(t); break;
    default: set_error("kron_nb_batch: q must be 2, 4, 6 or 8"); return XT_ERR_ARG;
    }
    note_launches(1);
    XT_CUDA(cudaGetLastError());
    return XT_OK;
}

int kron_spmm_df(DevCsr& K, DevCsr& M, int q, const double* dA, const double* dB, const float* x,
                 float2* y, cudaStream_t s, const int* skip)
{
    if (K.n != M.n || q < 1 || q > 8) {
        set_error("kron_spmm_df: K and M must have the same order and 1 <= q <= 8");
        return XT_ERR_ARG;
    }
    if (K.n == 0) return XT_OK;
    // node blocks: y must be 16-byte aligned (one float4 store per lane)
    if (K.nb.ok && q % 2 == 0 && reinterpret_cast<uintptr_t>(y) % 16 == 0 &&
        reinterpret_cast<uintptr_t>(x) % 8 == 0 && nb_enabled()) {
        switch (q) {
        case 2: return launch_nb<2>(K.nb, dA, dB, x, y, s, skip);
        case 4: return launch_nb<4>(K.nb, dA, dB, x, y, s, skip);
        case 6: return launch_nb<6>(K.nb, dA, dB, x, y, s, skip);
        default: return launch_nb<8>(K.nb, dA, dB, x, y, s, skip);
        }
    }
    XT_TRY(ensure_df(K, s));
    XT_TRY(ensure_df(M, s));
    switch (q) {
    case 1: return launch_df<1>(K, M, dA, dB, x, y, s);
    case 2: return launch_df<2>(K, M, dA, dB, x, y, s);
    case 3: return launch_df<3>(K, M, dA, dB, x, y, s);
    case 4: return launch_df<4>(K, M, dA, dB, x, y, s);
    case 5: return launch_df<5>(K, M, dA, dB, x, y, s);
    case 6: return launch_df<6>(K, M, dA, dB, x, y, s);
    case 7: return launch_df<7>(K, M, dA, dB, x, y, s);
    default: return launch_df<8>(K, M, dA, dB, x, y, s);
    }
}

int kron_spmm_bf16(DevCsr& K, DevCsr& M, int q, const double* dA, const double* dB,
                   double alpha, double beta, const float* x, float* y, cudaStream_t s)
{
    if (K.n != M.n || q < 1 || q > 8) {
        set_error("kron_spmm_bf16: K and M must have the same order and 1 <= q <= 8");
        return XT_ERR_ARG;
    }
    if (K.n == 0) return XT_OK;
    XT_TRY(ensure_bf16(K, s));
    XT_TRY(ensure_bf16(M, s));
    switch (q) {
    case 1: return launch_bf16<1>(K, M, dA, dB, alpha, beta, x, y, s);
    case 2: return launch_bf16<2>(K, M, dA, dB, alpha, beta, x, y, s);
    case 3: return launch_bf16<3>(K, M, dA, dB, alpha, beta, x, y, s);
    case 4: return launch_bf16<4>(K, M, dA, dB, alpha, beta, x, y, s);
    case 5: return launch_bf16<5>(K, M, dA, dB, alpha, beta, x, y, s);
    case 6: return launch_bf16<6>(K, M, dA, dB, alpha, beta, x, y, s);
    case 7: return launch_bf16<7>(K, M, dA, dB, alpha, beta, x, y, s);
    default: return launch_bf16<8>(K, M, dA, dB, alpha, beta, x, y, s);
    }
}

template int kron_spmm<double>(const DevCsr&, const DevCsr&, int, const double*,
                               const double*, double, double, const double*, double*,
                               cudaStream_t);
template int kron_spmm<float>(const DevCsr&, const DevCsr&, int, const double*,
                              const double*, double, double, const float*, float*,
                              cudaStream_t);

}  // namespace xt
