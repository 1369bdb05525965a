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
#include <cstring>

#include "df.cuh"
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

template <class T, int Q, int LANES, bool MERGED>
__global__ void __launch_bounds__(256)
k_kron_spmm(int p, const int* __restrict__ kptr, const int* __restrict__ kcol,
            const T* __restrict__ kval, const int* __restrict__ mptr,
            const int* __restrict__ mcol, const T* __restrict__ mval,
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
                const T vk = kval[k], vm = mval[k];
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
                const T v = kval[k];
                T xr[Q];
                load_row<T, Q>(x + (size_t)kcol[k] * Q, xr);
#pragma unroll
                for (int b = 0; b < Q; ++b) ak[b] = fma(v, xr[b], ak[b]);
            }
            const int m0 = act ? mptr[r] : 0, m1 = act ? mptr[r + 1] : 0;
#pragma unroll 4
            for (int k = m0 + lane; k < m1; k += LANES) {
                const T v = mval[k];
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

int kron_spmm_df(DevCsr& K, DevCsr& M, int q, const double* dA, const double* dB, const float* x,
                 float2* y, cudaStream_t s)
{
    if (K.n != M.n || q < 1 || q > 8) {
        set_error("kron_spmm_df: K and M must have the same order and 1 <= q <= 8");
        return XT_ERR_ARG;
    }
    if (K.n == 0) return XT_OK;
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

template int kron_spmm<double>(const DevCsr&, const DevCsr&, int, const double*,
                               const double*, double, double, const double*, double*,
                               cudaStream_t);
template int kron_spmm<float>(const DevCsr&, const DevCsr&, int, const double*,
                              const double*, double, double, const float*, float*,
                              cudaStream_t);

}  // namespace xt
