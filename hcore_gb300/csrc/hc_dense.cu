// hcore-gb300 — dense-C tile updates on sm_103a:
//   HCORE_dsyrk   (src/compute/hcore_dsyrk.c:47-189)
//       CD = alpha * AU (AV^T AV) AU^T + CD, strict upper triangle := 0
//   HCORE_dgemmcd (src/compute/hcore_dgemmcd.c:36-106)
//       CD = CD - Au (Av^T Bv) Bu^T (associated by the smaller rank, :72)
//   HCORE_duncompress (src/compute/hcore_duncompress.c:33-84)
//       CD = AU BV^T
//   HCORE_dgemmbdcd (src/compute/hcore_dgemmbdcd.c:35-122)
//       CD = alpha AU (AV^T BD) + beta CD
//   HCORE_dgemm_dense (src/compute/hcore_dgemm.c:1701-1715)
//       C = alpha op(A) op(B) + beta C
//
// Every contribution is first reduced to a rank-K' product beta CD +
// coef * P Q^T with P of size M x K' and Q of size N x K' (prep kernels: one
// CTA per syrk/gemmcd task, a tiled GEMM for the gemmbdcd product
// Q = BD^T AV; uncompress needs none), and all tasks that hit the same tile
// are then applied in list order by one tile kernel that keeps a 64 x 64
// block of CD in registers.  Zeroing the
// strict upper triangle after each syrk task reproduces the reference's
// sequential semantics exactly; the syrk's own upper-triangle products are
// never computed since they are overwritten by zero.
#include <cuda_runtime.h>

#include <climits>

#include "hc_internal.h"

namespace hc {

template <typename T>
__device__ __forceinline__ T wsum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// S = X^T Y (p x q, reduce over n rows), then the computed factor:
//   syrk:                       P = AU S                 (M x K)
//   gemmcd, a > b:              P = Au rr                (M x b)
//   gemmcd, a <= b:             Q = Bu rr^T              (M x a)
__global__ void __launch_bounds__(256) dense_prep_kernel(const hcore_dense_task *tasks,
                                                         const DenseWork *work, double *ws) {
    const hcore_dense_task t = tasks[blockIdx.x];
    if (t.kind > 1) return;  // uncompress: no prep; gemmbdcd: bdcd_prep_kernel
    const DenseWork w = work[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double *S = ws + w.ws;
    const double *X, *Y;
    int p, q, n, ldx, ldy;
    if (t.kind == 0) {  // AV^T AV over LDAU rows (hcore_dsyrk.c:57,103)
        X = t.Av; Y = t.Av; p = t.a; q = t.a; n = t.lda; ldx = t.lda; ldy = t.lda;
    } else {            // Av^T Bv over M rows (hcore_dgemmcd.c:66-70)
        X = t.Av; Y = t.Bv; p = t.a; q = t.b; n = t.M; ldx = t.M; ldy = t.M;
    }
    for (int e = warp; e < p * q; e += 8) {
        const int i = e % p, j = e / p;
        double s = 0;
        for (int l = lane; l < n; l += 32) s += X[(size_t)i * ldx + l] * Y[(size_t)j * ldy + l];
        s = wsum(s);
        if (lane == 0) S[(size_t)j * p + i] = s;
    }
    __syncthreads();
    double *out = S + (size_t)p * q;
    const int M = t.M;
    if (t.kind == 0) {  // P = AU S (M x a)
        for (long long e = tid; e < (long long)M * t.a; e += 256) {
            const int i = (int)(e % M), j = (int)(e / M);
            double s = 0;
            for (int l = 0; l < t.a; ++l) s += t.Au[(size_t)l * t.lda + i] * S[(size_t)j * p + l];
            out[(size_t)j * M + i] = s;
        }
    } else if (t.a > t.b) {  // P = Au rr (M x b)
        for (long long e = tid; e < (long long)M * t.b; e += 256) {
            const int i = (int)(e % M), j = (int)(e / M);
            double s = 0;
            for (int l = 0; l < t.a; ++l) s += t.Au[(size_t)l * M + i] * S[(size_t)j * p + l];
            out[(size_t)j * M + i] = s;
        }
    } else {  // Q = Bu rr^T (M x a)
        for (long long e = tid; e < (long long)M * t.a; e += 256) {
            const int i = (int)(e % M), j = (int)(e / M);
            double s = 0;
            for (int l = 0; l < t.b; ++l) s += t.Bu[(size_t)l * M + i] * S[(size_t)l * p + j];
            out[(size_t)j * M + i] = s;
        }
    }
}

// One CTA per (64 x 64 tile of CD, group).  Thread (tx, ty) owns a 4 x 4
// register block; K' is staged in chunks of 16 through shared memory.
constexpr int TB = 64, TK = 16;

// gemmbdcd prep: Q = BD^T AV (N x a, ld N) into the task's workspace, i.e.
// (AV^T BD)^T of hcore_dgemmbdcd.c:80-87/:99-106, summed over kdim rows.
// One CTA per (64 rows of Q, 64 columns of Q, task); both operands are read
// along their contiguous dimension (16 consecutive rows of a column).
__global__ void __launch_bounds__(256) bdcd_prep_kernel(const hcore_dense_task *tasks,
                                                        const DenseWork *work, const int *idx,
                                                        int tilesN, int tilesA, double *ws) {
    __shared__ double sB[TK][TB + 1];
    __shared__ double sA[TK][TB + 1];
    const int ti = blockIdx.x % tilesN;
    const int tj = (blockIdx.x / tilesN) % tilesA;
    const int q = blockIdx.x / (tilesN * tilesA);
    const int task = idx[q];
    const hcore_dense_task t = tasks[task];
    const int N = t.N ? t.N : t.M, K = t.kdim ? t.kdim : t.M, a = t.a;
    const int row0 = ti * TB, col0 = tj * TB;  // rows of Q (columns of BD), columns of Q
    if (row0 >= N || col0 >= a) return;
    double *Q = ws + work[task].ws;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += TK) {
        for (int e = threadIdx.x; e < TK * TB; e += 256) {
            const int kk = e % TK, r = e / TK;
            const int kg = k0 + kk;
            sB[kk][r] = (kg < K && row0 + r < N) ? t.Bd[(size_t)(row0 + r) * t.ldb + kg] : 0.0;
            sA[kk][r] = (kg < K && col0 + r < a) ? t.Av[(size_t)(col0 + r) * t.lda + kg] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            double bv[4], av[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) bv[u] = sB[kk][tx + 16 * u];
#pragma unroll
            for (int v = 0; v < 4; ++v) av[v] = sA[kk][ty + 16 * v];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] += bv[u] * av[v];
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = row0 + tx + 16 * u, j = col0 + ty + 16 * v;
            if (i < N && j < a) Q[(size_t)j * N + i] = acc[u][v];
        }
}

__global__ void __launch_bounds__(256) dense_tile_kernel(const hcore_dense_task *tasks,
                                                         const DenseWork *work,
                                                         const int *group_start,
                                                         const int *group_tasks, int tiles_per_dim) {
    __shared__ double sP[TK][TB + 1];
    __shared__ double sQ[TK][TB + 1];
    const int g = blockIdx.y;
    const int tile = blockIdx.x;
    const int bi = tile % tiles_per_dim, bj = tile / tiles_per_dim;
    const int g0 = group_start[g], g1 = group_start[g + 1];
    if (g0 == g1) return;
    const hcore_dense_task t0 = tasks[group_tasks[g0]];
    const int M = t0.M, N = t0.N ? t0.N : t0.M;
    const int row0 = bi * TB, col0 = bj * TB;
    if (row0 >= M || col0 >= N) return;
    double *CD = t0.CD;
    const int ldcd = t0.ldcd;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = row0 + tx + 16 * u, j = col0 + ty + 16 * v;
            acc[u][v] = (i < M && j < N) ? CD[(size_t)j * ldcd + i] : 0.0;
        }
    const bool strictly_upper = row0 + TB <= col0;  // every (i, j) here has i < j
    for (int gi = g0; gi < g1; ++gi) {
        const DenseWork w = work[group_tasks[gi]];
        if (w.beta != 1.0) {  // beta = 0 does not read CD (BLAS convention)
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = w.beta == 0.0 ? 0.0 : w.beta * acc[u][v];
        }
        if (!(w.syrk && strictly_upper)) {
            for (int k0 = 0; k0 < w.kk; k0 += TK) {
                // the task's coefficient is folded into P as it is staged
                // (once per element, not once per use)
                for (int e = threadIdx.x; e < TK * TB; e += 256) {
                    const int kk = e / TB, r = e % TB;
                    const int kg = k0 + kk;
                    sP[kk][r] = (kg < w.kk && row0 + r < M) ? w.coef * w.P[(size_t)kg * w.ldp + row0 + r] : 0.0;
                    sQ[kk][r] = (kg < w.kk && col0 + r < N) ? w.Q[(size_t)kg * w.ldq + col0 + r] : 0.0;
                }
                __syncthreads();
#pragma unroll
                for (int kk = 0; kk < TK; ++kk) {
                    double pv[4], qv[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) pv[u] = sP[kk][tx + 16 * u];
#pragma unroll
                    for (int v = 0; v < 4; ++v) qv[v] = sQ[kk][ty + 16 * v];
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int v = 0; v < 4; ++v) acc[u][v] += pv[u] * qv[v];
                }
                __syncthreads();
            }
        }
        if (w.syrk) {
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v)
                    if (row0 + tx + 16 * u < col0 + ty + 16 * v) acc[u][v] = 0.0;
        }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = row0 + tx + 16 * u, j = col0 + ty + 16 * v;
            if (i < M && j < N) CD[(size_t)j * ldcd + i] = acc[u][v];
        }
}

cudaError_t launch_dense_prep(const hcore_dense_task *d_tasks, const DenseWork *d_work, int n,
                              double *ws, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    dense_prep_kernel<<<n, 256, 0, s>>>(d_tasks, d_work, ws);
    return cudaGetLastError();
}

cudaError_t launch_bdcd_prep(const hcore_dense_task *d_tasks, const DenseWork *d_work,
                             const int *d_idx, int n_idx, int maxN, int maxA, double *ws,
                             cudaStream_t s) {
    if (n_idx <= 0 || maxN <= 0 || maxA <= 0) return cudaSuccess;
    const int tn = (maxN + TB - 1) / TB, ta = (maxA + TB - 1) / TB;
    const long long blocks = (long long)tn * ta * n_idx;
    if (blocks > INT_MAX) return cudaErrorInvalidValue;
    bdcd_prep_kernel<<<(unsigned)blocks, 256, 0, s>>>(d_tasks, d_work, d_idx, tn, ta, ws);
    return cudaGetLastError();
}

cudaError_t launch_dense_tiles(const hcore_dense_task *d_tasks, const DenseWork *d_work,
                               const int *d_group_start, const int *d_group_tasks, int ngroups,
                               int maxDim, cudaStream_t s) {
    if (ngroups <= 0) return cudaSuccess;
    const int tpd = (maxDim + TB - 1) / TB;
    dense_tile_kernel<<<dim3(tpd * tpd, ngroups), 256, 0, s>>>(d_tasks, d_work, d_group_start,
                                                               d_group_tasks, tpd);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// plain dense GEMM, C = alpha op(A) op(B) + beta C (HCORE_dgemm_dense)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) gemm_dense_kernel(int ta, int tb, int M, int N, int K,
                                                         T alpha, const T *A, int lda, const T *B,
                                                         int ldb, T beta, T *C, int ldc) {
    __shared__ T sA[TK][TB + 1];
    __shared__ T sB[TK][TB + 1];
    const int row0 = blockIdx.x * TB, col0 = blockIdx.y * TB;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += TK) {
        for (int e = threadIdx.x; e < TK * TB; e += 256) {
            const int kk = e / TB, r = e % TB;
            const int kg = k0 + kk, i = row0 + r, j = col0 + r;
            T av = 0, bv = 0;
            if (kg < K && i < M) av = ta ? A[(size_t)i * lda + kg] : A[(size_t)kg * lda + i];
            if (kg < K && j < N) bv = tb ? B[(size_t)kg * ldb + j] : B[(size_t)j * ldb + kg];
            sA[kk][r] = av;
            sB[kk][r] = bv;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            T pv[4], qv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) pv[u] = sA[kk][tx + 16 * u];
#pragma unroll
            for (int v = 0; v < 4; ++v) qv[v] = sB[kk][ty + 16 * v];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] += pv[u] * qv[v];
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = row0 + tx + 16 * u, j = col0 + ty + 16 * v;
            if (i < M && j < N) {
                T *c = C + (size_t)j * ldc + i;
                *c = alpha * acc[u][v] + (beta == T(0) ? T(0) : beta * *c);
            }
        }
}

template <typename T>
cudaError_t launch_gemm_dense(int ta, int tb, int M, int N, int K, T alpha, const T *A, int lda,
                              const T *B, int ldb, T beta, T *C, int ldc, cudaStream_t s) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    dim3 grid((M + TB - 1) / TB, (N + TB - 1) / TB);
    gemm_dense_kernel<T><<<grid, 256, 0, s>>>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
    return cudaGetLastError();
}
template cudaError_t launch_gemm_dense<double>(int, int, int, int, int, double, const double *, int,
                                               const double *, int, double, double *, int,
                                               cudaStream_t);
template cudaError_t launch_gemm_dense<float>(int, int, int, int, int, float, const float *, int,
                                              const float *, int, float, float *, int, cudaStream_t);

}  // namespace hc
