// hcore-gb300 — the steps either side of the Schur update in a tile low-rank
// Cholesky, on sm_103a:
//   HCORE_dtrsm  (src/compute/hcore_dtrsm.c:24-48): B = alpha op(A)^-1 B or
//                alpha B op(A)^-1, A triangular; in the TLR Cholesky B is a
//                tile's V factor and A the panel's diagonal Cholesky factor
//   HCORE_dpotrf (src/compute/hcore_dpotrf.c:23-34): Cholesky factor of a
//                dense diagonal tile
//
// TRSM.  Every task is cut into groups of up to S right-hand-side vectors
// (columns of B for the left side, rows of B for the right side), one CTA
// per group.  The CTA keeps its S vectors in shared memory for the whole
// solve and turns every case into a forward substitution with a lower
// triangular T' (transposing and/or reversing the index order of A).  T' is
// walked in 32-column blocks: the block's diagonal part is solved by one warp
// per vector (lane i holds x_i; 32 steps with a shuffle), then the rows below
// are updated with the block's 32 solved values, 64 rows at a time through a
// shared-memory tile of T' that every vector of the CTA reuses.  Tiles are
// read along A's contiguous dimension, so a transposed A is read coalesced
// too.  A task's groups share A, which stays in L2.
//
// POTRF.  Blocked right-looking Cholesky on the lower view of the tile (the
// transposed view for uplo 'U'), 64 columns per block, three launches per
// block: the diagonal block (left-looking columns in shared memory, the
// reference LAPACK's pivot test: a pivot that is not > 0, or is NaN, stops
// the factorization and is left in place), the panel below it
// (A_ik = A_ik L_kk^-T, 64 rows per CTA, the 64 components of a row spread
// over 4 threads), and the trailing lower triangle (A_ij -= A_ik A_jk^T,
// 32 x 32 tiles, 2 x 2 register blocks).  Every launch first reads the
// task's info and returns once a pivot has failed.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <vector>

#include "hc_host.h"
#include "hcore.h"
#include "hcore_d.h"

namespace hc {

constexpr int kTrBs = 32;  // diagonal block of T'
constexpr int kTrRc = 64;  // rows per trailing chunk

struct TrsmWork {
    int task, v0, nv, pad;
};

// T' = the lower triangular form of the task's system (see the file comment):
// element (i, j) of T' is A(p, q) or A(q, p), p and q the indices i, j taken
// in reverse order when the effective triangle is upper.
struct TrsmView {
    const double *A;
    int lda, n;
    bool tflag, rev;
    __device__ double at(int i, int j) const {
        const int p = rev ? n - 1 - i : i, q = rev ? n - 1 - j : j;
        return tflag ? A[(size_t)p * lda + q] : A[(size_t)q * lda + p];
    }
};

// T'(r0 + r, c0 + c) for r < rows, c < cols into T (zero elsewhere, R rows)
template <int R>
__device__ __forceinline__ void trsm_tile(double (*T)[kTrBs + 1], const TrsmView &v, int r0, int rows, int c0,
                          int cols) {
    for (int e = threadIdx.x; e < R * kTrBs; e += blockDim.x) {
        int r, c;
        if (v.tflag) {  // A(q, p): contiguous in q, i.e. along a row of T'
            c = e % kTrBs; r = e / kTrBs;
        } else {        // A(p, q): contiguous in p, i.e. along a column of T'
            r = e % R; c = e / R;
        }
        T[r][c] = (r < rows && c < cols) ? v.at(r0 + r, c0 + c) : 0.0;
    }
}

__global__ void __launch_bounds__(256) trsm_kernel(const hcore_trsm_task *tasks,
                                                   const TrsmWork *work, int S) {
    extern __shared__ double X[];  // X[i * S + v]
    __shared__ double Tt[kTrRc][kTrBs + 1];
    __shared__ double Td[kTrBs][kTrBs + 1];
    const TrsmWork w = work[blockIdx.x];
    const hcore_trsm_task t = tasks[w.task];
    const bool left = t.side == HCORE_Left;
    TrsmView v;
    v.A = t.A;
    v.lda = t.lda;
    v.n = left ? t.M : t.N;
    v.tflag = left ? t.trans != HCORE_NoTrans : t.trans == HCORE_NoTrans;
    v.rev = (t.uplo == HCORE_Lower) == v.tflag;  // effective triangle is upper
    const int n = v.n;
    const bool unit = t.diag == HCORE_Unit;
    // element i of vector u: B[i * es + u * vs]
    const size_t es = left ? 1 : (size_t)t.ldb, vs = left ? (size_t)t.ldb : 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (t.alpha == 0.0) {  // B = 0 without reading A (BLAS convention)
        for (int e = tid; e < n * w.nv; e += blockDim.x) {
            const int i = left ? e % n : e / w.nv, u = left ? e / n : e % w.nv;
            t.B[(size_t)i * es + (size_t)(w.v0 + u) * vs] = 0.0;
        }
        return;
    }
    for (int e = tid; e < n * S; e += blockDim.x) {
        const int i = left ? e % n : e / S, u = left ? e / n : e % S;
        double x = 0.0;
        if (u < w.nv) {
            const int ia = v.rev ? n - 1 - i : i;
            x = t.alpha * t.B[(size_t)ia * es + (size_t)(w.v0 + u) * vs];
        }
        X[i * S + u] = x;
    }
    __syncthreads();
    for (int b0 = 0; b0 < n; b0 += kTrBs) {
        const int bs = min(kTrBs, n - b0);
        trsm_tile<kTrBs>(Td, v, b0, bs, b0, bs);
        __syncthreads();
        if (warp < w.nv) {  // one warp per vector: forward substitution in the block
            double x = lane < bs ? X[(b0 + lane) * S + warp] : 0.0;
            // x_j = b_j / T'_jj as a product with the reciprocal (one division
            // per lane and block instead of one per step)
            const double rd = (unit || lane >= bs) ? 1.0 : 1.0 / Td[lane][lane];
            for (int j = 0; j < bs; ++j) {
                if (lane == j) x *= rd;
                const double xj = __shfl_sync(0xffffffffu, x, j);
                if (lane > j) x -= Td[lane][j] * xj;
            }
            if (lane < bs) X[(b0 + lane) * S + warp] = x;
        }
        __syncthreads();
        for (int r0 = b0 + bs; r0 < n; r0 += kTrRc) {
            const int rc = min(kTrRc, n - r0);
            trsm_tile<kTrRc>(Tt, v, r0, rc, b0, bs);
            __syncthreads();
            for (int o = tid; o < kTrRc * S; o += blockDim.x) {
                const int u = o % S, r = o / S;
                if (r < rc && u < w.nv) {
                    double acc = X[(r0 + r) * S + u];
#pragma unroll 8
                    for (int j = 0; j < bs; ++j) acc -= Tt[r][j] * X[(b0 + j) * S + u];
                    X[(r0 + r) * S + u] = acc;
                }
            }
            __syncthreads();
        }
    }
    for (int e = tid; e < n * w.nv; e += blockDim.x) {
        const int i = left ? e % n : e / w.nv, u = left ? e / n : e % w.nv;
        const int ia = v.rev ? n - 1 - i : i;
        t.B[(size_t)ia * es + (size_t)(w.v0 + u) * vs] = X[i * S + u];
    }
}

// ---------------------------------------------------------------------------
// POTRF
// ---------------------------------------------------------------------------
constexpr int kPb = 64;  // block width

// element (i, j), i >= j, of the lower view
struct PotrfView {
    double *A;
    int lda;
    bool up;
    __device__ double &at(int i, int j) const {
        return up ? A[(size_t)i * lda + j] : A[(size_t)j * lda + i];
    }
};

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// diagonal block [kb, kb + bs): left-looking columns (LAPACK dpotf2 order);
// a failing pivot is stored in place and ends the task (info = column + 1)
__global__ void __launch_bounds__(256) potrf_diag_kernel(const hcore_potrf_task *tasks, int *info,
                                                         int kb) {
    __shared__ double S[kPb][kPb + 1];
    __shared__ double rpiv;
    __shared__ int fail;
    const hcore_potrf_task t = tasks[blockIdx.x];
    if (info[blockIdx.x] != 0 || kb >= t.n) return;
    const int bs = min(kPb, t.n - kb);
    const PotrfView V{t.A, t.lda, t.uplo == 'U' || t.uplo == 'u'};
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int e = tid; e < kPb * kPb; e += 256) {
        const int i = e % kPb, j = e / kPb;
        S[i][j] = (i < bs && j <= i) ? V.at(kb + i, kb + j) : 0.0;
    }
    if (tid == 0) fail = -1;
    __syncthreads();
    const int row = tid >> 2, part = tid & 3;  // 4 threads per row
    for (int j = 0; j < bs; ++j) {
        if (warp == 0) {
            double s = 0.0;
            for (int l = lane; l < j; l += 32) s += S[j][l] * S[j][l];
            s = warp_sum_d(s);
            if (lane == 0) {
                const double d = S[j][j] - s;
                if (!(d > 0.0)) {  // not positive, or NaN
                    S[j][j] = d;
                    fail = j;
                } else {
                    const double l = sqrt(d);
                    S[j][j] = l;
                    rpiv = 1.0 / l;  // the column is scaled by the reciprocal, as dpotf2 does
                }
            }
        }
        __syncthreads();
        if (fail >= 0) break;
        double s = 0.0;
        if (row > j && row < bs)
            for (int l = part; l < j; l += 4) s += S[row][l] * S[j][l];
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (part == 0 && row > j && row < bs) S[row][j] = (S[row][j] - s) * rpiv;
        __syncthreads();
    }
    for (int e = tid; e < kPb * kPb; e += 256) {
        const int i = e % kPb, j = e / kPb;
        if (i < bs && j <= i) V.at(kb + i, kb + j) = S[i][j];
    }
    if (tid == 0 && fail >= 0) info[blockIdx.x] = kb + fail + 1;
}

// panel rows [r0, r0 + 64) below the diagonal block: X L_kk^T = A_ik.
// Thread (r, q) holds components q, q + 4, ... of row r in registers; the
// solve runs over the columns c in order, one barrier per column.
__global__ void __launch_bounds__(256) potrf_panel_kernel(const hcore_potrf_task *tasks,
                                                          const int *info, int kb) {
    __shared__ double Ls[kPb][kPb + 1];
    __shared__ double Xs[kPb][kPb + 1];
    __shared__ double rL[kPb];
    const hcore_potrf_task t = tasks[blockIdx.y];
    if (info[blockIdx.y] != 0 || kb >= t.n) return;
    const int bs = min(kPb, t.n - kb);
    const int r0 = kb + bs + blockIdx.x * kPb;
    if (r0 >= t.n) return;
    const int rows = min(kPb, t.n - r0);
    const PotrfView V{t.A, t.lda, t.uplo == 'U' || t.uplo == 'u'};
    const int tid = threadIdx.x;
    for (int e = tid; e < kPb * kPb; e += 256) {
        const int i = e % kPb, j = e / kPb;
        Ls[i][j] = (i < bs && j <= i) ? V.at(kb + i, kb + j) : 0.0;
    }
    const int r = tid & 63, q = tid >> 6;
    double a[kPb / 4];
#pragma unroll
    for (int m = 0; m < kPb / 4; ++m) {
        const int c = q + 4 * m;
        a[m] = (r < rows && c < bs) ? V.at(r0 + r, kb + c) : 0.0;
    }
    if (tid < bs) rL[tid] = 1.0 / V.at(kb + tid, kb + tid);
    __syncthreads();
    for (int c = 0; c < bs; ++c) {
        if (q == (c & 3)) {
#pragma unroll
            for (int m = 0; m < kPb / 4; ++m)
                if (q + 4 * m == c) {
                    a[m] *= rL[c];
                    Xs[r][c] = a[m];
                }
        }
        __syncthreads();
        const double xc = Xs[r][c];
#pragma unroll
        for (int m = 0; m < kPb / 4; ++m) {
            const int l = q + 4 * m;
            if (l > c && l < bs) a[m] -= xc * Ls[l][c];
        }
    }
    __syncthreads();
    for (int e = tid; e < kPb * kPb; e += 256) {
        const int i = e % kPb, j = e / kPb;
        if (i < rows && j < bs) V.at(r0 + i, kb + j) = Xs[i][j];
    }
}

// trailing lower triangle from row/column t0 = kb + bs: A_ij -= A_ik A_jk^T,
// one CTA per 32 x 32 tile (bi >= bj), 2 x 2 outputs per thread, K = bs
// staged 16 at a time.  Small tiles keep each CTA short: the update is on the
// factorization's critical path once per block.
constexpr int kUt = 32;
__global__ void __launch_bounds__(256) potrf_update_kernel(const hcore_potrf_task *tasks,
                                                           const int *info, int kb, int tiles) {
    __shared__ double sP[16][kUt + 1];
    __shared__ double sQ[16][kUt + 1];
    const hcore_potrf_task t = tasks[blockIdx.y];
    if (info[blockIdx.y] != 0 || kb >= t.n) return;
    const int bs = min(kPb, t.n - kb), t0 = kb + bs;
    const int bi = blockIdx.x % tiles, bj = blockIdx.x / tiles;
    if (bj > bi) return;
    const int i0 = t0 + bi * kUt, j0 = t0 + bj * kUt;
    if (i0 >= t.n) return;
    const PotrfView V{t.A, t.lda, t.uplo == 'U' || t.uplo == 'u'};
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[2][2] = {};
    for (int k0 = 0; k0 < bs; k0 += 16) {
        for (int e = threadIdx.x; e < 2 * 16 * kUt; e += 256) {
            const int which = e / (16 * kUt), f = e % (16 * kUt);
            int kk, rr;
            if (V.up) { kk = f % 16; rr = f / 16; } else { rr = f % kUt; kk = f / kUt; }
            const int kg = k0 + kk, base = which ? j0 : i0;
            const double x = (kg < bs && base + rr < t.n) ? V.at(base + rr, kb + kg) : 0.0;
            if (which) sQ[kk][rr] = x; else sP[kk][rr] = x;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            const double p0 = sP[kk][tx], p1 = sP[kk][tx + 16];
            const double q0 = sQ[kk][ty], q1 = sQ[kk][ty + 16];
            acc[0][0] += p0 * q0; acc[0][1] += p0 * q1;
            acc[1][0] += p1 * q0; acc[1][1] += p1 * q1;
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int w = 0; w < 2; ++w) {
            const int i = i0 + tx + 16 * u, j = j0 + ty + 16 * w;
            if (i < t.n && j <= i) V.at(i, j) -= acc[u][w];
        }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// vectors per CTA: up to 8 while the CTA's vectors take at most 64 KB of
// shared memory (two or more CTAs per SM), fewer for longer vectors, 0 if
// not even one fits
static int trsm_stride(int maxn) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const long long stat = (kTrRc + kTrBs) * (kTrBs + 1) * (long long)sizeof(double);
    const long long per = (long long)maxn * (long long)sizeof(double);
    for (int S = 8; S >= 1; S >>= 1)
        if (per * S <= 65536 && per * S + stat <= optin) return S;
    return per + stat <= optin ? 1 : 0;
}

static bool trsm_valid(const hcore_trsm_task &t) {
    const bool side = t.side == HCORE_Left || t.side == HCORE_Right;
    const bool uplo = t.uplo == HCORE_Upper || t.uplo == HCORE_Lower;
    const bool tr = t.trans == HCORE_NoTrans || t.trans == HCORE_Trans || t.trans == HCORE_ConjTrans;
    const bool dg = t.diag == HCORE_Unit || t.diag == HCORE_NonUnit;
    if (!side || !uplo || !tr || !dg || t.M < 0 || t.N < 0) return false;
    const int na = t.side == HCORE_Left ? t.M : t.N;
    if (t.M == 0 || t.N == 0) return true;
    return t.A && t.B && t.lda >= std::max(1, na) && t.ldb >= std::max(1, t.M);
}

// Run n TRSM tasks (device-accessible pointers) on stream s and wait.
static int run_trsm(int n, const hcore_trsm_task *tasks, cudaStream_t s) {
    std::vector<TrsmWork> work;
    int maxn = 1;
    for (int i = 0; i < n; ++i) {
        const hcore_trsm_task &t = tasks[i];
        if (!trsm_valid(t)) {
            set_error("hcore_gpu_trsm_batched: invalid task %d", i);
            return HCORE_GPU_EINVAL;
        }
        if (t.M == 0 || t.N == 0) continue;
        maxn = std::max(maxn, t.side == HCORE_Left ? t.M : t.N);
    }
    const int S = trsm_stride(maxn);
    if (S == 0) {
        set_error("hcore_gpu_trsm_batched: triangle of order %d does not fit shared memory", maxn);
        return HCORE_GPU_EINVAL;
    }
    for (int i = 0; i < n; ++i) {
        const hcore_trsm_task &t = tasks[i];
        if (t.M == 0 || t.N == 0) continue;
        const int nvec = t.side == HCORE_Left ? t.N : t.M;
        for (int v0 = 0; v0 < nvec; v0 += S) work.push_back({i, v0, std::min(S, nvec - v0), 0});
    }
    if (work.empty()) return HCORE_GPU_OK;
    if (work.size() > (size_t)INT_MAX) {
        set_error("hcore_gpu_trsm_batched: too many vector groups");
        return HCORE_GPU_EINVAL;
    }
    ThreadCtx &tc = thread_ctx();
    const size_t bt = al256(n * sizeof(hcore_trsm_task)), bw = al256(work.size() * sizeof(TrsmWork));
    char *arena = (char *)tc.dev_ensure(bt + bw);
    char *pin = (char *)tc.pin_ensure(bt + bw);
    if (!arena || !pin) {
        set_error("hcore_gpu_trsm_batched: out of memory");
        return HCORE_GPU_ENOMEM;
    }
    cudaStreamSynchronize(s);  // the previous call may still read the pinned buffer
    memcpy(pin, tasks, n * sizeof(hcore_trsm_task));
    memcpy(pin + bt, work.data(), work.size() * sizeof(TrsmWork));
    cudaMemcpyAsync(arena, pin, bt + bw, cudaMemcpyHostToDevice, s);
    const size_t smem = (size_t)maxn * S * sizeof(double);
    cudaError_t e = cudaFuncSetAttribute(trsm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e == cudaSuccess) {
        trsm_kernel<<<(unsigned)work.size(), 256, smem, s>>>(
            (const hcore_trsm_task *)arena, (const TrsmWork *)(arena + bt), S);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_trsm_batched: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    return HCORE_GPU_OK;
}

// LAPACKE_dpotrf_work's argument checks (its info is LAPACK's minus one)
static int potrf_arg_info(const hcore_potrf_task &t) {
    const char u = (char)t.uplo;
    if (u != 'L' && u != 'l' && u != 'U' && u != 'u') return -2;
    if (t.n < 0) return -3;
    if (t.lda < std::max(1, t.n)) return -5;
    return 0;
}

// Run n POTRF tasks on stream s and wait; info[i] as LAPACKE_dpotrf_work.
static int run_potrf(int n, const hcore_potrf_task *tasks, int *info, cudaStream_t s) {
    std::vector<hcore_potrf_task> run;
    std::vector<int> slot;
    int maxn = 0;
    for (int i = 0; i < n; ++i) {
        info[i] = potrf_arg_info(tasks[i]);
        if (info[i] != 0 || tasks[i].n == 0) continue;
        if (!tasks[i].A) {
            set_error("hcore_gpu_potrf_batched: task %d has no matrix", i);
            return HCORE_GPU_EINVAL;
        }
        run.push_back(tasks[i]);
        slot.push_back(i);
        maxn = std::max(maxn, tasks[i].n);
    }
    if (run.empty()) return HCORE_GPU_OK;
    const int nr = (int)run.size();
    if (nr > 65535) {
        set_error("hcore_gpu_potrf_batched: more than 65535 tiles in one call");
        return HCORE_GPU_EINVAL;
    }
    ThreadCtx &tc = thread_ctx();
    const size_t bt = al256(nr * sizeof(hcore_potrf_task)), bi = al256(nr * sizeof(int));
    char *arena = (char *)tc.dev_ensure(bt + bi);
    char *pin = (char *)tc.pin_ensure(bt + bi);
    if (!arena || !pin) {
        set_error("hcore_gpu_potrf_batched: out of memory");
        return HCORE_GPU_ENOMEM;
    }
    cudaStreamSynchronize(s);
    memcpy(pin, run.data(), nr * sizeof(hcore_potrf_task));
    memset(pin + bt, 0, nr * sizeof(int));
    cudaMemcpyAsync(arena, pin, bt + bi, cudaMemcpyHostToDevice, s);
    const hcore_potrf_task *d_t = (const hcore_potrf_task *)arena;
    int *d_info = (int *)(arena + bt);
    cudaError_t e = cudaSuccess;
    for (int kb = 0; kb < maxn && e == cudaSuccess; kb += kPb) {
        potrf_diag_kernel<<<nr, 256, 0, s>>>(d_t, d_info, kb);
        const int below = maxn - std::min(maxn, kb + kPb);
        if (below > 0) {
            const int panels = (below + kPb - 1) / kPb, tiles = (below + kUt - 1) / kUt;
            potrf_panel_kernel<<<dim3(panels, nr), 256, 0, s>>>(d_t, d_info, kb);
            potrf_update_kernel<<<dim3(tiles * tiles, nr), 256, 0, s>>>(d_t, d_info, kb, tiles);
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(pin + bt, d_info, nr * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_potrf_batched: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    for (int q = 0; q < nr; ++q) info[slot[q]] = ((const int *)(pin + bt))[q];
    return HCORE_GPU_OK;
}

// stage a host block (rows x cols, ld) into dst (ld rows) / back
static void stage_in(double *dst, const double *src, int rows, int cols, int ld, cudaStream_t s) {
    if (rows > 0 && cols > 0)
        cudaMemcpy2DAsync(dst, rows * sizeof(double), src, (size_t)ld * sizeof(double),
                          rows * sizeof(double), cols, cudaMemcpyHostToDevice, s);
}
static cudaError_t stage_out(double *dst, int ld, const double *src, int rows, int cols,
                             cudaStream_t s) {
    if (rows > 0 && cols > 0)
        cudaMemcpy2DAsync(dst, (size_t)ld * sizeof(double), src, rows * sizeof(double),
                          rows * sizeof(double), cols, cudaMemcpyDeviceToHost, s);
    return cudaStreamSynchronize(s);
}

// per-thread device buffer for the drop-ins' host operands
static double *tlr_buffer(size_t n, const char *fn) {
    static thread_local double *buf = nullptr;
    static thread_local size_t buf_n = 0;
    if (buf_n < n) {
        if (buf) {
            cudaStreamSynchronize(thread_ctx().stream);
            cudaFree(buf);
        }
        buf = nullptr;
        buf_n = 0;
        if (cudaMalloc(&buf, std::max<size_t>(n, 1) * sizeof(double)) != cudaSuccess)
            fatal("%s: cannot allocate %zu bytes of device memory\n", fn, n * sizeof(double));
        buf_n = n;
    }
    return buf;
}

}  // namespace hc

using namespace hc;

extern "C" {

int hcore_gpu_trsm_batched(int n, const hcore_trsm_task *tasks, void *stream) {
    if (n < 0 || (n > 0 && !tasks)) {
        set_error("hcore_gpu_trsm_batched: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    std::vector<hcore_trsm_task> tt(tasks, tasks + n);
    for (auto &t : tt) {
        if (t.M == 0 || t.N == 0) continue;
        t.A = (const double *)device_alias(t.A);
        t.B = (double *)device_alias(t.B);
        if (!t.A || !t.B) {
            set_error("hcore_gpu_trsm_batched: pointers must be device or pinned memory");
            return HCORE_GPU_EINVAL;
        }
    }
    return run_trsm(n, tt.data(), (cudaStream_t)stream);
}

int hcore_gpu_potrf_batched(int n, const hcore_potrf_task *tasks, int *info, void *stream) {
    if (n < 0 || (n > 0 && (!tasks || !info))) {
        set_error("hcore_gpu_potrf_batched: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    std::vector<hcore_potrf_task> tt(tasks, tasks + n);
    for (auto &t : tt) {
        if (t.n <= 0) continue;
        t.A = (double *)device_alias(t.A);
        if (!t.A) {
            set_error("hcore_gpu_potrf_batched: pointers must be device or pinned memory");
            return HCORE_GPU_EINVAL;
        }
    }
    return run_potrf(n, tt.data(), info, (cudaStream_t)stream);
}

// cblas_dtrsm(ColMajor, side, uplo, transA, diag, M, Brank, alpha, A, LDA,
// BV, LDBV) on the GPU; flops as hcore_dtrsm.c:41-46 (an invalid side is the
// reference's failed assert).
void HCORE_dtrsm(HCORE_enum side, HCORE_enum uplo, HCORE_enum transA, HCORE_enum diag, int M,
                 int Brank, double alpha, double *A, int LDA, double *BV, int LDBV,
                 flop_counter *flops) {
    if (side != HCORE_Left && side != HCORE_Right)
        fatal("HCORE_dtrsm: side is not CblasLeft or CblasRight\n");
    hcore_trsm_task t{};
    t.side = side; t.uplo = uplo; t.trans = transA; t.diag = diag; t.M = M; t.N = Brank;
    t.alpha = alpha; t.A = A; t.lda = LDA; t.B = BV; t.ldb = LDBV;
    const bool ok = trsm_valid(t);  // as cblas_dtrsm: report, leave BV, return
    if (!ok) fprintf(stderr, "HCORE_dtrsm: invalid argument, BV left unchanged\n");
    if (ok && M > 0 && Brank > 0) {
        ThreadCtx &tc = thread_ctx();
        const int na = side == HCORE_Left ? M : Brank;
        const bool dev = is_device_memory(A) && is_device_memory(BV);
        if (!dev) {
            double *buf = tlr_buffer((size_t)na * na + (size_t)M * Brank, "HCORE_dtrsm");
            stage_in(buf, A, na, na, LDA, tc.stream);
            stage_in(buf + (size_t)na * na, BV, M, Brank, LDBV, tc.stream);
            t.A = buf; t.lda = na; t.B = buf + (size_t)na * na; t.ldb = M;
        }
        if (run_trsm(1, &t, tc.stream)) fatal("HCORE_dtrsm: %s\n", last_error());
        if (!dev && stage_out(BV, LDBV, t.B, M, Brank, tc.stream) != cudaSuccess)
            fatal("HCORE_dtrsm: %s\n", cudaGetErrorString(cudaGetLastError()));
    }
    if (flops) flops->trsm += flop_counts('t', M, Brank, side == HCORE_Left ? 1 : 2, 0);
}

// *info = LAPACKE_dpotrf_work(LAPACK_COL_MAJOR, uplo, N, A, LDA) on the GPU;
// uplo is LAPACK's character ('L' or 'U'), as the reference passes it through
// unchanged; flops as hcore_dpotrf.c:33.
void HCORE_dpotrf(HCORE_enum uplo, int N, double *A, int LDA, int *info, flop_counter *flops) {
    hcore_potrf_task t{};
    t.uplo = uplo; t.n = N; t.A = A; t.lda = LDA;
    int r = potrf_arg_info(t);
    if (r != 0) {
        fprintf(stderr, " ** On entry to DPOTRF parameter number %d had an illegal value\n", -r - 1);
    } else if (N > 0) {
        ThreadCtx &tc = thread_ctx();
        const bool dev = is_device_memory(A);
        if (!dev) {
            t.A = tlr_buffer((size_t)N * N, "HCORE_dpotrf");
            t.lda = N;
            stage_in(t.A, A, N, N, LDA, tc.stream);
        }
        if (run_potrf(1, &t, &r, tc.stream)) fatal("HCORE_dpotrf: %s\n", last_error());
        if (!dev && stage_out(A, LDA, t.A, N, N, tc.stream) != cudaSuccess)
            fatal("HCORE_dpotrf: %s\n", cudaGetErrorString(cudaGetLastError()));
    }
    if (info) *info = r;
    if (flops) flops->potrf += flop_counts('c', N, 0, 0, 0);
}

}  // extern "C"
