// hcore-gb300 — native complex (FP64) low-rank recompression kernels.
//
// The complex update of HCORE_zgemm (src/compute/hcore_zgemm.c:663-976):
// C <- beta*C + alpha*A*B^T with X = XU*XV^T (plain transposes), then
// recompression by QR of [beta*CU | alpha*AU] and of [CV | BU*(AV^T BV)^T]
// (zgeqrf, :115), the SVD of T = R_A R_B^T (zgesvd, :327), truncation at the
// first sigma_i < acc, and the rebuild CU = Q_A [U_r; 0], CV = Q_B [conj(W_r)
// S_r; 0] (zunmqr, :483), where T = U S W^H.  (C = Q_A T Q_B^T, so the plain
// transpose puts conj(W) next to Q_B.)  Four phases, one grid each, as the
// real kernels (hc_kernels.cu):
//
//   zstack_kernel   UA = [beta CU | alpha AU], F = AV^T BV, G = BU F^T, VB = [CV | G]
//   zgeqrf_kernel   Householder QR of UA and VB (zlarfg conventions: beta real,
//                   tau complex, H = I - tau v v^H, Q^H applied to the trailing columns)
//   zgesvd_kernel   T = R_A R_B^T, QR with column pivoting T P = Q R (deflated
//                   as the real kernel's), one-sided Jacobi on B = R^H with
//                   complex column scales, rank rule;
//                   U_r = Q V_J, conj(W_r S_r) = conj(P (rotated B))
//   zapply_kernel   CU = Q_A [U_r; 0], CV = Q_B [conj(W_r S_r); 0]
//
// Complex arithmetic costs four real multiply-adds per product, so this is
// half the FP64 work of the order-2M real embedding, and a rank sum of 64
// keeps both Jacobi matrices in shared memory (the embedding's 128 does not).
#include <cuda_runtime.h>

#include <cfloat>

#include "hc_zinternal.h"

namespace hc {

__device__ __forceinline__ zd zmk(double re, double im) { return zd{re, im}; }
__device__ __forceinline__ zd zadd(zd a, zd b) { return zd{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ zd zsub(zd a, zd b) { return zd{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ zd zmul(zd a, zd b) {
    return zd{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
// conj(a) * b
__device__ __forceinline__ zd zcmul(zd a, zd b) {
    return zd{a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re};
}
__device__ __forceinline__ zd zconj(zd a) { return zd{a.re, -a.im}; }
__device__ __forceinline__ zd zscal(double s, zd a) { return zd{s * a.re, s * a.im}; }
__device__ __forceinline__ double zabs2(zd a) { return a.re * a.re + a.im * a.im; }
// acc + a * b
__device__ __forceinline__ zd zfma(zd a, zd b, zd acc) {
    return zd{fma(a.re, b.re, fma(-a.im, b.im, acc.re)), fma(a.re, b.im, fma(a.im, b.re, acc.im))};
}
// acc + conj(a) * b
__device__ __forceinline__ zd zcfma(zd a, zd b, zd acc) {
    return zd{fma(a.re, b.re, fma(a.im, b.im, acc.re)), fma(a.re, b.im, fma(-a.im, b.re, acc.im))};
}
// acc - a * b (four FMAs)
__device__ __forceinline__ zd zfms(zd a, zd b, zd acc) {
    return zd{fma(-a.re, b.re, fma(a.im, b.im, acc.re)), fma(-a.re, b.im, fma(-a.im, b.re, acc.im))};
}
// 1 / a
__device__ __forceinline__ zd zinv(zd a) {
    const double d = 1.0 / zabs2(a);
    return zd{a.re * d, -a.im * d};
}
__device__ __forceinline__ double zwarp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ zd zwarp_sum(zd v) { return zd{zwarp_sum(v.re), zwarp_sum(v.im)}; }
__device__ __forceinline__ double dmul_exp2(double x, int n) {
    return (x * __longlong_as_double((long long)(n / 2 + 1023) << 52)) *
           __longlong_as_double((long long)(n - n / 2 + 1023) << 52);
}

// ---------------------------------------------------------------------------
// phase 1: stack (hcore_zgemm.c:79-225 in complex arithmetic)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) zstack_kernel(const ZDesc *__restrict__ descs,
                                                     zd *__restrict__ ws) {
    const ZDesc d = descs[blockIdx.x];
    if (d.status0) return;
    const int M = d.M, a = d.a, b = d.b, c = d.c;
    const ZLayout L = zlayout(M, a, b, d.k);
    zd *UA = ws + d.ws + L.UA, *VB = ws + d.ws + L.VB, *F = ws + d.ws + L.F;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (long long e = tid; e < (long long)M * c; e += 256) {
        const int i = (int)(e % M), j = (int)(e / M);
        UA[(size_t)j * M + i] = zmul(d.beta, d.CU[(size_t)j * d.ldcu + i]);
        VB[(size_t)j * M + i] = d.CV[(size_t)j * d.ldcv + i];
    }
    for (long long e = tid; e < (long long)M * a; e += 256) {
        const int i = (int)(e % M), j = (int)(e / M);
        UA[(size_t)(c + j) * M + i] = zmul(d.alpha, d.AU[(size_t)j * d.ldau + i]);
    }
    // F = AV^T BV (a x b), one warp per entry
    for (int e = warp; e < a * b; e += 8) {
        const int p = e % a, q = e / a;
        const zd *x = d.AV + (size_t)p * d.ldav, *y = d.BV + (size_t)q * d.ldbv;
        zd s = zmk(0, 0);
        for (int l = lane; l < M; l += 32) s = zfma(x[l], y[l], s);
        s = zwarp_sum(s);
        if (lane == 0) F[(size_t)q * a + p] = s;
    }
    __syncthreads();
    // G = BU F^T (M x a) after CV in VB
    zd *G = VB + (size_t)c * M;
    for (long long e = tid; e < (long long)M * a; e += 256) {
        const int i = (int)(e % M), p = (int)(e / M);
        zd s = zmk(0, 0);
        for (int q = 0; q < b; ++q) s = zfma(d.BU[(size_t)q * d.ldbu + i], F[(size_t)q * a + p], s);
        G[(size_t)p * M + i] = s;
    }
}

// ---------------------------------------------------------------------------
// phase 2: Householder QR, one CTA (8 warps) per (update, side)
// ---------------------------------------------------------------------------
// zlarfg on (alpha, ||x||^2): beta = -sign(Re alpha) sqrt(|alpha|^2 + ||x||^2),
// tau = (beta - alpha) / beta, x scaled by 1 / (alpha - beta); tau = 0 when
// x = 0 and alpha is real
__device__ __forceinline__ void zlarfg(zd alpha, double xn2, double &beta, zd &tau, zd &scal) {
    if (xn2 == 0.0 && alpha.im == 0.0) {
        beta = alpha.re;
        tau = zmk(0, 0);
        scal = zmk(1, 0);
        return;
    }
    beta = -copysign(sqrt(zabs2(alpha) + xn2), alpha.re);
    tau = zmk((beta - alpha.re) / beta, -alpha.im / beta);
    scal = zinv(zmk(alpha.re - beta, alpha.im));
}

__global__ void __launch_bounds__(256) zgeqrf_kernel(const ZDesc *__restrict__ descs,
                                                     zd *__restrict__ ws) {
    extern __shared__ unsigned char zsm[];
    zd *sv = reinterpret_cast<zd *>(zsm);   // reflector v (M), zero above row j
    __shared__ double red[8];
    __shared__ zd s_tau, s_scal;
    const ZDesc d = descs[blockIdx.x];
    if (d.status0) return;
    const int M = d.M, k = d.k, side = blockIdx.y;
    const ZLayout L = zlayout(M, d.a, d.b, k);
    zd *A = ws + d.ws + (side ? L.VB : L.UA);
    zd *tau = ws + d.ws + (side ? L.tauB : L.tauA);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int j = 0; j < k; ++j) {
        zd *x = A + (size_t)j * M;
        double ss = 0;
        for (int i = j + 1 + tid; i < M; i += 256) ss += zabs2(x[i]);
        ss = zwarp_sum(ss);
        if (lane == 0) red[warp] = ss;
        __syncthreads();
        if (tid == 0) {
            double t = 0;
            for (int w = 0; w < 8; ++w) t += red[w];
            double beta;
            zd tj, scal;
            zlarfg(x[j], t, beta, tj, scal);
            s_tau = tj;
            tau[j] = tj;
            s_scal = scal;
            x[j] = zmk(beta, 0);          // R(j, j)
        }
        __syncthreads();
        const zd scal = s_scal;
        for (int i = tid; i < M; i += 256) {
            zd v = zmk(0, 0);
            if (i > j) {
                v = zmul(x[i], scal);
                x[i] = v;
            } else if (i == j) {
                v = zmk(1, 0);
            }
            sv[i] = v;
        }
        __syncthreads();
        // trailing columns: c <- c - conj(tau) (v^H c) v, one warp per column
        const zd tc = zconj(s_tau);
        if (s_tau.re != 0.0 || s_tau.im != 0.0)
            for (int col = j + 1 + warp; col < k; col += 8) {
                zd *y = A + (size_t)col * M;
                zd s = zmk(0, 0);
                for (int i = j + lane; i < M; i += 32) s = zcfma(sv[i], y[i], s);
                s = zmul(tc, zwarp_sum(s));
                for (int i = j + lane; i < M; i += 32) y[i] = zfms(s, sv[i], y[i]);
            }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// phase 3: SVD of T = R_A R_B^T, both Jacobi matrices in shared memory
// ---------------------------------------------------------------------------
__device__ __forceinline__ void zrr_pair(int round, int pi, int n, int &p, int &q) {
    if (pi == 0) {
        p = n - 1;
        q = round;
    } else {
        p = (round + pi) % (n - 1);
        q = (round - pi + (n - 1)) % (n - 1);
    }
}

// Shared memory: A (V_J, then the QRCP's working matrix) and B (R^H), each
// K x ld column-major (ld = K | 1), then per-column complex scales d,
// squared norms, complex QRCP taus, and two index arrays.
// (one CTA per SM at k near 64: its shared memory is the limit, so the
// registers need not be)
template <bool AGLOBAL>
__global__ void __launch_bounds__(256, 1) zgesvd_kernel(const ZDesc *__restrict__ descs,
                                                     zd *__restrict__ ws, int *__restrict__ rank,
                                                     int *__restrict__ status, int maxK, int G) {
    extern __shared__ unsigned char zsm[];
    __shared__ int s_piv, s_exp, s_conv, s_rot, s_bad;
    __shared__ double s_wmax[8];
    __shared__ double s_defl2;
    const ZDesc d = descs[blockIdx.x];
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31;
    if (d.status0) {
        if (tid == 0) {
            status[d.idx] = d.status0;
            rank[d.idx] = 0;
        }
        return;
    }
    const int M = d.M, k = d.k;
    const ZLayout L = zlayout(M, d.a, d.b, k);
    zd *base = ws + d.ws;
    const zd *UA = base + L.UA, *VB = base + L.VB;
    const int ld = zsvd_ld(maxK);
    // AGLOBAL: A (the QRCP's matrix, then V_J) in the workspace, only B in
    // shared memory, so that three CTAs fit an SM at k near 64
    zd *B = reinterpret_cast<zd *>(zsm) + (AGLOBAL ? 0 : (size_t)maxK * ld);
    zd *A = AGLOBAL ? base + L.W : reinterpret_cast<zd *>(zsm);
    const int ldA = AGLOBAL ? k : ld;
    zd *s_d = B + (size_t)maxK * ld;
    zd *s_tau = s_d + (maxK + 1);
    double *s_nrm = reinterpret_cast<double *>(s_tau + (maxK + 1));
    double *s_dn = s_nrm + (maxK + 1);   // norms at the last exact computation
    int *s_perm = reinterpret_cast<int *>(s_dn + (maxK + 1));
    int *s_pcol = s_perm + (maxK + 1);
    zd *Yg = base + L.Y;   // the QRCP's reflectors (k x k, ld k)
    auto ix = [ld](int i, int j) { return (size_t)j * ld + i; };
    auto ixA = [ldA](int i, int j) { return (size_t)j * ldA + i; };

    // T = triu(R_A) triu(R_B)^T
    double amax = 0;
    for (int e = tid; e < k * k; e += nthr) {
        const int i = e % k, j = e / k;
        zd s = zmk(0, 0);
        for (int l = max(i, j); l < k; ++l)
            s = zfma(UA[(size_t)l * M + i], VB[(size_t)l * M + j], s);
        A[ixA(i, j)] = s;
        amax = max(amax, max(fabs(s.re), fabs(s.im)));
    }
    for (int o = 16; o > 0; o >>= 1) amax = max(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if (lane == 0) s_wmax[tid >> 5] = amax;
    __syncthreads();
    if (tid == 0) {
        double m = 0;
        for (int w = 0; w < nthr / 32; ++w) m = max(m, s_wmax[w]);
        s_exp = (m > 0 && isfinite(m)) ? ilogb(m) : 0;
        s_bad = 0;
    }
    __syncthreads();
    const int sexp = s_exp;
    if (sexp != 0)
        for (int e = tid; e < k * k; e += nthr) {
            const int i = e % k, j = e / k;
            const zd v = A[ixA(i, j)];
            A[ixA(i, j)] = zmk(dmul_exp2(v.re, -sexp), dmul_exp2(v.im, -sexp));
        }
    __syncthreads();

    // QR with column pivoting, T P = Q R (lane per trailing column)
    for (int c = tid; c < k; c += nthr) {
        double s = 0;
        for (int i = 0; i < k; ++i) s += zabs2(A[ixA(i, c)]);
        s_nrm[c] = s;
        s_dn[c] = s;
        s_pcol[c] = c;
    }
    __syncthreads();
    // Deflation, as in the real kernel (gesvd_kernel): the QR stops at the
    // first step j >= 1 (the rank search starts at 1) whose trailing block has
    // ||R(j:k, j:k)||_F <= delta = min(1e-13 acc, 1e-16 ||T||_F) and the
    // Jacobi works on the first j rows of R.  Every singular value moves by at
    // most delta (Weyl); the dropped directions come out with singular value 0.
    if (tid == 0) {
        double f2 = 0;   // ||T||_F^2 of the scaled T
        for (int c = 0; c < k; ++c) f2 += s_nrm[c];
        double dl = -1.0;
        if (d.rk == 0 && d.acc > 0.0) dl = fmin(1e-13 * dmul_exp2(d.acc, -sexp), 1e-16 * sqrt(f2));
        s_defl2 = (dl >= 0.0 && isfinite(dl)) ? dl * dl : -1.0;
    }
    int kk = k;   // columns of R^H that the Jacobi rotates
    for (int j = 0; j < k; ++j) {
        if (tid < 32) {
            double best = -1, tail = 0;
            int bi = j;
            for (int c = j + lane; c < k; c += 32) {
                tail += s_nrm[c];
                if (s_nrm[c] > best) {
                    best = s_nrm[c];
                    bi = c;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                tail += __shfl_xor_sync(0xffffffffu, tail, o);
                if (ob > best || (ob == best && oi < bi)) {
                    best = ob;
                    bi = oi;
                }
            }
            if (lane == 0) s_piv = (j >= 1 && tail <= s_defl2) ? -1 : bi;
        }
        __syncthreads();
        const int pv = s_piv;
        if (pv < 0) {
            kk = j;
            break;
        }
        if (pv != j) {
            for (int i = tid; i < k; i += nthr) {
                const zd x = A[ixA(i, j)];
                A[ixA(i, j)] = A[ixA(i, pv)];
                A[ixA(i, pv)] = x;
            }
            if (tid == 0) {
                double x = s_nrm[j]; s_nrm[j] = s_nrm[pv]; s_nrm[pv] = x;
                x = s_dn[j]; s_dn[j] = s_dn[pv]; s_dn[pv] = x;
                const int ci = s_pcol[j]; s_pcol[j] = s_pcol[pv]; s_pcol[pv] = ci;
            }
        }
        __syncthreads();
        if (tid < 32) {   // reflector of column j, rows j..k-1
            double ss = 0;
            for (int i = j + 1 + lane; i < k; i += 32) ss += zabs2(A[ixA(i, j)]);
            ss = zwarp_sum(ss);
            double beta;
            zd tj, scal;
            zlarfg(A[ixA(j, j)], ss, beta, tj, scal);
            for (int i = j + 1 + lane; i < k; i += 32) A[ixA(i, j)] = zmul(A[ixA(i, j)], scal);
            __syncwarp();
            if (lane == 0) {
                A[ixA(j, j)] = zmk(beta, 0);
                s_tau[j] = tj;
            }
        }
        __syncthreads();
        // apply H_j^H to the trailing columns and downdate their norms
        const zd tc = zconj(s_tau[j]);
        for (int c = j + 1 + tid; c < k; c += nthr) {
            if (tc.re != 0.0 || tc.im != 0.0) {
                zd dot = A[ixA(j, c)];
                for (int i = j + 1; i < k; ++i) dot = zcfma(A[ixA(i, j)], A[ixA(i, c)], dot);
                const zd s = zmul(tc, dot);
                A[ixA(j, c)] = zsub(A[ixA(j, c)], s);
                for (int i = j + 1; i < k; ++i) A[ixA(i, c)] = zfms(s, A[ixA(i, j)], A[ixA(i, c)]);
            }
            double nn = s_nrm[c] - zabs2(A[ixA(j, c)]);
            if (nn <= s_dn[c] * (1.0 / 1024) || nn <= 0.0) {
                double s = 0;
                for (int i = j + 1; i < k; ++i) s += zabs2(A[ixA(i, c)]);
                nn = s;
                s_dn[c] = s;
            }
            s_nrm[c] = nn;
        }
        __syncthreads();
    }
    // reflectors to the workspace; B = R^H (rows kk.. of R dropped: B's
    // columns kk.. are zero; reflectors kk.. were never formed); A = I
    for (int h = kk + tid; h < k; h += nthr) s_tau[h] = zmk(0, 0);
    for (int e = tid; e < k * k; e += nthr) {
        const int i = e % k, j = e / k;
        const zd x = A[ixA(i, j)];
        Yg[(size_t)j * k + i] = (i > j && j < kk) ? x : zmk(0, 0);
        B[ix(j, i)] = (i <= j && i < kk) ? zconj(x) : zmk(0, 0);   // B(j, i) = conj(R(i, j))
    }
    __syncthreads();
    for (int e = tid; e < k * k; e += nthr) {
        const int i = e % k, j = e / k;
        A[ixA(i, j)] = zmk(i == j ? 1.0 : 0.0, 0);
    }
    for (int c = tid; c < k; c += nthr) {
        double s = 0;
        if (c < kk)
            for (int i = 0; i < k; ++i) s += zabs2(B[ix(i, c)]);
        s_nrm[c] = s;
        s_d[c] = zmk(1, 0);
    }
    __syncthreads();

    // one-sided Jacobi on B with complex column scales: true column j is
    // d_j x_j in B and in V_J (A).  For a pair with a_pq = P^H Q = |a_pq|
    // e^{i phi}: P' = c (P - t e^{-i phi} Q), Q' = c (e^{-i phi} Q + t P),
    // t the real Jacobi tangent of (a_pp, a_qq, |a_pq|); in scaled form
    // x_p -= f1 x_q, x_q += f2 x_p with f1 = t e^{-i phi} d_q / d_p,
    // f2 = t e^{i phi} d_p / d_q, d_p <- c d_p, d_q <- c e^{-i phi} d_q
    // (columns kk.. of B are zero and take no part; V_J's rows kk.. stay zero)
    const int n = kk + (kk & 1), np = n / 2;
    const int grp = tid / G, lig = tid % G, ngrp = nthr / G;
    const double tol = (double)(k > 8 ? k : 8) * DBL_EPSILON;
    const double tol2 = tol * tol, stop2 = tol;
    const double safmin = DBL_MIN / DBL_EPSILON;
    bool converged = (kk <= 1);
    for (int sweep = 0; sweep < kMaxSweeps && !converged; ++sweep) {
        if (tid == 0) s_rot = 0;
        bool big = false;
        __syncthreads();
        for (int round = 0; round < n - 1; ++round) {
            for (int bs = 0; bs < np; bs += ngrp) {
                const int pi = bs + grp;
                int p = 0, q = 0;
                if (pi < np) zrr_pair(round, pi, n, p, q);
                const bool valid = pi < np && p < kk && q < kk;
                zd *xp = B + ix(0, p), *xq = B + ix(0, q);
                zd dot = zmk(0, 0);
                if (valid)
                    for (int i = lig; i < k; i += G) dot = zcfma(xp[i], xq[i], dot);
                for (int o = G / 2; o > 0; o >>= 1) {
                    dot.re += __shfl_xor_sync(0xffffffffu, dot.re, o);
                    dot.im += __shfl_xor_sync(0xffffffffu, dot.im, o);
                }
                zd dp = zmk(1, 0), dq = zmk(1, 0);
                double app = 0, aqq = 0, amag2 = 0;
                zd apq = zmk(0, 0);
                if (valid) {
                    dp = s_d[p];
                    dq = s_d[q];
                    app = s_nrm[p];
                    aqq = s_nrm[q];
                    apq = zmul(zcmul(dp, dq), dot);   // conj(dp) dq x_p^H x_q
                    amag2 = zabs2(apq);
                }
                const double pq = app * aqq;
                const bool rot = valid && app > safmin && aqq > safmin && amag2 > 0.0 &&
                                 amag2 > tol2 * pq;
                double t = 0, cs = 1;
                zd ph = zmk(1, 0);
                if (rot) {
                    big |= amag2 > stop2 * pq;
                    const double am = sqrt(amag2);
                    ph = zscal(1.0 / am, apq);                // e^{i phi}
                    const double w = aqq - app, v = 2.0 * am;
                    const double h = sqrt(fma(w, w, v * v));
                    t = v / (fabs(w) + h);
                    if (w < 0.0) t = -t;
                    cs = rsqrt(fma(t, t, 1.0));
                    const zd f1 = zscal(t / zabs2(dp), zmul(zconj(ph), zmul(dq, zconj(dp))));
                    const zd f2 = zscal(t / zabs2(dq), zmul(ph, zmul(dp, zconj(dq))));
                    zd *vp = A + ixA(0, p), *vq = A + ixA(0, q);
                    int i = lig;
                    for (; i < kk; i += G) {
                        const zd a = xp[i], b = xq[i];
                        xp[i] = zfms(f1, b, a);
                        xq[i] = zfma(f2, a, b);
                        const zd u = vp[i], vv = vq[i];
                        vp[i] = zfms(f1, vv, u);
                        vq[i] = zfma(f2, u, vv);
                    }
                    for (; i < k; i += G) {   // V_J's rows kk.. are zero
                        const zd a = xp[i], b = xq[i];
                        xp[i] = zfms(f1, b, a);
                        xq[i] = zfma(f2, a, b);
                    }
                }
                double np_ = app - t * sqrt(amag2), nq_ = aqq + t * sqrt(amag2);
                const bool redo_p = rot && np_ < app * (1.0 / 64);
                const bool redo_q = rot && nq_ < aqq * (1.0 / 64);
                const zd dp2 = zscal(cs, dp), dq2 = zscal(cs, zcmul(ph, dq));   // c e^{-i phi} dq
                if (__any_sync(0xffffffffu, redo_p || redo_q)) {
                    double sp = 0, sq = 0;
                    if (redo_p || redo_q)
                        for (int i = lig; i < k; i += G) {
                            sp += zabs2(xp[i]);
                            sq += zabs2(xq[i]);
                        }
                    for (int o = G / 2; o > 0; o >>= 1) {
                        sp += __shfl_xor_sync(0xffffffffu, sp, o);
                        sq += __shfl_xor_sync(0xffffffffu, sq, o);
                    }
                    if (redo_p) np_ = zabs2(dp2) * sp;
                    if (redo_q) nq_ = zabs2(dq2) * sq;
                }
                if (rot && lig == 0) {
                    s_nrm[p] = np_;
                    s_nrm[q] = nq_;
                    s_d[p] = dp2;
                    s_d[q] = dq2;
                    s_rot = 1;
                }
            }
            __syncthreads();
        }
        // exact norms once per sweep; fold scales before they underflow
        for (int j = tid; j < kk; j += nthr) {
            zd *xj = B + ix(0, j);
            zd dj = s_d[j];
            if (zabs2(dj) < 1e-120) {
                zd *vj = A + ixA(0, j);
                for (int i = 0; i < k; ++i) {
                    xj[i] = zmul(dj, xj[i]);
                    vj[i] = zmul(dj, vj[i]);
                }
                dj = zmk(1, 0);
                s_d[j] = dj;
            }
            double s2 = 0;
            for (int i = 0; i < k; ++i) s2 += zabs2(xj[i]);
            s_nrm[j] = zabs2(dj) * s2;
        }
        const bool anybig = __any_sync(0xffffffffu, big);
        if (lane == 0) s_wmax[tid >> 5] = anybig ? 1.0 : 0.0;
        __syncthreads();
        if (tid == 0) {
            double m = 0;
            for (int w = 0; w < nthr / 32; ++w) m = max(m, s_wmax[w]);
            s_conv = (s_rot == 0 || m == 0.0) ? 1 : 0;
        }
        __syncthreads();
        converged = s_conv != 0;
        __syncthreads();
    }

    // singular values, sorted descending (ties by index, NaN last)
    double *s_sig = s_dn;
    for (int j = tid; j < k; j += nthr) {
        const double s = sqrt(s_nrm[j]);
        s_sig[j] = s;
        if (!isfinite(s)) s_bad = 1;
    }
    __syncthreads();
    for (int j = tid; j < k; j += nthr) {
        const double sj = s_sig[j] == s_sig[j] ? s_sig[j] : -1.0;
        int pos = 0;
        for (int i = 0; i < k; ++i) {
            const double si = s_sig[i] == s_sig[i] ? s_sig[i] : -1.0;
            pos += (si > sj) || (si == sj && i < j);
        }
        s_perm[pos] = j;
    }
    __syncthreads();
    zd *sig_out = base + L.sig;
    for (int t = tid; t < k; t += nthr) sig_out[t] = zmk(dmul_exp2(s_sig[s_perm[t]], sexp), 0);
    int r;
    if (d.rk != 0) {
        r = d.rk < k ? d.rk : k;
    } else {
        r = k;
        for (int i = 1; i < k; ++i)
            if (dmul_exp2(s_sig[s_perm[i]], sexp) < d.acc) {
                r = i;
                break;
            }
    }
    int st = HCORE_GPU_S_OK;
    if (!converged || s_bad) st = HCORE_GPU_S_NOCONV;
    else if (r > d.max_rank) st = HCORE_GPU_S_RANK_MAX;
    if (st == HCORE_GPU_S_OK) {
        // U_r = Q (true V_J columns), Q = H_0 ... H_{k-1}: lane per output
        // column, reflectors from last to first, H_h x = x - tau_h v_h (v_h^H x)
        for (int t = tid; t < r; t += nthr) {
            const int j = s_perm[t];
            zd *x = A + ixA(0, j);
            const zd dj = s_d[j];
            for (int i = 0; i < k; ++i) x[i] = zmul(dj, x[i]);
            for (int h = k - 1; h >= 0; --h) {
                const zd th = s_tau[h];
                if (th.re == 0.0 && th.im == 0.0) continue;
                const zd *y = Yg + (size_t)h * k;
                zd dot = x[h];
                for (int i = h + 1; i < k; ++i) dot = zcfma(y[i], x[i], dot);
                const zd s = zmul(th, dot);
                x[h] = zsub(x[h], s);
                for (int i = h + 1; i < k; ++i) x[i] = zfms(s, y[i], x[i]);
            }
        }
        __syncthreads();
        // Uo = U_r; Vo = conj(W_r S_r) with W S = P (rotated B), scaled back
        zd *Uo = base + L.Uo, *Vo = base + L.Vo;
        for (int e = tid; e < k * r; e += nthr) {
            const int i = e % k, t = e / k;
            const int j = s_perm[t];
            const zd w = zmul(s_d[j], B[ix(i, j)]);
            Vo[(size_t)t * k + s_pcol[i]] = zmk(dmul_exp2(w.re, sexp), -dmul_exp2(w.im, sexp));
            Uo[(size_t)t * k + i] = A[ixA(i, j)];
        }
    }
    if (tid == 0) {
        rank[d.idx] = r;
        status[d.idx] = st;
    }
}

// ---------------------------------------------------------------------------
// phase 4: rebuild, CU = Q_A [U_r; 0] (side 0), CV = Q_B [Vo_r; 0] (side 1);
// one warp per output column, RPL complex rows per lane in registers, the
// reflectors staged through shared memory kZApplyChunk at a time
// ---------------------------------------------------------------------------
template <int RPL>
__global__ void __launch_bounds__(256, 1) zapply_kernel(const ZDesc *__restrict__ descs,
                                                        const zd *__restrict__ ws,
                                                        const int *__restrict__ rank,
                                                        const int *__restrict__ status) {
    extern __shared__ unsigned char zsm[];
    zd *sv = reinterpret_cast<zd *>(zsm);
    __shared__ zd s_tau[kZApplyChunk];
    const ZDesc d = descs[blockIdx.x];
    if (d.status0 || status[d.idx] != HCORE_GPU_S_OK) return;
    const int r = rank[d.idx];
    const int col = blockIdx.z * 8 + (threadIdx.x >> 5);
    if (blockIdx.z * 8 >= r) return;
    const int side = blockIdx.y, M = d.M, k = d.k;
    const ZLayout L = zlayout(M, d.a, d.b, k);
    const zd *base = ws + d.ws;
    const zd *Y = base + (side ? L.VB : L.UA);
    const zd *tau = base + (side ? L.tauB : L.tauA);
    const zd *X0 = base + (side ? L.Vo : L.Uo);
    zd *out = side ? d.CVo : d.CUo;
    const int tid = threadIdx.x, lane = tid & 31;
    const bool active = col < r;
    constexpr int ROWS = 32 * RPL;
    zd x[RPL];
#pragma unroll
    for (int t = 0; t < RPL; ++t) {
        const int i = lane + 32 * t;
        x[t] = (active && i < k) ? X0[(size_t)col * k + i] : zmk(0, 0);
    }
    const int nch = (k + kZApplyChunk - 1) / kZApplyChunk;
    for (int ch = nch - 1; ch >= 0; --ch) {
        const int j0 = ch * kZApplyChunk, nj = min(kZApplyChunk, k - j0);
        __syncthreads();
        for (int e = tid; e < nj * ROWS; e += 256) {
            const int c = e / ROWS, i = e % ROWS, j = j0 + c;
            zd v = zmk(0, 0);
            if (i > j && i < M) v = Y[(size_t)j * M + i];
            else if (i == j) v = zmk(1, 0);
            sv[c * ROWS + i] = v;
        }
        if (tid < nj) s_tau[tid] = tau[j0 + tid];
        __syncthreads();
        if (!active) continue;
        for (int c = nj - 1; c >= 0; --c) {
            const zd tj = s_tau[c];
            if (tj.re == 0.0 && tj.im == 0.0) continue;
            const zd *v = sv + c * ROWS;
            zd s = zmk(0, 0);
#pragma unroll
            for (int t = 0; t < RPL; ++t) s = zcfma(v[lane + 32 * t], x[t], s);
            s = zmul(tj, zwarp_sum(s));
#pragma unroll
            for (int t = 0; t < RPL; ++t) x[t] = zfms(s, v[lane + 32 * t], x[t]);
        }
    }
    if (active) {
#pragma unroll
        for (int t = 0; t < RPL; ++t) {
            const int i = lane + 32 * t;
            if (i < M) out[(size_t)col * d.ldco + i] = x[t];
        }
    }
}

template <int RPL>
static void launch_zapply(const ZDesc *d_desc, int n, const zd *ws, const int *d_rank,
                          const int *d_status, int maxR, cudaStream_t s) {
    const size_t smem = (size_t)kZApplyChunk * 32 * RPL * sizeof(zd);
    cudaFuncSetAttribute(zapply_kernel<RPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    zapply_kernel<RPL><<<dim3(n, 2, (maxR + 7) / 8), 256, smem, s>>>(d_desc, ws, d_rank,
                                                                      d_status);
}

int zsvd_kmax() {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess)
        return 0;
    int kmax = 0;
    while (kmax < 256 && zsvd_smem_bytes(kmax + 1) + 1024 <= (size_t)optin) ++kmax;
    return kmax;
}

cudaError_t launch_zrecompress(const ZDesc *d_desc, int n, zd *ws, int *d_rank, int *d_status,
                               int maxM, int maxK, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int rpl = (maxM + 31) / 32;
    if (rpl > 32 || maxK > zsvd_kmax()) return cudaErrorInvalidValue;
    zstack_kernel<<<n, 256, 0, s>>>(d_desc, ws);
    const size_t qsm = (size_t)maxM * sizeof(zd);
    zgeqrf_kernel<<<dim3(n, 2), 256, qsm, s>>>(d_desc, ws);
    // lanes per column pair: as many as fit in 256 threads, at most 4
    const int np = (maxK + 1) / 2;
    int G = 1;
    while (G < 4 && 2 * G * np <= 256) G *= 2;
    const int nt = ((np * G + 31) / 32) * 32;
    // both Jacobi matrices in shared memory, unless that leaves one CTA per
    // SM while the batch has more updates than SMs: then V_J moves to the
    // workspace and three CTAs share an SM
    int dev = 0, sms = 1, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const bool aglobal = n > sms && 2 * zsvd_smem_bytes(maxK) > (size_t)optin;
    const size_t ssm = aglobal ? zsvd_smem_bytes_half(maxK) : zsvd_smem_bytes(maxK);
    cudaError_t e;
    if (aglobal) {
        e = cudaFuncSetAttribute(zgesvd_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)ssm);
        if (e != cudaSuccess) return e;
        zgesvd_kernel<true><<<n, nt < 32 ? 32 : nt, ssm, s>>>(d_desc, ws, d_rank, d_status, maxK, G);
    } else {
        e = cudaFuncSetAttribute(zgesvd_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)ssm);
        if (e != cudaSuccess) return e;
        zgesvd_kernel<false><<<n, nt < 32 ? 32 : nt, ssm, s>>>(d_desc, ws, d_rank, d_status, maxK, G);
    }
    if (rpl <= 4) launch_zapply<4>(d_desc, n, ws, d_rank, d_status, maxK, s);
    else if (rpl <= 8) launch_zapply<8>(d_desc, n, ws, d_rank, d_status, maxK, s);
    else if (rpl <= 16) launch_zapply<16>(d_desc, n, ws, d_rank, d_status, maxK, s);
    else launch_zapply<32>(d_desc, n, ws, d_rank, d_status, maxK, s);
    return cudaGetLastError();
}

}  // namespace hc
