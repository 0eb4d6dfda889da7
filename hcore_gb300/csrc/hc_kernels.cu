// hcore-gb300 — batched low-rank recompression kernels for sm_103a.
//
// One Schur update C <- beta*C + alpha*A*B^T (A, B, C in U*V^T form) follows
// the reference HCORE_dgemm (src/compute/hcore_dgemm.c:703-1012) as four
// batched phases, each a grid over the updates of the batch:
//
//   1. stack  (hcore_dgemm.c:79-225)  UA = [beta*CU | alpha*AU],
//              F = AV^T BV, G = BU F^T, VB = [CV | G]            -> workspace
//   2. geqrf  (hcore_dgemm.c:123, :216) Householder QR of UA and VB
//              (blockIdx.y selects the side), LAPACK dlarfg conventions
//   3. gesvd  (hcore_dgemm.c:296-503) T = R_A R_B^T, pivoted QR (in FP64
//              deflated below 1e-13 of the threshold), one-sided Jacobi SVD,
//              singular values sorted, rank rule, U_r and V_r S_r
//   4. apply  (hcore_dgemm.c:508-696) CU = Q_A [U_r; 0], CV = Q_B [V_r S_r; 0]
//              written straight into the caller's output factors
//
// In FP64 plans with a + c <= 64 the QR runs blocked, its trailing updates on
// the tensor cores (hc_qr_tc.cu), and the rebuild runs there too
// (hc_rebuild_tc.cu); this file keeps the panels and every other case.
//
// The scalar type T is double (HCORE_dgemm) or float (HCORE_sgemm); every
// step computes in T, like the reference's two copies.  With the plan flag
// HCORE_GPU_MIXED_FACTORS an FP64 plan computes the factor products (stack)
// and the Q.U rebuild in FP32 (compute type Tc = float, FP32 accumulation,
// FP64 storage) while the QRs, the SVD and the truncation stay FP64.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <mutex>

#include "hc_internal.h"

namespace hc {

template <typename T>
struct Lim;
template <>
struct Lim<double> {
    static constexpr double eps = DBL_EPSILON;
};
template <>
struct Lim<float> {
    static constexpr float eps = FLT_EPSILON;
};

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// binary exponent (floor(log2|x|), subnormals included), per precision
__device__ __forceinline__ int binary_exponent(double x) { return ilogb(x); }
__device__ __forceinline__ int binary_exponent(float x) { return ilogbf(x); }
// 2^n built from its bits, n within the normal exponent range
template <typename T>
__device__ __forceinline__ T exp2i(int n);
template <>
__device__ __forceinline__ double exp2i<double>(int n) {
    return __longlong_as_double((long long)(n + 1023) << 52);
}
template <>
__device__ __forceinline__ float exp2i<float>(int n) {
    return __int_as_float((n + 127) << 23);
}
// x * 2^n for |n| up to twice the normal exponent range: two exact multiplies
template <typename T>
__device__ __forceinline__ T mul_exp2(T x, int n) {
    return (x * exp2i<T>(n / 2)) * exp2i<T>(n - n / 2);
}

// -x by its sign bit (integer pipe; exact, NaN payloads kept)
__device__ __forceinline__ double flip_sign(double x) {
    return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ULL);
}
__device__ __forceinline__ float flip_sign(float x) {
    return __int_as_float(__float_as_int(x) ^ (int)0x80000000u);
}

// ---------------------------------------------------------------------------
// phase 1: stack the factors
// ---------------------------------------------------------------------------
// tc_products: the products F and G of updates that stack_tc_eligible
// accepts are left to the tensor-core kernel (hc_stack_tc.cu)
template <typename T, typename Tc>
__global__ void __launch_bounds__(kThreads) stack_kernel(const Desc *__restrict__ descs,
                                                         T *__restrict__ ws, bool tc_products) {
    const Desc d = descs[blockIdx.x];
    if (d.status0) return;
    const int M = d.M, a = d.a, b = d.b, c = d.c;
    const WsLayout L = ws_layout(d);
    T *UA = ws + d.ws + L.UA;
    T *VB = ws + d.ws + L.VB;
    T *F = ws + d.ws + L.F;
    const T alpha = (T)d.alpha, beta = (T)d.beta;
    const T *CU = (const T *)d.CU, *CV = (const T *)d.CV;
    const T *AU = (const T *)d.AU, *AV = (const T *)d.AV;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    // [beta*CU | alpha*AU] and [CV | .] (hcore_dgemm.c:106-114, :199-205).
    // The Schur update's coefficients 1 and -1 are applied without an FP64
    // instruction (a copy, a sign-bit flip on the integer pipe): same bits.
    const bool beta_one = beta == T(1), alpha_minus_one = alpha == T(-1);
    for (long long e = tid; e < (long long)M * c; e += kThreads) {
        const int i = (int)(e % M), j = (int)(e / M);
        const T x = CU[(size_t)j * d.ldc + i];
        UA[(size_t)j * M + i] = beta_one ? x : beta * x;
        VB[(size_t)j * M + i] = CV[(size_t)j * d.ldc + i];
    }
    for (long long e = tid; e < (long long)M * a; e += kThreads) {
        const int i = (int)(e % M), j = (int)(e / M);
        const T x = AU[(size_t)j * d.lda + i];
        UA[(size_t)(c + j) * M + i] = alpha_minus_one ? flip_sign(x) : alpha * x;
    }
    if (a == 0 || (tc_products && stack_tc_eligible(d))) return;
    T *G = VB + (size_t)c * M;
    if (d.Bd) {
        // dense B: G = B * AV (hcore_dgemm.c:262-271)
        const T *B = (const T *)d.Bd;
        for (long long e = tid; e < (long long)M * a; e += kThreads) {
            const int i = (int)(e % M), j = (int)(e / M);
            Tc s = 0;
            for (int l = 0; l < M; ++l)
                s += (Tc)B[(size_t)l * d.ldb + i] * (Tc)AV[(size_t)j * d.lda + l];
            G[(size_t)j * M + i] = (T)s;
        }
        return;
    }
    const T *BU = (const T *)d.BU, *BV = (const T *)d.BV;
    // F = AV^T BV, a x b, one warp per entry (hcore_dgemm.c:175-178)
    for (int e = warp; e < a * b; e += kWarps) {
        const int p = e % a, q = e / a;
        const T *x = AV + (size_t)p * d.lda;
        const T *y = BV + (size_t)q * d.ldb;
        Tc s = 0;
        for (int l = lane; l < M; l += 32) s += (Tc)x[l] * (Tc)y[l];
        s = warp_sum(s);
        if (lane == 0) F[(size_t)q * a + p] = (T)s;
    }
    __syncthreads();
    // G = BU F^T, M x a (hcore_dgemm.c:199-205)
    for (long long e = tid; e < (long long)M * a; e += kThreads) {
        const int i = (int)(e % M), p = (int)(e / M);
        Tc s = 0;
        for (int q = 0; q < b; ++q) s += (Tc)BU[(size_t)q * d.ldb + i] * (Tc)F[(size_t)q * a + p];
        G[(size_t)p * M + i] = (T)s;
    }
}

// ---------------------------------------------------------------------------
// phase 2: Householder QR of UA (blockIdx.y = 0) or VB (blockIdx.y = 1)
// ---------------------------------------------------------------------------
// Reflector j is H_j = I - tau_j v v^T with v(j) = 1, v(i<j) = 0 and v(i>j)
// stored below the diagonal, beta = -sign(alpha)*||x||, tau = (beta-alpha)/beta
// (LAPACK dlarfg); ||x|| = 0 gives tau = 0.  R ends up on and above the
// diagonal, as dgeqrf leaves it.
//
// FP64 issue slots are the scarce resource on this GPU, so a warp keeps the
// column it updates in registers (RPL rows per lane, row = lane + 32 t): one
// load, one dot, one axpy, one store per column and reflector.  The reflector
// vector is published in shared memory, zero outside rows j..M-1, so the dot
// and the axpy need no predicates.  Look-ahead: warp 0 updates column j+1
// first and turns it into reflector j+1 while the other warps finish step j,
// so there is a single barrier per column.
// lo/hi: range in which a plain sum of squares neither under- nor overflows;
// safmin = (smallest normal) / eps, the LAPACK dlamch('S')/dlamch('E')
// threshold below which 1/beta is not safe (a power of two).
template <typename T>
struct NormLim;
template <>
struct NormLim<double> {
    static constexpr double lo = 1e-280, hi = 1e280;
    static constexpr double safmin = DBL_MIN / DBL_EPSILON;
    static constexpr int max_shift = 1000;   // 2^(+-max_shift) is a normal double
};
template <>
struct NormLim<float> {
    static constexpr float lo = 1e-30f, hi = 1e30f;
    static constexpr float safmin = FLT_MIN / FLT_EPSILON;
    static constexpr int max_shift = 120;
};

// dlarfg's rescaling for a column whose beta is below safmin (subnormal
// entries; warp-uniform and rare, so kept out of line to spare the
// registers of the common path).  With alpha and ||x|| scaled by 2^s
// (|beta| -> ~1) tau follows, and v = x 2^s / (as - bs) is applied in two
// exact factors to the x that make_reflector published; beta stays
// unscaled.  Each lane rescales the rows it stored.  Returns tau.
template <typename T>
__device__ __noinline__ T rescale_reflector(T alpha, T xnorm, T beta, int j, int M, int lane,
                                            T *Aj, T *sv) {
    const int sh = -binary_exponent(beta);
    const T as = mul_exp2(alpha, sh);
    const T xs = mul_exp2(xnorm, sh);   // as, xs <= ~1: no overflow below
    const T bs = -copysign(sqrt(as * as + xs * xs), as);
    const T sc = exp2i<T>(sh - sh / 2) / (as - bs), post = exp2i<T>(sh / 2);
    for (int i = lane; i < M; i += 32) {
        if (i <= j) continue;
        const T v = (sv[i] * sc) * post;
        sv[i] = v;
        Aj[i] = v;
    }
    return (bs - as) / bs;
}

// Build reflector j from the register column x (already updated by all
// earlier reflectors); store the column back and publish v and tau.
// Tiny columns (subnormal entries, e.g. far-field interactions in FP32)
// take a scaled norm (dnrm2) and dlarfg's rescaling, so that no reciprocal
// overflows; both scale by powers of two only (exact, no division).
template <typename T, int RPL>
__device__ __forceinline__ void make_reflector(T (&x)[RPL], int j, int M, int lane, T *Aj,
                                               T *sv, T *s_tau, T *tau_out) {
    T alpha_l = 0, ss = 0;
#pragma unroll
    for (int t = 0; t < RPL; ++t) {
        const int i = lane + 32 * t;
        if (i == j) alpha_l = x[t];
        if (i > j && i < M) ss += x[t] * x[t];
    }
    const T alpha = __shfl_sync(0xffffffffu, alpha_l, j & 31);
    ss = warp_sum(ss);
    T xnorm;
    if (ss > NormLim<T>::lo && ss < NormLim<T>::hi) {
        xnorm = sqrt(ss);
    } else {  // scaled recomputation (dnrm2's guard against under/overflow)
        T amax = 0;
#pragma unroll
        for (int t = 0; t < RPL; ++t) {
            const int i = lane + 32 * t;
            if (i > j && i < M) amax = max(amax, abs(x[t]));
        }
        amax = warp_max(amax);
        T s2 = 0;
        int sc = 0;
        if (amax > T(0)) {
            // y = x 2^sc with |y| < 2 (sc clamped to a representable power)
            sc = min(max(-binary_exponent(amax), -NormLim<T>::max_shift), NormLim<T>::max_shift);
            const T f = exp2i<T>(sc);
#pragma unroll
            for (int t = 0; t < RPL; ++t) {
                const int i = lane + 32 * t;
                if (i > j && i < M) {
                    const T y = x[t] * f;
                    s2 += y * y;
                }
            }
        }
        xnorm = mul_exp2(sqrt(warp_sum(s2)), -sc);
    }
    T tj = 0, beta = alpha, scal = 1;
    bool rescale = false;
    if (xnorm > T(0)) {
        beta = -copysign(hypot(alpha, xnorm), alpha);
        if (abs(beta) >= NormLim<T>::safmin) {
            tj = (beta - alpha) / beta;
            scal = T(1) / (alpha - beta);
        } else if (beta == beta) {
            rescale = true;   // 1/(alpha - beta) would overflow: x is published as is
        }
    }
#pragma unroll
    for (int t = 0; t < RPL; ++t) {
        const int i = lane + 32 * t;
        T v = 0;
        if (i > j && i < M) {
            v = x[t] * scal;
            Aj[i] = v;
        } else if (i == j) {
            v = T(1);
            Aj[i] = beta;
        } else if (i < j) {
            Aj[i] = x[t];  // R entries above the diagonal
        }
        sv[i] = v;
    }
    if (rescale) tj = rescale_reflector(alpha, xnorm, beta, j, M, lane, Aj, sv);
    if (lane == 0) {
        *s_tau = tj;
        tau_out[j] = tj;
    }
}

// NW warps per CTA (a tuning choice): 8 gives the shortest path per update;
// 4 or 2 keep the same warps per SM in two or four times as many CTAs, so
// that one CTA's per-column barrier stall is covered by the others.
// panel < 0: all k columns; panel p >= 0: the columns [c0, c1) of the blocked
// QR's panel p (qr_panel_bounds), whose earlier columns are already factored
// and whose own columns already hold the earlier panels' updates.
template <typename T, int RPL, int NW>
__global__ void __launch_bounds__(NW * 32, (RPL <= 32 ? 2 : 1) * (8 / NW))
    geqrf_kernel(const Desc *__restrict__ descs, T *__restrict__ ws, int panel) {
    __shared__ T sv[2][32 * RPL];
    __shared__ T s_tau[2];
    const Desc d = descs[blockIdx.x];
    if (d.status0) return;
    const int M = d.M, k = d.k;
    int c0 = 0, c1 = k;
    if (panel >= 0 && !qr_panel_bounds(k, panel, c0, c1)) return;
    const WsLayout L = ws_layout(d);
    const int side = blockIdx.y;
    T *A = ws + d.ws + (side ? L.VB : L.UA);
    T *tau = ws + d.ws + (side ? L.tauB : L.tauA);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x[RPL];

    if (warp == 0) {
        const T *A0 = A + (size_t)c0 * M;
#pragma unroll
        for (int t = 0; t < RPL; ++t) {
            const int i = lane + 32 * t;
            x[t] = i < M ? A0[i] : T(0);
        }
        make_reflector<T, RPL>(x, c0, M, lane, A + (size_t)c0 * M, sv[0], &s_tau[0], tau);
    }
    __syncthreads();
    for (int j = c0; j + 1 < c1; ++j) {
        const int cur = (j - c0) & 1;
        const T *v = sv[cur];
        const T tj = s_tau[cur];
        for (int col = j + 1 + warp; col < c1; col += NW) {
            T *Ac = A + (size_t)col * M;
#pragma unroll
            for (int t = 0; t < RPL; ++t) {
                const int i = lane + 32 * t;
                x[t] = i < M ? Ac[i] : T(0);
            }
            if (tj != T(0)) {
                // two chains: four measured slower here (register pressure at
                // four CTAs per SM; other CTAs already hide the chain's latency)
                T d0 = 0, d1 = 0;
#pragma unroll
                for (int t = 0; t < RPL; t += 2) {
                    d0 += v[lane + 32 * t] * x[t];
                    if (t + 1 < RPL) d1 += v[lane + 32 * (t + 1)] * x[t + 1];
                }
                const T sc = tj * warp_sum(d0 + d1);
                // re-read v from shared memory instead of holding RPL values in registers
                const volatile T *vv = v;
#pragma unroll
                for (int t = 0; t < RPL; ++t) x[t] -= sc * vv[lane + 32 * t];
            }
            if (col == j + 1) {
                make_reflector<T, RPL>(x, j + 1, M, lane, Ac, sv[cur ^ 1], &s_tau[cur ^ 1], tau);
            } else {
#pragma unroll
                for (int t = 0; t < RPL; ++t) {
                    const int i = lane + 32 * t;
                    if (i >= j && i < M) Ac[i] = x[t];
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// phase 3: T = R_A R_B^T, SVD, rank rule
// ---------------------------------------------------------------------------
__device__ __forceinline__ void rr_pair(int round, int pi, int n, int &p, int &q) {
    // circle-method tournament on n (even) columns: n/2 disjoint pairs per
    // round, every pair exactly once in n-1 rounds
    if (pi == 0) {
        p = n - 1;
        q = round;
    } else {
        p = (round + pi) % (n - 1);
        q = (round - pi + (n - 1)) % (n - 1);
    }
}

template <typename T>
struct JacobiLim;
template <>
struct JacobiLim<double> {
    static constexpr double tiny_scale = 1e-60;  // fold a column scale below this
};
template <>
struct JacobiLim<float> {
    static constexpr float tiny_scale = 1e-12f;
};

// Lanes per column pair in the Jacobi sweeps of a bucket whose largest k is
// K.  A group of G lanes shares a pair's rows, which divides the per-round
// latency of one update by about G but repeats the rotation parameters in
// every lane of the group.  Shared-memory buckets take the plan's tuning
// (lanes for buckets of up to 24, up to 64 and more pairs; default two
// throughout, the autotuner's usual pick on a TLR panel).  Workspace buckets (k beyond the
// shared-memory limit): four lanes per pair, up to 1024 threads, to keep
// enough loads in flight on the L2-resident matrices.
constexpr int kSvdMaxThreads = 1024;
// A tuning value of 0 fills the warps: one lane per pair needs ceil(np/32)
// warps, and the pairs take as many lanes each (a power of two) as still fit
// in them.  On this GPU one FP64 warp instruction holds a sub-partition's
// pipe for about 64 cycles whatever its active lanes, so lanes left idle in a
// warp are free to share a pair's rows, while an extra warp would repeat the
// rotation-parameter arithmetic.
__host__ __device__ inline int svd_group(int K, bool smem, const int *lanes) {
    const int np = (K + 1) / 2;
    if (smem) {
        int g = np <= 24 ? lanes[0] : (np <= 64 ? lanes[1] : lanes[2]);
        if (g == 0) {
            const int w = (np + 31) / 32;
            g = 1;
            while (g < 32 && 2 * g * np <= 32 * w) g *= 2;
        }
        return g;
    }
    return np <= kSvdMaxThreads / 4 ? 4 : (np <= kSvdMaxThreads / 2 ? 2 : 1);
}
// Threads per CTA of the SVD kernel: G lanes for each of the K/2 pairs.
__host__ __device__ inline int svd_threads(int K, bool smem, const int *lanes) {
    const int np = (K + 1) / 2;
    const int cap = smem ? kThreads : kSvdMaxThreads;
    const int t = ((np * svd_group(K, smem, lanes) + 31) / 32) * 32;
    return t < 32 ? 32 : (t > cap ? cap : t);
}
__host__ __device__ inline int svd_ld(int k) { return k | 1; }

// Dynamic shared memory of the SVD kernel: `mats` K x ld matrices (2, 1 or 0:
// the launch mode), then the column scales, squared norms, singular values,
// Householder scalars, and two index arrays.
template <typename T>
__host__ __device__ inline size_t svd_smem_bytes(int K, int mats) {
    return (size_t)mats * K * svd_ld(K) * sizeof(T) + (size_t)4 * (K + 1) * sizeof(T) +
           (size_t)2 * (K + 1) * sizeof(int) + 64;
}

// Squared deflation bound of the SVD kernel's QR (described there): delta^2
// for an FP64 update ranked by accuracy, -1 (no deflation) otherwise.  f2 is
// ||T||_F^2 of T scaled by 2^-sexp.  One thread computes it once per update
// (a warp-wide sum there cost the Jacobi loops registers).
template <typename T>
__device__ __forceinline__ T deflation_bound2(T f2, int k, int rk, int rule, double acc, int sexp) {
    if constexpr (sizeof(T) != sizeof(double)) {
        return T(-1);
    } else {
        if (rk != 0 || !(acc > 0.0)) return T(-1);
        const T fro = sqrt(f2);
        const T thr = (rule & kRuleRelative) ? (T)acc * fro * rsqrt(T(k)) : mul_exp2((T)acc, -sexp);
        const T dl = min(T(1e-13) * thr, T(1e-16) * fro);
        return isfinite(dl) ? dl * dl : T(-1);
    }
}

// SVD of T = R_A R_B^T (k x k) by QR-preconditioned one-sided Jacobi
// (Drmac-Veselic): T P = Q R with column pivoting, then one-sided Jacobi on
// R^T, whose columns are graded by the pivoting, so the sweeps are few.
// With R^T V_J = U' S (U' orthonormal):  T = (Q V_J) S (P U')^T, hence
//   left vectors  U_T = Q V_J           (V_J accumulated by the rotations)
//   V_T S         = P (R^T V_J)         (the rotated columns, rows permuted).
// Written for the FP64 issue rate of this GPU (one warp FP64 instruction per
// ~80 cycles per SM sub-partition): lanes work on whole columns or pairs of
// columns and loop over rows, so no shuffle reductions are needed, and the
// rotations are scaled ("fast"): column j is d_j x_j in both R^T and V_J, so
// a rotation costs two FMAs per row and matrix.  Squared norms are tracked
// (exact in exact arithmetic), recomputed on strong cancellation and after
// every sweep.  Convergence: every pair orthogonal to k*eps relative to its
// norms (LAPACK dgesvj's criterion).
// Range safety (as LAPACK's sgesvd/dgesvd scale the matrix first): T is
// scaled by 2^-e so that its largest entry lies in [1, 2) (exact; the
// singular values and V S are scaled back by 2^e), and a column whose squared
// norm is below safmin is negligible (< 2^-485 relative in FP64, 2^-51 in
// FP32) and not rotated.  A non-finite singular value marks the update
// NOCONV; the sort below is a total order even then.
template <typename T, int MODE>
__global__ void __launch_bounds__(kSvdMaxThreads) gesvd_kernel(const Desc *__restrict__ descs,
                                                               T *__restrict__ ws,
                                                               int *__restrict__ rank,
                                                               int *__restrict__ status,
                                                               int *__restrict__ info, int maxK,
                                                               int G) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ int s_rot, s_piv, s_exp, s_conv;
    __shared__ T s_wmax[kSvdMaxThreads / 32];
    __shared__ T s_defl2;
    const Desc d = descs[blockIdx.x];
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31;
    if (d.status0) {
        if (tid == 0) {
            status[d.idx] = d.status0;
            rank[d.idx] = 0;
            if (info) info[d.idx] = 0;
        }
        return;
    }
    const int M = d.M, k = d.k;
    const WsLayout L = ws_layout(d);
    T *base = ws + d.ws;
    const T *UA = base + L.UA, *VB = base + L.VB;
    // the k x k working matrices: column-major in shared memory (odd ld: a
    // lane walking its own column is free of bank conflicts), row-major in
    // the workspace (the lanes of a warp own consecutive columns in the
    // tournament and in every lane-per-column loop: coalesced).  MODE 1: both
    // in shared memory; 2: B (R^T) in shared memory, A (V_J) in the
    // workspace; 0: both in the workspace.
    constexpr bool A_SM = MODE == 1, B_SM = MODE >= 1;
    const int ldA = A_SM ? svd_ld(k) : k, ldB = B_SM ? svd_ld(k) : k;
    // distance of rows i and i + 1 in a column
    const size_t rsA = A_SM ? 1 : (size_t)ldA, rsB = B_SM ? 1 : (size_t)ldB;
    auto ixA = [ldA](int i, int j) -> size_t {
        return A_SM ? (size_t)j * ldA + i : (size_t)i * ldA + j;
    };
    auto ixB = [ldB](int i, int j) -> size_t {
        return B_SM ? (size_t)j * ldB + i : (size_t)i * ldB + j;
    };
    T *A = A_SM ? reinterpret_cast<T *>(smem_raw) : base + L.W;   // T, then QR, then V_J
    T *B = B_SM ? reinterpret_cast<T *>(smem_raw) + (A_SM ? (size_t)maxK * svd_ld(maxK) : 0)
                : base + L.V;                                       // R^T, rotated
    const int nsm = (A_SM ? 1 : 0) + (B_SM ? 1 : 0);
    T *aux = reinterpret_cast<T *>(smem_raw + (size_t)nsm * maxK * svd_ld(maxK) * sizeof(T));
    T *s_d = aux, *s_nrm = aux + (maxK + 1), *s_sig = aux + 2 * (maxK + 1);
    T *s_tau = aux + 3 * (maxK + 1);
    int *s_perm = reinterpret_cast<int *>(aux + 4 * (maxK + 1));   // Jacobi sort
    int *s_pcol = s_perm + (maxK + 1);                                // QR pivots
    T *Yg = base + L.Uo;   // reflectors of Q (k x k, ld k) in the Uo slot until U_r is written

    // T = triu(R_A) triu(R_B)^T (hcore_dgemm.c:330-387)
    T amax = 0;
    for (int o = 0; o < k; ++o)
        for (int t = tid; t < k; t += nthr) {   // the lanes walk the contiguous index
            const int i = A_SM ? t : o, j = A_SM ? o : t;
            T s = 0;
            for (int l = max(i, j); l < k; ++l) s += UA[(size_t)l * M + i] * VB[(size_t)l * M + j];
            A[ixA(i, j)] = s;
            amax = max(amax, abs(s));
        }
    // scale T by 2^-e, e = exponent of its largest entry (nthr is a multiple of 32)
    amax = warp_max(amax);
    if (lane == 0) s_wmax[tid >> 5] = amax;
    __syncthreads();
    if (tid == 0) {
        T m = 0;
        for (int w = 0; w < nthr / 32; ++w) m = max(m, s_wmax[w]);
        s_exp = (m > T(0) && isfinite(m)) ? binary_exponent(m) : 0;
    }
    __syncthreads();
    const int sexp = s_exp;
    if (sexp != 0)
        for (int o = 0; o < k; ++o)
            for (int t = tid; t < k; t += nthr) A[(size_t)o * ldA + t] = mul_exp2(A[(size_t)o * ldA + t], -sexp);
    __syncthreads();

    // ---- QR with column pivoting, T P = Q R (lane per column) ----
    for (int c = tid; c < k; c += nthr) {
        T s = 0;
        for (int i = 0; i < k; ++i) s += A[ixA(i, c)] * A[ixA(i, c)];
        s_nrm[c] = s;   // partial column norms (rows j..k-1), squared
        s_d[c] = s;     // norms at the last exact computation
        s_pcol[c] = c;
    }
    __syncthreads();
    // Deflation (FP64 rank-by-accuracy updates): the QR stops at the first
    // step j whose trailing block R22 = R(j:k, j:k) has ||R22||_F <= delta,
    // and the Jacobi then runs on the first j rows of R only.  Dropping R22
    // moves every singular value by at most delta (Weyl), with
    //   delta = min(1e-13 thr, 1e-16 ||T||_F),
    // thr the truncation threshold (acc, or for the relative rule its lower
    // bound acc ||T||_F / sqrt(k)): a rank decision can change only for a
    // singular value within 1e-13 of the threshold, relative, and every
    // singular value stays within a few eps sigma_max of the full one (the
    // accuracy of dgesvd's small singular values).  The dropped directions
    // come out with singular value 0.  On the TLR panel's updates about half
    // of the columns are below this bound.
    if (tid == 0) {
        T f2 = 0;   // ||T||_F^2 of the scaled T
        for (int c = 0; c < k; ++c) f2 += s_nrm[c];
        s_defl2 = deflation_bound2(f2, k, d.rk, d.rule, d.acc, sexp);
    }
    int kk = k;   // columns of R^T that the Jacobi rotates
    // (the rank search keeps its first rank_start columns whatever their size)
    const int kfloor = d.rank_start < k ? (d.rank_start > 0 ? d.rank_start : 0) : k;
    for (int j = 0; j < k; ++j) {
        // pivot: the largest remaining partial norm (warp 0); deflation test
        if (tid < 32) {
            T best = -1, tail = 0;
            int bi = j;
            for (int c = j + lane; c < k; c += 32) {
                tail += s_nrm[c];
                if (s_nrm[c] > best) {
                    best = s_nrm[c];
                    bi = c;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const T ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                tail += __shfl_xor_sync(0xffffffffu, tail, o);
                if (ob > best || (ob == best && oi < bi)) {
                    best = ob;
                    bi = oi;
                }
            }
            if (lane == 0) s_piv = (j >= kfloor && tail <= s_defl2) ? -1 : bi;
        }
        __syncthreads();
        const int pv = s_piv;
        if (pv < 0) {
            kk = j;
            break;
        }
        if (pv != j) {
            for (int i = tid; i < k; i += nthr) {
                const T x = A[ixA(i, j)];
                A[ixA(i, j)] = A[ixA(i, pv)];
                A[ixA(i, pv)] = x;
            }
            if (tid == 0) {
                T x = s_nrm[j]; s_nrm[j] = s_nrm[pv]; s_nrm[pv] = x;
                x = s_d[j]; s_d[j] = s_d[pv]; s_d[pv] = x;
                const int ci = s_pcol[j]; s_pcol[j] = s_pcol[pv]; s_pcol[pv] = ci;
            }
        }
        __syncthreads();
        // reflector of column j, rows j..k-1 (dlarfg), by warp 0: the lanes
        // split the sum of squares and the scaling
        if (tid < 32) {
            T *aj = A + ixA(0, j);
            const T alpha = aj[j * rsA];
            T ss = 0;
            for (int i = j + 1 + lane; i < k; i += 32) ss += aj[i * rsA] * aj[i * rsA];
            ss = warp_sum(ss);
            T tj = 0;
            if (ss > T(0)) {
                const T beta = -copysign(sqrt(alpha * alpha + ss), alpha);
                tj = (beta - alpha) / beta;
                const T scal = T(1) / (alpha - beta);
                for (int i = j + 1 + lane; i < k; i += 32) aj[i * rsA] *= scal;
                __syncwarp();
                if (lane == 0) aj[j * rsA] = beta;
            }
            if (lane == 0) s_tau[j] = tj;
        }
        __syncthreads();
        // apply to the trailing columns and downdate their norms (lane per column)
        const T tj = s_tau[j];
        for (int c = j + 1 + tid; c < k; c += nthr) {
            T *ac = A + ixA(0, c);
            const T *aj = A + ixA(0, j);
            if (tj != T(0)) {
                T dot = ac[j * rsA], dot2 = 0;
                int i = j + 1;
                for (; i + 1 < k; i += 2) {
                    dot += aj[i * rsA] * ac[i * rsA];
                    dot2 += aj[(i + 1) * rsA] * ac[(i + 1) * rsA];
                }
                if (i < k) dot += aj[i * rsA] * ac[i * rsA];
                const T s = tj * (dot + dot2);
                ac[j * rsA] -= s;
                for (int i = j + 1; i < k; ++i) ac[i * rsA] -= s * aj[i * rsA];
            }
            // partial norm of rows j+1..k-1 (dlaqp2's downdate with recomputation)
            const T rjc = ac[j * rsA];
            T nn = s_nrm[c] - rjc * rjc;
            if (nn <= s_d[c] * T(1.0 / 1024) || nn <= T(0)) {
                T s = 0;
                for (int i = j + 1; i < k; ++i) s += ac[i * rsA] * ac[i * rsA];
                nn = s;
                s_d[c] = s;
            }
            s_nrm[c] = nn;
        }
        __syncthreads();
    }
    // Q's reflectors to global (read back when forming U_T = Q V_J); B = R^T
    // (rows kk.. of R dropped: B's columns kk.. are zero); A = I (V_J).
    // Reflectors kk.. were never formed: tau 0.
    for (int h = kk + tid; h < k; h += nthr) s_tau[h] = T(0);
    for (int j = 0; j < k; ++j)
        for (int i = tid; i < k; i += nthr) {
            const T x = A[ixA(i, j)];
            Yg[(size_t)j * k + i] = (i > j && j < kk) ? x : T(0);
            B[ixB(j, i)] = (i <= j && i < kk) ? x : T(0);   // B(j, i) = R(i, j)
        }
    __syncthreads();
    for (int o = 0; o < k; ++o)
        for (int t = tid; t < k; t += nthr) A[(size_t)o * ldA + t] = o == t ? T(1) : T(0);
    for (int c = tid; c < k; c += nthr) {
        T s = 0;
        if (c < kk)
            for (int i = 0; i < k; ++i) s += B[ixB(i, c)] * B[ixB(i, c)];
        s_nrm[c] = s;
        s_d[c] = T(1);
    }
    if (tid == 0) s_piv = 0;   // reused below: set when a singular value is not finite
    __syncthreads();

    // ---- one-sided Jacobi on B = R^T, rotations accumulated in A ----
    // G lanes per pair (rows i = lig, lig+G, ...); every lane runs the same
    // number of iterations so that the full-warp shuffles stay converged
    // (columns kk.. of B are zero and take no part; V_J's rows kk.. stay zero)
    const int n = kk + (kk & 1);
    const int np = n / 2;
    const int grp = tid / G, lig = tid % G, ngrp = nthr / G;
    const T tol = T(k > 8 ? k : 8) * Lim<T>::eps;
    // Stop after a sweep with no rotation, or after one whose largest relative
    // off-diagonal |a_pq| / sqrt(a_pp a_qq) was at most sqrt(tol): cyclic
    // Jacobi converges quadratically, so the next sweep would only rotate by
    // angles near tol, moving the singular values at second order (the
    // product U S V^T is exact after every sweep; only orthogonality remains).
    // Both tests compare squares (a_pq^2 against tol^2 a_pp a_qq), so they
    // take no square root or division.
    const T tol2 = tol * tol;
    const T stop2 = tol;   // (sqrt(tol))^2
    bool converged = (kk <= 1);
    int sweeps = 0;
    for (int sweep = 0; sweep < kMaxSweeps && !converged; ++sweep) {
        if (tid == 0) s_rot = 0;
        bool sweep_big = false;   // this thread rotated a pair above sqrt(tol)
        __syncthreads();
        for (int round = 0; round < n - 1; ++round) {
            for (int base = 0; base < np; base += ngrp) {
                const int pi = base + grp;
                int p = 0, q = 0;
                if (pi < np) rr_pair(round, pi, n, p, q);
                const bool valid = pi < np && p < kk && q < kk;
                T *xp = B + ixB(0, p), *xq = B + ixB(0, q);
                T dot = 0;
                if (valid) {
                    // four partial sums: the chain of dependent FMAs is a quarter
                    // as long (one update's Jacobi round is latency-bound)
                    T d1 = 0, d2 = 0, d3 = 0;
                    int i = lig;
                    for (; i + 3 * G < k; i += 4 * G) {
                        dot += xp[i * rsB] * xq[i * rsB];
                        d1 += xp[(i + G) * rsB] * xq[(i + G) * rsB];
                        d2 += xp[(i + 2 * G) * rsB] * xq[(i + 2 * G) * rsB];
                        d3 += xp[(i + 3 * G) * rsB] * xq[(i + 3 * G) * rsB];
                    }
                    for (; i < k; i += G) dot += xp[i * rsB] * xq[i * rsB];
                    dot = (dot + d1) + (d2 + d3);
                }
                for (int o = G / 2; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
                T dp = 1, dq = 1, app = 0, aqq = 0, apq = 0;
                if (valid) {
                    dp = s_d[p];
                    dq = s_d[q];
                    app = s_nrm[p];
                    aqq = s_nrm[q];
                    apq = dp * dq * dot;
                }
                // the squared norms are at most 4k (T is scaled to entries
                // below 2), so the products below cannot overflow
                const T apq2 = apq * apq, pq = app * aqq;
                const bool rot = valid && app > NormLim<T>::safmin && aqq > NormLim<T>::safmin &&
                                 apq != T(0) && apq2 > tol2 * pq;
                T t = 0, cs = 1;
                if (rot) {
                    sweep_big |= apq2 > stop2 * pq;
                    // t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)), zeta = w / v with
                    // w = a_qq - a_pp, v = 2 a_pq, taken as |v| / (|w| + sqrt(w^2 + v^2))
                    // with the sign of w v (w = 0 gives t = sign(v)): one square
                    // root and one division, and no overflow for tiny a_pq
                    const T w = aqq - app, v = T(2) * apq;
                    const T h = sqrt(fma(w, w, v * v));
                    t = abs(v) / (abs(w) + h);
                    if ((w < T(0)) != (v < T(0))) t = -t;
                    cs = rsqrt(fma(t, t, T(1)));
                    // true columns p' = c (p - t q), q' = c (q + t p), in B and V_J;
                    // with scales d: f1 = t dq / dp, f2 = t dp / dq from one reciprocal
                    const T inv = T(1) / (dp * dq);
                    const T f1 = t * (dq * dq) * inv, f2 = t * (dp * dp) * inv;
                    T *vp = A + ixA(0, p), *vq = A + ixA(0, q);
                    // two rows per iteration, all loads before the stores: the rows
                    // are distinct, so the loads of the second row need not wait
                    // for the stores of the first
                    // (shared-memory modes only: the workspace mode has no registers
                    // to spare at 1024 threads)
                    // (V_J's rows kk.. are zero in every column the Jacobi
                    // rotates: rows from kk on update B alone)
                    int i = lig;
                    if (MODE != 0)
                    for (; i + G < kk; i += 2 * G) {
                        const size_t r0 = (size_t)i, r1 = (size_t)(i + G);
                        const T a0 = xp[r0 * rsB], b0 = xq[r0 * rsB];
                        const T a1 = xp[r1 * rsB], b1 = xq[r1 * rsB];
                        const T u0 = vp[r0 * rsA], v0 = vq[r0 * rsA];
                        const T u1 = vp[r1 * rsA], v1 = vq[r1 * rsA];
                        xp[r0 * rsB] = a0 - f1 * b0;
                        xq[r0 * rsB] = b0 + f2 * a0;
                        xp[r1 * rsB] = a1 - f1 * b1;
                        xq[r1 * rsB] = b1 + f2 * a1;
                        vp[r0 * rsA] = u0 - f1 * v0;
                        vq[r0 * rsA] = v0 + f2 * u0;
                        vp[r1 * rsA] = u1 - f1 * v1;
                        vq[r1 * rsA] = v1 + f2 * u1;
                    }
                    for (; i < kk; i += G) {
                        const T a = xp[i * rsB], b = xq[i * rsB];
                        xp[i * rsB] = a - f1 * b;
                        xq[i * rsB] = b + f2 * a;
                        const T u = vp[i * rsA], v = vq[i * rsA];
                        vp[i * rsA] = u - f1 * v;
                        vq[i * rsA] = v + f2 * u;
                    }
                    if (MODE != 0)
                    for (; i + G < k; i += 2 * G) {
                        const size_t r0 = (size_t)i, r1 = (size_t)(i + G);
                        const T a0 = xp[r0 * rsB], b0 = xq[r0 * rsB];
                        const T a1 = xp[r1 * rsB], b1 = xq[r1 * rsB];
                        xp[r0 * rsB] = a0 - f1 * b0;
                        xq[r0 * rsB] = b0 + f2 * a0;
                        xp[r1 * rsB] = a1 - f1 * b1;
                        xq[r1 * rsB] = b1 + f2 * a1;
                    }
                    for (; i < k; i += G) {
                        const T a = xp[i * rsB], b = xq[i * rsB];
                        xp[i * rsB] = a - f1 * b;
                        xq[i * rsB] = b + f2 * a;
                    }
                }
                T np_ = app - t * apq, nq_ = aqq + t * apq;
                const T dp2 = dp * cs, dq2 = dq * cs;
                // strong cancellation in a tracked norm: recompute (warp-uniform)
                const bool redo_p = rot && np_ < app * T(1.0 / 64);
                const bool redo_q = rot && nq_ < aqq * T(1.0 / 64);
                if (__any_sync(0xffffffffu, redo_p || redo_q)) {
                    T sp = 0, sq = 0;
                    if (redo_p || redo_q)
                        for (int i = lig; i < k; i += G) {
                            sp += xp[i * rsB] * xp[i * rsB];
                            sq += xq[i * rsB] * xq[i * rsB];
                        }
                    for (int o = G / 2; o > 0; o >>= 1) {
                        sp += __shfl_xor_sync(0xffffffffu, sp, o);
                        sq += __shfl_xor_sync(0xffffffffu, sq, o);
                    }
                    if (redo_p) np_ = dp2 * dp2 * sp;
                    if (redo_q) nq_ = dq2 * dq2 * sq;
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
            T *xj = B + ixB(0, j);
            T dj = s_d[j];
            if (dj < JacobiLim<T>::tiny_scale) {
                T *vj = A + ixA(0, j);
                for (int i = 0; i < k; ++i) {
                    xj[i * rsB] *= dj;
                    vj[i * rsA] *= dj;
                }
                dj = T(1);
                s_d[j] = dj;
            }
            T s2 = 0, s3 = 0;
            int i = 0;
            for (; i + 1 < k; i += 2) {
                s2 += xj[i * rsB] * xj[i * rsB];
                s3 += xj[(i + 1) * rsB] * xj[(i + 1) * rsB];
            }
            if (i < k) s2 += xj[i * rsB] * xj[i * rsB];
            s_nrm[j] = dj * dj * (s2 + s3);
        }
        ++sweeps;
        const bool big = __any_sync(0xffffffffu, sweep_big);
        if (lane == 0) s_wmax[tid >> 5] = big ? T(1) : T(0);
        __syncthreads();
        if (tid == 0) {
            T m = 0;
            for (int w = 0; w < nthr / 32; ++w) m = max(m, s_wmax[w]);
            s_conv = (s_rot == 0 || m == T(0)) ? 1 : 0;
        }
        __syncthreads();
        converged = s_conv != 0;
        __syncthreads();
    }

    // singular values = true column norms of B (of the scaled T); sort
    // descending, ties by index, NaN last: a total order, so s_perm is a
    // permutation whatever the values
    for (int j = tid; j < k; j += nthr) {
        const T s = sqrt(s_nrm[j]);
        s_sig[j] = s;
        if (!isfinite(s)) s_piv = 1;
    }
    __syncthreads();
    const bool finite = s_piv == 0;
    for (int j = tid; j < k; j += nthr) {
        const T sj = s_sig[j] == s_sig[j] ? s_sig[j] : T(-1);
        int pos = 0;
        for (int i = 0; i < k; ++i) {
            const T si = s_sig[i] == s_sig[i] ? s_sig[i] : T(-1);
            pos += (si > sj) || (si == sj && i < j);
        }
        s_perm[pos] = j;
    }
    __syncthreads();
    T *sig_out = base + L.sig;
    for (int t = tid; t < k; t += nthr) sig_out[t] = mul_exp2(s_sig[s_perm[t]], sexp);

    // rank rule (hcore_dgemm.c:444-464; the fast rules start at i = 2; the
    // compressor's starts at 0, may compare with acc * sigma_max and caps
    // the rank at max_rank)
    int r;
    if (d.rk != 0) {
        r = d.rk < k ? d.rk : k;
    } else {
        const T thr = (d.rule & kRuleRelative) ? (T)d.acc * mul_exp2(s_sig[s_perm[0]], sexp)
                                               : (T)d.acc;
        r = k;
        for (int i = d.rank_start; i < k; ++i)
            if (mul_exp2(s_sig[s_perm[i]], sexp) < thr) {
                r = i;
                break;
            }
    }
    if ((d.rule & kRuleCapRank) && r > d.max_rank) r = d.max_rank;
    int st = HCORE_GPU_S_OK;
    if (!converged || !finite) st = HCORE_GPU_S_NOCONV;
    else if (r > d.max_rank) st = HCORE_GPU_S_RANK_MAX;
    else if (r > d.storage_rank) st = HCORE_GPU_S_STORAGE;

    // U_r and V_r S_r of an accepted update, and of one whose rank only
    // exceeds its storage limit (rebuilt later into larger storage).  st is
    // uniform in the CTA.
    if (st == HCORE_GPU_S_OK || st == HCORE_GPU_S_STORAGE) {
        // U_r = Q (V_J's true columns), Q = H_0 ... H_{k-1}: lane per output
        // column, in place in V_J's column, reflectors (in the Uo slot) from
        // last to first.
        for (int t = tid; t < r; t += nthr) {
            const int j = s_perm[t];
            T *x = A + ixA(0, j);   // each lane owns the column of its own j
            const T dj = s_d[j];
            for (int i = 0; i < k; ++i) x[i * rsA] *= dj;
            for (int h = k - 1; h >= 0; --h) {
                const T th = s_tau[h];
                if (th == T(0)) continue;
                const T *y = Yg + (size_t)h * k;
                T dot = x[h * rsA];
                for (int i = h + 1; i < k; ++i) dot += y[i] * x[i * rsA];
                const T s = th * dot;
                x[h * rsA] -= s;
                for (int i = h + 1; i < k; ++i) x[i * rsA] -= s * y[i];
            }
        }
        __syncthreads();   // the reflectors are dead from here on
        // V_r S_r = P (B's true columns): row P(i) of the output is row i of
        // B (the rows S V^T of hcore_dgemm.c:484-489, transposed); U_r
        T *Uo = base + L.Uo, *Vo = base + L.Vo;
        for (int e = tid; e < k * r; e += nthr) {
            const int i = e % k, t = e / k;
            const int j = s_perm[t];
            Vo[(size_t)t * k + s_pcol[i]] = mul_exp2(s_d[j] * B[ixB(i, j)], sexp);
            Uo[(size_t)t * k + i] = A[ixA(i, j)];
        }
    }
    if (tid == 0) {
        rank[d.idx] = r;
        status[d.idx] = st;
        if (info) info[d.idx] = sweeps;
    }
}

// ---------------------------------------------------------------------------
// phase 4: CU = Q_A [U_r; 0], CV = Q_B [V_r S_r; 0]   (dormqr 'L','N')
// ---------------------------------------------------------------------------
// A CTA owns up to kWarps output columns of one (update, side), one per warp,
// each kept in registers (RPL rows per lane, row = lane + 32 t) for the whole
// product.  The k reflectors are applied last to first, staged through
// shared memory kApplyChunk at a time (one coalesced load per CTA, zero
// outside rows j..M-1 so that the dot and the axpy need no predicates); the
// column is stored once, coalesced, into the caller's factor.  blockIdx.z
// selects the group of columns; groups past the new rank exit at once.
constexpr int kApplyChunk = 8;

template <typename T, int RPL, typename Tc>
__global__ void __launch_bounds__(kThreads, RPL <= 32 ? 2 : 1) apply_kernel(const Desc *__restrict__ descs,
                                                         const T *__restrict__ ws,
                                                         const int *__restrict__ rank,
                                                         const int *__restrict__ status) {
    extern __shared__ unsigned char smem_raw[];
    Tc *sv = reinterpret_cast<Tc *>(smem_raw);   // kApplyChunk x (32 RPL)
    __shared__ Tc s_tau[kApplyChunk];
    const Desc d = descs[blockIdx.x];
    if (d.status0 || status[d.idx] != HCORE_GPU_S_OK) return;
    const int r = rank[d.idx];
    const int col0 = blockIdx.z * kWarps;
    if (col0 >= r) return;
    const int side = blockIdx.y;
    const int M = d.M, k = d.k;
    const WsLayout L = ws_layout(d);
    const T *base = ws + d.ws;
    const T *Y = base + (side ? L.VB : L.UA);
    const T *tau = base + (side ? L.tauB : L.tauA);
    const T *X0 = base + (side ? L.Vo : L.Uo);
    T *out = (T *)(side ? d.CVo : d.CUo);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int col = col0 + warp;
    const bool active = col < r;
    constexpr int ROWS = 32 * RPL;

    Tc x[RPL];
#pragma unroll
    for (int t = 0; t < RPL; ++t) {
        const int i = lane + 32 * t;
        x[t] = (active && i < k) ? (Tc)X0[(size_t)col * k + i] : Tc(0);
    }
    const int nch = (k + kApplyChunk - 1) / kApplyChunk;
    for (int ch = nch - 1; ch >= 0; --ch) {
        const int j0 = ch * kApplyChunk;
        const int nj = min(kApplyChunk, k - j0);
        __syncthreads();  // the previous chunk is no longer read
        for (int e = tid; e < nj * ROWS; e += kThreads) {
            const int c = e / ROWS, i = e % ROWS;
            const int j = j0 + c;
            Tc v = Tc(0);
            if (i > j && i < M) v = (Tc)Y[(size_t)j * M + i];
            else if (i == j) v = Tc(1);
            sv[c * ROWS + i] = v;
        }
        if (tid < nj) s_tau[tid] = (Tc)tau[j0 + tid];
        __syncthreads();
        if (!active) continue;
        for (int c = nj - 1; c >= 0; --c) {
            const Tc tj = s_tau[c];
            if (tj == Tc(0)) continue;
            const Tc *v = sv + c * ROWS;
            Tc d0 = 0, d1 = 0;
#pragma unroll
            for (int t = 0; t < RPL; t += 2) {
                d0 += v[lane + 32 * t] * x[t];
                if (t + 1 < RPL) d1 += v[lane + 32 * (t + 1)] * x[t + 1];
            }
            const Tc s = tj * warp_sum(d0 + d1);
            const volatile Tc *vv = v;  // re-read rather than hold RPL values in registers
#pragma unroll
            for (int t = 0; t < RPL; ++t) x[t] -= s * vv[lane + 32 * t];
        }
    }
    if (active) {
#pragma unroll
        for (int t = 0; t < RPL; ++t) {
            const int i = lane + 32 * t;
            if (i < M) out[(size_t)col * d.ldco + i] = (T)x[t];
        }
    }
}

// ---------------------------------------------------------------------------
template <typename T, int RPL, typename Tc>
static void launch_apply(const Desc *d_desc, int n, const T *ws, const int *d_rank,
                         const int *d_status, int maxK, cudaStream_t s) {
    const int groups = (maxK + kWarps - 1) / kWarps;   // the new rank is at most k
    const size_t smem = (size_t)kApplyChunk * 32 * RPL * sizeof(Tc);
    apply_kernel<T, RPL, Tc><<<dim3(n, 2, groups), kThreads, smem, s>>>(d_desc, ws, d_rank,
                                                                       d_status);
}

template <typename T, typename Tc>
static void launch_apply_all(const Desc *d_desc, int n, const T *ws, const int *d_rank,
                             const int *d_status, int maxK, int rpl, cudaStream_t s) {
    if (rpl <= 4) launch_apply<T, 4, Tc>(d_desc, n, ws, d_rank, d_status, maxK, s);
    else if (rpl <= 8) launch_apply<T, 8, Tc>(d_desc, n, ws, d_rank, d_status, maxK, s);
    else if (rpl <= 16) launch_apply<T, 16, Tc>(d_desc, n, ws, d_rank, d_status, maxK, s);
    else if (rpl <= 32) launch_apply<T, 32, Tc>(d_desc, n, ws, d_rank, d_status, maxK, s);
    else launch_apply<T, 64, Tc>(d_desc, n, ws, d_rank, d_status, maxK, s);
}

template <typename T, typename Tc>
static cudaError_t set_apply_smem() {
    const int s64 = kApplyChunk * 32 * 64 * (int)sizeof(Tc);
    cudaError_t e = cudaFuncSetAttribute(apply_kernel<T, 64, Tc>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, s64);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(apply_kernel<T, 32, Tc>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, s64 / 2);
    return e;
}

template <typename T, int RPL>
static void launch_geqrf(const Desc *d_desc, int n, T *ws, int warps, int panel, cudaStream_t s) {
    if (n <= 0) return;
    if (warps == 2) geqrf_kernel<T, RPL, 2><<<dim3(n, 2), 64, 0, s>>>(d_desc, ws, panel);
    else if (warps == 4) geqrf_kernel<T, RPL, 4><<<dim3(n, 2), 128, 0, s>>>(d_desc, ws, panel);
    else geqrf_kernel<T, RPL, 8><<<dim3(n, 2), 256, 0, s>>>(d_desc, ws, panel);
}

template <typename T>
static void launch_geqrf_all(const Desc *d_desc, int n, T *ws, int warps, int rpl, int panel,
                             cudaStream_t s) {
    if (rpl <= 4) launch_geqrf<T, 4>(d_desc, n, ws, warps, panel, s);
    else if (rpl <= 8) launch_geqrf<T, 8>(d_desc, n, ws, warps, panel, s);
    else if (rpl <= 16) launch_geqrf<T, 16>(d_desc, n, ws, warps, panel, s);
    else if (rpl <= 32) launch_geqrf<T, 32>(d_desc, n, ws, warps, panel, s);
    else launch_geqrf<T, 64>(d_desc, n, ws, warps, panel, s);
}

// Launch plan of the blocked QR over a shape's k-sorted buckets: the
// descriptors above kTcMaxK (a prefix) take the unblocked kernel; for the
// rest, panel p runs over every descriptor that has one, and the trailing
// update after panel p once per update-size class.  fn(kind, start, count,
// panel, class): kind 0 unblocked QR, 1 panel, 2 trailing update.
template <typename F>
static void qr_plan(const LaunchShape &shape, int n, F &&fn) {
    int split = 0;  // first descriptor with k <= kTcMaxK
    int b = 0;
    while (b < shape.nbuckets && shape.buckets[b].K > kTcMaxK) split += shape.buckets[b++].count;
    if (split > 0) fn(0, 0, split, -1, 0);
    if (split >= n || b >= shape.nbuckets) return;
    const int kmax = shape.buckets[b].K;
    for (int p = 0; p < kQrPanels; ++p) {
        int c0, c1;
        if (!qr_panel_bounds(kmax, p, c0, c1)) break;
        fn(1, split, n - split, p, 0);
        // trailing updates: descriptors whose panel p is not their last
        int bb = b, start = split;
        while (bb < shape.nbuckets) {
            const int K = shape.buckets[bb].K;
            if (!qr_panel_bounds(K, p, c0, c1) || c1 >= K) break;  // sorted: none below
            const int cls = qr_update_class(K - 16 * p);
            int count = 0;
            while (bb < shape.nbuckets && qr_panel_bounds(shape.buckets[bb].K, p, c0, c1) &&
                   c1 < shape.buckets[bb].K && qr_update_class(shape.buckets[bb].K - 16 * p) == cls)
                count += shape.buckets[bb++].count;
            if (count > 0) fn(2, start, count, p, cls);
            start += count;
        }
    }
}

int qr_launches(const LaunchShape &shape, bool fp64) {
    if (!fp64 || !shape.tc_qr || shape.nbuckets <= 0) return 1;
    int c = 0;
    int n = 0;
    for (int b = 0; b < shape.nbuckets; ++b) n += shape.buckets[b].count;
    qr_plan(shape, n, [&](int, int, int count, int, int) { c += count > 0; });
    return c;
}

template <typename T>
static cudaError_t configure_recompress_once(int dev, int *svd_smem_kmax, int *svd_half_kmax);

// The kernel attributes are per device and do not depend on the plan, so
// they are set once per device and scalar type; later calls (every drop-in
// call, every plan) only read the cached limits.
template <typename T>
cudaError_t configure_recompress(int maxK, int *svd_smem_kmax, int *svd_half_kmax) {
    (void)maxK;
    constexpr int kDevices = 64;
    static std::mutex mu;
    static int done[kDevices], kmax_c[kDevices], khalf_c[kDevices];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kDevices) return configure_recompress_once<T>(dev, svd_smem_kmax, svd_half_kmax);
    std::lock_guard<std::mutex> lk(mu);
    if (!done[dev]) {
        e = configure_recompress_once<T>(dev, &kmax_c[dev], &khalf_c[dev]);
        if (e != cudaSuccess) return e;
        done[dev] = 1;
    }
    *svd_smem_kmax = kmax_c[dev];
    if (svd_half_kmax) *svd_half_kmax = khalf_c[dev];
    return cudaSuccess;
}

template <typename T>
static cudaError_t configure_recompress_once(int dev, int *svd_smem_kmax, int *svd_half_kmax) {
    // the Jacobi matrices live in shared memory when they fit (k <= 119 in FP64,
    // 168 in FP32, with 227 KB per CTA); R^T alone up to k = 167 in FP64
    int optin = 0;
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    // dynamic shared memory the SVD kernel may take next to its static arrays
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, gesvd_kernel<T, 1>);
    if (e != cudaSuccess) return e;
    const int dyn_max = optin - (int)fa.sharedSizeBytes;
    int kmax = 0;
    while (kmax < kMaxK && svd_smem_bytes<T>(kmax + 1, 2) <= (size_t)dyn_max) ++kmax;
    *svd_smem_kmax = kmax;
    int khalf = kmax;
    while (khalf < kMaxK && svd_smem_bytes<T>(khalf + 1, 1) <= (size_t)dyn_max) ++khalf;
    if (svd_half_kmax) *svd_half_kmax = khalf;
    e = set_apply_smem<T, T>();
    if (e == cudaSuccess) e = set_apply_smem<T, float>();
    if (e == cudaSuccess && sizeof(T) == sizeof(double)) e = configure_rebuild_tc();
    if (e == cudaSuccess && sizeof(T) == sizeof(double)) e = configure_qr_tc();
    if (e == cudaSuccess && sizeof(T) == sizeof(double)) e = configure_stack_tc();
    if (e != cudaSuccess) return e;
    // the attribute is per kernel, not per plan: allow the largest size any
    // plan may launch with, so plans of different k coexist
    e = cudaFuncSetAttribute(gesvd_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             dyn_max);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(gesvd_kernel<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 dyn_max);
    return e;
}

int bucket_edge(int k, int width) {
    static const int fine[] = {8, 16, 24, 32, 40, 48, 56, 64, 80, 96, 112, 128,
                               160, 192, 224, 256, 320, 384, 448, 512};
    static const int coarse[] = {16, 32, 48, 64, 96, 128, 192, 256, 384, 512};
    if (width >= 16) {
        for (int e : coarse)
            if (k <= e) return e;
    } else {
        for (int e : fine)
            if (k <= e) return e;
    }
    return kMaxK;
}

template <typename T>
cudaError_t launch_recompress(const Desc *d_desc, int n, T *ws, int *d_rank, int *d_status,
                              int *d_info, const LaunchShape &shape, cudaStream_t s,
                              unsigned phases) {
    if (n <= 0) return cudaSuccess;
    const int maxM = shape.maxM;
    if (shape.maxK > kMaxK || maxM > 32 * kMaxRowsPerLane) return cudaErrorInvalidValue;
    const int rpl = (maxM + 31) / 32;
    const bool mixed = shape.mixed && sizeof(T) == sizeof(double);
    if (phases & kPhaseStack) {
        if (mixed) {
            stack_kernel<T, float><<<n, kThreads, 0, s>>>(d_desc, ws, false);
        } else {
            const bool tcs = sizeof(T) == sizeof(double) && shape.tc_stack;
            stack_kernel<T, T><<<n, kThreads, 0, s>>>(d_desc, ws, tcs);
            if (tcs) launch_stack_tc(d_desc, n, (double *)ws, d_status, s);
        }
    }
    if (phases & kPhaseQR) {
        const int qw = shape.qr_warps;
        if (sizeof(T) == sizeof(double) && shape.tc_qr && shape.nbuckets > 0) {
            qr_plan(shape, n, [&](int kind, int start, int count, int p, int cls) {
                if (count <= 0) return;
                if (kind == 2)
                    launch_qr_update_tc(d_desc + start, count, (double *)ws, p, d_status, cls, s);
                else
                    launch_geqrf_all<T>(d_desc + start, count, ws, qw, rpl, p, s);
            });
        } else {
            launch_geqrf_all<T>(d_desc, n, ws, qw, rpl, -1, s);
        }
    }
    if (phases & kPhaseSVD) {
        // buckets run concurrently (largest k first) when the plan provides
        // side streams; otherwise back to back on s
        const bool forked = shape.fork != nullptr && shape.nbuckets > 1;
        if (forked) cudaEventRecord(shape.fork, s);
        for (int b = 0; b < shape.nbuckets; ++b) {
            const Bucket &bk = shape.buckets[b];
            if (bk.count <= 0) continue;
            const int K = bk.K;
            // both Jacobi matrices in shared memory, only R^T there (V_J in
            // the workspace), or both in the workspace
            const int mode = K <= shape.svd_smem_kmax ? 1 : (K <= shape.svd_half_kmax ? 2 : 0);
            cudaStream_t sb = forked ? shape.side[b] : s;
            if (forked) cudaStreamWaitEvent(sb, shape.fork, 0);
            const int G = svd_group(K, mode == 1, shape.svd_lanes);
            const int nt = svd_threads(K, mode == 1, shape.svd_lanes);
            if (mode == 1)
                gesvd_kernel<T, 1><<<bk.count, nt, svd_smem_bytes<T>(K, 2), sb>>>(
                    d_desc + bk.start, ws, d_rank, d_status, d_info, K, G);
            else if (mode == 2)
                gesvd_kernel<T, 2><<<bk.count, nt, svd_smem_bytes<T>(K, 1), sb>>>(
                    d_desc + bk.start, ws, d_rank, d_status, d_info, K, G);
            else
                gesvd_kernel<T, 0><<<bk.count, nt, svd_smem_bytes<T>(K, 0), sb>>>(
                    d_desc + bk.start, ws, d_rank, d_status, d_info, K, G);
            if (forked) {
                cudaEventRecord(shape.join[b], sb);
                cudaStreamWaitEvent(s, shape.join[b], 0);
            }
        }
    }
    if (phases & kPhaseApply) {
        const int ncols = shape.maxR > 0 ? std::min(shape.maxR, shape.maxK) : shape.maxK;
        if (mixed) {
            launch_apply_all<T, float>(d_desc, n, ws, d_rank, d_status, ncols, rpl, s);
        } else if (sizeof(T) == sizeof(double) && shape.tc_rebuild && shape.nbuckets > 0) {
            // descriptors are sorted by decreasing k: the buckets above
            // kTcMaxK take the DFMA kernel, the rest one tensor-core launch
            // per padded-k class
            int b = 0;
            while (b < shape.nbuckets) {
                const int cls = tc_rebuild_class(shape.buckets[b].K);
                const int start = shape.buckets[b].start;
                int count = 0;
                while (b < shape.nbuckets && tc_rebuild_class(shape.buckets[b].K) == cls)
                    count += shape.buckets[b++].count;
                if (count <= 0) continue;
                if (cls == 0)
                    launch_apply_all<T, T>(d_desc + start, count, ws, d_rank, d_status, ncols,
                                           rpl, s);
                else
                    launch_rebuild_tc(d_desc + start, count, (const double *)ws, d_rank,
                                      d_status, cls, s);
            }
        } else {
            launch_apply_all<T, T>(d_desc, n, ws, d_rank, d_status, ncols, rpl, s);
        }
    }
    return cudaGetLastError();
}

int rebuild_launches(const LaunchShape &shape, bool fp64) {
    if (!fp64 || shape.mixed || !shape.tc_rebuild || shape.nbuckets <= 0) return 1;
    int launches = 0, b = 0;
    while (b < shape.nbuckets) {
        const int cls = tc_rebuild_class(shape.buckets[b].K);
        int count = 0;
        while (b < shape.nbuckets && tc_rebuild_class(shape.buckets[b].K) == cls)
            count += shape.buckets[b++].count;
        launches += count > 0;
    }
    return launches;
}

// Rebuild of updates that ended with HCORE_GPU_S_STORAGE: their U_r and
// V_r S_r are still in the workspace, so only the rebuild phase runs again,
// over descriptors that point at the new output storage.
// cap[q] > 0 keeps the leading cap[q] singular triplets only (the fixed-rank
// truncation of HCORE_dgemm's rk argument, applied after the fact).
__global__ void storage_to_ok_kernel(const int *__restrict__ idx, const int *__restrict__ cap,
                                     int n, int *__restrict__ status, int *__restrict__ rank) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n || status[idx[q]] != HCORE_GPU_S_STORAGE) return;
    status[idx[q]] = HCORE_GPU_S_OK;
    if (cap && cap[q] > 0 && rank[idx[q]] > cap[q]) rank[idx[q]] = cap[q];
}

template <typename T>
cudaError_t launch_rebuild(const Desc *d_desc, const int *d_idx, const int *d_cap, int n, T *ws,
                           int *d_rank, int *d_status, int maxM, int maxK, bool mixed,
                           bool tc_rebuild, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (maxK > kMaxK || maxM > 32 * kMaxRowsPerLane) return cudaErrorInvalidValue;
    storage_to_ok_kernel<<<(n + 255) / 256, 256, 0, s>>>(d_idx, d_cap, n, d_status, d_rank);
    const int rpl = (maxM + 31) / 32;
    if (mixed && sizeof(T) == sizeof(double))
        launch_apply_all<T, float>(d_desc, n, ws, d_rank, d_status, maxK, rpl, s);
    else if (sizeof(T) == sizeof(double) && tc_rebuild && tc_rebuild_class(maxK) > 0)
        launch_rebuild_tc(d_desc, n, (const double *)ws, d_rank, d_status,
                          tc_rebuild_class(maxK), s);
    else
        launch_apply_all<T, T>(d_desc, n, ws, d_rank, d_status, maxK, rpl, s);
    return cudaGetLastError();
}
template cudaError_t launch_rebuild<double>(const Desc *, const int *, const int *, int, double *,
                                            int *, int *, int, int, bool, bool, cudaStream_t);
template cudaError_t launch_rebuild<float>(const Desc *, const int *, const int *, int, float *,
                                           int *, int *, int, int, bool, bool, cudaStream_t);

template cudaError_t configure_recompress<double>(int, int *, int *);
template cudaError_t configure_recompress<float>(int, int *, int *);
template cudaError_t launch_recompress<double>(const Desc *, int, double *, int *, int *, int *,
                                               const LaunchShape &, cudaStream_t, unsigned);
template cudaError_t launch_recompress<float>(const Desc *, int, float *, int *, int *, int *,
                                              const LaunchShape &, cudaStream_t, unsigned);

}  // namespace hc
