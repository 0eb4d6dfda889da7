// hcore-gb300: the rebuild phase (CU = Q_A [U_r; 0], CV = Q_B [V_r S_r; 0])
// on the tensor cores, FP64-accurate.
//
// Reference step: src/compute/hcore_dgemm.c:508-696 (__newu / __newv: dormqr
// 'L','N' of the k Householder reflectors from dgeqrf onto the k x r core
// factor).  The DFMA kernel (apply_kernel in hc_kernels.cu) applies the
// reflectors one by one, 2 M k r FP64 FMAs per side.  Here the same product is
// formed through the compact WY representation Q = I - Y T Y^T (Schreiber and
// Van Loan 1989) as
//
//     Q X = X - Y Z,   z_j = tau_j (y_j^T X - sum_{i>j} (y_j^T y_i) z_i)
//
// (j = k-1 .. 0; X = [X0; 0]), so that the two products with a long dimension,
// the Gram matrix Y^T Y (inner dimension M) and Y Z (M x r, inner dimension
// k), run on the tensor cores, and only O(k^2 r) FP64 work stays on the FP64
// pipe.
//
// FP64 accuracy on bf16 tensor cores: the error-free splitting of Ozaki,
// Ogita, Oishi and Rump (2012), in the fixed-point form of Mukunoki, Ozaki,
// Ogita and Imamura (2020).  Every value x of a row (or column) with common
// scale 2^E becomes the integer X = round(x 2^(55-E)), |X| < 2^55, written as
// seven balanced base-256 digits a_0..a_6 in [-128, 128]; each digit is exact
// in bf16.  A product of two digits is at most 2^14, so a sum of up to 1024
// of them is an integer below 2^24 and the tensor core's FP32 accumulator
// holds it exactly (checked on this GPU up to 1.6e7).  The digit products of
// equal weight d = i + l accumulate in one tensor-memory accumulator per d.
// Planes d = 0..7 are kept (34 slice pairs): the dropped terms (d >= 8) are
// below 2^-61 of the largest product.  Dropping d = 7 as well would leave a
// systematic error of ~1e-14 in the Gram matrix (measured in a CPU
// emulation); with it, the rebuilt factors agree with an extended-precision
// reflector application to about 1e-15, as close as the FP64 path.  Each
// accumulator is read back with tcgen05.ld and the eight are combined exactly
// in 64-bit integers, then converted to FP64 once.
//
// One CTA (8 warps) per (update, side).  Shared-memory operands use the
// K-major, no-swizzle core-matrix layout of hc_tc.cuh.
#include <algorithm>
#include <mutex>

#include "hc_digits.cuh"
#include "hc_internal.h"

namespace hc {
namespace {
using namespace dg;

constexpr int kTcThreads = 256;

constexpr int cmax(int a, int b) { return a > b ? a : b; }
constexpr int pow2_at_least(int x) {
    int p = 32;
    while (p < x) p *= 2;
    return p;
}

// Shared-memory plan of the KP variant (KP: padded k, a multiple of 16).
//   R0: the Gram's seven digit slices (KP rows x 128 rows of Y each; the
//       last is read as a 128-row operand, so 16 row groups past its start
//       stay inside R0), later the FP64 matrices G, Y_top, X0 / Z (KP x KP
//       each), later the seven slices of a 128-row tile of Y (128 x KP).
//       The eighth Gram slice position (inside R0) holds zeros.
//   R1: the seven digit slices of Z^T (r rounded up to 16 rows x KP each,
//       consecutive), then a zero slice.
template <int KP>
struct TcCfg {
    static constexpr int kSliceG = (KP / 8) * 2048;
    static constexpr int kR0G = 6 * kSliceG + 16 * 2048;
    static constexpr int kSliceA = 256 * KP;
    static constexpr int kR0A = 7 * kSliceA;
    static constexpr int kR0D = 3 * 8 * KP * KP;
    static constexpr int kR0 = cmax(cmax(kR0G, kR0A), kR0D);
    static constexpr int kSliceB = 2 * KP * KP;  // largest Z slice (r <= KP rows)
    static constexpr int kR1 = 8 * kSliceB;       // seven slices and a zero one
    static constexpr int kMisc = 2048;
    static constexpr int kTmemCols = pow2_at_least(kPlanes * KP);
    // Tensor-memory budget by shared memory: every tensor-core CTA of this
    // library takes at least 175 KB with 512 columns, 113 KB with 256 and
    // 62 KB with 128, so the CTAs that fit on one SM (228 KB) never hold more
    // than 512 columns together and no allocation waits for another CTA's.
    static constexpr int kSmem =
        cmax(kR0 + kR1 + kMisc,
             kTmemCols == 512 ? 175 * 1024 : kTmemCols == 256 ? 113 * 1024 : 62 * 1024);
};

// Y(i, j) of the reflector block: unit diagonal, zero above it
__device__ __forceinline__ double yelem(const double *Y, int M, int k, int i, int j) {
    if (j >= k || i >= M || i < j) return 0.0;
    return i == j ? 1.0 : Y[(size_t)j * M + i];
}

// Combine shifts S: the combined sum is T = value 2^(110 - E_x - E_y - S).
// Gram: |y_j^T y_l| <= ||y_j|| ||y_l|| <= 2 (a Householder vector has
// ||v||^2 = 2 / tau <= 2), for any partial sum over rows too, and E = 1, so
// T <= 2^(109 - S) = 2^61 with S = 48; its last place is 2^-60.  Output:
// |(Y Z)_rc| <= k 2^(E_r + E_c) with k <= 64, so T <= 2^61 with S = 55.
constexpr int kShiftGram = 48;
constexpr int kShiftOut = 55;

// Eight warps per CTA: the two warp groups (warps 0-3 and 4-7) see the same
// 128 tensor-memory lanes and split the accumulator column blocks between
// them.  Every |y| of a Householder block is at most 1 (dlarfg), so Y takes
// the one scale 2^1 in both products; the output's error is then absolute,
// 2^-55 |Z| per term, as a normwise-stable reflector application's is.
template <int KP>
__device__ __forceinline__ void rebuild_tc_body(const Desc *__restrict__ descs,
                                                const double *__restrict__ ws,
                                                const int *__restrict__ rank,
                                                int *__restrict__ status) {
    using C = TcCfg<KP>;
    constexpr int kItems = KP / 16;            // 8-value slicing items per thread
    constexpr int kBlk = KP / 16;              // 8-column accumulator blocks per warp group
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *R0 = sm, *R1 = sm + C::kR0, *misc = sm + C::kR0 + C::kR1;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(misc);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(misc + 8);
    int *zE = reinterpret_cast<int *>(misc + 16);              // KP column scales of Z
    double *s_tau = reinterpret_cast<double *>(misc + 16 + 4 * KP);

    const Desc d = descs[blockIdx.x];
    if (d.status0 || status[d.idx] != HCORE_GPU_S_OK) return;
    const int r = rank[d.idx];
    if (r <= 0) return;
    const int side = blockIdx.y;
    const int M = d.M, k = d.k;
    const WsLayout L = ws_layout(d);
    const double *Y = ws + d.ws + (side ? L.VB : L.UA);
    const double *tau = ws + d.ws + (side ? L.tauB : L.tauA);
    const double *X0 = ws + d.ws + (side ? L.Vo : L.Uo);
    double *out = (double *)(side ? d.CVo : d.CUo);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int lrow = tid & 127;                // tensor-memory lane of this thread
    const int wg = tid >> 7;                   // warp group
    const int rp = (r + 15) & ~15;
    const int zslice = 2 * rp * KP;            // bytes of one digit slice of Z^T

    if (warp == 0) tc::tmem_alloc(tslot, C::kTmemCols);
    if (tid == 0) tc::mbar_init(mbar, 1);
    if (tid < KP) s_tau[tid] = tid < k ? tau[tid] : 0.0;
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot;
    const uint32_t lane_base = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
    const uint32_t r0 = tc::smem_u32(R0), r1 = tc::smem_u32(R1);
    uint32_t phase = 0;
    bool failed = false;

    // wait for the MMAs committed last; uniform across the CTA
    auto wait_mma = [&]() -> bool {
        const bool ok = tc::mbar_wait(mbar, phase, kTcWaitCycles);
        phase ^= 1u;
        return __syncthreads_and(ok) != 0;
    };
    auto issue = [&](uint32_t a0, int a_stride, uint32_t a_sbo, uint32_t b0, int b_stride,
                     uint32_t b_sbo, int ksteps, int pstride) {
        issue_planes(tbase, mbar, a0, a_stride, a_sbo, b0, b_stride, b_sbo, ksteps, pstride);
    };

    // ---- 1. Gram G = Y^T Y, 128 rows of Y per pass ---------------------------
    // Item q of a thread: column j = (jh + 2 q) * 8 + jj, rows g*8 .. g*8+7 of
    // the chunk; the next chunk's values are loaded while the MMAs run.
    long long accG[kBlk][8];
#pragma unroll
    for (int m = 0; m < kBlk; ++m)
#pragma unroll
        for (int e = 0; e < 8; ++e) accG[m][e] = 0;
    {
        const int jj = tid & 7, g = (tid >> 3) & 15, jh = tid >> 7;
        const int nchunks = (M + 127) / 128;
        double pre[kItems][8];
        auto load_chunk = [&](int ch) {
            const int i0 = ch * 128 + g * 8;
#pragma unroll
            for (int q = 0; q < kItems; ++q)
#pragma unroll
                for (int t = 0; t < 8; ++t) pre[q][t] = yelem(Y, M, k, i0 + t, (jh + 2 * q) * 8 + jj);
        };
        load_chunk(0);
        // the eighth Gram slice: zeros (the B run of plane 7 with i = 0 ends there)
        for (int e = tid; e < C::kSliceG / 16; e += kTcThreads)
            reinterpret_cast<uint4 *>(R0 + 7 * C::kSliceG)[e] = make_uint4(0, 0, 0, 0);
        for (int ch = 0; ch < nchunks; ++ch) {
#pragma unroll
            for (int q = 0; q < kItems; ++q) {
                unsigned char *dst = R0 + (jh + 2 * q) * 2048 + g * 128 + jj * 16;
                if ((jh + 2 * q) * 8 + jj < k) slice8(pre[q], 1, dst, C::kSliceG);
                else zero8(dst, C::kSliceG);   // padding column of Y
            }
            tc::fence_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (tid == 0)
                issue(r0, C::kSliceG, 2048, r0, C::kSliceG, 2048, 8, KP);
            if (ch + 1 < nchunks) load_chunk(ch + 1);
            if (!wait_mma()) {
                failed = true;
                break;
            }
            tc::fence_after_sync();
#pragma unroll
            for (int m = 0; m < kBlk; ++m)
                combine_planes<kShiftGram>(accG[m], lane_base + (wg + 2 * m) * 8, KP);
            tc::fence_before_sync();
            __syncthreads();  // slices and accumulators are free again
            tc::fence_after_sync();
        }
    }

    // ---- 2. Z (FP64, shared memory) -----------------------------------------
    double *Gs = reinterpret_cast<double *>(R0);  // KP x KP, column-major
    double *Yt = Gs + KP * KP;                    // top k x k block of Y
    double *Xs = Yt + KP * KP;                    // X0, then Z
    if (!failed) {
        // G = T 2^(S - 110 + 1 + 1)
        if (lrow < k) {
            const double f = __longlong_as_double((long long)(kShiftGram - 108 + 1023) << 52);
            static_assert(kShiftGram - 108 >= -1022, "normal scale factor");
#pragma unroll
            for (int m = 0; m < kBlk; ++m) {
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int c = (wg + 2 * m) * 8 + e;
                    if (c < k) Gs[lrow + c * KP] = (double)accG[m][e] * f;
                }
            }
        }
        for (int e = tid; e < k * k; e += kTcThreads) {
            const int i = e % k, j = e / k;
            Yt[i + j * KP] = yelem(Y, M, k, i, j);
        }
        for (int e = tid; e < k * r; e += kTcThreads) {
            const int i = e % k, c = e / k;
            Xs[i + c * KP] = X0[(size_t)c * k + i];
        }
        __syncthreads();
        // W = Y_top^T X0, kept in registers until every thread has read X0
        double wv[(KP * KP + kTcThreads - 1) / kTcThreads];
        int nw = 0;
        for (int e = tid; e < k * r; e += kTcThreads, ++nw) {
            const int j = e % k, c = e / k;
            double w0 = Xs[j + c * KP], w1 = 0.0;
            int i = j + 1;
            for (; i + 1 < k; i += 2) {
                w0 += Yt[i + j * KP] * Xs[i + c * KP];
                w1 += Yt[i + 1 + j * KP] * Xs[i + 1 + c * KP];
            }
            if (i < k) w0 += Yt[i + j * KP] * Xs[i + c * KP];
            wv[nw] = w0 + w1;
        }
        __syncthreads();
        double *Ws = Yt;  // Y_top is no longer read: it holds w', Xs receives z
        nw = 0;
        for (int e = tid; e < k * r; e += kTcThreads, ++nw) {
            const int j = e % k, c = e / k;
            Ws[j + c * KP] = wv[nw];
        }
        __syncthreads();
        // Back substitution (diag(1/tau) + strict upper part of G) Z = W:
        // z_j = tau_j (w_j - sum_{i>j} G_ji z_i), in blocks of 8 rows from the
        // bottom.  A block's rows are solved one column per thread, then one
        // pass takes the block's z out of every row above it.
        for (int b1 = k; b1 > 0; b1 -= 8) {
            const int b0 = max(0, b1 - 8);
            if (tid < r) {
                const int c = tid;
                for (int j = b1 - 1; j >= b0; --j) {
                    double w = Ws[j + c * KP];
                    for (int i = j + 1; i < b1; ++i) w -= Gs[j + i * KP] * Xs[i + c * KP];
                    Xs[j + c * KP] = s_tau[j] * w;
                }
            }
            __syncthreads();
            for (int e = tid; e < b0 * r; e += kTcThreads) {
                const int i = e % b0, c = e / b0;
                double w = Ws[i + c * KP];
                for (int j = b0; j < b1; ++j) w -= Gs[i + j * KP] * Xs[j + c * KP];
                Ws[i + c * KP] = w;
            }
            __syncthreads();
        }
        // column scales of Z, then its digit slices (B operand: row c, K = j)
        if (tid < r) {
            int ef = 0;
            for (int j = 0; j < k; ++j) ef = max(ef, exp_field(Xs[j + tid * KP]));
            zE[tid] = ef - 1022;
        }
        __syncthreads();
        for (int it = tid; it < rp * (KP / 8); it += kTcThreads) {
            const int cc = it & 7, rest = it >> 3;
            const int jb = rest % (KP / 8), cb = rest / (KP / 8);
            const int c = cb * 8 + cc;
            double x[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int j = jb * 8 + t;
                x[t] = (c < r && j < k) ? Xs[j + c * KP] : 0.0;
            }
            slice8(x, c < r ? zE[c] : 0, R1 + cb * (16 * KP) + jb * 128 + cc * 16, zslice);
        }
        for (int e = tid; e < zslice / 16; e += kTcThreads)
            reinterpret_cast<uint4 *>(R1 + 7 * zslice)[e] = make_uint4(0, 0, 0, 0);
        __syncthreads();
    }

    // ---- 3. out = X - Y Z, 128 rows per tile ----------------------------------
    if (!failed) {
        const int jh = tid >> 7;
        const int ntiles = (M + 127) / 128;
        double pre[kItems][8];
        auto load_tile = [&](int tile) {
            const int row = tile * 128 + lrow;
#pragma unroll
            for (int q = 0; q < kItems; ++q)
#pragma unroll
                for (int t = 0; t < 8; ++t) pre[q][t] = yelem(Y, M, k, row, (jh + 2 * q) * 8 + t);
        };
        load_tile(0);
        for (int tile = 0; tile < ntiles; ++tile) {
            const int row = tile * 128 + lrow;
#pragma unroll
            for (int q = 0; q < kItems; ++q) {
                unsigned char *dst =
                    R0 + (lrow >> 3) * (16 * KP) + (jh + 2 * q) * 128 + (lrow & 7) * 16;
                if ((jh + 2 * q) * 8 < k) slice8(pre[q], 1, dst, C::kSliceA);
                else zero8(dst, C::kSliceA);   // padding columns of Y
            }
            tc::fence_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (tid == 0)
                issue(r0, C::kSliceA, 16 * KP, r1, zslice, 16 * KP, KP / 16, rp);
            if (tile + 1 < ntiles) load_tile(tile + 1);
            if (!wait_mma()) {
                failed = true;
                break;
            }
            tc::fence_after_sync();
#pragma unroll
            for (int m = 0; m < kBlk; ++m) {
                const int cb = wg + 2 * m;  // 8-column block
                if (cb * 8 >= rp) continue;
                long long a8[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) a8[e] = 0;
                combine_planes<kShiftOut>(a8, lane_base + cb * 8, rp);
                if (row < M) {
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const int c = cb * 8 + e;
                        if (c < r) {
                            // rows below k: out = -(Y Z) exactly; above: X0 - (Y Z)
                            const int p = 1 + zE[c] - kShiftOut;
                            bool ok;
                            double v = i64_times_pow2(row < k ? a8[e] : -a8[e], p, ok);
                            if (!ok) v = scale2((double)(row < k ? a8[e] : -a8[e]), p);
                            if (row < k) v = X0[(size_t)c * k + row] - v;
                            out[(size_t)c * d.ldco + row] = v;
                        }
                    }
                }
            }
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
        }
    }

    if (failed) {
        // give up on this update; let MMAs still in flight finish before the
        // columns are released
        if (tid == 0) status[d.idx] = HCORE_GPU_S_TIMEOUT;
        tc::mbar_wait(mbar, phase ^ 1u, kTcWaitCycles);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, C::kTmemCols);
}

// Two CTAs per SM for KP <= 32 (128 registers a thread); one for the wider
// variants, whose registers are capped so that other kernels' CTAs (the QR and
// SVD of other stream groups) still fit beside it on the SM.
template <int KP>
__global__ void __launch_bounds__(kTcThreads, 2)
    rebuild_tc_kernel(const Desc *__restrict__ descs, const double *__restrict__ ws,
                      const int *__restrict__ rank, int *__restrict__ status) {
    rebuild_tc_body<KP>(descs, ws, rank, status);
}
template <int KP>
__global__ void __maxnreg__(168)
    rebuild_tc_wide_kernel(const Desc *__restrict__ descs, const double *__restrict__ ws,
                           const int *__restrict__ rank, int *__restrict__ status) {
    rebuild_tc_body<KP>(descs, ws, rank, status);
}

template <int KP>
cudaError_t set_tc_smem() {
    if constexpr (KP <= 32)
        return cudaFuncSetAttribute(rebuild_tc_kernel<KP>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, TcCfg<KP>::kSmem);
    else
        return cudaFuncSetAttribute(rebuild_tc_wide_kernel<KP>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, TcCfg<KP>::kSmem);
}

}  // namespace

int tc_rebuild_class(int k) {
    if (k <= 16) return 16;
    if (k <= 32) return 32;
    if (k <= 48) return 48;
    if (k <= kTcMaxK) return 64;
    return 0;
}

cudaError_t configure_rebuild_tc() {
    cudaError_t e = set_tc_smem<16>();
    if (e == cudaSuccess) e = set_tc_smem<32>();
    if (e == cudaSuccess) e = set_tc_smem<48>();
    if (e == cudaSuccess) e = set_tc_smem<64>();
    return e;
}

void launch_rebuild_tc(const Desc *d_desc, int n, const double *ws, const int *d_rank,
                       int *d_status, int kclass, cudaStream_t s) {
    if (n <= 0) return;
    const dim3 grid(n, 2);
    switch (kclass) {
        case 16:
            rebuild_tc_kernel<16><<<grid, kTcThreads, TcCfg<16>::kSmem, s>>>(d_desc, ws, d_rank,
                                                                            d_status);
            break;
        case 32:
            rebuild_tc_kernel<32><<<grid, kTcThreads, TcCfg<32>::kSmem, s>>>(d_desc, ws, d_rank,
                                                                            d_status);
            break;
        case 48:
            rebuild_tc_wide_kernel<48><<<grid, kTcThreads, TcCfg<48>::kSmem, s>>>(
                d_desc, ws, d_rank, d_status);
            break;
        default:
            rebuild_tc_wide_kernel<64><<<grid, kTcThreads, TcCfg<64>::kSmem, s>>>(
                d_desc, ws, d_rank, d_status);
            break;
    }
}

}  // namespace hc
