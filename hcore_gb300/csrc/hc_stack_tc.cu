// hcore-gb300: the stack phase's factor products on the tensor cores,
// FP64-accurate.
//
// Reference steps: src/compute/hcore_dgemm.c:175-178 (F = AV^T BV, a x b) and
// :199-205 (G = BU F^T, M x a, the second half of VB = [CV | G]).  The stack
// kernel (hc_kernels.cu) still copies [beta CU | alpha AU] and CV; for
// updates with 1 <= a <= 64, 1 <= b <= 32 and a low-rank B it leaves F and G
// to this kernel, which forms them as exact digit products (hc_digits.cuh):
//   F: inner dimension M, 64-row chunks; each chunk's eight planes are
//      combined exactly in 64-bit integers and added to an FP64 sum, since
//      a general inner product has no small bound (|F_pq| <= M 2^(E_p + E_q)).
//   G: inner dimension b, 128-row tiles of BU, in passes of at most 32 of
//      F's rows; written once into the workspace.
// Scales: each column of AV and BV, each row of BU and each row of F takes
// its own power of two.
//
// One CTA (8 warps) per update.
#include "hc_digits.cuh"
#include "hc_internal.h"

namespace hc {
namespace {
using namespace dg;

constexpr int kSThreads = 256;
constexpr int kSTmemCols = 256;
constexpr int kAP = 64;   // rows of the F pass's A operand (a <= 64)
constexpr int kBP = 32;   // rows of its B operand, and K of the G pass (b <= 32)
// combine shifts: F chunk |sum| <= 64 2^(E_p + E_q), so T <= 2^61 with S = 55;
// G |sum| <= 32 2^(E_r + E_p), so T <= 2^61 with S = 54
constexpr int kShiftF = 55;
constexpr int kShiftG = 54;

// shared memory (bytes)
constexpr int kSliceFA = (kAP / 8) * 1024;        // AV^T chunk: 64 rows x 64
constexpr int kR0 = 6 * kSliceFA + 16 * 1024;     // last slice read as 128 rows
constexpr int kSliceFB = (kBP / 8) * 1024;        // BV^T chunk: 32 rows x 64
constexpr int kRB = 8 * kSliceFB;                 // seven slices and a zero slice
constexpr int kSliceGA = 16 * (kBP / 8) * 128;    // BU tile: 128 rows x 32
constexpr int kRF = kAP * kBP * 8;                // F, FP64 (p + 64 q)
constexpr int kMisc = 2048;
constexpr int kSmem = kR0 + kRB + kRF + kMisc;    // >= 113 KB (256 columns)
static_assert(kSmem >= 113 * 1024, "tensor-memory rule: 256 columns need 113 KB");
static_assert(7 * kSliceGA <= kR0, "G pass A slices fit in R0");

static_assert(kAP == kStackTcMaxA && kBP == kStackTcMaxB, "limits shared with the stack kernel");

__global__ void __maxnreg__(128) stack_tc_kernel(const Desc *__restrict__ descs,
                                                 double *__restrict__ ws,
                                                 int *__restrict__ status) {
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *R0 = sm, *RB = sm + kR0;
    double *Fs = reinterpret_cast<double *>(sm + kR0 + kRB);
    unsigned char *misc = sm + kR0 + kRB + kRF;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(misc);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(misc + 8);
    int *eA = reinterpret_cast<int *>(misc + 16);   // 64 column scales of AV
    int *eB = eA + kAP;                             // 32 column scales of BV
    int *eF = eB + kBP;                             // 64 row scales of F

    const Desc d = descs[blockIdx.x];
    if (!stack_tc_eligible(d)) return;
    const int M = d.M, a = d.a, b = d.b, c = d.c;
    const WsLayout L = ws_layout(d);
    double *F = ws + d.ws + L.F;
    double *G = ws + d.ws + L.VB + (size_t)c * M;
    const double *AV = (const double *)d.AV, *BV = (const double *)d.BV;
    const double *BU = (const double *)d.BU;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int lrow = tid & 127, wg = tid >> 7;

    if (warp == 0) tc::tmem_alloc(tslot, kSTmemCols);
    if (tid == 0) tc::mbar_init(mbar, 1);
    if (tid < kAP + kBP) eA[tid] = 0;   // eA and eB are contiguous
    for (int e = tid; e < kSliceFB / 16; e += kSThreads)
        reinterpret_cast<uint4 *>(RB + 7 * kSliceFB)[e] = make_uint4(0, 0, 0, 0);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot;
    const uint32_t lane_base = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
    const uint32_t r0 = tc::smem_u32(R0), rb = tc::smem_u32(RB);
    uint32_t phase = 0;
    bool failed = false, timed_out = false;
    auto wait_mma = [&]() -> bool {
        const bool ok = tc::mbar_wait(mbar, phase, kTcWaitCycles);
        phase ^= 1u;
        return __syncthreads_and(ok) != 0;
    };

    // ---- 0. column scales of AV and BV ---------------------------------------
    {
        const int ngroups = (M + 7) / 8;
        for (int e = tid; e < (a + b) * ngroups; e += kSThreads) {
            const int col = e % (a + b), i0 = (e / (a + b)) * 8;
            const double *x = col < a ? AV + (size_t)col * d.lda : BV + (size_t)(col - a) * d.ldb;
            int ef = 0;
            for (int t = 0; t < 8 && i0 + t < M; ++t) ef = max(ef, exp_field(x[i0 + t]));
            atomicMax(col < a ? &eA[col] : &eB[col - a], ef);
        }
        __syncthreads();
        // a NaN or infinity in AV or BV (exponent field 2047): F and G become
        // NaN, as the FP64 products would make them, so that the SVD reports
        // the update as not converged
        bool nonfinite = tid < a ? eA[tid] == 2047 : (tid >= kAP && tid < kAP + b && eB[tid - kAP] == 2047);
        nonfinite = __syncthreads_or(nonfinite) != 0;
        if (nonfinite) {
            const double qnan = __longlong_as_double(0x7FF8000000000000LL);
            for (int e = tid; e < a * b; e += kSThreads) F[e] = qnan;
            for (long long e = tid; e < (long long)a * M; e += kSThreads) G[e] = qnan;
            failed = true;   // skip the products
        }
        if (tid < kAP + kBP) eA[tid] -= 1022;
        __syncthreads();
    }

    // ---- 1. F = AV^T BV, 64 rows per pass --------------------------------------
    // Item (operand row r, 8-row group g of the chunk): r < 64 a column of AV,
    // 64 <= r < 96 a column of BV.  The drain adds each chunk's combined sum
    // to FP64 accumulators: lane = row p of F, 8-column blocks of q.
    double accF[2][8];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int e = 0; e < 8; ++e) accF[m][e] = 0.0;
    {
        const int nchunks = (M + 63) / 64;
        for (int ch = 0; ch < nchunks && !failed; ++ch) {
            for (int it = tid; it < (kAP + kBP) * 8; it += kSThreads) {
                const int r = it >> 3, g = it & 7;
                const int i0 = ch * 64 + g * 8;
                double x[8];
                if (r < kAP) {
                    unsigned char *dst = R0 + (r >> 3) * 1024 + g * 128 + (r & 7) * 16;
                    if (r < a) {
#pragma unroll
                        for (int t = 0; t < 8; ++t)
                            x[t] = i0 + t < M ? AV[(size_t)r * d.lda + i0 + t] : 0.0;
                        slice8(x, eA[r], dst, kSliceFA);
                    } else {
                        zero8(dst, kSliceFA);
                    }
                } else {
                    const int q = r - kAP;
                    unsigned char *dst = RB + (q >> 3) * 1024 + g * 128 + (q & 7) * 16;
                    if (q < b) {
#pragma unroll
                        for (int t = 0; t < 8; ++t)
                            x[t] = i0 + t < M ? BV[(size_t)q * d.ldb + i0 + t] : 0.0;
                        slice8(x, eB[q], dst, kSliceFB);
                    } else {
                        zero8(dst, kSliceFB);
                    }
                }
            }
            tc::fence_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (tid == 0)
                issue_planes(tbase, mbar, r0, kSliceFA, 1024, rb, kSliceFB, 1024, 4, kBP);
            if (!wait_mma()) {
                failed = timed_out = true;
                break;
            }
            tc::fence_after_sync();
            if (lrow < kAP) {   // lanes 64..127 hold padding rows (warps 2, 3, 6, 7)
#pragma unroll
                for (int m = 0; m < 2; ++m) {
                    long long t8[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) t8[e] = 0;
                    combine_planes<kShiftF>(t8, lane_base + (wg + 2 * m) * 8, kBP);
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const int q = (wg + 2 * m) * 8 + e;
                        if (lrow < a && q < b)
                            accF[m][e] += scale2((double)t8[e], kShiftF - 110 + eA[lrow] + eB[q]);
                    }
                }
            }
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
        }
    }

    // ---- 2. F to the workspace and shared memory, row scales of F -------------
    if (!failed) {
        if (lrow < a) {
#pragma unroll
            for (int m = 0; m < 2; ++m)
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int q = (wg + 2 * m) * 8 + e;
                    if (q < b) {
                        Fs[lrow + kAP * q] = accF[m][e];
                        F[(size_t)q * a + lrow] = accF[m][e];
                    }
                }
        }
        __syncthreads();
        if (tid < a) {
            int ef = 0;
            for (int q = 0; q < b; ++q) ef = max(ef, exp_field(Fs[tid + kAP * q]));
            eF[tid] = ef - 1022;
        }
        __syncthreads();
    }

    // ---- 3. G = BU F^T, 128 rows per tile, at most 32 of F's rows per pass ----
    if (!failed) {
        const int ap = (a + 15) & ~15;
        const int ntiles = (M + 127) / 128;
        const int row_l = lrow;   // tile row of this thread (both warp groups)
        for (int pg = 0; pg < ap && !failed; pg += 32) {
            const int gw = min(32, ap - pg);
            // digit slices of F's rows pg .. pg + gw - 1 (B: row p, K = q), in RB
            for (int it = tid; it < gw * (kBP / 8); it += kSThreads) {
                const int pp = it / (kBP / 8), qb = it % (kBP / 8), p = pg + pp;
                double x[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const int q = qb * 8 + t;
                    x[t] = (p < a && q < b) ? Fs[p + kAP * q] : 0.0;
                }
                slice8(x, p < a ? eF[p] : 0, RB + (pp >> 3) * (kBP / 8 * 128) + qb * 128 +
                                                  (pp & 7) * 16,
                       gw * kBP * 2);
            }
            for (int e = tid; e < gw * kBP * 2 / 16; e += kSThreads)
                reinterpret_cast<uint4 *>(RB + 7 * gw * kBP * 2)[e] = make_uint4(0, 0, 0, 0);
            for (int tile = 0; tile < ntiles; ++tile) {
                const int row = tile * 128 + row_l;
                // one row of BU per thread pair: warp group wg slices q block wg .. of the row
                int ef = 0;
                for (int q = 0; q < b; ++q)
                    if (row < M) ef = max(ef, exp_field(BU[(size_t)q * d.ldb + row]));
                const int Er = ef - 1022;
#pragma unroll
                for (int m = 0; m < kBP / 16; ++m) {
                    const int qb = wg + 2 * m;
                    unsigned char *dst =
                        R0 + (row_l >> 3) * (kBP / 8 * 128) + qb * 128 + (row_l & 7) * 16;
                    if (qb * 8 < b) {
                        double x[8];
#pragma unroll
                        for (int t = 0; t < 8; ++t) {
                            const int q = qb * 8 + t;
                            x[t] = (row < M && q < b) ? BU[(size_t)q * d.ldb + row] : 0.0;
                        }
                        slice8(x, Er, dst, kSliceGA);
                    } else {
                        zero8(dst, kSliceGA);
                    }
                }
                tc::fence_async_smem();
                tc::fence_before_sync();
                __syncthreads();
                tc::fence_after_sync();
                if (tid == 0)
                    issue_planes(tbase, mbar, r0, kSliceGA, kBP / 8 * 128, rb, gw * kBP * 2,
                                 kBP / 8 * 128, kBP / 16, gw);
                if (!wait_mma()) {
                    failed = timed_out = true;
                    break;
                }
                tc::fence_after_sync();
#pragma unroll
                for (int m = 0; m < 2; ++m) {
                    const int cb = wg + 2 * m;
                    if (cb * 8 >= gw) continue;
                    long long t8[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) t8[e] = 0;
                    combine_planes<kShiftG>(t8, lane_base + cb * 8, gw);
                    if (row < M) {
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            const int p = pg + cb * 8 + e;
                            if (p < a) {
                                const int pw = kShiftG + Er + eF[p] - 110;
                                bool ok;
                                double v = i64_times_pow2(t8[e], pw, ok);
                                if (!ok) v = scale2((double)t8[e], pw);
                                G[(size_t)p * M + row] = v;
                            }
                        }
                    }
                }
                tc::fence_before_sync();
                __syncthreads();
                tc::fence_after_sync();
            }
        }
    }

    if (timed_out) {
        if (tid == 0) status[d.idx] = HCORE_GPU_S_TIMEOUT;
        tc::mbar_wait(mbar, phase ^ 1u, kTcWaitCycles);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, kSTmemCols);
}

}  // namespace

cudaError_t configure_stack_tc() {
    return cudaFuncSetAttribute(stack_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                kSmem);
}

void launch_stack_tc(const Desc *d_desc, int n, double *ws, int *d_status, cudaStream_t s) {
    if (n <= 0) return;
    stack_tc_kernel<<<n, kSThreads, kSmem, s>>>(d_desc, ws, d_status);
}

}  // namespace hc
