// hcore-gb300: the blocked Householder QR's trailing update on the tensor
// cores, FP64-accurate.
//
// Reference step: the two dgeqrf calls of the recompression,
// src/compute/hcore_dgemm.c:123-124 (QR of [beta CU | alpha AU]) and :216-217
// (QR of [CV | G]).  The QR phase factors 16-column panels with the FP64
// register kernel (geqrf_kernel with a panel index; the last panel takes up
// to 20 columns) and, between panels, applies the panel's reflectors
// H_c0 ... H_c1-1 to the columns on its right:
//
//     A_t <- Q_p^T A_t = A_t - Y_p W',   W' = T_p^T (Y_p^T A_t),
//
// where (diag(1/tau) + strict lower part of Y_p^T Y_p) W' = Y_p^T A_t, i.e.
// w'_j = tau_j (w_j - sum_{i<j} (y_j^T y_i) w'_i) for j = 0..15: the same
// sequence as applying the reflectors one after the other (the compact WY
// form of Schreiber and Van Loan 1989).  The two products with a long
// dimension, [Y_p | A_t]^T Y_p (inner dimension M) and Y_p W' (M x n_t,
// inner dimension 16), run as exact digit products on the tensor cores
// (hc_digits.cuh); the FP64 pipe does the 16-row forward substitution and one
// subtraction per updated entry.
//
// One CTA (8 warps) per (update, side) and panel.  Scales: Householder
// vectors take 2^1 (|y| <= 1), each trailing column of A_t and each column of
// W' its own power of two.
#include "hc_digits.cuh"
#include "hc_internal.h"

namespace hc {
namespace {
using namespace dg;

constexpr int kQWorkers = 256;              // warps 0-7: slicing, drains, FP64 work
constexpr int kQThreads = kQWorkers + 32;   // warp 8: issues the MMAs
constexpr int kQTmemCols = 256;
// combine shifts S (T = value 2^(110 - E_x - E_y - S)): Gram pass rows
// |y_j^T y_l| <= 2 and |y_l^T a_c| <= sqrt(2 M) 2^E_c <= 2^6 2^E_c (M <=
// 2048), so T <= 2^61 with S = 54; output |(Y_p W')_rc| <= 16 2^(1 + E_c), so
// T <= 2^61 with S = 53.
constexpr int kShiftW = 54;
constexpr int kShiftU = 53;

// Shared memory of the RP variant (RP = 16 + n_t rounded up to 16):
//   R0: two buffers of seven digit slices of [Y_p | A_t]^T (RP rows x 64
//       rows of A each; a slice is read as a 128-row operand, so the space
//       after the second buffer covers 16 row groups past its last slice);
//       after the Gram pass: two buffers of the output pass's seven slices
//       of a 128-row tile of Y_p (128 x 16), the digit slices of W'^T and
//       the FP64 matrices G_p (16 x 16), W (16 x n_t), W'
//   RB: two buffers of the seven digit slices of Y_p^T (16 rows x 64) and a
//       zero slice
// While the MMAs of one chunk run, the threads slice the next chunk into the
// other buffer; the Gram's accumulators (8 planes x 16 columns) are double
// buffered in tensor memory too, so a chunk's drain overlaps the next
// chunk's MMAs.
template <int RP>
struct QrCfg {
    static constexpr int kSliceA = (RP / 8) * 1024;
    static constexpr int kBufA = 7 * kSliceA;
    static constexpr int kSliceB = 2 * 1024;
    static constexpr int kBufB = 8 * kSliceB;
    static constexpr int kRB = 2 * kBufB;
    static constexpr int kMisc = 2048;
    // output pass layout inside R0
    static constexpr int kOutA = 0;                    // 2 buffers x 7 x 4096
    static constexpr int kOutB = 2 * 7 * 4096;         // 8 slices x (32 rows x 32 B), per group
    static constexpr int kG = kOutB + 8 * 32 * 32;     // G_p, 16 x 16 doubles
    static constexpr int kW = kG + 16 * 16 * 8;        // W, 16 x 48 doubles
    static constexpr int kWp = kW + 16 * 48 * 8;       // W', 16 x 48 doubles
    static constexpr int kOutEnd = kWp + 16 * 48 * 8;
    static constexpr int kGramEnd = 13 * kSliceA + 16 * 1024;
    static constexpr int kR0 = kGramEnd > kOutEnd ? kGramEnd : kOutEnd;
    // at least 113 KB with 256 tensor-memory columns (the library's rule, see
    // the rebuild kernel): CTAs on one SM never hold more than 512 columns
    static constexpr int kSmem =
        (kR0 + kRB + kMisc) > 113 * 1024 ? (kR0 + kRB + kMisc) : 113 * 1024;
};

// entry (i, l) of the panel's reflector block Y_p (column c0 + l of A):
// unit diagonal at row c0 + l, zero above it
__device__ __forceinline__ double ypanel(const double *A, int M, int c0, int i, int l) {
    const int j = c0 + l;
    if (i >= M || i < j) return 0.0;
    return i == j ? 1.0 : A[(size_t)j * M + i];
}

// registers capped so that FP64 QR panel CTAs of other stream groups still
// fit beside it on the SM
template <int RP>
__global__ void __maxnreg__(128)
    qr_update_tc_kernel(const Desc *__restrict__ descs, double *__restrict__ ws, int panel,
                        int *__restrict__ status) {
    using C = QrCfg<RP>;
    constexpr int kItems = RP / 16;
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *R0 = sm, *RB = sm + C::kR0, *misc = sm + C::kR0 + C::kRB;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(misc);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(misc + 8);
    int *colE = reinterpret_cast<int *>(misc + 16);       // 48 trailing-column scales
    int *wE = colE + 48;                                  // 48 column scales of W'
    double *s_tau = reinterpret_cast<double *>(misc + 16 + 4 * 96);  // 16

    const Desc d = descs[blockIdx.x];
    if (d.status0) return;
    const int M = d.M, k = d.k;
    int c0, c1;
    if (!qr_panel_bounds(k, panel, c0, c1) || c1 >= k) return;
    const int nt = k - c1;                      // 5 .. 48 trailing columns
    const int side = blockIdx.y;
    const WsLayout L = ws_layout(d);
    double *A = ws + d.ws + (side ? L.VB : L.UA);
    const double *tau = ws + d.ws + (side ? L.tauB : L.tauA);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int lrow = tid & 127, wg = tid >> 7;
    const bool worker = tid < kQWorkers, issuer = tid == kQWorkers;

    if (warp == 0) tc::tmem_alloc(tslot, kQTmemCols);
    if (tid == 0) tc::mbar_init(mbar, 1);
    if (tid < 48) colE[tid] = 0;
    if (tid < 16) s_tau[tid] = tau[c0 + tid];
    for (int e = tid; e < C::kSliceB / 16; e += kQThreads) {
        reinterpret_cast<uint4 *>(RB + 7 * C::kSliceB)[e] = make_uint4(0, 0, 0, 0);
        reinterpret_cast<uint4 *>(RB + C::kBufB + 7 * C::kSliceB)[e] = make_uint4(0, 0, 0, 0);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot;
    const uint32_t lane_base = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
    const uint32_t r0 = tc::smem_u32(R0), rb = tc::smem_u32(RB);
    uint32_t phase = 0;
    bool failed = false;
    auto wait_mma = [&]() -> bool {
        const bool ok = tc::mbar_wait(mbar, phase, kTcWaitCycles);
        phase ^= 1u;
        return __syncthreads_and(ok) != 0;
    };

    // ---- 0. scale of each trailing column (its largest exponent) ------------
    {
        const int ngroups = (M + 7) / 8, total = nt * ngroups;
        for (int e0 = tid; e0 < total; e0 += 4 * kQThreads) {
            double v[4][8];   // four items' loads in flight before any is used
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int e = e0 + u * kQThreads;
                const int c = e % nt, i0 = (e / nt) * 8;
#pragma unroll
                for (int t = 0; t < 8; ++t)
                    v[u][t] = (e < total && i0 + t < M) ? A[(size_t)(c1 + c) * M + i0 + t] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int e = e0 + u * kQThreads;
                if (e < total) {
                    int ef = 0;
#pragma unroll
                    for (int t = 0; t < 8; ++t) ef = max(ef, exp_field(v[u][t]));
                    atomicMax(&colE[e % nt], ef);
                }
            }
        }
        __syncthreads();
        if (tid < nt) colE[tid] -= 1022;
        __syncthreads();
    }

    // ---- 1. [Y_p | A_t]^T Y_p, 64 rows of A per pass, double buffered -------
    // Item it of a chunk: operand row jr = (it >> 6) * 8 + (it & 7) (a
    // reflector c0 + jr for jr < 16, else trailing column c1 + jr - 16), the
    // eight A rows ((it >> 3) & 7) * 8 .. + 7 of the chunk.
    long long accW[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) accW[e] = 0;
    {
        constexpr int kIt = RP * 8, kMaxIt = (kIt + kQWorkers - 1) / kQWorkers;
        const int nchunks = (M + 63) / 64;
        double pre[kMaxIt][8];
        auto value = [&](int i, int jr) -> double {
            if (jr < 16) return ypanel(A, M, c0, i, jr);
            const int c = jr - 16;
            return (c < nt && i < M) ? A[(size_t)(c1 + c) * M + i] : 0.0;
        };
        auto load_chunk = [&](int ch) {
            if (!worker) return;
#pragma unroll
            for (int q = 0; q < kMaxIt; ++q) {
                const int it = tid + q * kQWorkers;
                if (it < kIt) {
                    const int jr = (it >> 6) * 8 + (it & 7), i0 = ch * 64 + ((it >> 3) & 7) * 8;
#pragma unroll
                    for (int t = 0; t < 8; ++t) pre[q][t] = value(i0 + t, jr);
                }
            }
        };
        auto slice_chunk = [&](int buf) {
            if (!worker) return;
#pragma unroll
            for (int q = 0; q < kMaxIt; ++q) {
                const int it = tid + q * kQWorkers;
                if (it < kIt) {
                    const int jj = it & 7, g = (it >> 3) & 7, jb = it >> 6, jr = jb * 8 + jj;
                    const int off = jb * 1024 + g * 128 + jj * 16;
                    unsigned char *dst = R0 + buf * C::kBufA + off;
                    if (jr < 16)   // the reflector rows are the B operand too
                        slice8(pre[q], 1, dst, C::kSliceA, RB + buf * C::kBufB + off, C::kSliceB);
                    else if (jr - 16 < nt)
                        slice8(pre[q], colE[jr - 16], dst, C::kSliceA);
                    else
                        zero8(dst, C::kSliceA);
                }
            }
        };
        auto issue_chunk = [&](int buf) {
            issue_planes(tbase + buf * 128, mbar, r0 + buf * C::kBufA, C::kSliceA, 1024,
                         rb + buf * C::kBufB, C::kSliceB, 1024, 4, 16);
        };
        load_chunk(0);
        slice_chunk(0);
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (issuer) issue_chunk(0);
        if (nchunks > 1) load_chunk(1);
        for (int ch = 0; ch < nchunks; ++ch) {
            const int cur = ch & 1;
            // slice chunk ch + 1 while the MMAs of chunk ch run (its buffer's
            // last reader, chunk ch - 1, is done)
            if (ch + 1 < nchunks) {
                slice_chunk(cur ^ 1);
                tc::fence_async_smem();
            }
            if (!wait_mma()) {   // chunk ch done; every thread's slicing and last drain too
                failed = true;
                break;
            }
            tc::fence_after_sync();
            if (issuer && ch + 1 < nchunks) issue_chunk(cur ^ 1);
            if (ch + 2 < nchunks) load_chunk(ch + 2);
            if (worker) combine_planes<kShiftW>(accW, lane_base + cur * 128 + wg * 8, 16);
            tc::fence_before_sync();
        }
        __syncthreads();
    }

    // ---- 2. G_p, W, and W' by forward substitution (FP64) --------------------
    double *Gs = reinterpret_cast<double *>(R0 + C::kG);   // (j, l) at j + 16 l
    double *Wm = reinterpret_cast<double *>(R0 + C::kW);   // (l, c) at l + 16 c
    double *Wp = reinterpret_cast<double *>(R0 + C::kWp);  // W', same layout
    if (!failed) {
        if (worker && lrow < 16 + nt) {
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int l = wg * 8 + e;
                if (lrow < 16) {
                    Gs[lrow + 16 * l] = scale2((double)accW[e], kShiftW - 108);
                } else {
                    const int c = lrow - 16;
                    Wm[l + 16 * c] = scale2((double)accW[e], kShiftW + 1 + colE[c] - 110);
                }
            }
        }
        __syncthreads();
        if (tid < nt) {
            const int c = tid;
            int ef = 0;
            for (int j = 0; j < 16; ++j) {
                double w = Wm[j + 16 * c];
                for (int i = 0; i < j; ++i) w -= Gs[j + 16 * i] * Wp[i + 16 * c];
                w *= s_tau[j];
                Wp[j + 16 * c] = w;
                ef = max(ef, exp_field(w));
            }
            wE[c] = ef - 1022;
        }
        __syncthreads();
    }

    // ---- 3. A_t -= Y_p W', 128 rows per tile, at most 32 columns per pass ----
    if (!failed) {
        const int ntp = (nt + 15) & ~15;
        const int tile0 = c0 / 128, ntiles = (M + 127) / 128;
        for (int cg = 0; cg < ntp && !failed; cg += 32) {
            const int gw = min(32, ntp - cg);
            // digit slices of W'^T for columns cg .. cg + gw - 1 (B: row c, K = l)
            for (int it = tid; it < gw * 2; it += kQThreads) {
                const int cc = it >> 1, lb = it & 1, c = cg + cc;
                double x[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) x[t] = c < nt ? Wp[lb * 8 + t + 16 * c] : 0.0;
                slice8(x, c < nt ? wE[c] : 0,
                       R0 + C::kOutB + (cc >> 3) * 256 + lb * 128 + (cc & 7) * 16, gw * 32);
            }
            for (int e = tid; e < gw * 2; e += kQThreads)
                reinterpret_cast<uint4 *>(R0 + C::kOutB + 7 * gw * 32)[e] = make_uint4(0, 0, 0, 0);
            double pre[8];
            double old[2][8];   // the entries this thread updates, loaded before the wait
            const int jh = tid >> 7;
            auto load_tile = [&](int tile) {
                if (!worker) return;
                const int row = tile * 128 + lrow;
#pragma unroll
                for (int t = 0; t < 8; ++t) pre[t] = ypanel(A, M, c0, row, jh * 8 + t);
            };
            auto load_old = [&](int tile) {
                if (!worker) return;
                const int row = tile * 128 + lrow;
#pragma unroll
                for (int m = 0; m < 2; ++m)
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const int c = cg + (wg + 2 * m) * 8 + e;
                        old[m][e] = (c < nt && row < M && row >= c0)
                                        ? A[(size_t)(c1 + c) * M + row] : 0.0;
                    }
            };
            auto slice_tile = [&](int buf) {
                if (!worker) return;
                slice8(pre, 1,
                       R0 + C::kOutA + buf * 7 * 4096 + (lrow >> 3) * 256 + jh * 128 +
                           (lrow & 7) * 16,
                       4096);
            };
            auto issue_tile = [&](int buf) {
                issue_planes(tbase, mbar, r0 + C::kOutA + buf * 7 * 4096, 4096, 256,
                             r0 + C::kOutB, gw * 32, 256, 1, gw);
            };
            load_tile(tile0);
            slice_tile(0);
            tc::fence_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (issuer) issue_tile(0);
            if (tile0 + 1 < ntiles) load_tile(tile0 + 1);
            for (int tile = tile0; tile < ntiles; ++tile) {
                const int cur = (tile - tile0) & 1;
                const int row = tile * 128 + lrow;
                load_old(tile);
                // slice the next tile while this tile's MMAs run
                if (tile + 1 < ntiles) {
                    slice_tile(cur ^ 1);
                    tc::fence_async_smem();
                }
                if (!wait_mma()) {
                    failed = true;
                    break;
                }
                tc::fence_after_sync();
                if (worker) {
#pragma unroll
                    for (int m = 0; m < 2; ++m) {
                        const int cb = wg + 2 * m;  // 8-column block of this pass
                        if (cb * 8 >= gw) continue;
                        long long a8[8];
#pragma unroll
                        for (int e = 0; e < 8; ++e) a8[e] = 0;
                        combine_planes<kShiftU>(a8, lane_base + cb * 8, gw);
                        if (row < M && row >= c0) {
#pragma unroll
                            for (int e = 0; e < 8; ++e) {
                                const int c = cg + cb * 8 + e;
                                if (c < nt) {
                                    const int p = kShiftU + 1 + wE[c] - 110;
                                    bool ok;
                                    double v = i64_times_pow2(-a8[e], p, ok);
                                    if (!ok) v = scale2((double)(-a8[e]), p);
                                    A[(size_t)(c1 + c) * M + row] = old[m][e] + v;
                                }
                            }
                        }
                    }
                }
                tc::fence_before_sync();
                __syncthreads();   // the accumulators are read before the next tile's MMAs
                tc::fence_after_sync();
                if (issuer && tile + 1 < ntiles) issue_tile(cur ^ 1);
                if (tile + 2 < ntiles) load_tile(tile + 2);
            }
        }
    }

    if (failed) {
        if (tid == 0) status[d.idx] = HCORE_GPU_S_TIMEOUT;
        tc::mbar_wait(mbar, phase ^ 1u, kTcWaitCycles);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, kQTmemCols);
}

template <int RP>
cudaError_t set_qr_smem() {
    return cudaFuncSetAttribute(qr_update_tc_kernel<RP>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, QrCfg<RP>::kSmem);
}

}  // namespace

int qr_update_class(int rows) {
    if (rows <= 32) return 32;
    if (rows <= 48) return 48;
    if (rows <= 64) return 64;
    return 0;
}

cudaError_t configure_qr_tc() {
    cudaError_t e = set_qr_smem<32>();
    if (e == cudaSuccess) e = set_qr_smem<48>();
    if (e == cudaSuccess) e = set_qr_smem<64>();
    return e;
}

void launch_qr_update_tc(const Desc *d_desc, int n, double *ws, int panel, int *d_status,
                         int rclass, cudaStream_t s) {
    if (n <= 0) return;
    const dim3 grid(n, 2);
    if (rclass == 32)
        qr_update_tc_kernel<32><<<grid, kQThreads, QrCfg<32>::kSmem, s>>>(d_desc, ws, panel,
                                                                         d_status);
    else if (rclass == 48)
        qr_update_tc_kernel<48><<<grid, kQThreads, QrCfg<48>::kSmem, s>>>(d_desc, ws, panel,
                                                                         d_status);
    else
        qr_update_tc_kernel<64><<<grid, kQThreads, QrCfg<64>::kSmem, s>>>(d_desc, ws, panel,
                                                                         d_status);
}

}  // namespace hc
