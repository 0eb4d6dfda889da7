// hcore-gb300 internal definitions shared by the kernels and the host API.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hcore_gb300.h"

namespace hc {

// Per-update descriptor as the kernels see it (device resident, one per task).
// All pointers are device-accessible (device memory, or pinned host memory
// through its device alias).  Offsets are in elements of the plan's scalar.
struct Desc {
    const void *AU, *AV, *BU, *BV, *Bd, *CU, *CV;
    void *CUo, *CVo;
    long long ws;        // start of this update's workspace
    double alpha, beta, acc;
    int lda, ldb, ldc, ldco;
    int M, a, b, c, k;
    int rk;              // fixed output rank (0: by acc)
    int max_rank;        // largest accepted new rank (reference: maxrk)
    int storage_rank;    // second limit (split API storage_maxrank), INT_MAX if none
    int rank_start;      // rank search starts here (1, or 2 for the fast rules)
    int status0;         // non-zero: rejected on the host, skip
    int idx;             // task index (rank/status slots)
    int rule;            // rank rule bits (kRule*): 0 for HCORE_dgemm's rule
};
// rank rule bits of a descriptor: cap the rank at max_rank instead of
// reporting RANK_MAX; compare with acc * sigma_max instead of acc
constexpr int kRuleCapRank = 1, kRuleRelative = 2;

// Workspace layout of one update (element offsets from Desc::ws), k = a + c:
//   UA  M*k   stacked [beta CU | alpha AU], then its QR (R on top, reflectors below)
//   VB  M*k   stacked [CV | G], then its QR
//   tauA k, tauB k, sig k
//   F   a*b   AV^T BV
//   W   k*k   Jacobi working matrix (used when it does not fit shared memory)
//   V   k*k   Jacobi right vectors (same)
//   Uo  k*k   U_r (k x r, ld k); the SVD's QR reflectors until U_r is written
//   Vo  k*k   V_r S_r (k x r, ld k)
// U_r and V_r S_r are kept for an update whose rank exceeds its storage
// limit too, so that it can be rebuilt into larger storage without being
// recompressed (hcore_gpu_plan_rebuild).
struct WsLayout {
    long long UA, VB, tauA, tauB, sig, F, W, V, Uo, Vo, total;
};

__host__ __device__ inline long long hc_align32(long long x) { return (x + 31) & ~31LL; }

__host__ __device__ inline WsLayout ws_layout(int M, int a, int b, int k) {
    const long long u = k;
    WsLayout L;
    long long o = 0;
    L.UA = o; o = hc_align32(o + (long long)M * k);
    L.VB = o; o = hc_align32(o + (long long)M * k);
    L.tauA = o; o = hc_align32(o + k);
    L.tauB = o; o = hc_align32(o + k);
    L.sig = o; o = hc_align32(o + k);
    L.F = o; o = hc_align32(o + (long long)a * b);
    L.W = o; o = hc_align32(o + (long long)k * k);
    L.V = o; o = hc_align32(o + (long long)k * k);
    L.Uo = o; o = hc_align32(o + (long long)k * u);
    L.Vo = o; o = hc_align32(o + (long long)k * u);
    L.total = o;
    return L;
}
__host__ __device__ inline WsLayout ws_layout(const Desc &d) {
    return ws_layout(d.M, d.a, d.b, d.k);
}

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxSweeps = 40;
constexpr int kMaxRowsPerLane = 64;  // apply kernel keeps a column in registers: M <= 2048

constexpr unsigned kPhaseStack = 1u, kPhaseQR = 2u, kPhaseSVD = 4u, kPhaseApply = 8u;
constexpr unsigned kPhaseAll = 15u;
constexpr int kMaxK = 512;  // largest a + c a plan accepts

// Rank buckets: the descriptors of a plan are sorted by decreasing k and the
// SVD phase is launched once per bucket of similar k, each launch sized (CTA
// width, shared memory) for its own largest k.
constexpr int kMaxBuckets = 24;
struct Bucket {
    int start, count, K;
};
struct LaunchShape {
    int maxM = 1, maxK = 1, svd_smem_kmax = 0;
    // largest k whose R^T alone fits shared memory (the SVD's mode with V_J
    // in the workspace); 0: that mode is not used
    int svd_half_kmax = 0;
    // most output columns an accepted update may have, max of
    // min(k, storage_rank): the rebuild's grid (0: maxK)
    int maxR = 0;
    // tuning: lanes per column pair of shared-memory SVD buckets with <= 24,
    // <= 64 and more pairs; rank-bucket edge spacing
    int svd_lanes[3] = {2, 2, 2};
    int bucket_width = 8;
    int qr_warps = 4;   // warps per QR CTA (2, 4 or 8)
    bool mixed = false;  // FP32 factor products and rebuild (HCORE_GPU_MIXED_FACTORS)
    // FP64 plans: the rebuild of updates with k <= kTcMaxK on the tensor cores
    // (hc_rebuild_tc.cu); off: the DFMA reflector kernel for every update
    bool tc_rebuild = true;
    // FP64 plans: the QR of updates with k <= kTcMaxK blocked, with the
    // trailing updates on the tensor cores; off: the unblocked FP64 kernel
    bool tc_qr = true;
    // FP64 plans, opt-in (HCORE_GPU_TC_STACK): the stack's products F and G on
    // the tensor cores for updates that stack_tc_eligible accepts
    bool tc_stack = false;
    int nbuckets = 0;
    Bucket buckets[kMaxBuckets];
    // optional fork/join resources so the bucket launches overlap: one stream
    // per bucket, a fork event and one join event per bucket (plan-owned)
    cudaStream_t side[kMaxBuckets] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kMaxBuckets] = {};
};
// smallest bucket edge >= k (edges every `width` up to 64, then coarser)
int bucket_edge(int k, int width);

// launchers (hc_kernels.cu).  configure_recompress sets kernel attributes
// (not capturable) and returns the largest k whose Jacobi matrices fit in
// shared memory; launch_recompress only launches (capturable).
template <typename T>
cudaError_t configure_recompress(int maxK, int *svd_smem_kmax, int *svd_half_kmax = nullptr);
template <typename T>
cudaError_t launch_recompress(const Desc *d_desc, int n, T *ws, int *d_rank, int *d_status,
                              int *d_info, const LaunchShape &shape, cudaStream_t s,
                              unsigned phases);
// rebuild phase only, for listed updates whose status is STORAGE (set to
// OK; d_cap, if not null, caps their rank)
template <typename T>
cudaError_t launch_rebuild(const Desc *d_desc, const int *d_idx, const int *d_cap, int n, T *ws,
                           int *d_rank, int *d_status, int maxM, int maxK, bool mixed,
                           bool tc_rebuild, cudaStream_t s);

// tensor-core rebuild (hc_rebuild_tc.cu): FP64-accurate Q.U products for
// updates with k <= kTcMaxK.  tc_rebuild_class(k) is the kernel variant
// (padded k: 16, 32, 48 or 64; 0 above kTcMaxK); configure_rebuild_tc sets
// the variants' shared-memory attributes (not capturable).
constexpr int kTcMaxK = 64;
// kernel launches of the rebuild phase of one execute (hc_kernels.cu)
int rebuild_launches(const LaunchShape &shape, bool fp64);

// Blocked QR (FP64 plans, a + c <= kTcMaxK): 16-column panels factored by the
// FP64 register kernel, the last panel taking the rest when it is at most 20
// columns wide (on the TLR panel workload the QR phase took 10.7, 10.1, 9.85
// and 10.1 ms with limits 32, 24, 20 and 16); between panels the trailing
// columns are updated on the tensor cores (hc_qr_tc.cu).  Returns false when
// panel p does not exist.
__host__ __device__ inline bool qr_panel_bounds(int k, int p, int &c0, int &c1) {
    const int q = k > 20 ? (k - 20 + 15) / 16 : 0;   // full panels before the last
    if (p < 0 || p > q) return false;
    c0 = 16 * p;
    c1 = p < q ? c0 + 16 : k;
    return true;
}
constexpr int kQrPanels = 4;  // panels of the widest blocked QR (k = 64)
// tensor-core trailing update: variant by 16 + (columns right of the panel)
// rounded up (32, 48 or 64; 0 above 64); launches only
int qr_update_class(int rows);
cudaError_t configure_qr_tc();
void launch_qr_update_tc(const Desc *d_desc, int n, double *ws, int panel, int *d_status,
                         int rclass, cudaStream_t s);
// kernel launches of the QR phase of one execute (hc_kernels.cu)
int qr_launches(const LaunchShape &shape, bool fp64);

// Stack phase products on the tensor cores (hc_stack_tc.cu): F = AV^T BV and
// G = BU F^T of updates with a low-rank B, 1 <= a <= 64 and 1 <= b <= 32; the
// stack kernel then only copies the stacked factors of those updates.
constexpr int kStackTcMaxA = 64, kStackTcMaxB = 32;
__host__ __device__ inline bool stack_tc_eligible(const Desc &d) {
    return !d.status0 && !d.Bd && d.a >= 1 && d.a <= kStackTcMaxA && d.b >= 1 &&
           d.b <= kStackTcMaxB;
}
cudaError_t configure_stack_tc();
void launch_stack_tc(const Desc *d_desc, int n, double *ws, int *d_status, cudaStream_t s);
int tc_rebuild_class(int k);
cudaError_t configure_rebuild_tc();
void launch_rebuild_tc(const Desc *d_desc, int n, const double *ws, const int *d_rank,
                       int *d_status, int kclass, cudaStream_t s);

// dense-C updates (hc_dense.cu): per-task rank-K' form coef * P Q^T
struct DenseWork {
    const double *P;  // M x K' (ldp): computed into the workspace, or an input factor
    const double *Q;  // N x K' (ldq)
    int ldp, ldq, kk;
    double coef;      // CD = beta CD + coef P Q^T
    double beta;
    int syrk;         // 1: zero the strict upper triangle after this task
    long long ws;     // workspace offset (doubles): S (p x q), then the computed factor
};
cudaError_t launch_dense_prep(const hcore_dense_task *d_tasks, const DenseWork *d_work, int n,
                              double *ws, cudaStream_t s);
// Q = Bd^T Av (N x a) of the gemmbdcd tasks listed in d_idx
cudaError_t launch_bdcd_prep(const hcore_dense_task *d_tasks, const DenseWork *d_work,
                             const int *d_idx, int n_idx, int maxN, int maxA, double *ws,
                             cudaStream_t s);
cudaError_t launch_dense_tiles(const hcore_dense_task *d_tasks, const DenseWork *d_work,
                               const int *d_group_start, const int *d_group_tasks, int ngroups,
                               int maxDim, cudaStream_t s);
template <typename T>
cudaError_t launch_gemm_dense(int ta, int tb, int M, int N, int K, T alpha, const T *A, int lda,
                              const T *B, int ldb, T beta, T *C, int ldc, cudaStream_t s);

}  // namespace hc
