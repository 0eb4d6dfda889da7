/*
 * hcore-gb300 — batched GPU API (new; the reference has no batched entry
 * point, every HCORE_* call there recompresses one tile on one CPU thread).
 *
 * A batch is a list of independent low-rank updates
 *     C_i <- beta_i * C_i + alpha_i * A_i * B_i^T
 * (the Schur updates of a TLR Cholesky panel, for instance), each with the
 * semantics of HCORE_dgemm (src/compute/hcore_dgemm.c:703-1012): stack,
 * Householder QR of both stacked factors, SVD of R_A R_B^T, truncation with the
 * absolute threshold acc (first i >= min_rank_start with sigma_i < acc), and
 * rebuild CU = Q_A U_r, CV = Q_B V_r S_r.  In FP64 the SVD drops the part of
 * R_A R_B^T below delta = min(1e-13 acc, 1e-16 ||R_A R_B^T||_F) after its
 * pivoted QR: every singular value moves by at most delta, so a rank differs
 * from the full SVD's only for a singular value within 1e-13 of acc,
 * relative, and the dropped singular values are reported as 0.
 *
 * Pointers in a task may be device memory or pinned (page-locked) host
 * memory; both are read and written directly by the kernels.  Outputs may
 * alias inputs (a task's own C, updated in place as in the reference, or
 * another task's inputs): the results are those of reading every input of
 * the batch before writing any output.
 *
 * Usage without a GPU-side rank array in the caller's hands:
 *     hcore_gpu_dgemm_batched(n, tasks, ranks, status, stream)   (synchronous)
 * Capturable form (no host work, no allocation inside execute):
 *     hcore_gpu_plan_create(&p, HCORE_GPU_F64, n, tasks, flags);
 *     hcore_gpu_plan_execute(p, stream);      // may be captured in a graph
 *     hcore_gpu_plan_results(p, ranks, status, stream);
 *     hcore_gpu_plan_destroy(p);
 *
 * Return values: 0 on success, a negative HCORE_GPU_E* code otherwise (the
 * message is available from hcore_gpu_last_error()).  Per-task outcomes are
 * reported in the status array (HCORE_GPU_S*).
 */
#ifndef HCORE_GB300_H
#define HCORE_GB300_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

/* precision of a plan */
#define HCORE_GPU_F64 0 /* HCORE_dgemm semantics, everything in FP64 */
#define HCORE_GPU_F32 1 /* HCORE_sgemm semantics, everything in FP32 */

/* return codes */
#define HCORE_GPU_OK 0
#define HCORE_GPU_EINVAL (-1)   /* bad argument (see hcore_gpu_last_error) */
#define HCORE_GPU_ECUDA (-2)    /* CUDA runtime error */
#define HCORE_GPU_ENOMEM (-3)   /* device allocation failed */
#define HCORE_GPU_ETASK (-4)    /* at least one task reported a non-zero status */

/* per-task status (what the reference would have exit(-1)-ed on) */
#define HCORE_GPU_S_OK 0
#define HCORE_GPU_S_ZERO_RANK 1 /* hcore_dgemm.c:743-746 */
#define HCORE_GPU_S_RANK_SUM 2  /* a + c > 2*maxrk, hcore_dgemm.c:91-95 */
#define HCORE_GPU_S_LDNEWV 3    /* a + c > ld_newV, hcore_dgemm.c:924-927 */
#define HCORE_GPU_S_RANK_MAX 4  /* new rank > maxrk, hcore_dgemm.c:465-468 */
#define HCORE_GPU_S_STORAGE 5   /* new rank > storage maxrank, :1648-1651 */
#define HCORE_GPU_S_NOCONV 6    /* Jacobi SVD did not converge, or a value was not finite */
#define HCORE_GPU_S_SHAPE 7     /* a + c > M */
#define HCORE_GPU_S_TIMEOUT 8   /* a tensor-core wait gave up; the update's output is not written */

/* flags of a plan */
#define HCORE_GPU_FAST_RULES 0x1 /* HCORE_dgemm_fast: rank search from i=2, no maxrk checks */
/* Host input factors that several updates read (a panel tile) or that are
 * pageable are merged into contiguous segments, mirrored on the device, and
 * refreshed by one copy per segment at the start of every execute, so they
 * cross the host link once.  A pinned host range that only one update reads
 * (its own C tile) is not copied: its stack kernel reads it in place,
 * overlapped with the other stream groups' work.  With pinned inputs,
 * execute stays capturable.  Outputs in pinned host memory are written in
 * place by the rebuild kernel. */
#define HCORE_GPU_STAGE_INPUTS 0x2
/* FP64 plans only: the factor products F = AV^T BV, G = BU F^T and the Q.U
 * rebuild run in FP32 with FP32 accumulation (FP64 storage), the QRs, the SVD
 * and the truncation stay FP64.  Meant for loose accuracies (1e-4 .. 1e-6);
 * the rebuild's FP32 rounding (~1e-7 relative) is far below such acc. */
#define HCORE_GPU_MIXED_FACTORS 0x4
/* FP64 plans run the rebuild (Q.U products) of updates with a + c <= 64 on
 * the tensor cores, FP64-accurate (exact bf16 digit products, see
 * hc_rebuild_tc.cu).  This flag keeps the FP64 (DFMA) reflector kernel for
 * every update instead. */
#define HCORE_GPU_DFMA_REBUILD 0x8
/* FP64 plans factor the stacked matrices of updates with a + c <= 64 as a
 * blocked Householder QR: 16-column panels in FP64, the trailing columns
 * updated between panels on the tensor cores, FP64-accurate (hc_qr_tc.cu).
 * This flag keeps the unblocked FP64 QR for every update instead. */
#define HCORE_GPU_UNBLOCKED_QR 0x10
/* FP64 plans: form the stack's products F = AV^T BV and G = BU F^T of updates
 * with a low-rank B, 1 <= a <= 64 and 1 <= b <= 32 on the tensor cores,
 * FP64-accurate (hc_stack_tc.cu), instead of in FP64.  Off by default: on the
 * TLR panel workload (a, b ~ 17) it measured slower than the FP64 products. */
#define HCORE_GPU_TC_STACK 0x20

/* One low-rank update.  Factors are column-major with the given leading
 * dimensions; every factor has M rows.  Ranks are plain ints. */
typedef struct hcore_lr_task {
    int M;
    int a, b, c;          /* ranks of A, B and C (c may be 0) */
    int rk;               /* fixed output rank (0: decided by acc) */
    int maxrk;            /* computational max rank: a + c <= 2*maxrk, new rank <= maxrk */
    int ld_newv;          /* reference's ld_newV rule: a + c must not exceed it (0: 2*maxrk) */
    int storage_maxrank;  /* new rank must not exceed it (0: no extra limit) */
    double alpha, beta, acc;
    const void *AU, *AV;
    int lda;
    const void *BU, *BV; /* BU == NULL and Bdense != NULL selects dense B */
    int ldb;
    const void *Bdense;  /* M x M dense B (HCORE_dgemm_qr_svd_b_dense form) or NULL */
    const void *CU, *CV;
    int ldc;
    void *CUo, *CVo;     /* outputs: the first r columns are written */
    int ldco;
} hcore_lr_task;

typedef struct hcore_gpu_plan_s *hcore_gpu_plan;

int hcore_gpu_plan_create(hcore_gpu_plan *plan, int precision, int n, const hcore_lr_task *tasks,
                          unsigned flags);
int hcore_gpu_plan_execute(hcore_gpu_plan plan, void *stream);
/* run only some of the four phases (bit 0 stack, 1 QR, 2 SVD, 3 rebuild),
 * in that order; for per-phase timing.  Phases read what earlier phases left
 * in the plan's workspace. */
#define HCORE_GPU_PHASE_STACK 0x1
#define HCORE_GPU_PHASE_QR 0x2
#define HCORE_GPU_PHASE_SVD 0x4
#define HCORE_GPU_PHASE_REBUILD 0x8
int hcore_gpu_plan_execute_phases(hcore_gpu_plan plan, void *stream, unsigned phases);
/* device array of the n new ranks / statuses (valid after execute completes) */
const int *hcore_gpu_plan_device_ranks(hcore_gpu_plan plan);
const int *hcore_gpu_plan_device_status(hcore_gpu_plan plan);
/* copy ranks and statuses to host arrays (either may be NULL) and wait */
int hcore_gpu_plan_results(hcore_gpu_plan plan, int *ranks, int *status, void *stream);
/* Rebuild tasks that ended with HCORE_GPU_S_STORAGE (new rank above their
 * storage_maxrank, e.g. a predicted capacity) into new output storage
 * without recompressing them: the rank, U_r and V_r S_r the last execute
 * found are still in the plan's workspace, so only the rebuild phase runs,
 * for these n tasks.  Task task_idx[q] is written to CUo[q]/CVo[q] (leading
 * dimension ldco[q], room for its new rank) and its status becomes
 * HCORE_GPU_S_OK.  With max_rank non-NULL, a task whose rank exceeds
 * max_rank[q] > 0 keeps its leading max_rank[q] singular triplets only (the
 * truncation HCORE_dgemm's fixed rank rk would have made; its reported rank
 * becomes max_rank[q]).  Tasks with another status are not written.  Call
 * after the execute that produced the statuses and before the next one; the
 * first call (or one with more tasks than any before) allocates. */
int hcore_gpu_plan_rebuild(hcore_gpu_plan plan, int n, const int *task_idx, void *const *CUo,
                           void *const *CVo, const int *ldco, const int *max_rank, void *stream);
/* copy the k singular values of task i (descending) to host (diagnostics;
 * in FP64 the values below the SVD's deflation bound are 0) */
int hcore_gpu_plan_sigma(hcore_gpu_plan plan, int i, double *sigma, int *k, void *stream);
/* Jacobi sweeps each task's SVD took (diagnostics; valid after execute) */
int hcore_gpu_plan_sweeps(hcore_gpu_plan plan, int *sweeps, void *stream);
/* kernel launches one execute makes (stack, QR, one SVD launch per rank
 * bucket, rebuild; per stream group) */
int hcore_gpu_plan_launches(hcore_gpu_plan plan);
/* bytes of device workspace the plan holds */
size_t hcore_gpu_plan_workspace_bytes(hcore_gpu_plan plan);
/* bytes copied host->device by every execute (HCORE_GPU_STAGE_INPUTS) */
size_t hcore_gpu_plan_staged_bytes(hcore_gpu_plan plan);
/* bytes of pinned host inputs that one update each reads in place over the
 * host link during every execute (HCORE_GPU_STAGE_INPUTS leaves them there) */
size_t hcore_gpu_plan_zero_copy_bytes(hcore_gpu_plan plan);
int hcore_gpu_plan_destroy(hcore_gpu_plan plan);

/* Launch-shape tuning of a plan (no counterpart in the reference).
 *   stream_groups      updates are dealt into this many concurrent groups
 *   svd_lanes[3]       lanes per column pair of the shared-memory SVD buckets
 *                      with <= 24, <= 64 and more column pairs (1..32, a
 *                      power of two; 0: as many as fit in the warps that one
 *                      lane per pair needs)
 *   bucket_width       rank-bucket edges every 8 (fine) or 16 (coarse)
 *   phase_sync         0: each group runs its four phases as soon as it can
 *                      (phases of different groups overlap); 1: every group
 *                      finishes a phase before any group starts the next
 *   qr_warps           warps per Householder-QR CTA: 8 (shortest path per
 *                      update), 4 or 2 (two or four times the CTAs per SM)
 * hcore_gpu_tuning_default fills the built-in choice (16 groups, 2 lanes per
 * pair, width 8, no phase sync, 4 QR warps: the autotuner's pick on a TLR
 * panel of 1953 updates; HCORE_GPU_STREAMS overrides the groups).  hcore_gpu_autotune
 * times plans of the given tasks over a search of these parameters
 * (coordinate descent; each candidate's execute captured in a CUDA graph on
 * a private stream and replayed `reps` times) and returns the fastest; the
 * tasks' outputs must not alias their inputs (the batch runs many times)
 * and are overwritten.  `stream` is not used (reserved).  Results do not
 * depend on the tuning beyond rounding (the SVD's reduction order follows
 * the lanes). */
typedef struct hcore_gpu_tuning {
    int stream_groups;
    int svd_lanes[3];
    int bucket_width;
    int phase_sync;
    int qr_warps;
} hcore_gpu_tuning;
int hcore_gpu_tuning_default(hcore_gpu_tuning *tuning);
int hcore_gpu_plan_create_tuned(hcore_gpu_plan *plan, int precision, int n,
                                const hcore_lr_task *tasks, unsigned flags,
                                const hcore_gpu_tuning *tuning);
int hcore_gpu_autotune(int precision, int n, const hcore_lr_task *tasks, unsigned flags, int reps,
                       void *stream, hcore_gpu_tuning *best, double *best_ms);

/* one-shot synchronous batch: create, execute, results, destroy */
int hcore_gpu_dgemm_batched(int n, const hcore_lr_task *tasks, int *ranks, int *status,
                            void *stream);
int hcore_gpu_sgemm_batched(int n, const hcore_lr_task *tasks, int *ranks, int *status,
                            void *stream);

/* Dense-C tile operations batched over output tiles.  Each task writes one
 * dense M x N tile CD (ld ldcd; N = 0 means N = M):
 *   kind 0 (syrk, HCORE_dsyrk):       CD += alpha * Au (Av^T Av) Au^T, strict
 *                                     upper set to 0 (N = M)
 *   kind 1 (gemmcd, HCORE_dgemmcd):   CD -= Au (Av^T Bv) Bu^T (N = M)
 *   kind 2 (uncompress, HCORE_duncompress): CD = Au Bv^T, Au M x a (lda),
 *                                     Bv N x a (ldb); alpha and beta unused
 *   kind 3 (gemmbdcd, HCORE_dgemmbdcd): CD = alpha Au (Av^T Bd) + beta CD,
 *                                     Au M x a (lda), Av kdim x a (lda),
 *                                     Bd kdim x N (ldb); kdim = 0 means M
 * Tasks that share a CD are applied in list order by one CTA group, so the
 * result is that of running them one after another. */
typedef struct hcore_dense_task {
    int kind;
    int M;
    int a, b;             /* ranks (b: gemmcd only) */
    double alpha;
    const double *Au, *Av;
    int lda;              /* leading dimension of Au/Av (syrk: also the row count of Av) */
    const double *Bu, *Bv;
    int ldb;              /* leading dimension of Bu/Bv, or of Bd */
    double *CD;
    int ldcd;
    int N;                /* columns of CD (0: M) */
    double beta;          /* gemmbdcd only */
    int kdim;             /* gemmbdcd: rows of Av and Bd (0: M) */
    const double *Bd;     /* gemmbdcd: dense B */
} hcore_dense_task;

int hcore_gpu_dense_batched(int n, const hcore_dense_task *tasks, void *stream);

/* The same as a plan: create validates, groups and uploads once; execute only
 * launches (capturable) and applies every task again to the current tiles. */
typedef struct hcore_gpu_dense_plan_s *hcore_gpu_dense_plan;
int hcore_gpu_dense_plan_create(hcore_gpu_dense_plan *plan, int n, const hcore_dense_task *tasks);
int hcore_gpu_dense_plan_execute(hcore_gpu_dense_plan plan, void *stream);
int hcore_gpu_dense_plan_destroy(hcore_gpu_dense_plan plan);

/* Triangular solves with many right-hand sides (HCORE_dtrsm semantics,
 * cblas_dtrsm column-major): B = alpha op(A)^-1 B (side HCORE_Left, A M x M)
 * or B = alpha B op(A)^-1 (HCORE_Right, A N x N), B M x N.  side, uplo,
 * trans and diag take the HCORE_/CBLAS enum values.  In a TLR Cholesky each
 * task is one V factor of a panel (Left, Lower, NoTrans, M = nb, N = its
 * rank) and all tasks share the diagonal tile's factor A.  Synchronous. */
typedef struct hcore_trsm_task {
    int side, uplo, trans, diag;
    int M, N;
    double alpha;
    const double *A;
    int lda;
    double *B;
    int ldb;
} hcore_trsm_task;
int hcore_gpu_trsm_batched(int n, const hcore_trsm_task *tasks, void *stream);

/* Cholesky factorization of dense tiles (HCORE_dpotrf semantics: LAPACK's
 * dpotrf through LAPACKE_dpotrf_work).  uplo is LAPACK's character, 'L'
 * (A = L L^T, lower triangle overwritten) or 'U' (A = U^T U, upper); the
 * other triangle is not touched.  info[i] (host array) receives
 * LAPACKE_dpotrf_work's value: 0, -2/-3/-5 for a bad uplo/n/lda, or j > 0
 * when the leading minor of order j is not positive definite (the failing
 * pivot is left in A(j-1, j-1), and the factorization stops there).
 * Synchronous. */
typedef struct hcore_potrf_task {
    int uplo;
    int n;
    double *A;
    int lda;
} hcore_potrf_task;
int hcore_gpu_potrf_batched(int n, const hcore_potrf_task *tasks, int *info, void *stream);

/* Tile compression (the reference's compressor semantics, generate_compress
 * in testing/testing_dgemm.c:119-236): a dense M x M tile D (ld ldd) becomes
 * U and V (M x r each, ld ldo) with D ~ U V^T, U the first r left singular
 * vectors, V = (S V^T)^T, r the number of leading singular values >= acc
 * (relative = 1: >= acc * sigma_max), capped at maxrank; r may be 0.  A
 * truncated pivoted QR finds the tile's range first, so ranks agree with a
 * full SVD's except for singular values within 1e-3 * threshold of it.
 * Status per tile: OK, NOCONV (non-finite input), RANK_MAX (the range needs
 * more than min(M, 512) columns).  M <= 2048.  Synchronous. */
typedef struct hcore_compress_task {
    int M;
    const double *D;
    int ldd;
    double acc;
    int relative;
    int maxrank;
    double *U, *V;
    int ldo;
} hcore_compress_task;
int hcore_gpu_compress_batched(int n, const hcore_compress_task *tasks, int *ranks, int *status,
                               void *stream);

/* A tile low-rank (TLR) symmetric matrix, lower triangle, as HiCMA holds it
 * for its Cholesky: nt x nt tiles of order nb, dense diagonal tiles D[i]
 * (column-major, ld ldd) and low-rank tiles A_ij = U_ij V_ij^T for i > j,
 * whose factors (nb x maxrank storage each, ld nb) are U[i + j*nt] and
 * V[i + j*nt] with rank rank[i + j*nt] (host array; entries with i <= j are
 * not used).  Device (or pinned host) pointers. */
typedef struct hcore_tlr_matrix {
    int nt, nb;
    double *const *D;
    int ldd;
    double *const *U, *const *V;
    int *rank;
    int maxrank;
} hcore_tlr_matrix;

/* Panel step k of the TLR Cholesky A = L L^T (no single counterpart in the
 * reference: it chains HiCMA's per-tile calls of HCORE_dpotrf
 * (src/compute/hcore_dpotrf.c:23-34), HCORE_dtrsm (hcore_dtrsm.c:24-48),
 * HCORE_dsyrk (hcore_dsyrk.c:47-189) and HCORE_dgemm (hcore_dgemm.c:703)):
 *   D_kk = L_kk L_kk^T (lower triangle overwritten; info = LAPACK's info),
 *   V_ik <- L_kk^-1 V_ik for every panel tile i > k,
 *   D_ii <- D_ii - U_ik (V_ik^T V_ik) U_ik^T for i > k (strict upper set to 0),
 *   A_ij <- A_ij - A_ik A_jk^T for k < j < i, recompressed in place with the
 *   reference's absolute rule at acc, a + c <= 2 maxrk, new rank <= maxrk and
 *   <= the tile storage (maxrank); rank[] is updated.
 * Tiles of rank 0 contribute nothing (no call is made for them).  The SYRK
 * batch and the recompression plan run concurrently.  status (nt*nt host
 * array, may be NULL) receives each Schur update's status at [i + j*nt]; a
 * failed update leaves its tile unchanged.  Synchronous.  Returns
 * HCORE_GPU_OK, HCORE_GPU_ETASK (POTRF info != 0, or an update failed),
 * EINVAL, ENOMEM or ECUDA. */
int hcore_gpu_tlr_panel_step(const hcore_tlr_matrix *A, int k, double acc, int maxrk, int *info,
                             int *status, void *stream);

/* FP64 issue-rate probes (no counterpart in the reference): the measured
 * ceiling that the FP64 phases are compared with.  Each form runs `chains`
 * independent accumulator chains per thread (2, 4 or 8) in
 * blocks_per_sm x SM-count CTAs of 128 threads for `iters` iterations, with
 * no memory traffic; one warm-up launch, then one launch timed with CUDA
 * events on `stream`.  Returns TFLOP/s and the timed launch's milliseconds. */
#define HCORE_PROBE_DFMA 0                 /* fma.rn.f64 */
#define HCORE_PROBE_DMMA_8x8x4 1           /* mma.sync m8n8k4 f64 */
#define HCORE_PROBE_DMMA_16x8x4 2          /* mma.sync m16n8k4 f64 */
#define HCORE_PROBE_DMMA_16x8x8 3          /* mma.sync m16n8k8 f64 */
#define HCORE_PROBE_DMMA_16x8x16 4         /* mma.sync m16n8k16 f64, distinct B */
#define HCORE_PROBE_DMMA_16x8x16_B_ONE_REG 5 /* the four B operands one register */
#define HCORE_PROBE_DMMA_16x8x16_B_EQUAL 6 /* four B registers holding one value */
int hcore_gpu_fp64_probe(int kind, int chains, int blocks_per_sm, int iters, void *stream,
                         double *tflops, double *ms);
/* the m16n8k16 DMMA form with distinct operands, 4 chains, 8 CTAs per SM
 * (about 0.3 s), in TFLOP/s; -1 on error */
double hcore_gpu_fp64_peak(void *stream);

/* One update with HCORE_dgemm's semantics that allocates no memory (no
 * counterpart in the reference).  For callers that cannot call cudaMalloc:
 * a task-runtime worker that must not stall the other workers' streams
 * (cudaMalloc/cudaFree may synchronise the device), or a runtime that
 * reserved all the device memory it may use up front.  The workspace is one
 * fixed-size device array of the library (3 MiB, reserved on every GPU that
 * loads the library until exit), enough for M = 1024 with a + c <= 128 and
 * a*b <= 16384; larger updates are rejected with HCORE_GPU_EINVAL and a
 * message before anything is launched.  Factors are device (or pinned host)
 * memory; CU/CV are updated in place (first new_rank columns; storage must
 * hold max(c, new rank) columns).  The first call on a device sets up that
 * device (the array's device address, the SVD kernel's shared-memory
 * attributes), so make it before any stream capture.  All calls share the
 * array: calls that can overlap on the GPU race and must be serialised by
 * the caller.  The call waits for its stream to finish the update.  A CUDA
 * error already pending when it is called is left pending and reported as
 * HCORE_GPU_ECUDA without launching anything.  Returns HCORE_GPU_OK,
 * HCORE_GPU_ETASK (status set), EINVAL or ECUDA. */
int hcore_gpu_dgemm_noalloc(int M, double alpha, const double *AU, const double *AV, int a,
                            int lda, const double *BU, const double *BV, int b, int ldb,
                            double beta, double *CU, double *CV, int c, int ldc, int rk,
                            int maxrk, double acc, int *new_rank, int *status, void *stream);

/* Rank predictor (no counterpart in the reference): a 6 -> 64 -> 64 -> 1
 * MLP with ReLU, FP32 weights and BF16 activations, trained and run by the
 * library's own CUDA kernels.  It predicts an update's output rank from cheap
 * features so that output slots, workspace and launch shapes can be sized
 * before the batch runs; the SVD still decides every rank (a task whose rank
 * exceeds its predicted capacity gets HCORE_GPU_S_STORAGE and is rerun).
 * Parameters (FP32): W1[6][64] (in x out), b1[64], W2[64][64], b2[64],
 * w3[64], b3.  Inputs are row-major n x 6 FP32 device arrays, targets and
 * outputs n FP32 device arrays.  Loss: mean of 0.5 (y - t)^2; optimiser Adam
 * (0.9, 0.999, 1e-8). */
#define HCORE_MLP_INPUTS 6
#define HCORE_MLP_HIDDEN 64
#define HCORE_MLP_PARAMS (6 * 64 + 64 + 64 * 64 + 64 + 64 + 1)
typedef struct hcore_gpu_mlp_s *hcore_gpu_mlp;
/* He-uniform weights from a seeded generator, zero biases */
int hcore_gpu_mlp_create(hcore_gpu_mlp *mlp, unsigned long long seed);
/* copy the HCORE_MLP_PARAMS parameters to (set = 0) or from (set = 1) host;
 * setting them also clears the optimiser state */
int hcore_gpu_mlp_params(hcore_gpu_mlp mlp, float *params, int set);
/* gradient of the mean loss over all n samples (host array of
 * HCORE_MLP_PARAMS) and the loss itself; synchronous */
int hcore_gpu_mlp_gradient(hcore_gpu_mlp mlp, const float *x, const float *y, int n, float *grad,
                           float *loss, void *stream);
/* minibatch Adam: `epochs` passes over the n samples in a fresh seeded order
 * each time; epoch_loss (host, may be NULL) receives each epoch's mean
 * training loss; synchronous */
int hcore_gpu_mlp_train(hcore_gpu_mlp mlp, const float *x, const float *y, int n, int epochs,
                        int batch, float lr, unsigned long long seed, float *epoch_loss,
                        void *stream);
/* forward pass of n samples into out (device); asynchronous on stream */
int hcore_gpu_mlp_predict(hcore_gpu_mlp mlp, const float *x, int n, float *out, void *stream);
int hcore_gpu_mlp_destroy(hcore_gpu_mlp mlp);

/* library-owned per-thread stream used by the drop-in HCORE_* entry points */
void *hcore_gpu_thread_stream(void);
const char *hcore_gpu_last_error(void);
int hcore_gpu_version(void);

#ifdef __cplusplus
}
#endif
#endif
