/*
 * hcore-gb300 — complex (double _Complex) drop-in entry points, replacing the
 * declarations of src/include/hcore_z.h that the reference defines
 * (src/compute/hcore_zgemm.c:663-976, src/compute/hcore_zuncompress.c:35-86).
 *
 * The prototype is the reference's.  C++ sees double _Complex as a struct of
 * two doubles, real part first: the same layout and the same argument passing
 * (two floating-point registers on x86-64 and AArch64) as C's type.
 */
#ifndef HCORE_GB300_HCORE_Z_H
#define HCORE_GB300_HCORE_Z_H
#include "flop_util_structs.h"
#include "hcore.h"
#ifdef __cplusplus
extern "C" {
typedef struct hcore_dcomplex {
    double re, im;
} hcore_dcomplex;
#else
typedef double _Complex hcore_dcomplex;
#endif

/* C = beta*C + alpha*A*B^T (plain transposes: X = XU*XV^T) with A, B, C low
 * rank and complex, then recompression to the first i >= 1 singular values
 * with sigma_i >= acc (or rk).  Ranks as double* (value in, new rank of C out
 * in Crk[0]).  Limits of this library: M <= 1024, Ark + Crk <= 256. */
void HCORE_zgemm(HCORE_enum transA, int transB, int M, int N, hcore_dcomplex alpha,
                 hcore_dcomplex *AU, hcore_dcomplex *AV, double *Ark, int LDA, hcore_dcomplex *BU,
                 hcore_dcomplex *BV, double *Brk, int LDB, hcore_dcomplex beta,
                 hcore_dcomplex *CU, hcore_dcomplex *CV, double *Crk, int LDC, int rk, int maxrk,
                 double acc, hcore_dcomplex *work, flop_counter *flops);

/* CD = AU*BV^T (M x N, complex, plain transpose) from factors of rank
 * Ark == Brk; alpha and beta are not used.  Replaces src/include/hcore_z.h:76-88
 * (src/compute/hcore_zuncompress.c:35-86). */
void HCORE_zuncompress(HCORE_enum transA, HCORE_enum transB, int M, int N, hcore_dcomplex alpha,
                       hcore_dcomplex *AU, double *Ark, int LDA, hcore_dcomplex *BV, double *Brk,
                       int LDB, hcore_dcomplex beta, hcore_dcomplex *CD, int LDC);

/* Batched complex updates on the GPU (the same semantics per task, statuses
 * HCORE_GPU_S_* instead of exit; no counterpart in the reference).  Batches
 * whose tasks all have M <= 1024 and a + c within the complex SVD's
 * shared-memory limit (84 on GB300) run on the native complex kernels; other
 * batches, or any batch with HCORE_GPU_ZGEMM_EMBED=1 in the environment, run
 * as one real plan of order 2M.  CU/CV are updated in place (room for
 * max(c, new rank) columns); pointers may be host or device memory.
 * Synchronous.  Returns HCORE_GPU_OK, HCORE_GPU_ETASK (a task's status is
 * set) or a negative error. */
typedef struct hcore_zlr_task {
    int M, a, b, c;
    int rk, maxrk;
    hcore_dcomplex alpha, beta;
    double acc;
    const hcore_dcomplex *AU, *AV;
    int lda;
    const hcore_dcomplex *BU, *BV;
    int ldb;
    hcore_dcomplex *CU, *CV;
    int ldc;
} hcore_zlr_task;
int hcore_gpu_zgemm_batched(int n, const hcore_zlr_task *tasks, int *ranks, int *status,
                            void *stream);

#ifdef __cplusplus
}
#endif
#endif
