/*
 * hcore-gb300 — FP64 drop-in entry points (replacing src/include/hcore_d.h).
 *
 * Every prototype below is identical to the reference's so that a caller such
 * as HiCMA links against libhcore_gb300.so unchanged.  The work runs on the
 * GPU; pointers may be ordinary (pageable) host memory, pinned host memory or
 * device memory: the library stages host data through its own per-thread
 * stream and device arena and returns when the results are back in the
 * caller's buffers.  Errors keep the reference's behaviour (message on stderr
 * and exit(-1)) at the same conditions.
 *
 * Globals: the library defines the reference's tuning/verbosity globals and,
 * like the reference, leaves `use_scratch` to the caller (it is referenced
 * weakly; an undefined use_scratch reads as 0).
 */
#ifndef HCORE_GB300_HCORE_D_H
#define HCORE_GB300_HCORE_D_H
#ifdef __cplusplus
extern "C" {
#endif
#include "flop_util_structs.h"
#include "hcore.h"

/* hcore_dgemm.c:37,41-43 (defined by the library); use_scratch is the
 * caller's (hcore_dgemm.c:38) */
extern int use_trmm;
extern int gemm_print_index;
extern int gemm_print_mat;
extern int hc_nelm_limit;
/* hcore_dsyrk.c:21, hcore_dgemmcd.c:24-26 */
extern int syrk_print_index;
extern int gemmcd_print_index;
extern int gemmcd_print_mat;
extern int gemmcd_use_scratch;
/* hcore_dgemmbdcd.c:25-26 */
extern int gemmbdcd_print_index;
extern int gemmbdcd_print_mat;

/* C = beta*C + alpha*A*B^T with A, B, C low rank, then recompression.
 * Replaces src/include/hcore_d.h:25-46 (src/compute/hcore_dgemm.c:703-1012).
 * Ranks are passed as double* (value in, new rank of C out in Crk[0]). */
void HCORE_dgemm(HCORE_enum transA, int transB, int M, int N, double alpha, double *AU,
                 double *AV, double *Ark, int LDA, double *BU, double *BV, double *Brk,
                 int LDB, double beta, double *CU, double *CV, double *Crk, int LDC, int rk,
                 int maxrk, double acc, double *work, flop_counter *flops);

/* Same update with the "fast" rules: rank search starts at 2, no maxrank
 * checks, no flop counter.  Replaces src/include/hcore_d.h:47-67
 * (src/compute/hcore_dgemm_fast.c:59-426). */
void HCORE_dgemm_fast(HCORE_enum transA, int transB, int M, int N, double alpha, double *AU,
                      double *AV, double *Ark, int LDA, double *BU, double *BV, double *Brk,
                      int LDB, double beta, double *CU, double *CV, double *Crk, int LDC, int rk,
                      int maxrk, double acc, double *work);

/* Dense C update CD -= Au (Av^T Bv) Bu^T (alpha, beta, LDA, LDB, LDC are
 * ignored and every leading dimension is M, as in the reference).
 * Replaces src/include/hcore_d.h:68-86 (src/compute/hcore_dgemmcd.c:36-106). */
void HCORE_dgemmcd(HCORE_enum transA, HCORE_enum transB, int M, double alpha, double *Au,
                   double *Av, int Arank, int LDA, double *Bu, double *Bv, int Brank, int LDB,
                   double beta, double *CD, int LDC, int maxrank, double *work,
                   flop_counter *flops);

/* CD = alpha*AU (AV^T AV) AU^T + CD, strict upper triangle set to zero
 * (beta, uplo, trans ignored; AV has LDAU rows).  Replaces
 * src/include/hcore_d.h:107-116 (src/compute/hcore_dsyrk.c:47-189). */
void HCORE_dsyrk(HCORE_enum uplo, HCORE_enum trans, int M, int K, double alpha,
                 const double *AU, int LDAU, const double *AV, int LDAV, double beta,
                 double *CD, int LDCD, double *work, flop_counter *flops);

/* First half of the update with a dense B (QR, QR, SVD; the new rank is
 * returned in *_p_new_UVrk).  Replaces src/include/hcore_d.h:146-186
 * (src/compute/hcore_dgemm.c:1022-1303). */
void HCORE_dgemm_qr_svd_b_dense(int transA, int transB, int M, int N, double alpha, double *AU,
                                double *AV, int *Ark, int LDA, double *B, int LDB, double beta,
                                double *CU, double *CV, int *Crk, int LDC, int rk,
                                int storage_maxrank, int maxrk, double acc, double *work,
                                flop_counter *flops, double **_p_work_new, double **_p__CU,
                                double **_p__CV, int *_p_CU_ncols, int *_p_new_UVrk,
                                double **_p_newU, int *_p_ld_newU, double **_p_qrtauA,
                                int *_p_CV_ncols, double **_p_newV, int *_p_ld_newV,
                                double **_p_qrtauB, int *_p_use_CUV_clone, double **_p_CUclone,
                                int *_p_ld_CUclone, double **_p__CU_save, double **_p_CVclone,
                                int *_p_ld_CVclone, double **_p__CV_save);

/* First half of the low-rank update (QR, QR, SVD, rank decision).  Replaces
 * src/include/hcore_d.h:187-229 (src/compute/hcore_dgemm.c:1312-1597). */
void HCORE_dgemm_qr_svd(int transA, int transB, int M, int N, double alpha, double *AU,
                        double *AV, int *Ark, int LDA, double *BU, double *BV, int *Brk, int LDB,
                        double beta, double *CU, double *CV, int *Crk, int LDC, int rk,
                        int storage_maxrank, int maxrk, double acc, double *work,
                        flop_counter *flops, double **_p_work_new, double **_p__CU,
                        double **_p__CV, int *_p_CU_ncols, int *_p_new_UVrk, double **_p_newU,
                        int *_p_ld_newU, double **_p_qrtauA, int *_p_CV_ncols, double **_p_newV,
                        int *_p_ld_newV, double **_p_qrtauB, int *_p_use_CUV_clone,
                        double **_p_CUclone, int *_p_ld_CUclone, double **_p__CU_save,
                        double **_p_CVclone, int *_p_ld_CVclone, double **_p__CV_save);

/* Second half: rebuild CU = Q_A U_r and CV = Q_B (S_r V_r^T)^T into
 * _CU_save/_CV_save and set Crk[0].  Replaces src/include/hcore_d.h:230-267
 * (src/compute/hcore_dgemm.c:1602-1699). */
void HCORE_dgemm_ormqr(int transA, int transB, int M, int N, double alpha, double *AU,
                       double *AV, int *Ark, int LDA, double beta, double *CU, double *CV,
                       int *Crk, int LDC, int rk, int storage_maxrank, int maxrk, double acc,
                       double *work, flop_counter *flops, double *_CU, double *_CV,
                       int CU_ncols, int new_UVrk, double *newU, int ld_newU, double *qrtauA,
                       int CV_ncols, double *newV, int ld_newV, double *qrtauB,
                       int use_CUV_clone, double *CUclone, int ld_CUclone, double *_CU_save,
                       double *CVclone, int ld_CVclone, double *_CV_save);

/* CD = alpha*AU*(AV^T*BD) + beta*CD, a low-rank A times a dense B.  With
 * transA == HCORE_Trans the product AV^T*BD sums over M rows and CD has LDA
 * rows; otherwise it sums over LDB rows and CD has M rows.  Replaces
 * src/include/hcore_d.h:87-101 (src/compute/hcore_dgemmbdcd.c:35-122). */
void HCORE_dgemmbdcd(HCORE_enum transA, HCORE_enum transB, int M, int N, double alpha,
                     double *AU, double *AV, double *Ark, int LDA, double *BD, int LDB,
                     double beta, double *CD, int LDC, double *work, flop_counter *flops);

/* CD = AU*BV^T (M x N) from factors of rank Ark == Brk; alpha and beta are
 * not used.  Replaces src/include/hcore_d.h:126-139
 * (src/compute/hcore_duncompress.c:33-84). */
void HCORE_duncompress(HCORE_enum transA, HCORE_enum transB, int M, int N, double alpha,
                       double *AU, double *Ark, int LDA, double *BV, double *Brk, int LDB,
                       double beta, double *CD, int LDC);

/* Triangular solve on a factor: cblas_dtrsm(ColMajor, side, uplo, transA,
 * diag, M, Brank, alpha, A, LDA, BV, LDBV).  Replaces
 * src/include/hcore_d.h:117-125 (src/compute/hcore_dtrsm.c:24-48). */
void HCORE_dtrsm(HCORE_enum side, HCORE_enum uplo, HCORE_enum transA, HCORE_enum diag, int M,
                 int Brank, double alpha, double *A, int LDA, double *BV, int LDBV,
                 flop_counter *flops);

/* Cholesky factorization of a dense tile: *info = LAPACKE_dpotrf_work(
 * LAPACK_COL_MAJOR, uplo, N, A, LDA), uplo being LAPACK's 'L' or 'U'.
 * Replaces src/include/hcore_d.h:102-106 (src/compute/hcore_dpotrf.c:23-34). */
void HCORE_dpotrf(HCORE_enum uplo, int N, double *A, int LDA, int *info, flop_counter *flops);

/* Plain dense C = alpha*op(A)*op(B) + beta*C.  Replaces
 * src/include/hcore_d.h:269-278 (src/compute/hcore_dgemm.c:1701-1715). */
void HCORE_dgemm_dense(HCORE_enum transA, int transB, int M, int N, int K, double alpha,
                       const double *A, int LDA, const double *B, int LDB, double beta,
                       double *C, int LDC);

#ifdef __cplusplus
}
#endif
#endif
