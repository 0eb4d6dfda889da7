/*
 * hcore-gb300 — FP32 drop-in entry points (replacing src/include/hcore_s.h).
 * Same contract as hcore_d.h in single precision: the whole update runs in
 * FP32 on the GPU, as the reference's float copy does on the CPU.
 */
#ifndef HCORE_GB300_HCORE_S_H
#define HCORE_GB300_HCORE_S_H
#ifdef __cplusplus
extern "C" {
#endif
#include "flop_util_structs.h"
#include "hcore.h"

/* src/compute/hcore_sgemm.c:37,41-43 */
extern int sgemm_use_trmm;
extern int sgemm_print_index;
extern int sgemm_print_mat;
extern int shc_nelm_limit;

/* Replaces src/include/hcore_s.h:25-46 (src/compute/hcore_sgemm.c:703). */
void HCORE_sgemm(HCORE_enum transA, HCORE_enum transB, int M, int N, float alpha, float *AU,
                 float *AV, float *Ark, int LDA, float *BU, float *BV, float *Brk, int LDB,
                 float beta, float *CU, float *CV, float *Crk, int LDC, int rk, int maxrk,
                 float acc, float *work, flop_counter *flops);

/* Replaces src/include/hcore_s.h:146-186 (src/compute/hcore_sgemm.c:1022). */
void HCORE_sgemm_qr_svd_b_dense(int transA, int transB, int M, int N, float alpha, float *AU,
                                float *AV, int *Ark, int LDA, float *B, int LDB, float beta,
                                float *CU, float *CV, int *Crk, int LDC, int rk,
                                int storage_maxrank, int maxrk, float acc, float *work,
                                flop_counter *flops, float **_p_work_new, float **_p__CU,
                                float **_p__CV, int *_p_CU_ncols, int *_p_new_UVrk,
                                float **_p_newU, int *_p_ld_newU, float **_p_qrtauA,
                                int *_p_CV_ncols, float **_p_newV, int *_p_ld_newV,
                                float **_p_qrtauB, int *_p_use_CUV_clone, float **_p_CUclone,
                                int *_p_ld_CUclone, float **_p__CU_save, float **_p_CVclone,
                                int *_p_ld_CVclone, float **_p__CV_save);

/* Replaces src/include/hcore_s.h:187-229 (src/compute/hcore_sgemm.c:1312). */
void HCORE_sgemm_qr_svd(int transA, int transB, int M, int N, float alpha, float *AU, float *AV,
                        int *Ark, int LDA, float *BU, float *BV, int *Brk, int LDB, float beta,
                        float *CU, float *CV, int *Crk, int LDC, int rk, int storage_maxrank,
                        int maxrk, float acc, float *work, flop_counter *flops,
                        float **_p_work_new, float **_p__CU, float **_p__CV, int *_p_CU_ncols,
                        int *_p_new_UVrk, float **_p_newU, int *_p_ld_newU, float **_p_qrtauA,
                        int *_p_CV_ncols, float **_p_newV, int *_p_ld_newV, float **_p_qrtauB,
                        int *_p_use_CUV_clone, float **_p_CUclone, int *_p_ld_CUclone,
                        float **_p__CU_save, float **_p_CVclone, int *_p_ld_CVclone,
                        float **_p__CV_save);

/* Replaces src/include/hcore_s.h:230-267 (src/compute/hcore_sgemm.c:1602). */
void HCORE_sgemm_ormqr(int transA, int transB, int M, int N, float alpha, float *AU, float *AV,
                       int *Ark, int LDA, float beta, float *CU, float *CV, int *Crk, int LDC,
                       int rk, int storage_maxrank, int maxrk, float acc, float *work,
                       flop_counter *flops, float *_CU, float *_CV, int CU_ncols, int new_UVrk,
                       float *newU, int ld_newU, float *qrtauA, int CV_ncols, float *newV,
                       int ld_newV, float *qrtauB, int use_CUV_clone, float *CUclone,
                       int ld_CUclone, float *_CU_save, float *CVclone, int ld_CVclone,
                       float *_CV_save);

/* Replaces src/include/hcore_s.h:269-278 (src/compute/hcore_sgemm.c:1701). */
void HCORE_sgemm_dense(HCORE_enum transA, int transB, int M, int N, int K, float alpha,
                       const float *A, int LDA, const float *B, int LDB, float beta, float *C,
                       int LDC);

#ifdef __cplusplus
}
#endif
#endif
