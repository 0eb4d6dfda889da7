/*
 * ORACLE — declarations of the CPU restatement (test infrastructure only).
 * See hcore_port_impl.h for the reference lines each function follows.
 */
#ifndef HCORE_PORT_H
#define HCORE_PORT_H

/* status codes standing in for the reference's exit(-1) sites */
#define PORT_OK 0
#define PORT_E_ZERO_RANK 1  /* hcore_dgemm.c:743-746 and :879-882 */
#define PORT_E_RANK_SUM 2   /* __qra :91-95 */
#define PORT_E_LDNEWV 3     /* hcore_dgemm.c:924-927 */
#define PORT_E_RANK_MAX 4   /* __svd :465-468 */
#define PORT_E_STORAGE 5    /* HCORE_dgemm_ormqr :1648-1651 */
#define PORT_E_LAPACK 6     /* LAPACK info != 0 */
#define PORT_E_SHAPE 7      /* k = a + c > M: the reference reads past R */

unsigned long port_flop_counts(char op, unsigned long a, unsigned long b, unsigned long c,
                               unsigned long d);
void port_set_threads(int n);
int port_dlatms(int m, int n, char dist, int *iseed, char sym, double *d, int mode,
                double cond, double dmax, int kl, int ku, char pack, double *a, int lda);

int port_dgemm(int M, double alpha, const double *AU, const double *AV, int a, int lda,
               const double *BU, const double *BV, int b, int ldb, const double *dense_B,
               double beta, double *CU, double *CV, int *c_inout, int ldc, int rk, int maxrk,
               int storage_maxrank, double acc, int variant, double *sigma_out,
               unsigned long *flops_update);
int port_sgemm(int M, float alpha, const float *AU, const float *AV, int a, int lda,
               const float *BU, const float *BV, int b, int ldb, const float *dense_B,
               float beta, float *CU, float *CV, int *c_inout, int ldc, int rk, int maxrk,
               int storage_maxrank, float acc, int variant, float *sigma_out,
               unsigned long *flops_update);
int port_dgemm_list(int nb, const double *U, const double *V, const long long *off, int n,
                    const int *sa, const int *sb, const int *sc, double alpha, double beta,
                    int maxrk, double acc, int variant);
int port_dsyrk(int M, int K, double alpha, const double *AU, int LDAU, const double *AV,
               double *CD, int LDCD, unsigned long *flops_syrk);
int port_dgemmcd(int M, const double *Au, const double *Av, int Arank, const double *Bu,
                 const double *Bv, int Brank, double *CD);
void port_duncompress(int M, int N, const double *AU, int a, int LDA, const double *BV, int LDB,
                      double *CD, int LDC);
void port_dgemmbdcd(int transA, int M, int N, double alpha, const double *AU, const double *AV,
                    int a, int LDA, const double *BD, int LDB, double beta, double *CD, int LDC,
                    unsigned long *flops_update);
void port_dtrsm(int side, int uplo, int transA, int diag, int M, int Brank, double alpha,
                const double *A, int LDA, double *BV, int LDBV, unsigned long *flops_trsm);
int port_dpotrf(int uplo, int N, double *A, int LDA, unsigned long *flops_potrf);
int port_dcompress(int M, int N, const double *D, int ldd, double acc, int relative, int maxrank,
                   double *U, double *V, int ldo, int *rank, double *sigma);
#endif
