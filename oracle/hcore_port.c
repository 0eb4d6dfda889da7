/*
 * ORACLE — CPU restatement of the reference HCORE low-rank path (test
 * infrastructure; never part of the GPU product).
 *
 * Built by oracle/build.py into oracle/_build/libhcore_port.so on whichever
 * machine runs the tests, linked against the LAPACK/BLAS that SciPy bundles
 * (OpenBLAS, symbols prefixed "scipy_").  The reference itself pins no
 * LAPACK version (CMakeLists.txt:49-144 accepts any CBLAS/LAPACKE); the
 * oracle's is whatever SciPy wheel is installed, and its results are pinned
 * against the reference's own known-answer tests and against outputs of the
 * reference compiled from source (tests/golden/).
 *
 * The double and float bodies come from hcore_port_impl.h.
 */
#include <stdlib.h>
#include <string.h>

#include "hcore_port.h"

enum { CblasColMajor = 102 };
enum { CblasNoTrans = 111, CblasTrans = 112 };
#define LAPACK_COL_MAJOR 102

void scipy_cblas_dgemm(int, int, int, int, int, int, double, const double *, int,
                       const double *, int, double, double *, int);
void scipy_cblas_sgemm(int, int, int, int, int, int, float, const float *, int,
                       const float *, int, float, float *, int);
int scipy_LAPACKE_dgeqrf(int, int, int, double *, int, double *);
int scipy_LAPACKE_sgeqrf(int, int, int, float *, int, float *);
int scipy_LAPACKE_dgesvd(int, char, char, int, int, double *, int, double *, double *,
                         int, double *, int, double *);
int scipy_LAPACKE_sgesvd(int, char, char, int, int, float *, int, float *, float *, int,
                         float *, int, float *);
int scipy_LAPACKE_dormqr(int, char, char, int, int, int, const double *, int,
                         const double *, double *, int);
int scipy_LAPACKE_sormqr(int, char, char, int, int, int, const float *, int,
                         const float *, float *, int);
int scipy_LAPACKE_dlatms(int, int, int, char, int *, char, double *, int, double, double,
                         int, int, char, double *, int);
void scipy_openblas_set_num_threads(int);

/* src/misc/descutil/flop_counts.c:3-70, restated.  The 'q' formula divides
 * in single precision (2*n*n*n/3.0f) exactly as the reference does, so the
 * integer totals agree bit for bit. */
unsigned long port_flop_counts(char op, unsigned long a, unsigned long b, unsigned long c,
                               unsigned long d)
{
    unsigned long res = 0;
    if (op == 'q') {
        unsigned long m = a, n = b;
        res = 2 * m * n * n - (unsigned long)((float)(2 * n * n * n) / 3.0f) + 2 * m * n +
              (unsigned long)((float)(17 * n) / 3.0f);
    } else if (op == 'm') {
        res = a * b * c * 2;
    } else if (op == 's') {
        res = 22 * a * a * a;
    } else if (op == 'o') {
        unsigned long m = a, n = b, k = c;
        if (d == 1)
            res = 4 * n * m * k - 2 * n * k * k + 3 * n * k;
        else if (d == 2)
            res = 4 * n * m * k - 2 * m * k * k + 2 * m * k + n * k - k * k / 2 + k / 2;
    } else if (op == 'c') {
        unsigned long n = a;
        res = (unsigned long)(n * n * n / 3 - n * n / 2.0 + n / 6);
    } else if (op == 't' || op == 'r') {
        unsigned long m = a, n = b;
        if (c == 1) res = n * m * m;
        else if (c == 2) res = m * n * n;
    }
    return res;
}

void port_set_threads(int n) { scipy_openblas_set_num_threads(n); }

/* LAPACKE_dlatms, used by the reference tests' generate_compress
 * (testing/testing_dgemm.c:159) to build their known-answer inputs. */
int port_dlatms(int m, int n, char dist, int *iseed, char sym, double *d, int mode,
                double cond, double dmax, int kl, int ku, char pack, double *a, int lda)
{
    return scipy_LAPACKE_dlatms(LAPACK_COL_MAJOR, m, n, dist, iseed, sym, d, mode, cond,
                                dmax, kl, ku, pack, a, lda);
}

#define REAL double
#define PFX(name) port_d##name
#define LAPACKE_(name) scipy_LAPACKE_d##name
#define cblas_(name) scipy_cblas_d##name
#include "hcore_port_impl.h"
#undef REAL
#undef PFX
#undef LAPACKE_
#undef cblas_

#define REAL float
#define PFX(name) port_s##name
#define LAPACKE_(name) scipy_LAPACKE_s##name
#define cblas_(name) scipy_cblas_s##name
#include "hcore_port_impl.h"
#undef REAL
#undef PFX
#undef LAPACKE_
#undef cblas_

/* ---- the tile steps either side of the update (FP64 only, as in the
 * reference): the same BLAS/LAPACK calls in the same order ---- */
/* A list of Schur-type updates over two factor arenas, as a benchmark's CPU
 * baseline runs them: update u reads tiles sa[u], sb[u] and sc[u], whose
 * factors are column-major nb x rank blocks at U + off[t], V + off[t] (rank
 * = (off[t+1] - off[t]) / nb), and runs port_dgemm on a copy of C (so the
 * list can be repeated on the same inputs).  The loop is in C so that the
 * timed work is the reference's sequence of calls and not interpreter
 * overhead.  Returns the number of updates whose status was not PORT_OK,
 * or -1 if the scratch could not be allocated. */
int port_dgemm_list(int nb, const double *U, const double *V, const long long *off, int n,
                    const int *sa, const int *sb, const int *sc, double alpha, double beta,
                    int maxrk, double acc, int variant)
{
    int kmax = 1, bad = 0;
    for (int u = 0; u < n; ++u) {
        const int a = (int)((off[sa[u] + 1] - off[sa[u]]) / nb);
        const int c = (int)((off[sc[u] + 1] - off[sc[u]]) / nb);
        if (a + c > kmax) kmax = a + c;
    }
    double *CU = (double *)malloc(sizeof(double) * (size_t)nb * kmax);
    double *CV = (double *)malloc(sizeof(double) * (size_t)nb * kmax);
    if (!CU || !CV) {
        free(CU);
        free(CV);
        return -1;
    }
    for (int u = 0; u < n; ++u) {
        const long long oa = off[sa[u]], ob = off[sb[u]], oc = off[sc[u]];
        const int a = (int)((off[sa[u] + 1] - oa) / nb);
        const int b = (int)((off[sb[u] + 1] - ob) / nb);
        int c = (int)((off[sc[u] + 1] - oc) / nb);
        memcpy(CU, U + oc, sizeof(double) * (size_t)nb * c);
        memcpy(CV, V + oc, sizeof(double) * (size_t)nb * c);
        unsigned long fl = 0;
        const int st = port_dgemm(nb, alpha, U + oa, V + oa, a, nb, U + ob, V + ob, b, nb, NULL,
                                  beta, CU, CV, &c, nb, 0, maxrk, maxrk, acc, variant, NULL, &fl);
        if (st != PORT_OK) ++bad;
    }
    free(CU);
    free(CV);
    return bad;
}

void scipy_cblas_dtrsm(int, int, int, int, int, int, int, double, const double *, int,
                       double *, int);
int scipy_LAPACKE_dpotrf_work(int, char, int, double *, int);

/* HCORE_duncompress (src/compute/hcore_duncompress.c:33-84): CD = AU BV^T */
void port_duncompress(int M, int N, const double *AU, int a, int LDA, const double *BV, int LDB,
                      double *CD, int LDC)
{
    scipy_cblas_dgemm(CblasColMajor, CblasNoTrans, CblasTrans, M, N, a, 1.0, AU, LDA, BV, LDB,
                      0.0, CD, LDC);
}

/* HCORE_dgemmbdcd (src/compute/hcore_dgemmbdcd.c:35-122): AVBD = AV^T BD
 * (a x N, ld a) over K = M rows (transA == Trans) or LDB rows, then
 * CD = alpha AU AVBD + beta CD with LDA (Trans) or M rows.  With a = 0 the
 * reference's GEMMs get a leading dimension of 0, which BLAS rejects, so CD
 * stays as it was. */
void port_dgemmbdcd(int transA, int M, int N, double alpha, const double *AU, const double *AV,
                    int a, int LDA, const double *BD, int LDB, double beta, double *CD, int LDC,
                    unsigned long *flops_update)
{
    const int tr = transA == CblasTrans;
    const int K = tr ? M : LDB, rows = tr ? LDA : M;
    if (a > 0) {
        double *AVBD = malloc((size_t)a * (N > 0 ? N : 1) * sizeof(double));
        scipy_cblas_dgemm(CblasColMajor, CblasTrans, CblasNoTrans, a, N, K, 1.0, AV, LDA, BD,
                          LDB, 0.0, AVBD, a);
        scipy_cblas_dgemm(CblasColMajor, CblasNoTrans, CblasNoTrans, rows, N, a, alpha, AU, LDA,
                          AVBD, a, beta, CD, LDC);
        free(AVBD);
    }
    if (flops_update)
        *flops_update += port_flop_counts('m', a, N, K, 0) + port_flop_counts('m', rows, N, a, 0);
}

/* HCORE_dtrsm (src/compute/hcore_dtrsm.c:24-48) */
void port_dtrsm(int side, int uplo, int transA, int diag, int M, int Brank, double alpha,
                const double *A, int LDA, double *BV, int LDBV, unsigned long *flops_trsm)
{
    scipy_cblas_dtrsm(CblasColMajor, side, uplo, transA, diag, M, Brank, alpha, A, LDA, BV, LDBV);
    if (flops_trsm) *flops_trsm += port_flop_counts('t', M, Brank, side == 141 ? 1 : 2, 0);
}

/* HCORE_dpotrf (src/compute/hcore_dpotrf.c:23-34) */
int port_dpotrf(int uplo, int N, double *A, int LDA, unsigned long *flops_potrf)
{
    const int info = scipy_LAPACKE_dpotrf_work(LAPACK_COL_MAJOR, (char)uplo, N, A, LDA);
    if (flops_potrf) *flops_potrf += port_flop_counts('c', N, 0, 0, 0);
    return info;
}

/* The reference's tile compressor, generate_compress
 * (testing/testing_dgemm.c:119-236) after its dlatms step: dgesvd('A','A')
 * of the M x N tile, rank = the number of leading singular values >= thr
 * (:194; thr = acc, or acc * sigma_max when relative), capped at maxrank
 * (:195-197); U = the first r left vectors (:204), V = (S V^T)^T (:173-176,
 * :209).  sigma (min(M, N)) receives the singular values. */
int port_dcompress(int M, int N, const double *D, int ldd, double acc, int relative, int maxrank,
                   double *U, double *V, int ldo, int *rank, double *sigma)
{
    const int mn = M < N ? M : N;
    double *A = malloc((size_t)M * N * sizeof(double));
    double *tU = malloc((size_t)M * M * sizeof(double));
    double *tV = malloc((size_t)N * N * sizeof(double));
    double *sup = malloc((size_t)(mn > 1 ? mn : 1) * sizeof(double));
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < M; ++i) A[(size_t)j * M + i] = D[(size_t)j * ldd + i];
    const int info = scipy_LAPACKE_dgesvd(LAPACK_COL_MAJOR, 'A', 'A', M, N, A, M, sigma, tU, M,
                                          tV, N, sup);
    int r = 0;
    if (info == 0) {
        const double thr = relative ? acc * sigma[0] : acc;
        while (r < mn && sigma[r] >= thr) ++r;
        if (r > maxrank) r = maxrank;
        for (int t = 0; t < r; ++t) {
            for (int i = 0; i < M; ++i) U[(size_t)t * ldo + i] = tU[(size_t)t * M + i];
            for (int i = 0; i < N; ++i) V[(size_t)t * ldo + i] = sigma[t] * tV[(size_t)i * N + t];
        }
    }
    *rank = r;
    free(A); free(tU); free(tV); free(sup);
    return info == 0 ? PORT_OK : PORT_E_LAPACK;
}

/* ---- HCORE_zgemm (src/compute/hcore_zgemm.c:663-976), restated with the
 * same complex LAPACK/BLAS calls: __zqra stacks [beta*CU | alpha*AU] and
 * zgeqrf (:65-135); __zqrb F = AV^T BV, G = BU F^T, [CV | G], zgeqrf
 * (:138-220; plain transposes); __zsvd T = R_A R_B^T, zgesvd('A','A'), the
 * rank rule, rows of V^H scaled by sigma (:222-430); __znewu zunmqr('L','N')
 * (:435-560); __znewv conj, zunmqr('R','C'), conj, transpose (:561-640),
 * i.e. CV = (S_r V^H_r Q_B^T)^T.  ld_newV = maxrk as in HCORE_dgemm. ---- */
#include <complex.h>
typedef double _Complex zdouble;
void scipy_cblas_zgemm(int, int, int, int, int, int, const void *, const void *, int,
                       const void *, int, const void *, void *, int);
int scipy_LAPACKE_zgeqrf(int, int, int, zdouble *, int, zdouble *);
int scipy_LAPACKE_zgesvd(int, char, char, int, int, zdouble *, int, double *, zdouble *, int,
                         zdouble *, int, double *);
int scipy_LAPACKE_zunmqr(int, char, char, int, int, int, const zdouble *, int, const zdouble *,
                         zdouble *, int);

int port_zgemm(int M, zdouble alpha, const zdouble *AU, const zdouble *AV, int a, int lda,
               const zdouble *BU, const zdouble *BV, int b, int ldb, zdouble beta, zdouble *CU,
               zdouble *CV, int *c_inout, int ldc, int rk, int maxrk, double acc,
               unsigned long *flops_update)
{
    const int c = *c_inout;
    if (a == 0 || b == 0 || c == 0) return PORT_E_ZERO_RANK;  /* :703-706 */
    if (a + c > 2 * maxrk) return PORT_E_RANK_SUM;
    const int k = a + c;
    if (k > M) return PORT_E_SHAPE;
    if (maxrk < k) return PORT_E_LDNEWV;
    unsigned long fl = 0;
    const zdouble one = 1.0, zero = 0.0;
    zdouble *UA = calloc((size_t)M * k, sizeof(zdouble)), *VB = calloc((size_t)M * k, sizeof(zdouble));
    zdouble *tauA = calloc(k, sizeof(zdouble)), *tauB = calloc(k, sizeof(zdouble));
    zdouble *T = calloc((size_t)k * k, sizeof(zdouble)), *U = calloc((size_t)k * k, sizeof(zdouble));
    zdouble *VT = calloc((size_t)k * k, sizeof(zdouble)), *F = calloc((size_t)a * b, sizeof(zdouble));
    double *s = calloc(k, sizeof(double)), *superb = calloc(k, sizeof(double));
    int status = PORT_OK, i, j, l, r;
    for (j = 0; j < c; j++)
        for (i = 0; i < M; i++) UA[(size_t)j * M + i] = beta * CU[(size_t)j * ldc + i];
    for (j = 0; j < a; j++)
        for (i = 0; i < M; i++) UA[(size_t)(c + j) * M + i] = alpha * AU[(size_t)j * lda + i];
    if (scipy_LAPACKE_zgeqrf(LAPACK_COL_MAJOR, M, k, UA, M, tauA)) { status = PORT_E_LAPACK; goto done; }
    fl += port_flop_counts('q', M, k, 0, 0);
    for (j = 0; j < c; j++)
        for (i = 0; i < M; i++) VB[(size_t)j * M + i] = CV[(size_t)j * ldc + i];
    scipy_cblas_zgemm(CblasColMajor, CblasTrans, CblasNoTrans, a, b, M, &one, AV, lda, BV, ldb,
                      &zero, F, a);
    scipy_cblas_zgemm(CblasColMajor, CblasNoTrans, CblasTrans, M, a, b, &one, BU, ldb, F, a,
                      &zero, VB + (size_t)c * M, M);
    fl += port_flop_counts('m', a, b, M, 0) + port_flop_counts('m', M, a, b, 0);
    if (scipy_LAPACKE_zgeqrf(LAPACK_COL_MAJOR, M, k, VB, M, tauB)) { status = PORT_E_LAPACK; goto done; }
    fl += port_flop_counts('q', M, k, 0, 0);
    for (j = 0; j < k; j++)
        for (i = 0; i < k; i++) {
            zdouble t = 0;
            for (l = (i > j ? i : j); l < k; l++) t += UA[(size_t)l * M + i] * VB[(size_t)l * M + j];
            T[(size_t)j * k + i] = t;
        }
    if (scipy_LAPACKE_zgesvd(LAPACK_COL_MAJOR, 'A', 'A', k, k, T, k, s, U, k, VT, k, superb)) {
        status = PORT_E_LAPACK; goto done;
    }
    fl += port_flop_counts('s', k, 0, 0, 0);
    if (rk != 0) {
        r = rk > k ? k : rk;
    } else {
        r = k;
        for (i = 1; i < k; i++)
            if (s[i] < acc) { r = i; break; }
    }
    if (r > maxrk) { status = PORT_E_RANK_MAX; goto done; }
    for (i = 0; i < r; i++)
        for (j = 0; j < k; j++) VT[(size_t)j * k + i] *= s[i];
    fl += (unsigned long)r * (unsigned long)k;
    {   /* CU = Q_A [U_r; 0] */
        zdouble *X = calloc((size_t)M * r, sizeof(zdouble));
        for (j = 0; j < r; j++)
            for (i = 0; i < k; i++) X[(size_t)j * M + i] = U[(size_t)j * k + i];
        if (scipy_LAPACKE_zunmqr(LAPACK_COL_MAJOR, 'L', 'N', M, r, k, UA, M, tauA, X, M)) {
            free(X); status = PORT_E_LAPACK; goto done;
        }
        fl += port_flop_counts('o', M, r, k, 1);
        for (j = 0; j < r; j++)
            for (i = 0; i < M; i++) CU[(size_t)j * ldc + i] = X[(size_t)j * M + i];
        free(X);
    }
    {   /* CV = (S_r V^H_r Q_B^T)^T = conj(conj(S_r V^H_r) Q_B^H)^T */
        zdouble *X = calloc((size_t)r * M, sizeof(zdouble));
        for (j = 0; j < k; j++)
            for (i = 0; i < r; i++) X[(size_t)j * r + i] = conj(VT[(size_t)j * k + i]);
        if (scipy_LAPACKE_zunmqr(LAPACK_COL_MAJOR, 'R', 'C', r, M, k, VB, M, tauB, X, r)) {
            free(X); status = PORT_E_LAPACK; goto done;
        }
        fl += port_flop_counts('o', r, M, k, 2);
        for (j = 0; j < r; j++)
            for (i = 0; i < M; i++) CV[(size_t)j * ldc + i] = conj(X[(size_t)i * r + j]);
        free(X);
    }
    *c_inout = r;
done:
    if (flops_update) *flops_update += fl;
    free(UA); free(VB); free(tauA); free(tauB); free(T); free(U); free(VT); free(F);
    free(s); free(superb);
    return status;
}
