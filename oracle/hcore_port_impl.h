/*
 * ORACLE — CPU restatement of the reference HCORE low-rank update path.
 * Test infrastructure only: tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it as the checker.  The GPU product never links it.
 *
 * This body is included twice by hcore_port.c: once with REAL=double
 * (prefix port_d*) and once with REAL=float (prefix port_s*).  It calls the
 * same LAPACK/BLAS routines, in the same order and with the same shapes, as
 * the reference:
 *
 *   src/compute/hcore_dgemm.c:703-1012  HCORE_dgemm
 *     __qra   :79-137   stack [beta*CU | alpha*AU], dgeqrf
 *     __qrb   :149-225  F = AV^T BV, G = BU F^T, stack [CV | G], dgeqrf
 *     __svd   :296-503  T = R_A R_B^T, dgesvd('A','A'), rank rule, S*V^T
 *     __newu  :508-617  zero-pad U, dormqr('L','N'), copy
 *     __newv  :622-696  zero-pad S*V^T, dormqr('R','T'), transpose
 *   src/compute/hcore_dgemm.c:1022-1303 HCORE_dgemm_qr_svd_b_dense (dense B)
 *   src/compute/hcore_dgemm.c:1312-1699 split API (ld_newV = 2*maxrk)
 *   src/compute/hcore_dgemm_fast.c:59-426 HCORE_dgemm_fast (rank loop from 2)
 *   src/compute/hcore_dsyrk.c:47-189   HCORE_dsyrk
 *   src/compute/hcore_dgemmcd.c:36-106 HCORE_dgemmcd
 *
 * Where the reference calls exit(-1) this restatement returns a status code
 * (PORT_E_*), so tests can check the error behaviour without ending the
 * process.  Flop accounting follows src/misc/descutil/flop_counts.c:3-70.
 */

/* ---- one low-rank x low-rank update, C <- beta*C + alpha*A*B^T ---------- */
/* variant: 0 = HCORE_dgemm (ld_newV = maxrk, rank search from i=1)
 *          1 = HCORE_dgemm_fast (no maxrk checks, rank search from i=2)
 *          2 = split API HCORE_dgemm_qr_svd + HCORE_dgemm_ormqr
 *              (ld_newV = 2*maxrk, storage_maxrank checked in phase 2)
 * dense_B != NULL selects the HCORE_dgemm_qr_svd_b_dense form (variant 2).
 * c_inout: rank of C in, new rank out.  sigma_out (optional): k values. */
int PFX(gemm)(int M, REAL alpha,
              const REAL *AU, const REAL *AV, int a, int lda,
              const REAL *BU, const REAL *BV, int b, int ldb,
              const REAL *dense_B,
              REAL beta, REAL *CU, REAL *CV, int *c_inout, int ldc,
              int rk, int maxrk, int storage_maxrank, REAL acc, int variant,
              REAL *sigma_out, unsigned long *flops_update)
{
    int c = *c_inout;
    unsigned long fl = 0;
    /* hcore_dgemm.c:740-746 (HCORE_dgemm only; the split API has the check
     * commented out at :1366-1369) */
    if (variant == 0 && (a == 0 || b == 0 || c == 0)) return PORT_E_ZERO_RANK;
    /* __qra :91-95 */
    if (variant != 1 && a + c > 2 * maxrk) return PORT_E_RANK_SUM;
    const int k = a + c;
    if (k == 0) return PORT_E_ZERO_RANK;                 /* :879-882 */
    if (k > M) return PORT_E_SHAPE;  /* T would be read past R's rows */
    const int ld_newV = (variant == 0) ? maxrk : (variant == 2 ? 2 * maxrk : k);
    if (variant != 1 && ld_newV < k) return PORT_E_LDNEWV; /* :924-927, :1494 */

    REAL *UA = (REAL *)calloc((size_t)M * k, sizeof(REAL));
    REAL *VB = (REAL *)calloc((size_t)M * k, sizeof(REAL));
    REAL *tauA = (REAL *)calloc(k, sizeof(REAL));
    REAL *tauB = (REAL *)calloc(k, sizeof(REAL));
    REAL *T = (REAL *)calloc((size_t)k * k, sizeof(REAL));
    REAL *U = (REAL *)calloc((size_t)k * k, sizeof(REAL));
    REAL *VT = (REAL *)calloc((size_t)k * k, sizeof(REAL));
    REAL *s = (REAL *)calloc(k, sizeof(REAL));
    REAL *superb = (REAL *)calloc(k, sizeof(REAL));
    int status = PORT_OK, info, i, j;

    /* __qra: UA = [beta*CU | alpha*AU] then dgeqrf (:106-124) */
    for (j = 0; j < c; j++)
        for (i = 0; i < M; i++) UA[(size_t)j * M + i] = beta * CU[(size_t)j * ldc + i];
    for (j = 0; j < a; j++)
        for (i = 0; i < M; i++) UA[(size_t)(c + j) * M + i] = alpha * AU[(size_t)j * lda + i];
    info = LAPACKE_(geqrf)(LAPACK_COL_MAJOR, M, k, UA, M, tauA);
    if (info) { status = PORT_E_LAPACK; goto done; }
    fl += port_flop_counts('q', M, k, 0, 0);

    /* __qrb: VB = [CV | G] (:175-217) */
    for (j = 0; j < c; j++)
        for (i = 0; i < M; i++) VB[(size_t)j * M + i] = CV[(size_t)j * ldc + i];
    if (dense_B) {
        /* __qrb_b_dense :262-271: G = B * AV (M x a) */
        if (a > 0)
            cblas_(gemm)(CblasColMajor, CblasNoTrans, CblasNoTrans, M, a, M, 1,
                         dense_B, ldb, AV, lda, 0, VB + (size_t)c * M, M);
        fl += port_flop_counts('m', M, a, M, 0);
    } else {
        REAL *F = (REAL *)calloc((size_t)(a > 0 ? a : 1) * (b > 0 ? b : 1), sizeof(REAL));
        if (a > 0 && b > 0) {
            cblas_(gemm)(CblasColMajor, CblasTrans, CblasNoTrans, a, b, M, 1,
                         AV, lda, BV, ldb, 0, F, a);
            cblas_(gemm)(CblasColMajor, CblasNoTrans, CblasTrans, M, a, b, 1,
                         BU, ldb, F, a, 0, VB + (size_t)c * M, M);
        }
        fl += port_flop_counts('m', a, b, M, 0);
        fl += port_flop_counts('m', M, a, b, 0);
        free(F);
    }
    info = LAPACKE_(geqrf)(LAPACK_COL_MAJOR, M, k, VB, M, tauB);
    if (info) { status = PORT_E_LAPACK; goto done; }
    fl += port_flop_counts('q', M, k, 0, 0);

    /* __svd: T = triu(R_A) * triu(R_B)^T (:330-387), dgesvd (:403-406) */
    for (j = 0; j < k; j++)
        for (i = 0; i < k; i++) {
            REAL acc_t = 0;
            int l;
            for (l = (i > j ? i : j); l < k; l++)
                acc_t += UA[(size_t)l * M + i] * VB[(size_t)l * M + j];
            T[(size_t)j * k + i] = acc_t;
        }
    info = LAPACKE_(gesvd)(LAPACK_COL_MAJOR, 'A', 'A', k, k, T, k, s, U, k, VT, k, superb);
    if (info) { status = PORT_E_LAPACK; goto done; }
    fl += port_flop_counts('s', k, 0, 0, 0);
    if (sigma_out)
        for (i = 0; i < k; i++) sigma_out[i] = s[i];

    /* rank rule (:444-464; dgemm_fast :306-323 starts at i=2) */
    int r;
    if (rk != 0) {
        r = rk > k ? k : rk;
    } else {
        r = k;
        for (i = (variant == 1 ? 2 : 1); i < k; i++)
            if (s[i] < acc) { r = i; break; }
    }
    if (variant != 1 && r > maxrk) { status = PORT_E_RANK_MAX; goto done; } /* :465 */
    if (variant == 2 && r > storage_maxrank) { status = PORT_E_STORAGE; goto done; } /* :1648 */
    /* scale rows of V^T by sigma (:484-489) */
    for (i = 0; i < r; i++)
        for (j = 0; j < k; j++) VT[(size_t)j * k + i] *= s[i];
    fl += (unsigned long)r * (unsigned long)k;

    /* __newu: CU = Q_A [U_r; 0] (:536-597) */
    {
        REAL *X = (REAL *)calloc((size_t)M * (r > 0 ? r : 1), sizeof(REAL));
        for (j = 0; j < r; j++)
            for (i = 0; i < k; i++) X[(size_t)j * M + i] = U[(size_t)j * k + i];
        if (r > 0) {
            info = LAPACKE_(ormqr)(LAPACK_COL_MAJOR, 'L', 'N', M, r, k, UA, M, tauA, X, M);
            if (info) { free(X); status = PORT_E_LAPACK; goto done; }
        }
        fl += port_flop_counts('o', M, r, k, 1);
        for (j = 0; j < r; j++)
            for (i = 0; i < M; i++) CU[(size_t)j * ldc + i] = X[(size_t)j * M + i];
        free(X);
    }
    /* __newv: CV = ([S_r V_r^T, 0] Q_B^T)^T (:646-673) */
    {
        const int ldx = r > 0 ? r : 1;
        REAL *X = (REAL *)calloc((size_t)ldx * M, sizeof(REAL));
        for (j = 0; j < k; j++)
            for (i = 0; i < r; i++) X[(size_t)j * ldx + i] = VT[(size_t)j * k + i];
        if (r > 0) {
            info = LAPACKE_(ormqr)(LAPACK_COL_MAJOR, 'R', 'T', r, M, k, VB, M, tauB, X, ldx);
            if (info) { free(X); status = PORT_E_LAPACK; goto done; }
        }
        fl += port_flop_counts('o', r, M, k, 2);
        for (j = 0; j < r; j++)
            for (i = 0; i < M; i++) CV[(size_t)j * ldc + i] = X[(size_t)i * ldx + j];
        free(X);
    }
    *c_inout = r;

done:
    if (flops_update) *flops_update += fl;
    free(UA); free(VB); free(tauA); free(tauB); free(T); free(U); free(VT);
    free(s); free(superb);
    return status;
}

/* ---- HCORE_dsyrk: CD = alpha * AU (AV^T AV) AU^T + CD, strict upper := 0
 * (src/compute/hcore_dsyrk.c:47-189).  As in the reference, beta and uplo
 * are ignored, the row count of AV is LDAU (:57) and every leading dimension
 * of AU/AV is LDAU. */
int PFX(syrk)(int M, int K, REAL alpha, const REAL *AU, int LDAU, const REAL *AV,
              REAL *CD, int LDCD, unsigned long *flops_syrk)
{
    const int N = LDAU;
    REAL *S = (REAL *)calloc((size_t)(K > 0 ? K : 1) * (K > 0 ? K : 1), sizeof(REAL));
    REAL *W = (REAL *)calloc((size_t)M * (K > 0 ? K : 1), sizeof(REAL));
    int i, j;
    if (K > 0) {
        cblas_(gemm)(CblasColMajor, CblasTrans, CblasNoTrans, K, K, N, 1, AV, LDAU, AV,
                     LDAU, 0, S, K);
        cblas_(gemm)(CblasColMajor, CblasNoTrans, CblasNoTrans, M, K, K, 1, AU, LDAU, S, K,
                     0, W, M);
        cblas_(gemm)(CblasColMajor, CblasNoTrans, CblasTrans, M, M, K, alpha, W, M, AU,
                     LDAU, 1, CD, LDCD);
    }
    for (j = 1; j < M; j++)
        for (i = 0; i < j; i++) CD[(size_t)j * LDCD + i] = 0;
    if (flops_syrk)
        *flops_syrk += port_flop_counts('m', K, K, N, 0) + port_flop_counts('m', M, K, K, 0) +
                       port_flop_counts('m', M, M, K, 0);
    free(S); free(W);
    return PORT_OK;
}

/* ---- HCORE_dgemmcd: CD -= Au (Av^T Bv) Bu^T, alpha/beta/LD* ignored, every
 * leading dimension is M (src/compute/hcore_dgemmcd.c:36-106).  The
 * association follows the rank comparison at :72. */
int PFX(gemmcd)(int M, const REAL *Au, const REAL *Av, int Arank, const REAL *Bu,
                const REAL *Bv, int Brank, REAL *CD)
{
    REAL *rr = (REAL *)calloc((size_t)(Arank > 0 ? Arank : 1) * (Brank > 0 ? Brank : 1),
                              sizeof(REAL));
    REAL *mbr = (REAL *)calloc((size_t)M * (Arank > Brank ? (Brank > 0 ? Brank : 1)
                                                          : (Arank > 0 ? Arank : 1)),
                               sizeof(REAL));
    if (Arank > 0 && Brank > 0) {
        cblas_(gemm)(CblasColMajor, CblasTrans, CblasNoTrans, Arank, Brank, M, 1, Av, M, Bv,
                     M, 0, rr, Arank);
        if (Arank > Brank) {
            cblas_(gemm)(CblasColMajor, CblasNoTrans, CblasNoTrans, M, Brank, Arank, 1, Au, M,
                         rr, Arank, 0, mbr, M);
            cblas_(gemm)(CblasColMajor, CblasNoTrans, CblasTrans, M, M, Brank, -1, mbr, M, Bu,
                         M, 1, CD, M);
        } else {
            cblas_(gemm)(CblasColMajor, CblasNoTrans, CblasTrans, Arank, M, Brank, 1, rr,
                         Arank, Bu, M, 0, mbr, Arank);
            cblas_(gemm)(CblasColMajor, CblasNoTrans, CblasNoTrans, M, M, Arank, -1, Au, M,
                         mbr, Arank, 1, CD, M);
        }
    }
    free(rr); free(mbr);
    return PORT_OK;
}
