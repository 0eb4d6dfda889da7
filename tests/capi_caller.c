/*
 * A compiled C caller of the drop-in library: what a HiCMA-style program
 * sees.  It includes the library's public headers, links
 * -lhcore_gb300, defines `use_scratch` as the reference's own test programs
 * do (testing/testing_dgemm.c:23), and calls HCORE_dgemm, HCORE_sgemm,
 * HCORE_dsyrk and HCORE_dgemmcd on inputs read from raw files.
 *
 * Usage: capi_caller DIR
 *   DIR/cases.txt lists one call per line:
 *     dgemm  NAME M a b c alpha beta acc maxrk rk
 *     sgemm  NAME M a b c alpha beta acc maxrk rk
 *     dsyrk  NAME M K alpha
 *     dgemmcd NAME M a b
 *     kat    NAME M ranka rankb rankc acc      (dgemm known-answer gate)
 *   Inputs are DIR/NAME_<field>.bin, column-major, M rows, ld = M (FP32 for
 *   sgemm, FP64 otherwise).  Outputs: DIR/NAME_CUo.bin, NAME_CVo.bin (new
 *   rank columns), NAME_CDo.bin, and one line per call on stdout:
 *     NAME rank=<r> flops=<f> [err=<inf-norm> PASS|FAIL]
 *
 * The kat case mirrors the reference's known-answer program
 * (testing/testing_dgemm.c:250-392): C + A B^T is formed densely from the
 * dense A, B, C it was compressed from, and the inf-norm of its difference to
 * CU CV^T must stay below 10 * acc.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hcore_d.h"
#include "hcore_s.h"

int use_scratch = 0;

static char g_dir[4096];

static void *read_file(const char *name, const char *field, size_t bytes) {
    char path[8192];
    snprintf(path, sizeof path, "%s/%s_%s.bin", g_dir, name, field);
    FILE *f = fopen(path, "rb");
    if (!f) {
        fprintf(stderr, "cannot open %s\n", path);
        exit(2);
    }
    void *p = calloc(bytes ? bytes : 1, 1);
    if (bytes && fread(p, 1, bytes, f) != bytes) {
        fprintf(stderr, "short read %s\n", path);
        exit(2);
    }
    fclose(f);
    return p;
}

static void write_file(const char *name, const char *field, const void *p, size_t bytes) {
    char path[8192];
    snprintf(path, sizeof path, "%s/%s_%s.bin", g_dir, name, field);
    FILE *f = fopen(path, "wb");
    if (!f || (bytes && fwrite(p, 1, bytes, f) != bytes)) {
        fprintf(stderr, "cannot write %s\n", path);
        exit(2);
    }
    fclose(f);
}

/* factors with room for `cols` columns, the first `k` read from the file */
static double *dfactor(const char *name, const char *field, int M, int k, int cols) {
    double *in = (double *)read_file(name, field, sizeof(double) * (size_t)M * k);
    double *out = (double *)calloc((size_t)M * (cols > k ? cols : k) + 1, sizeof(double));
    memcpy(out, in, sizeof(double) * (size_t)M * k);
    free(in);
    return out;
}

static float *sfactor(const char *name, const char *field, int M, int k, int cols) {
    float *in = (float *)read_file(name, field, sizeof(float) * (size_t)M * k);
    float *out = (float *)calloc((size_t)M * (cols > k ? cols : k) + 1, sizeof(float));
    memcpy(out, in, sizeof(float) * (size_t)M * k);
    free(in);
    return out;
}

static void run_dgemm(const char *name, int M, int a, int b, int c, double alpha, double beta,
                      double acc, int maxrk, int rk) {
    double *AU = dfactor(name, "AU", M, a, a), *AV = dfactor(name, "AV", M, a, a);
    double *BU = dfactor(name, "BU", M, b, b), *BV = dfactor(name, "BV", M, b, b);
    double *CU = dfactor(name, "CU", M, c, a + c), *CV = dfactor(name, "CV", M, c, a + c);
    double ra = a, rb = b, rc = c;
    flop_counter fc;
    memset(&fc, 0, sizeof fc);
    HCORE_dgemm(HCORE_NoTrans, HCORE_Trans, M, M, alpha, AU, AV, &ra, M, BU, BV, &rb, M, beta, CU,
                CV, &rc, M, rk, maxrk, acc, NULL, &fc);
    const int r = (int)rc;
    write_file(name, "CUo", CU, sizeof(double) * (size_t)M * r);
    write_file(name, "CVo", CV, sizeof(double) * (size_t)M * r);
    printf("%s rank=%d flops=%lu\n", name, r, (unsigned long)fc.update);
    free(AU), free(AV), free(BU), free(BV), free(CU), free(CV);
}

static void run_sgemm(const char *name, int M, int a, int b, int c, float alpha, float beta,
                      float acc, int maxrk, int rk) {
    float *AU = sfactor(name, "AU", M, a, a), *AV = sfactor(name, "AV", M, a, a);
    float *BU = sfactor(name, "BU", M, b, b), *BV = sfactor(name, "BV", M, b, b);
    float *CU = sfactor(name, "CU", M, c, a + c), *CV = sfactor(name, "CV", M, c, a + c);
    float ra = (float)a, rb = (float)b, rc = (float)c;
    flop_counter fc;
    memset(&fc, 0, sizeof fc);
    HCORE_sgemm(HCORE_NoTrans, HCORE_Trans, M, M, alpha, AU, AV, &ra, M, BU, BV, &rb, M, beta, CU,
                CV, &rc, M, rk, maxrk, acc, NULL, &fc);
    const int r = (int)rc;
    write_file(name, "CUo", CU, sizeof(float) * (size_t)M * r);
    write_file(name, "CVo", CV, sizeof(float) * (size_t)M * r);
    printf("%s rank=%d flops=%lu\n", name, r, (unsigned long)fc.update);
    free(AU), free(AV), free(BU), free(BV), free(CU), free(CV);
}

static void run_dsyrk(const char *name, int M, int K, double alpha) {
    double *AU = dfactor(name, "AU", M, K, K), *AV = dfactor(name, "AV", M, K, K);
    double *CD = dfactor(name, "CD", M, M, M);
    flop_counter fc;
    memset(&fc, 0, sizeof fc);
    HCORE_dsyrk(HCORE_Lower, HCORE_NoTrans, M, K, alpha, AU, M, AV, M, 1.0, CD, M, NULL, &fc);
    write_file(name, "CDo", CD, sizeof(double) * (size_t)M * M);
    printf("%s rank=0 flops=%lu\n", name, (unsigned long)fc.syrk);
    free(AU), free(AV), free(CD);
}

static void run_dgemmcd(const char *name, int M, int a, int b) {
    double *Au = dfactor(name, "Au", M, a, a), *Av = dfactor(name, "Av", M, a, a);
    double *Bu = dfactor(name, "Bu", M, b, b), *Bv = dfactor(name, "Bv", M, b, b);
    double *CD = dfactor(name, "CD", M, M, M);
    flop_counter fc;
    memset(&fc, 0, sizeof fc);
    HCORE_dgemmcd(HCORE_NoTrans, HCORE_Trans, M, -1.0, Au, Av, a, M, Bu, Bv, b, M, 1.0, CD, M,
                  a > b ? a : b, NULL, &fc);
    write_file(name, "CDo", CD, sizeof(double) * (size_t)M * M);
    printf("%s rank=0 flops=0\n", name);
    free(Au), free(Av), free(Bu), free(Bv), free(CD);
}

/* testing_dgemm.c's gate: || (C + A B^T) - CU CV^T ||_inf < 10 acc */
static void run_kat(const char *name, int M, int a, int b, int c, double acc) {
    double *A = dfactor(name, "A", M, M, M), *B = dfactor(name, "B", M, M, M);
    double *Cd = dfactor(name, "C", M, M, M);
    double *AU = dfactor(name, "AU", M, a, a), *AV = dfactor(name, "AV", M, a, a);
    double *BU = dfactor(name, "BU", M, b, b), *BV = dfactor(name, "BV", M, b, b);
    double *CU = dfactor(name, "CU", M, c, M), *CV = dfactor(name, "CV", M, c, M);
    double ra = a, rb = b, rc = c;
    flop_counter fc;
    memset(&fc, 0, sizeof fc);
    HCORE_dgemm(HCORE_NoTrans, HCORE_Trans, M, M, 1.0, AU, AV, &ra, M, BU, BV, &rb, M, 1.0, CU,
                CV, &rc, M, 0, M, acc, NULL, &fc);
    const int r = (int)rc;
    double worst = 0.0;
    for (int i = 0; i < M; ++i) {
        double row = 0.0;
        for (int j = 0; j < M; ++j) {
            double exact = Cd[i + (size_t)j * M];
            for (int l = 0; l < M; ++l) exact += A[i + (size_t)l * M] * B[j + (size_t)l * M];
            double got = 0.0;
            for (int l = 0; l < r; ++l) got += CU[i + (size_t)l * M] * CV[j + (size_t)l * M];
            row += fabs(exact - got);
        }
        if (row > worst) worst = row;
    }
    write_file(name, "CUo", CU, sizeof(double) * (size_t)M * r);
    write_file(name, "CVo", CV, sizeof(double) * (size_t)M * r);
    printf("%s rank=%d flops=%lu err=%.6e %s\n", name, r, (unsigned long)fc.update, worst,
           worst < 10.0 * acc ? "PASS" : "FAIL");
    free(A), free(B), free(Cd), free(AU), free(AV), free(BU), free(BV), free(CU), free(CV);
}

int main(int argc, char **argv) {
    if (argc != 2) {
        fprintf(stderr, "usage: %s DIR\n", argv[0]);
        return 2;
    }
    snprintf(g_dir, sizeof g_dir, "%s", argv[1]);
    char path[8192];
    snprintf(path, sizeof path, "%s/cases.txt", g_dir);
    FILE *f = fopen(path, "r");
    if (!f) {
        fprintf(stderr, "cannot open %s\n", path);
        return 2;
    }
    char kind[32], name[256];
    while (fscanf(f, "%31s %255s", kind, name) == 2) {
        int M, a, b, c, maxrk, rk, K;
        double alpha, beta, acc;
        if (!strcmp(kind, "dgemm") || !strcmp(kind, "sgemm")) {
            if (fscanf(f, "%d %d %d %d %lf %lf %lf %d %d", &M, &a, &b, &c, &alpha, &beta, &acc,
                       &maxrk, &rk) != 9)
                return 3;
            if (kind[0] == 'd')
                run_dgemm(name, M, a, b, c, alpha, beta, acc, maxrk, rk);
            else
                run_sgemm(name, M, a, b, c, (float)alpha, (float)beta, (float)acc, maxrk, rk);
        } else if (!strcmp(kind, "dsyrk")) {
            if (fscanf(f, "%d %d %lf", &M, &K, &alpha) != 3) return 3;
            run_dsyrk(name, M, K, alpha);
        } else if (!strcmp(kind, "dgemmcd")) {
            if (fscanf(f, "%d %d %d", &M, &a, &b) != 3) return 3;
            run_dgemmcd(name, M, a, b);
        } else if (!strcmp(kind, "kat")) {
            if (fscanf(f, "%d %d %d %d %lf", &M, &a, &b, &c, &acc) != 5) return 3;
            run_kat(name, M, a, b, c, acc);
        } else {
            fprintf(stderr, "unknown call %s\n", kind);
            return 3;
        }
        fflush(stdout);
    }
    fclose(f);
    return 0;
}
