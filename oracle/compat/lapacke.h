/*
 * Oracle-only compatibility header (test infrastructure, never shipped).
 *
 * Maps the LAPACKE and Fortran-LAPACK names used by the reference HCORE
 * sources and tests to SciPy's bundled OpenBLAS ("scipy_" prefix, LP64).
 * The tests call MKL-style dlange()/dlamch() helpers; those are mapped to the
 * Fortran entry points.
 */
#ifndef ORACLE_COMPAT_LAPACKE_H
#define ORACLE_COMPAT_LAPACKE_H
#define LAPACK_COL_MAJOR 102

#define ORACLE_LE(name) scipy_LAPACKE_##name
#define LAPACKE_dgeqrf      ORACLE_LE(dgeqrf)
#define LAPACKE_sgeqrf      ORACLE_LE(sgeqrf)
#define LAPACKE_dgesvd      ORACLE_LE(dgesvd)
#define LAPACKE_sgesvd      ORACLE_LE(sgesvd)
#define LAPACKE_dgesvd_work ORACLE_LE(dgesvd_work)
#define LAPACKE_sgesvd_work ORACLE_LE(sgesvd_work)
#define LAPACKE_dormqr      ORACLE_LE(dormqr)
#define LAPACKE_sormqr      ORACLE_LE(sormqr)
#define LAPACKE_dorgqr      ORACLE_LE(dorgqr)
#define LAPACKE_dlacpy      ORACLE_LE(dlacpy)
#define LAPACKE_slacpy      ORACLE_LE(slacpy)
#define LAPACKE_dge_trans   ORACLE_LE(dge_trans)
#define LAPACKE_sge_trans   ORACLE_LE(sge_trans)
#define LAPACKE_dlatms      ORACLE_LE(dlatms)
#define LAPACKE_slatms      ORACLE_LE(slatms)
#define LAPACKE_dpotrf      ORACLE_LE(dpotrf)
#define LAPACKE_dpotrf_work ORACLE_LE(dpotrf_work)
#define dlacpy_ scipy_dlacpy_
#define slacpy_ scipy_slacpy_
#define dlaset_ scipy_dlaset_
#define slaset_ scipy_slaset_
#define dlange(a, b, c, d, e, f) scipy_dlange_(a, b, c, d, e, f)
#define slange(a, b, c, d, e, f) scipy_slange_(a, b, c, d, e, f)
#define dlamch(a) scipy_dlamch_(a)
#define slamch(a) scipy_slamch_(a)

int LAPACKE_dgeqrf(int, int, int, double *, int, double *);
int LAPACKE_sgeqrf(int, int, int, float *, int, float *);
int LAPACKE_dgesvd(int, char, char, int, int, double *, int, double *, double *, int,
                   double *, int, double *);
int LAPACKE_sgesvd(int, char, char, int, int, float *, int, float *, float *, int,
                   float *, int, float *);
int LAPACKE_dgesvd_work(int, char, char, int, int, double *, int, double *, double *,
                        int, double *, int, double *, int);
int LAPACKE_sgesvd_work(int, char, char, int, int, float *, int, float *, float *,
                        int, float *, int, float *, int);
int LAPACKE_dormqr(int, char, char, int, int, int, const double *, int, const double *,
                   double *, int);
int LAPACKE_sormqr(int, char, char, int, int, int, const float *, int, const float *,
                   float *, int);
int LAPACKE_dorgqr(int, int, int, int, double *, int, const double *);
int LAPACKE_dlacpy(int, char, int, int, const double *, int, double *, int);
int LAPACKE_slacpy(int, char, int, int, const float *, int, float *, int);
void LAPACKE_dge_trans(int, int, int, const double *, int, double *, int);
void LAPACKE_sge_trans(int, int, int, const float *, int, float *, int);
int LAPACKE_dlatms(int, int, int, char, int *, char, double *, int, double, double,
                   int, int, char, double *, int);
int LAPACKE_slatms(int, int, int, char, int *, char, float *, int, float, float,
                   int, int, char, float *, int);
int LAPACKE_dpotrf(int, char, int, double *, int);
int LAPACKE_dpotrf_work(int, char, int, double *, int);
void scipy_dlacpy_(const char *, const int *, const int *, const double *, const int *,
                   double *, const int *);
void scipy_slacpy_(const char *, const int *, const int *, const float *, const int *,
                   float *, const int *);
void scipy_dlaset_(const char *, const int *, const int *, const double *,
                   const double *, double *, const int *);
void scipy_slaset_(const char *, const int *, const int *, const float *,
                   const float *, float *, const int *);
double scipy_dlange_(const char *, const int *, const int *, const double *,
                     const int *, double *);
float scipy_slange_(const char *, const int *, const int *, const float *,
                    const int *, float *);
double scipy_dlamch_(const char *);
float scipy_slamch_(const char *);

/* complex (hcore_zgemm.c) */
#define LAPACKE_zgeqrf    ORACLE_LE(zgeqrf)
#define LAPACKE_zgesvd    ORACLE_LE(zgesvd)
#define LAPACKE_zunmqr    ORACLE_LE(zunmqr)
#define LAPACKE_zlacpy    ORACLE_LE(zlacpy)
#define LAPACKE_zge_trans ORACLE_LE(zge_trans)
#define zlacpy_ scipy_zlacpy_
#define zlaset_ scipy_zlaset_
int LAPACKE_zgeqrf(int, int, int, double _Complex *, int, double _Complex *);
int LAPACKE_zgesvd(int, char, char, int, int, double _Complex *, int, double *,
                   double _Complex *, int, double _Complex *, int, double *);
int LAPACKE_zunmqr(int, char, char, int, int, int, const double _Complex *, int,
                   const double _Complex *, double _Complex *, int);
int LAPACKE_zlacpy(int, char, int, int, const double _Complex *, int, double _Complex *, int);
void LAPACKE_zge_trans(int, int, int, const double _Complex *, int, double _Complex *, int);
void scipy_zlacpy_(const char *, const int *, const int *, const double _Complex *,
                   const int *, double _Complex *, const int *);
void scipy_zlaset_(const char *, const int *, const int *, const double _Complex *,
                   const double _Complex *, double _Complex *, const int *);
#endif
