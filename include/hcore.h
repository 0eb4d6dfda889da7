/*
 * hcore-gb300 — drop-in replacement of HCORE's tile low-rank kernels on one
 * GB300 GPU.  Common enums, replacing the reference's src/include/hcore.h.
 *
 * The enum values equal the CBLAS ones, as in the reference
 * (src/include/hcore.h:30-44), because callers pass CblasNoTrans etc.
 * straight through (testing/testing_dgemm.c:329-330).  Unlike the reference
 * this header pulls in no BLAS/LAPACK header: the GPU library needs none.
 */
#ifndef HCORE_GB300_HCORE_H
#define HCORE_GB300_HCORE_H

#ifndef hcore_min
#define hcore_min(a, b) ((a) < (b) ? (a) : (b))
#endif
#ifndef hcore_max
#define hcore_max(a, b) ((a) < (b) ? (b) : (a))
#endif

#define HCORE_NoTrans 111
#define HCORE_Trans 112
#define HCORE_ConjTrans 113

#define HCORE_Upper 121
#define HCORE_Lower 122
#define HCORE_UpperLower 123

#define HCORE_NonUnit 131
#define HCORE_Unit 132

#define HCORE_Left 141
#define HCORE_Right 142

typedef int HCORE_enum;
#endif
