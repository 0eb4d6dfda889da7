// hcore-gb300 internal definitions of the native complex recompression
// (hc_zkernels.cu) shared with its host side (hc_dropin.cu).
#pragma once
#include <cuda_runtime.h>

#include "hc_internal.h"

namespace hc {

// a double-precision complex number, real part first (the layout of C's
// double _Complex and of hcore_dcomplex)
struct zd {
    double re, im;
};

// Per-update descriptor of the complex phases (device resident).  Pointers
// are device-accessible; offsets are in complex elements.
struct ZDesc {
    const zd *AU, *AV, *BU, *BV, *CU, *CV;
    zd *CUo, *CVo;
    long long ws;
    zd alpha, beta;
    double acc;
    int ldau, ldav, ldbu, ldbv, ldcu, ldcv, ldco;   // leading dimension of each factor
    int M, a, b, c, k;
    int rk;          // fixed output rank (0: by acc)
    int max_rank;    // largest accepted new rank (maxrk)
    int idx;
    int status0;     // non-zero: rejected on the host, skip
};

// Workspace of one update (complex elements, each region rounded up to 16):
//   UA M*k | VB M*k | tauA k | tauB k | sig k | F a*b | Y k*k (the SVD's QR
//   reflectors) | Uo k*k (U_r) | Vo k*k (conj(W_r S_r)) | W k*k (the SVD's
//   V_J when it does not stay in shared memory)
struct ZLayout {
    long long UA, VB, tauA, tauB, sig, F, Y, Uo, Vo, W, total;
};
__host__ __device__ inline long long zalign16(long long x) { return (x + 15) & ~15LL; }
__host__ __device__ inline ZLayout zlayout(int M, int a, int b, int k) {
    ZLayout L;
    long long o = 0;
    L.UA = o; o = zalign16(o + (long long)M * k);
    L.VB = o; o = zalign16(o + (long long)M * k);
    L.tauA = o; o = zalign16(o + k);
    L.tauB = o; o = zalign16(o + k);
    L.sig = o; o = zalign16(o + k);
    L.F = o; o = zalign16(o + (long long)a * b);
    L.Y = o; o = zalign16(o + (long long)k * k);
    L.Uo = o; o = zalign16(o + (long long)k * k);
    L.Vo = o; o = zalign16(o + (long long)k * k);
    L.W = o; o = zalign16(o + (long long)k * k);
    L.total = o;
    return L;
}

// the complex SVD kernel's shared memory for order K: two K x (K|1) complex
// matrices, complex scales and reflector taus, two double and two int arrays
__host__ __device__ inline int zsvd_ld(int K) { return K | 1; }
__host__ __device__ inline size_t zsvd_smem_bytes(int K) {
    return (size_t)2 * K * zsvd_ld(K) * sizeof(zd) + (size_t)2 * (K + 1) * sizeof(zd) +
           (size_t)2 * (K + 1) * sizeof(double) + (size_t)2 * (K + 1) * sizeof(int) + 64;
}
// the same with V_J in the workspace: one matrix in shared memory
__host__ __device__ inline size_t zsvd_smem_bytes_half(int K) {
    return zsvd_smem_bytes(K) - (size_t)K * zsvd_ld(K) * sizeof(zd);
}
constexpr int kZApplyChunk = 4;   // reflectors staged per pass of the complex rebuild

// largest rank sum k = a + c the complex kernels take on this device (both
// Jacobi matrices in shared memory); 0 if the device cannot be queried
int zsvd_kmax();
// the four complex phases over n descriptors (M <= 1024, k <= zsvd_kmax())
cudaError_t launch_zrecompress(const ZDesc *d_desc, int n, zd *ws, int *d_rank, int *d_status,
                               int maxM, int maxK, cudaStream_t s);

}  // namespace hc
