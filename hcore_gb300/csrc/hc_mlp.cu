// hcore-gb300 — rank predictor: a 6 -> 64 -> 64 -> 1 MLP (ReLU) with FP32
// weights and BF16 activations, trained and evaluated by the kernels below
// (no counterpart in the reference, which sizes nothing ahead of its
// per-tile LAPACK calls).
//
// Parameters (FP32, one array of kMlpParams):
//   W1 [6][64] (in x out)  b1 [64]  W2 [64][64]  b2 [64]  w3 [64]  b3
// Forward for one sample x (6 features):
//   z1 = b1 + x W1, h1 = bf16(relu(z1)), z2 = b2 + h1 W2, h2 = bf16(relu(z2)),
//   y  = b3 + h2 . w3
// Each sum is taken in input order with separately rounded products and
// additions (no FMA contraction), so a CPU restatement with FP32 numpy ops
// in the same order reproduces the forward bit for bit.  Loss: mean over the
// batch of 0.5 (y - t)^2; the backward treats the BF16 rounding as identity
// (straight-through) and accumulates in FP32.  Optimiser: Adam.
//
// Layout of the work: one CTA of 128 threads takes 128 samples, one per
// thread, with the parameters in shared memory (read as broadcasts).  The
// per-sample activations and deltas are staged in shared memory and the
// weight gradients (sums over the CTA's samples) are formed cooperatively,
// then added to the global gradient with one atomic per parameter per CTA.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "hc_host.h"
#include "hc_internal.h"

namespace hc {

constexpr int kIn = HCORE_MLP_INPUTS, kHid = HCORE_MLP_HIDDEN;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kIn * kHid, kOffW2 = kOffB1 + kHid,
              kOffB2 = kOffW2 + kHid * kHid, kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid;
constexpr int kMlpParams = kOffB3 + 1;
static_assert(kMlpParams == HCORE_MLP_PARAMS, "parameter layout");
constexpr int kMlpThreads = 128;   // samples per CTA

__device__ __forceinline__ float bf16_round(float x) {
    return __bfloat162float(__float2bfloat16_rn(x));
}

// forward of one sample; h1/h2 are the BF16-rounded activations, m1/m2 the
// ReLU masks (bit j: z_j > 0)
__device__ __forceinline__ float mlp_forward(const float *P, const float (&x)[kIn],
                                             float (&h1)[kHid], float (&h2)[kHid],
                                             uint64_t &m1, uint64_t &m2) {
    float z[kHid];
#pragma unroll
    for (int j = 0; j < kHid; ++j) z[j] = P[kOffB1 + j];
#pragma unroll
    for (int i = 0; i < kIn; ++i)
#pragma unroll
        for (int j = 0; j < kHid; ++j) z[j] = __fadd_rn(z[j], __fmul_rn(x[i], P[kOffW1 + i * kHid + j]));
    m1 = 0;
#pragma unroll
    for (int j = 0; j < kHid; ++j) {
        if (z[j] > 0.f) m1 |= 1ull << j;
        h1[j] = bf16_round(fmaxf(z[j], 0.f));
    }
#pragma unroll
    for (int j = 0; j < kHid; ++j) z[j] = P[kOffB2 + j];
#pragma unroll
    for (int i = 0; i < kHid; ++i) {   // fully unrolled: h1 stays in registers
        const float hi = h1[i];
#pragma unroll
        for (int j = 0; j < kHid; ++j) z[j] = __fadd_rn(z[j], __fmul_rn(hi, P[kOffW2 + i * kHid + j]));
    }
    m2 = 0;
#pragma unroll
    for (int j = 0; j < kHid; ++j) {
        if (z[j] > 0.f) m2 |= 1ull << j;
        h2[j] = bf16_round(fmaxf(z[j], 0.f));
    }
    float y = P[kOffB3];
#pragma unroll
    for (int j = 0; j < kHid; ++j) y = __fadd_rn(y, __fmul_rn(h2[j], P[kOffW3 + j]));
    return y;
}

__device__ __forceinline__ void load_params(float *sP, const float *P) {
    for (int e = threadIdx.x; e < kMlpParams; e += blockDim.x) sP[e] = P[e];
}

// sample s of the batch -> row of X: (pa * (b0 + s) + pc) mod n, a bijection
// of 0..n-1 when gcd(pa, n) = 1 (the training loop's per-epoch shuffle)
__device__ __forceinline__ long long mlp_row(long long g, long long pa, long long pc, long long n) {
    return (long long)(((unsigned long long)pa * (unsigned long long)g + (unsigned long long)pc) %
                       (unsigned long long)n);
}

// rows padded to an odd number of 32-bit words: a thread writing its own
// row and a warp reading one column both stay free of bank conflicts
struct MlpSmem {
    float P[kMlpParams + 3];
    __nv_bfloat16 H1[kMlpThreads][kHid + 2];
    __nv_bfloat16 H2[kMlpThreads][kHid + 2];
    float DZ1[kMlpThreads][kHid + 1];
    float DZ2[kMlpThreads][kHid + 1];
    float X[kMlpThreads][kIn + 1];
    float DY[kMlpThreads];
    float red[kMlpThreads / 32];
};

// One minibatch: samples b0 .. b0+cnt-1 (shuffled rows), gradient of
// inv_cnt * sum 0.5 (y - t)^2 added to G; loss_scale * sum 0.5 (y - t)^2 added
// to *loss.
__global__ void __launch_bounds__(kMlpThreads) mlp_fwd_bwd_kernel(
    const float *__restrict__ Pg, float *__restrict__ G, const float *__restrict__ X,
    const float *__restrict__ Y, long long n, long long b0, int cnt, long long pa, long long pc,
    float inv_cnt, float *__restrict__ loss, float loss_scale) {
    extern __shared__ __align__(16) unsigned char mlp_smem_raw[];
    MlpSmem &S = *reinterpret_cast<MlpSmem *>(mlp_smem_raw);
    const int tid = threadIdx.x;
    load_params(S.P, Pg);
    __syncthreads();
    const int s = blockIdx.x * kMlpThreads + tid;
    const bool valid = s < cnt;
    float x[kIn], t = 0.f;
    if (valid) {
        const long long row = mlp_row(b0 + s, pa, pc, n);
#pragma unroll
        for (int i = 0; i < kIn; ++i) x[i] = X[row * kIn + i];
        t = Y[row];
    } else {
#pragma unroll
        for (int i = 0; i < kIn; ++i) x[i] = 0.f;
    }
    float h1[kHid], h2[kHid];
    uint64_t m1, m2;
    const float y = mlp_forward(S.P, x, h1, h2, m1, m2);
    const float e = valid ? y - t : 0.f;
    const float dy = e * inv_cnt;
    // stage this sample's activations and deltas
#pragma unroll
    for (int i = 0; i < kIn; ++i) S.X[tid][i] = x[i];
    S.DY[tid] = dy;
    float dz2[kHid];
#pragma unroll
    for (int j = 0; j < kHid; ++j) {
        S.H1[tid][j] = __float2bfloat16_rn(h1[j]);   // exact: h1 is BF16 already
        S.H2[tid][j] = __float2bfloat16_rn(h2[j]);
        dz2[j] = ((m2 >> j) & 1) ? dy * S.P[kOffW3 + j] : 0.f;
        S.DZ2[tid][j] = dz2[j];
    }
    // dz1 = (W2 dz2) masked by relu'(z1)
#pragma unroll 4
    for (int i = 0; i < kHid; ++i) {
        float a = 0.f;
#pragma unroll
        for (int j = 0; j < kHid; ++j) a += S.P[kOffW2 + i * kHid + j] * dz2[j];
        S.DZ1[tid][i] = ((m1 >> i) & 1) ? a : 0.f;
    }
    // loss of the CTA
    float l = 0.5f * e * e;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((tid & 31) == 0) S.red[tid >> 5] = l;
    __syncthreads();
    const int ns = min(kMlpThreads, cnt - blockIdx.x * kMlpThreads);
    if (tid == 0) {
        float tot = 0.f;
        for (int w = 0; w < kMlpThreads / 32; ++w) tot += S.red[w];
        atomicAdd(loss, tot * loss_scale);
    }
    // dW2[i][j] = sum_s h1[s][i] dz2[s][j]: thread -> column j, rows i = i0, i0+2, ...
    {
        const int j = tid & (kHid - 1), i0 = tid >> 6;
        float acc[kHid / 2];
#pragma unroll
        for (int q = 0; q < kHid / 2; ++q) acc[q] = 0.f;
        for (int ss = 0; ss < ns; ++ss) {
            const float d = S.DZ2[ss][j];
#pragma unroll
            for (int q = 0; q < kHid / 2; ++q) acc[q] += __bfloat162float(S.H1[ss][i0 + 2 * q]) * d;
        }
#pragma unroll
        for (int q = 0; q < kHid / 2; ++q) atomicAdd(&G[kOffW2 + (i0 + 2 * q) * kHid + j], acc[q]);
    }
    // db2, dw3 (threads 0..63), db1 (64..127)
    if (tid < kHid) {
        float a = 0.f, b = 0.f;
        for (int ss = 0; ss < ns; ++ss) {
            a += S.DZ2[ss][tid];
            b += S.DY[ss] * __bfloat162float(S.H2[ss][tid]);
        }
        atomicAdd(&G[kOffB2 + tid], a);
        atomicAdd(&G[kOffW3 + tid], b);
    } else {
        const int j = tid - kHid;
        float a = 0.f;
        for (int ss = 0; ss < ns; ++ss) a += S.DZ1[ss][j];
        atomicAdd(&G[kOffB1 + j], a);
    }
    // dW1[i][j] = sum_s x[s][i] dz1[s][j] (384 entries, 3 per thread)
    for (int e2 = tid; e2 < kIn * kHid; e2 += kMlpThreads) {
        const int i = e2 / kHid, j = e2 % kHid;
        float a = 0.f;
        for (int ss = 0; ss < ns; ++ss) a += S.X[ss][i] * S.DZ1[ss][j];
        atomicAdd(&G[kOffW1 + e2], a);
    }
    if (tid == 0) {
        float a = 0.f;
        for (int ss = 0; ss < ns; ++ss) a += S.DY[ss];
        atomicAdd(&G[kOffB3], a);
    }
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8); c1 = 1/(1 - beta1^t),
// c2 = 1/(1 - beta2^t).  The gradient is cleared for the next step.
__global__ void mlp_adam_kernel(float *__restrict__ P, float *__restrict__ G,
                                float *__restrict__ Mo, float *__restrict__ Vo, float lr, float c1,
                                float c2) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kMlpParams) return;
    const float g = G[e];
    const float m = 0.9f * Mo[e] + 0.1f * g;
    const float v = 0.999f * Vo[e] + 0.001f * g * g;
    Mo[e] = m;
    Vo[e] = v;
    P[e] -= lr * (m * c1) / (sqrtf(v * c2) + 1e-8f);
    G[e] = 0.f;
}

__global__ void __launch_bounds__(kMlpThreads) mlp_predict_kernel(const float *__restrict__ Pg,
                                                                  const float *__restrict__ X,
                                                                  long long n, float *__restrict__ out) {
    __shared__ float sP[kMlpParams + 3];
    load_params(sP, Pg);
    __syncthreads();
    const long long s = (long long)blockIdx.x * kMlpThreads + threadIdx.x;
    if (s >= n) return;
    float x[kIn], h1[kHid], h2[kHid];
    uint64_t m1, m2;
#pragma unroll
    for (int i = 0; i < kIn; ++i) x[i] = X[s * kIn + i];
    out[s] = mlp_forward(sP, x, h1, h2, m1, m2);
}

}  // namespace hc

using namespace hc;

struct hcore_gpu_mlp_s {
    float *d_p = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr, *d_loss = nullptr;
    int d_loss_len = 0;
    long long step = 0;
};

namespace {

uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

float uniform_pm(uint64_t &s, float bound) {   // U(-bound, bound)
    const double u = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
    return (float)((2.0 * u - 1.0) * bound);
}

cudaError_t mlp_smem_attr() {
    return cudaFuncSetAttribute(mlp_fwd_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sizeof(MlpSmem));
}

int mlp_fail(const char *what, cudaError_t e) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return HCORE_GPU_ECUDA;
}

cudaError_t launch_fwd_bwd(hcore_gpu_mlp m, const float *X, const float *Y, long long n,
                           long long b0, int cnt, long long pa, long long pc, float *loss,
                           float loss_scale, cudaStream_t s) {
    const int grid = (cnt + kMlpThreads - 1) / kMlpThreads;
    mlp_fwd_bwd_kernel<<<grid, kMlpThreads, sizeof(MlpSmem), s>>>(
        m->d_p, m->d_g, X, Y, n, b0, cnt, pa, pc, 1.0f / (float)cnt, loss, loss_scale);
    return cudaGetLastError();
}

}  // namespace

extern "C" int hcore_gpu_mlp_create(hcore_gpu_mlp *out, unsigned long long seed) {
    if (!out) {
        set_error("hcore_gpu_mlp_create: null output");
        return HCORE_GPU_EINVAL;
    }
    *out = nullptr;
    auto *m = new hcore_gpu_mlp_s;
    cudaError_t e = cudaMalloc(&m->d_p, 4 * sizeof(float) * kMlpParams);
    if (e != cudaSuccess) {
        delete m;
        set_error("hcore_gpu_mlp_create: cudaMalloc: %s", cudaGetErrorString(e));
        return HCORE_GPU_ENOMEM;
    }
    m->d_g = m->d_p + kMlpParams;
    m->d_m = m->d_g + kMlpParams;
    m->d_v = m->d_m + kMlpParams;
    // He-uniform weights (bound sqrt(6 / fan_in)), zero biases
    std::vector<float> p(kMlpParams, 0.f);
    uint64_t st = seed;
    for (int i = 0; i < kIn * kHid; ++i) p[kOffW1 + i] = uniform_pm(st, std::sqrt(6.f / kIn));
    for (int i = 0; i < kHid * kHid; ++i) p[kOffW2 + i] = uniform_pm(st, std::sqrt(6.f / kHid));
    for (int i = 0; i < kHid; ++i) p[kOffW3 + i] = uniform_pm(st, std::sqrt(6.f / kHid));
    e = cudaMemcpy(m->d_p, p.data(), sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(m->d_g, 0, 3 * sizeof(float) * kMlpParams);
    if (e == cudaSuccess) e = mlp_smem_attr();
    if (e != cudaSuccess) {
        cudaFree(m->d_p);
        delete m;
        return mlp_fail("hcore_gpu_mlp_create", e);
    }
    *out = m;
    return HCORE_GPU_OK;
}

extern "C" int hcore_gpu_mlp_params(hcore_gpu_mlp m, float *host, int set) {
    if (!m || !host) {
        set_error("hcore_gpu_mlp_params: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    cudaError_t e;
    if (set) {
        e = cudaMemcpy(m->d_p, host, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemset(m->d_g, 0, 3 * sizeof(float) * kMlpParams);
        m->step = 0;
    } else {
        e = cudaMemcpy(host, m->d_p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost);
    }
    return e == cudaSuccess ? HCORE_GPU_OK : mlp_fail("hcore_gpu_mlp_params", e);
}

static int ensure_loss(hcore_gpu_mlp m, int len) {
    if (m->d_loss_len >= len) return HCORE_GPU_OK;
    if (m->d_loss) cudaFree(m->d_loss);
    m->d_loss = nullptr;
    m->d_loss_len = 0;
    cudaError_t e = cudaMalloc(&m->d_loss, sizeof(float) * len);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_mlp: cudaMalloc: %s", cudaGetErrorString(e));
        return HCORE_GPU_ENOMEM;
    }
    m->d_loss_len = len;
    return HCORE_GPU_OK;
}

extern "C" int hcore_gpu_mlp_gradient(hcore_gpu_mlp m, const float *x, const float *y, int n,
                                      float *grad, float *loss, void *stream) {
    if (!m || !x || !y || n <= 0 || !grad) {
        set_error("hcore_gpu_mlp_gradient: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    if (int rc = ensure_loss(m, 1)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(m->d_g, 0, sizeof(float) * kMlpParams, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->d_loss, 0, sizeof(float), s);
    if (e == cudaSuccess) e = launch_fwd_bwd(m, x, y, n, 0, n, 1, 0, m->d_loss, 1.0f / n, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(grad, m->d_g, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, s);
    float l = 0.f;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->d_g, 0, sizeof(float) * kMlpParams, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return mlp_fail("hcore_gpu_mlp_gradient", e);
    if (loss) *loss = l;
    return HCORE_GPU_OK;
}

extern "C" int hcore_gpu_mlp_train(hcore_gpu_mlp m, const float *x, const float *y, int n,
                                   int epochs, int batch, float lr, unsigned long long seed,
                                   float *epoch_loss, void *stream) {
    if (!m || !x || !y || n <= 0 || epochs <= 0 || batch <= 0 || !(lr > 0.f)) {
        set_error("hcore_gpu_mlp_train: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    if (int rc = ensure_loss(m, epochs)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(m->d_loss, 0, sizeof(float) * epochs, s);
    uint64_t st = seed;
    for (int ep = 0; ep < epochs && e == cudaSuccess; ++ep) {
        // per-epoch shuffle: row = (pa * i + pc) mod n with gcd(pa, n) = 1
        long long pa = 1, pc = 0;
        if (n > 1) {
            do {
                pa = 1 + (long long)(splitmix64(st) % (uint64_t)(n - 1));
            } while (std::gcd(pa, (long long)n) != 1);
            pc = (long long)(splitmix64(st) % (uint64_t)n);
        }
        for (long long b0 = 0; b0 < n && e == cudaSuccess; b0 += batch) {
            const int cnt = (int)std::min<long long>(batch, n - b0);
            e = launch_fwd_bwd(m, x, y, n, b0, cnt, pa, pc, m->d_loss + ep, 1.0f / n, s);
            if (e != cudaSuccess) break;
            ++m->step;
            const double c1 = 1.0 / (1.0 - std::pow(0.9, (double)m->step));
            const double c2 = 1.0 / (1.0 - std::pow(0.999, (double)m->step));
            mlp_adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, s>>>(m->d_p, m->d_g, m->d_m, m->d_v,
                                                                   lr, (float)c1, (float)c2);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess && epoch_loss)
        e = cudaMemcpyAsync(epoch_loss, m->d_loss, sizeof(float) * epochs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? HCORE_GPU_OK : mlp_fail("hcore_gpu_mlp_train", e);
}

extern "C" int hcore_gpu_mlp_predict(hcore_gpu_mlp m, const float *x, int n, float *out,
                                     void *stream) {
    if (!m || n < 0 || (n > 0 && (!x || !out))) {
        set_error("hcore_gpu_mlp_predict: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    if (n == 0) return HCORE_GPU_OK;
    mlp_predict_kernel<<<(n + kMlpThreads - 1) / kMlpThreads, kMlpThreads, 0,
                         (cudaStream_t)stream>>>(m->d_p, x, n, out);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HCORE_GPU_OK : mlp_fail("hcore_gpu_mlp_predict", e);
}

extern "C" int hcore_gpu_mlp_destroy(hcore_gpu_mlp m) {
    if (!m) return HCORE_GPU_OK;
    cudaFree(m->d_p);
    if (m->d_loss) cudaFree(m->d_loss);
    delete m;
    return HCORE_GPU_OK;
}
