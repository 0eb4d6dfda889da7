// hcore-gb300 — one low-rank update that allocates no memory.
//
// Some callers cannot call cudaMalloc.  A worker thread of a task runtime
// (StarPU, PaRSEC) that runs tile updates next to other workers' streams
// must not allocate: cudaMalloc and cudaFree may synchronise the whole
// device and stall every other worker.  A runtime that reserved all of the
// device memory it may use up front (its own pool allocator) cannot let a
// library take more.  For such callers hcore_gpu_dgemm_noalloc runs the same
// four phases as the batched plans with all of its workspace in one
// file-scope device array of fixed size.
//
// The array is reserved on every GPU that loads the library, until the
// process exits.  Host code must not hand the array's name to a kernel (in
// host code it is only a stand-in for the symbol): the device address comes
// from cudaGetSymbolAddress, once per device, on the first call made with
// that device current; the same set-up also sets the SVD kernel's shared
// memory attributes.  That first call should therefore come before any
// stream capture.  Every call uses the same array, so calls that may overlap
// on the GPU (different streams, or different host threads) race on it and
// must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "hc_host.h"

namespace hc {

// workspace capacity in doubles: M = 1024 rows with a + c <= 128 and
// a*b <= 128*128 fit (ws_layout(1024, 128, 128, 128, no storage limit) is
// 344448 doubles)
constexpr long long kNoAllocWsElems = 393216;                // 3 MiB
constexpr size_t kNoAllocDescOff = kNoAllocWsElems * sizeof(double);
constexpr size_t kNoAllocRankOff = kNoAllocDescOff + 512;   // rank, status
constexpr size_t kNoAllocBytes = kNoAllocRankOff + 256;
static_assert(sizeof(Desc) <= 512, "descriptor slot too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// writes the descriptor (passed by value) into its slot and clears the rank
// and status that the SVD phase fills in
__global__ void noalloc_setup_kernel(Desc d) {
    if (threadIdx.x == 0) {
        *reinterpret_cast<Desc *>(g_noalloc_scratch + kNoAllocDescOff) = d;
        int *rs = reinterpret_cast<int *>(g_noalloc_scratch + kNoAllocRankOff);
        rs[0] = 0;
        rs[1] = 0;
    }
}

constexpr int kNoAllocMaxDevices = 64;
struct NoAllocDevice {
    unsigned char *addr = nullptr;  // device address of g_noalloc_scratch
    int svd_smem_kmax = 0;          // SVD shared-memory limits on this device
    int svd_half_kmax = 0;
};
static std::mutex g_noalloc_mu;
static NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];

// once per device, with that device current: the scratch array's device
// address and the SVD kernel's shared-memory attributes (neither changes
// afterwards, so later calls make no set-up call at all)
static cudaError_t noalloc_device(NoAllocDevice *out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if (!d.addr) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        int kmax = 0, khalf = 0;
        e = configure_recompress<double>(kMaxK, &kmax, &khalf);
        if (e != cudaSuccess) return e;
        d.svd_smem_kmax = kmax;
        d.svd_half_kmax = khalf;
        d.addr = static_cast<unsigned char *>(p);
    }
    *out = d;
    return cudaSuccess;
}

}  // namespace hc

using namespace hc;

extern "C" int hcore_gpu_dgemm_noalloc(int M, double alpha, const double *AU, const double *AV,
                                       int a, int lda, const double *BU, const double *BV, int b,
                                       int ldb, double beta, double *CU, double *CV, int c,
                                       int ldc, int rk, int maxrk, double acc, int *new_rank,
                                       int *status, void *stream) {
    hcore_lr_task t{};
    t.M = M;
    t.a = a;
    t.b = b;
    t.c = c;
    t.rk = rk;
    t.maxrk = maxrk;
    t.ld_newv = maxrk;  // HCORE_dgemm's rule (hcore_dgemm.c:851, :924)
    t.alpha = alpha;
    t.beta = beta;
    t.acc = acc;
    t.AU = AU;
    t.AV = AV;
    t.lda = lda;
    t.BU = BU;
    t.BV = BV;
    t.ldb = ldb;
    t.CU = CU;
    t.CV = CV;
    t.ldc = ldc;
    t.CUo = CU;
    t.CVo = CV;
    t.ldco = ldc;
    Desc d;
    int k = 0;
    const int st0 = fill_desc(t, 0, true, d, k);
    if (st0) {
        if (status) *status = st0;
        set_error("hcore_gpu_dgemm_noalloc: task rejected (status %d)", st0);
        return HCORE_GPU_ETASK;
    }
    const long long need = ws_layout(d).total;
    if (need > kNoAllocWsElems) {
        set_error("hcore_gpu_dgemm_noalloc: M=%d, a+c=%d, a*b=%d needs %lld doubles of "
                  "workspace; the fixed scratch holds %lld (e.g. M=1024 with a+c <= 128)",
                  M, k, a * b, need, kNoAllocWsElems);
        return HCORE_GPU_EINVAL;
    }
    // an error left pending by the caller's own earlier work stays the
    // caller's: report it as such and leave it pending
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        set_error("hcore_gpu_dgemm_noalloc: an earlier CUDA error is pending (%s); nothing "
                  "was launched", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    NoAllocDevice nd;
    e = noalloc_device(&nd);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_dgemm_noalloc: device set-up (cudaGetSymbolAddress, kernel "
                  "attributes) failed: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    unsigned char *base = nd.addr;
    d.ws = 0;
    d.idx = 0;
    d.status0 = 0;
    cudaStream_t s = (cudaStream_t)stream;
    LaunchShape shape;
    shape.maxM = M;
    shape.maxK = k;
    shape.nbuckets = 1;
    shape.buckets[0] = Bucket{0, 1, k};
    shape.svd_smem_kmax = nd.svd_smem_kmax;
    shape.svd_half_kmax = nd.svd_half_kmax;
    noalloc_setup_kernel<<<1, 32, 0, s>>>(d);
    e = cudaGetLastError();
    int *rs = reinterpret_cast<int *>(base + kNoAllocRankOff);
    if (e == cudaSuccess)
        e = launch_recompress<double>(reinterpret_cast<const Desc *>(base + kNoAllocDescOff), 1,
                                      reinterpret_cast<double *>(base), rs, rs + 1, nullptr, shape,
                                      s, kPhaseAll);
    int out[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, rs, sizeof out, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_dgemm_noalloc: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    if (status) *status = out[1];
    if (out[1] != HCORE_GPU_S_OK) {
        set_error("hcore_gpu_dgemm_noalloc: task failed on the GPU (status %d)", out[1]);
        return HCORE_GPU_ETASK;
    }
    if (new_rank) *new_rank = out[0];
    return HCORE_GPU_OK;
}
