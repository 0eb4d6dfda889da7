// hcore-gb300 — one low-rank update that allocates no memory.
//
// Some callers cannot call cudaMalloc: a task runtime worker that must not
// stall the other streams of the device (cudaMalloc/cudaFree synchronise
// implicitly), code that runs while another stream of the process is being
// captured in global mode (where allocation calls are refused), or a caller
// held to a fixed device-memory budget that it reserved up front.  For them,
// hcore_gpu_dgemm_noalloc runs the same four phases as the batched plans
// with all of its workspace in one file-scope device array of fixed size.
//
// The array is reserved on every GPU that loads the library, until the
// process exits.  Host code must not hand the array's name to a kernel (in
// host code it is only a stand-in for the symbol): the device address comes
// from cudaGetSymbolAddress, once per device, on the first call made with
// that device current.  That first call should therefore come before any
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
static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_addr[kNoAllocMaxDevices];

// device address of the scratch array on the current device (set-up once)
static cudaError_t noalloc_scratch(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_noalloc_addr[dev];
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
    unsigned char *base = nullptr;
    cudaError_t e = noalloc_scratch(&base);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_dgemm_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    d.ws = 0;
    d.idx = 0;
    d.status0 = 0;
    cudaStream_t s = (cudaStream_t)stream;
    LaunchShape shape;
    shape.maxM = M;
    shape.maxK = k;
    shape.nbuckets = 1;
    shape.buckets[0] = Bucket{0, 1, k};
    e = configure_recompress<double>(k, &shape.svd_smem_kmax, &shape.svd_half_kmax);
    if (e == cudaSuccess) {
        noalloc_setup_kernel<<<1, 32, 0, s>>>(d);
        e = cudaGetLastError();
    }
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
