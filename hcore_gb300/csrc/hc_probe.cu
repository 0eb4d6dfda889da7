// hcore-gb300 — FP64 issue-rate probes: the roofline denominator of the
// FP64 phases.  The driver's measured peaks cover HBM and bf16 only, so the
// FP64 ceiling is measured here, live, by kernels with a fixed trip count and
// no memory traffic.  Several forms are measured so that the ceiling is not
// an artefact of one instruction form:
//
//   DFMA             fma.rn.f64 on independent accumulators
//   DMMA m8n8k4      mma.sync f64 (the first FP64 MMA shape)
//   DMMA m16n8k4 / m16n8k8 / m16n8k16
//   DMMA m16n8k16, B in one register: the four B operands name the same
//                    register (the compiler is given one variable)
//   DMMA m16n8k16, B equal values in distinct registers: B loaded at run time
//                    from a buffer that holds one value four times
//
// The last two separate a register-operand effect (fewer distinct registers
// read per instruction) from a data-dependent one (equal values).
#include <cuda_runtime.h>

#include "hcore_gb300.h"

namespace hc {

template <int KIND>
struct ProbeShape;
// flops per warp-level instruction
template <> struct ProbeShape<HCORE_PROBE_DFMA> { static constexpr double flops = 2.0 * 32; };
template <> struct ProbeShape<HCORE_PROBE_DMMA_8x8x4> { static constexpr double flops = 2.0 * 8 * 8 * 4; };
template <> struct ProbeShape<HCORE_PROBE_DMMA_16x8x4> { static constexpr double flops = 2.0 * 16 * 8 * 4; };
template <> struct ProbeShape<HCORE_PROBE_DMMA_16x8x8> { static constexpr double flops = 2.0 * 16 * 8 * 8; };
template <> struct ProbeShape<HCORE_PROBE_DMMA_16x8x16> { static constexpr double flops = 2.0 * 16 * 8 * 16; };
template <> struct ProbeShape<HCORE_PROBE_DMMA_16x8x16_B_ONE_REG> { static constexpr double flops = 2.0 * 16 * 8 * 16; };
template <> struct ProbeShape<HCORE_PROBE_DMMA_16x8x16_B_EQUAL> { static constexpr double flops = 2.0 * 16 * 8 * 16; };

// CH independent accumulator chains per thread; `seed` (device memory) holds
// the B values that the run-time-loaded forms read
template <int KIND, int CH>
__global__ void __launch_bounds__(128) fp64_probe_kernel(const double *__restrict__ seed,
                                                         double *out, int iters) {
    double a[8], b[4], c[CH][4];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = 1e-3 * (threadIdx.x + i + 1);
    if (KIND == HCORE_PROBE_DMMA_16x8x16_B_EQUAL) {
#pragma unroll
        for (int i = 0; i < 4; ++i) b[i] = seed[4];   // one value, four loads
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) b[i] = seed[i];   // four distinct values
    }
#pragma unroll
    for (int j = 0; j < CH; ++j)
#pragma unroll
        for (int i = 0; i < 4; ++i) c[j][i] = 0.0;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int j = 0; j < CH; ++j) {
            if (KIND == HCORE_PROBE_DFMA) {
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    asm volatile("fma.rn.f64 %0, %1, %2, %0;" : "+d"(c[j][i]) : "d"(a[i]), "d"(b[i]));
            } else if (KIND == HCORE_PROBE_DMMA_8x8x4) {
                asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, "
                             "{%0,%1};"
                             : "+d"(c[j][0]), "+d"(c[j][1])
                             : "d"(a[j & 7]), "d"(b[j & 3]));
            } else if (KIND == HCORE_PROBE_DMMA_16x8x4) {
                asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                             "{%4,%5}, {%6}, {%0,%1,%2,%3};"
                             : "+d"(c[j][0]), "+d"(c[j][1]), "+d"(c[j][2]), "+d"(c[j][3])
                             : "d"(a[0]), "d"(a[1]), "d"(b[0]));
            } else if (KIND == HCORE_PROBE_DMMA_16x8x8) {
                asm volatile("mma.sync.aligned.m16n8k8.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                             "{%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
                             : "+d"(c[j][0]), "+d"(c[j][1]), "+d"(c[j][2]), "+d"(c[j][3])
                             : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(b[0]), "d"(b[1]));
            } else if (KIND == HCORE_PROBE_DMMA_16x8x16_B_ONE_REG) {
                asm volatile("mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                             "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%12,%12,%12}, {%0,%1,%2,%3};"
                             : "+d"(c[j][0]), "+d"(c[j][1]), "+d"(c[j][2]), "+d"(c[j][3])
                             : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]),
                               "d"(a[6]), "d"(a[7]), "d"(b[0]));
            } else {  // m16n8k16, distinct or run-time-equal B registers
                asm volatile("mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                             "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};"
                             : "+d"(c[j][0]), "+d"(c[j][1]), "+d"(c[j][2]), "+d"(c[j][3])
                             : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]),
                               "d"(a[6]), "d"(a[7]), "d"(b[0]), "d"(b[1]), "d"(b[2]), "d"(b[3]));
            }
        }
    }
    double s = 0;
#pragma unroll
    for (int j = 0; j < CH; ++j) s += c[j][0] + c[j][1] + c[j][2] + c[j][3];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// instructions per thread per iteration of one probe form
template <int KIND>
constexpr int probe_instr_per_chain() { return KIND == HCORE_PROBE_DFMA ? 4 : 1; }

template <int KIND, int CH>
static cudaError_t run_probe(const double *seed, double *out, int blocks, int iters,
                             cudaStream_t s, double *flops) {
    fp64_probe_kernel<KIND, CH><<<blocks, 128, 0, s>>>(seed, out, iters);
    const double warps = (double)blocks * 128 / 32;
    *flops = ProbeShape<KIND>::flops * probe_instr_per_chain<KIND>() * CH * (double)iters * warps;
    return cudaGetLastError();
}

template <int KIND>
static cudaError_t run_kind(int chains, const double *seed, double *out, int blocks, int iters,
                            cudaStream_t s, double *flops) {
    switch (chains) {
        case 2: return run_probe<KIND, 2>(seed, out, blocks, iters, s, flops);
        case 4: return run_probe<KIND, 4>(seed, out, blocks, iters, s, flops);
        case 8: return run_probe<KIND, 8>(seed, out, blocks, iters, s, flops);
        default: return cudaErrorInvalidValue;
    }
}

static cudaError_t dispatch(int kind, int chains, const double *seed, double *out, int blocks,
                            int iters, cudaStream_t s, double *flops) {
    switch (kind) {
        case HCORE_PROBE_DFMA: return run_kind<HCORE_PROBE_DFMA>(chains, seed, out, blocks, iters, s, flops);
        case HCORE_PROBE_DMMA_8x8x4: return run_kind<HCORE_PROBE_DMMA_8x8x4>(chains, seed, out, blocks, iters, s, flops);
        case HCORE_PROBE_DMMA_16x8x4: return run_kind<HCORE_PROBE_DMMA_16x8x4>(chains, seed, out, blocks, iters, s, flops);
        case HCORE_PROBE_DMMA_16x8x8: return run_kind<HCORE_PROBE_DMMA_16x8x8>(chains, seed, out, blocks, iters, s, flops);
        case HCORE_PROBE_DMMA_16x8x16: return run_kind<HCORE_PROBE_DMMA_16x8x16>(chains, seed, out, blocks, iters, s, flops);
        case HCORE_PROBE_DMMA_16x8x16_B_ONE_REG: return run_kind<HCORE_PROBE_DMMA_16x8x16_B_ONE_REG>(chains, seed, out, blocks, iters, s, flops);
        case HCORE_PROBE_DMMA_16x8x16_B_EQUAL: return run_kind<HCORE_PROBE_DMMA_16x8x16_B_EQUAL>(chains, seed, out, blocks, iters, s, flops);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace hc

extern "C" int hcore_gpu_fp64_probe(int kind, int chains, int blocks_per_sm, int iters,
                                    void *stream, double *tflops, double *ms_out) {
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return HCORE_GPU_ECUDA;
    if (blocks_per_sm < 1 || blocks_per_sm > 16 || iters < 1) return HCORE_GPU_EINVAL;
    const int blocks = sms * blocks_per_sm;
    double *buf = nullptr;
    // B seeds: four distinct values, then the value the equal-B form repeats
    const double seed_h[5] = {0.999, 0.9989, 0.9988, 0.9987, 0.9986};
    if (cudaMalloc(&buf, (5 + (size_t)blocks * 128) * sizeof(double)) != cudaSuccess)
        return HCORE_GPU_ENOMEM;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double flops = 0;
    cudaError_t e = cudaMemcpyAsync(buf, seed_h, sizeof seed_h, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    // warm-up launch (module load, clocks up), then the timed one
    if (e == cudaSuccess) e = hc::dispatch(kind, chains, buf, buf + 5, blocks, 64, s, &flops);
    if (e == cudaSuccess) e = cudaEventRecord(e0, s);
    if (e == cudaSuccess) e = hc::dispatch(kind, chains, buf, buf + 5, blocks, iters, s, &flops);
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(buf);
    if (e == cudaErrorInvalidValue) return HCORE_GPU_EINVAL;
    if (e != cudaSuccess) return HCORE_GPU_ECUDA;
    if (tflops) *tflops = ms > 0 ? flops / (ms * 1e-3) / 1e12 : 0.0;
    if (ms_out) *ms_out = ms;
    return HCORE_GPU_OK;
}

extern "C" double hcore_gpu_fp64_peak(void *stream) {
    double t = -1.0;
    if (hcore_gpu_fp64_probe(HCORE_PROBE_DMMA_16x8x16, 4, 8, 4096, stream, &t, nullptr) !=
        HCORE_GPU_OK)
        return -1.0;
    return t;
}
